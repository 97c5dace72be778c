// TEST INFRASTRUCTURE ONLY — the reference's own GPU matvec as a checker
// and a same-GPU baseline.
//
// Compiles the reference's Hubbard_mv_<double> kernel
// (MBL_test/include/HubMatrix_GPU.cuh:114-161), unmodified and read where it
// lies in the reference checkout, into a device-only cubin for sm_103a
// (`make -C oracle ref`).  Nothing here is host code: tests load the cubin
// with the CUDA driver API (oracle/refkernel.py) and launch it the way
// Hubbard::Hubbard_mv does (HubMatrix_GPU.cuh:163-182).
//
// The reference header pulls in MAGMA_LAPACK.h for the host tridiagonal
// solver, which needs MAGMA; its include guard is defined here and the two
// host functions it declares are declared instead (never called or defined:
// the cubin holds device code only).
#define __MAGMA_LAPACK__
namespace LAPACK {
void dsted(int n, double* d, double* e, int il, int iu, double* m, double* z);
}
namespace LAPACKf77 {
void dsted(int n, double* d, double* e, double* m, double* z);
}

#include "HubMatrix_GPU.cuh"

// The real instantiation (entry _Z11Hubbard_mv_IdEvPKdPKiS1_S3_S3_S3_PT_S5_mmiidiii).
template __global__ void Hubbard_mv_<double>(const double*, const int*, const double*, const int*, const int*,
                                             const int*, double*, double*, const unsigned long, const unsigned long,
                                             const int, const int, const double, const int, const int, const int);
