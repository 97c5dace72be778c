// ed_dense.cu — the operator as a dense matrix (Hubbard::Write,
// MBL_test/include/HubMatrix_GPU.cuh:184-240): row i = u * dim_dn + d gets the
// up-term entries at columns u' * dim_dn + d, the down-term entries at
// u * dim_dn + d' and the diagonal eps_up(u) + eps_dn(d) + U popc(s_up & s_dn
// & mask), in FP64 from the class coefficients (not the fixed-point scale).
// For the small sectors the dense-ED drivers use (TotalSpinFull_*, tED).
#include <cuda_runtime.h>

#include <algorithm>
#include <complex>
#include <vector>

#include "../../include/ed_hubbard.h"
#include "ed_internal.hpp"

namespace ed {
namespace {

struct DenseArgs {
    const uint32_t *upPtr, *upEnt, *dnPtr, *dnEnt;
    const double2 *coefUP, *coefDN;  // class coefficients (re, im)
    const double2 *diagUP, *diagDN;  // folded site terms (re, im)
    const uint64_t *stUP, *stDN;
    uint64_t mask;
    double U;
    int64_t dimUP, dimDN;
    int cplx;
};

__device__ __forceinline__ void dense_put(double* H, int64_t D, int64_t r, int64_t c, double2 v, int cplx) {
    if (cplx) {
        double2* p = reinterpret_cast<double2*>(H) + (size_t)r * D + c;
        p->x += v.x;
        p->y += v.y;
    } else {
        H[(size_t)r * D + c] += v.x;
    }
}

// One thread per row; every row writes only its own row of H.
__global__ void k_write_dense(DenseArgs g, double* __restrict__ H) {
    const int64_t D = g.dimUP * g.dimDN;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t u = i / g.dimDN, d = i - u * g.dimDN;
        for (uint32_t q = g.upPtr[u]; q < g.upPtr[u + 1]; ++q) {
            const uint32_t e = g.upEnt[q];
            double2 c = g.coefUP[(e >> kClassShift) & kClassMask];
            if (e & kSignBit) c = make_double2(-c.x, -c.y);
            dense_put(H, D, i, (int64_t)(e & kColMask) * g.dimDN + d, c, g.cplx);
        }
        for (uint32_t q = g.dnPtr[d]; q < g.dnPtr[d + 1]; ++q) {
            const uint32_t e = g.dnEnt[q];
            double2 c = g.coefDN[(e >> kClassShift) & kClassMask];
            if (e & kSignBit) c = make_double2(-c.x, -c.y);
            dense_put(H, D, i, u * g.dimDN + (int64_t)(e & kColMask), c, g.cplx);
        }
        const double2 a = g.diagUP[u], b = g.diagDN[d];
        const double dd = g.U * (double)__popcll(g.stUP[u] & g.stDN[d] & g.mask);
        dense_put(H, D, i, i, make_double2(a.x + b.x + dd, a.y + b.y), g.cplx);
    }
}

}  // namespace
}  // namespace ed

extern "C" {

ed_status ed_op_write_dense(ed_op* op, double* H, int mem, void* stream) {
    using namespace ed;
    if (!op || !H || (mem != ED_MEM_HOST && mem != ED_MEM_DEVICE)) return ED_ERR_ARG;
    const int64_t D = op->D;
    if (D > 65536) return ED_ERR_RANGE;  // D^2 values
    if (cudaSetDevice(op->device) != cudaSuccess) return ED_ERR_CUDA;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const int W = op->cplx ? 2 : 1;
    const size_t bytes = sizeof(double) * (size_t)W * D * D;
    auto cplx2 = [](const std::vector<std::complex<double>>& v) {
        std::vector<double2> o(std::max<size_t>(v.size(), 1), make_double2(0.0, 0.0));
        for (size_t k = 0; k < v.size(); ++k) o[k] = make_double2(v[k].real(), v[k].imag());
        return o;
    };
    auto diag2 = [](const SpinTable& t) {
        std::vector<double2> o(t.count);
        for (int64_t k = 0; k < t.count; ++k) o[k] = make_double2(t.diag_re[k], t.diag_im.empty() ? 0.0 : t.diag_im[k]);
        return o;
    };
    const std::vector<double2> cu = cplx2(op->tup.coef), cd = cplx2(op->tdn.coef), du = diag2(op->tup),
                               dd = diag2(op->tdn);
    double* dH = mem == ED_MEM_DEVICE ? H : nullptr;
    double2 *dcu = nullptr, *dcd = nullptr, *ddu = nullptr, *ddd = nullptr;
    ed_status st = ED_OK;
    if ((mem == ED_MEM_HOST && cudaMallocAsync(&dH, bytes, s) != cudaSuccess) ||
        cudaMallocAsync(&dcu, sizeof(double2) * cu.size(), s) != cudaSuccess ||
        cudaMallocAsync(&dcd, sizeof(double2) * cd.size(), s) != cudaSuccess ||
        cudaMallocAsync(&ddu, sizeof(double2) * du.size(), s) != cudaSuccess ||
        cudaMallocAsync(&ddd, sizeof(double2) * dd.size(), s) != cudaSuccess)
        st = ED_ERR_ALLOC;
    if (st == ED_OK &&
        (cudaMemcpyAsync(dcu, cu.data(), sizeof(double2) * cu.size(), cudaMemcpyHostToDevice, s) != cudaSuccess ||
         cudaMemcpyAsync(dcd, cd.data(), sizeof(double2) * cd.size(), cudaMemcpyHostToDevice, s) != cudaSuccess ||
         cudaMemcpyAsync(ddu, du.data(), sizeof(double2) * du.size(), cudaMemcpyHostToDevice, s) != cudaSuccess ||
         cudaMemcpyAsync(ddd, dd.data(), sizeof(double2) * dd.size(), cudaMemcpyHostToDevice, s) != cudaSuccess ||
         cudaMemsetAsync(dH, 0, bytes, s) != cudaSuccess))
        st = ED_ERR_CUDA;
    if (st == ED_OK) {
        const MvArgs& a = op->mv;
        DenseArgs g{a.upPtr, a.upEntC, a.dnPtr, a.dnEntC, dcu, dcd, ddu, ddd, a.stUP, a.stDN, a.mask, op->U,
                    op->dimUP, op->dimDN, op->cplx ? 1 : 0};
        const int64_t blocks = std::min<int64_t>((D + 255) / 256, 152 * 8);
        k_write_dense<<<(int)std::max<int64_t>(blocks, 1), 256, 0, s>>>(g, dH);
        if (cudaGetLastError() != cudaSuccess) st = ED_ERR_CUDA;
    }
    if (st == ED_OK && mem == ED_MEM_HOST && cudaMemcpyAsync(H, dH, bytes, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        st = ED_ERR_CUDA;
    if (mem == ED_MEM_HOST) cudaFreeAsync(dH, s);
    cudaFreeAsync(dcu, s);
    cudaFreeAsync(dcd, s);
    cudaFreeAsync(ddu, s);
    cudaFreeAsync(ddd, s);
    if (cudaStreamSynchronize(s) != cudaSuccess && st == ED_OK) st = ED_ERR_CUDA;
    return st;
}

}  // extern "C"
