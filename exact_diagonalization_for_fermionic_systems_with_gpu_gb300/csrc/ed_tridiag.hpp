// ed_tridiag.hpp — eigenpairs of a symmetric tridiagonal matrix, on the host.
#pragma once

#include <vector>

namespace ed {

// Lowest eigenvalue of T (diagonal a[0..n-1], off-diagonal off[0..n-2]);
// when z is not null it receives the unit eigenvector (largest component
// positive).
double tridiag_lowest_host(int n, const double* a, const double* off, double* z);

// One plane rotation of the tridiagonal QR iteration: plane (k, k+1),
// matrix [[c, s], [-s, c]].
struct TriRot {
    int k;
    double c, s;
};

// All eigenvalues (in evals, unsorted) and the rotations whose product
// Z = G_1 ... G_K diagonalises T (Z^T T Z = diag(evals)).  False when the
// iteration did not converge.
bool tridiag_eigen_rotations(int n, const double* a, const double* off, std::vector<double>* evals,
                             std::vector<TriRot>* rots);
void tri_apply_zt(const std::vector<TriRot>& rots, double* v);  // v <- Z^T v
void tri_apply_z(const std::vector<TriRot>& rots, double* v);   // v <- Z v

// out[t][k] = (exp(-i T times[t]) e_0)_k as interleaved (re, im), n_times x 2n doubles.
bool tridiag_expm_e0(int n, const double* a, const double* off, int n_times, const double* times, double* out);

// Singular values of the upper bidiagonal (d, e) (both overwritten; the
// values, unsorted and nonnegative, in d).  False when not converged.
bool bidiag_singular_values(int n, double* d, double* e);

}  // namespace ed
