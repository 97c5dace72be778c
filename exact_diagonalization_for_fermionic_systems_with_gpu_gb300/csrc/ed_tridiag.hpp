// ed_tridiag.hpp — lowest eigenpair of a symmetric tridiagonal matrix.
#pragma once

namespace ed {

// Lowest eigenvalue of T (diagonal a[0..n-1], off-diagonal off[0..n-2]);
// when z is not null it receives the unit eigenvector (largest component
// positive).
double tridiag_lowest_host(int n, const double* a, const double* off, double* z);

}  // namespace ed
