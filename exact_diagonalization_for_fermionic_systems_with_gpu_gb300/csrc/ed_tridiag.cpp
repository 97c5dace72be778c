// ed_tridiag.cpp — lowest eigenpair of the Lanczos tridiagonal T, on the host.
//
// Replaces the reference's CPU LAPACK dstedc call (LAPACKf77::dsted,
// MBL_test/include/MAGMA_LAPACK.h:296-326, called from
// HubMatrix_GPU.cuh:591) for the pair Lanczos uses: the lowest eigenvalue
// m[0] and its eigenvector z.  T is small (one row per Lanczos step) and
// already on the host when the solve finishes, so this costs tens of
// microseconds where a single-thread device solve costs milliseconds.
//
// Eigenvalue: bisection on the Sturm count (eigenvalues below x from the
// signs of the LDL^T pivots q_k = a_k - x - b_{k-1}^2 / q_{k-1}, tiny pivots
// replaced by -pivmin as in LAPACK's dstebz) from a Gershgorin bracket down to
// adjacent floating-point numbers.
// Eigenvector: inverse iteration at that eigenvalue with a pivoted
// tridiagonal LU (four solves from the flat start vector), normalised with
// its largest component positive.
#include "ed_tridiag.hpp"

#include <algorithm>
#include <cmath>
#include <limits>
#include <vector>

namespace ed {

namespace {

int sturm_count(int n, const double* a, const double* b2, double pivmin, double x) {
    int c = 0;
    double q = a[0] - x;
    if (std::fabs(q) < pivmin) q = -pivmin;
    c += q < 0.0;
    for (int k = 1; k < n; ++k) {
        q = (a[k] - x) - b2[k - 1] / q;
        if (std::fabs(q) < pivmin) q = -pivmin;
        c += q < 0.0;
    }
    return c;
}

}  // namespace

double tridiag_lowest_host(int n, const double* a, const double* off, double* z) {
    if (n == 1) {
        if (z) z[0] = 1.0;
        return a[0];
    }
    std::vector<double> b2(n - 1);
    double lo = 1e300, hi = -1e300, bmax = 0.0;
    for (int i = 0; i < n; ++i) {
        const double r = (i > 0 ? std::fabs(off[i - 1]) : 0.0) + (i < n - 1 ? std::fabs(off[i]) : 0.0);
        lo = std::min(lo, a[i] - r);
        hi = std::max(hi, a[i] + r);
        if (i < n - 1) {
            b2[i] = off[i] * off[i];
            bmax = std::max(bmax, b2[i]);
        }
    }
    const double pad = 1e-12 * (std::fabs(lo) + std::fabs(hi)) + 1e-300;
    lo -= pad;
    hi += pad;
    const double pivmin = std::numeric_limits<double>::min() * std::max(1.0, bmax);
    for (int it = 0; it < 2100; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;  // adjacent numbers
        if (sturm_count(n, a, b2.data(), pivmin, mid) >= 1)
            hi = mid;
        else
            lo = mid;
    }
    const double lam = 0.5 * (lo + hi);
    if (!z) return lam;

    // pivoted LU of T - lam I: dl multipliers, dd diagonal, du / du2 the two
    // upper diagonals created by row exchanges
    std::vector<double> dl(n), dd(n), du(n), du2(n);
    std::vector<char> piv(n);
    double scale = 0.0;
    for (int i = 0; i < n; ++i) scale = std::max(scale, std::fabs(a[i]) + (i < n - 1 ? std::fabs(off[i]) : 0.0));
    const double pert = scale * 4e-16 + 1e-300;
    for (int i = 0; i < n; ++i) {
        dd[i] = a[i] - lam;
        du[i] = i < n - 1 ? off[i] : 0.0;
        dl[i] = i < n - 1 ? off[i] : 0.0;
        du2[i] = 0.0;
    }
    for (int k = 0; k < n - 1; ++k) {
        if (std::fabs(dd[k]) >= std::fabs(dl[k])) {
            piv[k] = 0;
            if (dd[k] == 0.0) dd[k] = pert;
            const double m = dl[k] / dd[k];
            dl[k] = m;
            dd[k + 1] -= m * du[k];
        } else {
            piv[k] = 1;
            const double m = dd[k] / dl[k];
            dd[k] = dl[k];
            dl[k] = m;
            const double t = du[k];
            du[k] = dd[k + 1];
            dd[k + 1] = t - m * dd[k + 1];
            if (k < n - 2) {
                du2[k] = du[k + 1];
                du[k + 1] = -m * du[k + 1];
            }
        }
    }
    if (dd[n - 1] == 0.0) dd[n - 1] = pert;
    const double z0 = 1.0 / std::sqrt((double)n);
    for (int i = 0; i < n; ++i) z[i] = z0;
    for (int iter = 0; iter < 4; ++iter) {
        for (int k = 0; k < n - 1; ++k) {
            if (piv[k]) {
                const double t = z[k];
                z[k] = z[k + 1];
                z[k + 1] = t - dl[k] * z[k];
            } else {
                z[k + 1] -= dl[k] * z[k];
            }
        }
        z[n - 1] /= dd[n - 1];
        z[n - 2] = (z[n - 2] - du[n - 2] * z[n - 1]) / dd[n - 2];
        for (int k = n - 3; k >= 0; --k) z[k] = (z[k] - du[k] * z[k + 1] - du2[k] * z[k + 2]) / dd[k];
        double nrm = 0.0, big = 0.0;
        int ib = 0;
        for (int i = 0; i < n; ++i) {
            nrm += z[i] * z[i];
            if (std::fabs(z[i]) > big) {
                big = std::fabs(z[i]);
                ib = i;
            }
        }
        const double inv = (z[ib] < 0.0 ? -1.0 : 1.0) / std::sqrt(nrm);
        for (int i = 0; i < n; ++i) z[i] *= inv;
    }
    return lam;
}

}  // namespace ed
