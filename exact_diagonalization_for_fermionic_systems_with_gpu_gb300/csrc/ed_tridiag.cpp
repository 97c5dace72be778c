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

// ----------------------------------------------------------------------------
// All eigenpairs: implicit symmetric tridiagonal QR with the Wilkinson shift
// (Golub & Van Loan, Matrix Computations, 4th ed., Algorithms 8.3.2-8.3.3):
// each step chases the bulge of one shifted rotation down the unreduced block
// [l, m]; off-diagonals below eps (|a_i| + |a_{i+1}|) deflate.  The rotations
// G_1 .. G_K (plane (k, k+1), [[c, s], [-s, c]]) are recorded in order, so
// Z = G_1 G_2 ... G_K holds the eigenvectors as columns and Z^T T Z = diag(m).
// Applying the rotations to one vector costs O(K) = O(n^2) instead of the
// O(n^3) of forming Z; this is what the Krylov propagator needs
// (exp(-i T t) e_0 = Z exp(-i diag(m) t) Z^T e_0, HubMatrix_GPU.cuh:684-690).
bool tridiag_eigen_rotations(int n, const double* a_in, const double* off, std::vector<double>* evals,
                             std::vector<TriRot>* rots) {
    std::vector<double> a(a_in, a_in + n), b(std::max(n - 1, 0));
    for (int i = 0; i + 1 < n; ++i) b[i] = off[i];
    rots->clear();
    const double eps = std::numeric_limits<double>::epsilon();
    int m = n - 1;
    long long iters = 0;
    const long long max_iters = 60LL * std::max(n, 1);
    while (m > 0) {
        if (std::fabs(b[m - 1]) <= eps * (std::fabs(a[m - 1]) + std::fabs(a[m]))) {
            b[m - 1] = 0.0;
            --m;
            continue;
        }
        int l = m - 1;
        while (l > 0 && std::fabs(b[l - 1]) > eps * (std::fabs(a[l - 1]) + std::fabs(a[l]))) --l;
        if (l > 0) b[l - 1] = 0.0;
        if (++iters > max_iters) return false;
        // Wilkinson shift from the trailing 2x2 of the block
        const double d = 0.5 * (a[m - 1] - a[m]);
        const double bb = b[m - 1];
        const double den = d + (d >= 0.0 ? 1.0 : -1.0) * std::hypot(d, bb);
        const double mu = den != 0.0 ? a[m] - bb * bb / den : a[m] - std::fabs(bb);
        double x = a[l] - mu, z = b[l];
        for (int k = l; k < m; ++k) {
            // rotation in plane (k, k+1) that zeroes z against x
            double r = std::hypot(x, z);
            double c = 1.0, s = 0.0;
            if (r != 0.0) {
                c = x / r;
                s = -z / r;
            }
            if (k > l) b[k - 1] = r;  // the bulge at (k-1, k+1) is gone
            const double ak = a[k], ak1 = a[k + 1], e = b[k];
            a[k] = c * c * ak - 2.0 * c * s * e + s * s * ak1;
            a[k + 1] = s * s * ak + 2.0 * c * s * e + c * c * ak1;
            b[k] = c * s * (ak - ak1) + (c * c - s * s) * e;
            rots->push_back(TriRot{k, c, s});
            if (k + 1 < m) {
                const double f = b[k + 1];
                z = -s * f;  // new bulge at (k, k+2)
                b[k + 1] = c * f;
                x = b[k];
            }
        }
    }
    evals->assign(a.begin(), a.end());
    return true;
}

// v <- Z^T v: G_1^T first
void tri_apply_zt(const std::vector<TriRot>& rots, double* v) {
    for (const TriRot& g : rots) {
        const double x = v[g.k], y = v[g.k + 1];
        v[g.k] = g.c * x - g.s * y;
        v[g.k + 1] = g.s * x + g.c * y;
    }
}

// v <- Z v: G_K first
void tri_apply_z(const std::vector<TriRot>& rots, double* v) {
    for (auto it = rots.rbegin(); it != rots.rend(); ++it) {
        const TriRot& g = *it;
        const double x = v[g.k], y = v[g.k + 1];
        v[g.k] = g.c * x + g.s * y;
        v[g.k + 1] = -g.s * x + g.c * y;
    }
}

bool tridiag_expm_e0(int n, const double* a, const double* off, int n_times, const double* times, double* out) {
    std::vector<double> m;
    std::vector<TriRot> rots;
    if (!tridiag_eigen_rotations(n, a, off, &m, &rots)) return false;
    std::vector<double> y(n, 0.0), re(n), im(n);
    y[0] = 1.0;
    tri_apply_zt(rots, y.data());
    for (int t = 0; t < n_times; ++t) {
        for (int j = 0; j < n; ++j) {
            const double ph = m[j] * times[t];
            re[j] = std::cos(ph) * y[j];
            im[j] = -std::sin(ph) * y[j];
        }
        tri_apply_z(rots, re.data());
        tri_apply_z(rots, im.data());
        double* o = out + (size_t)2 * n * t;
        for (int k = 0; k < n; ++k) {
            o[2 * k] = re[k];
            o[2 * k + 1] = im[k];
        }
    }
    return true;
}

}  // namespace ed

namespace ed {

// sqrt(a^2 + b^2) without hypot's scaling (the bidiagonal entries here are
// O(1) down to ~1e-150; a square that underflows gives a zero rotation angle,
// which costs nothing at the eps |B| accuracy sought).
inline double rot_norm(double a, double b) { return std::sqrt(a * a + b * b); }

// Singular values of an upper bidiagonal B (d[0..n-1] diagonal, e[0..n-2]
// superdiagonal; both overwritten, |values| left in d): the Golub-Kahan SVD
// step with a Wilkinson shift from the trailing 2x2 of B^T B (Golub & Van
// Loan, Matrix Computations, 4th ed., Algorithms 8.6.1-8.6.2).  A
// superdiagonal entry deflates when |e_i| <= eps |B|; a diagonal entry with
// |d_k| <= eps |B| is set to zero and its row is cleared by rotations from the
// left, which moves the entry along the row until it leaves the block.
// Absolute accuracy eps |B|, as LAPACK's gesvd gives after a Householder
// bidiagonalisation.  False when 60 n sweeps did not converge.
bool bidiag_singular_values(int n, double* d, double* e) {
    if (n <= 0) return true;
    const double eps = std::numeric_limits<double>::epsilon();
    double bnorm = 0.0;
    for (int i = 0; i < n; ++i) bnorm = std::max(bnorm, std::fabs(d[i]) + (i + 1 < n ? std::fabs(e[i]) : 0.0));
    if (bnorm == 0.0) return true;
    const double tol = eps * bnorm;
    int q = n - 1;  // bottom of the active block
    long long iters = 0;
    const long long max_iters = 60LL * n;
    while (q > 0) {
        if (std::fabs(e[q - 1]) <= tol) {
            e[q - 1] = 0.0;
            --q;
            continue;
        }
        int p = q - 1;
        while (p > 0 && std::fabs(e[p - 1]) > tol) --p;
        if (++iters > max_iters) return false;
        // a (near-)zero diagonal entry in [p, q): clear its row
        int z = -1;
        for (int k = p; k < q; ++k)
            if (std::fabs(d[k]) <= tol) { z = k; break; }
        if (z >= 0) {
            d[z] = 0.0;
            double f = e[z];
            e[z] = 0.0;
            for (int j = z + 1; j <= q && f != 0.0; ++j) {
                // rotate rows (z, j) so that the entry f in row z, column j
                // goes to zero against d[j]
                const double r = rot_norm(d[j], f);
                const double ir = 1.0 / r;
                const double c = d[j] * ir, s = f * ir;
                d[j] = r;
                if (j < q) {
                    f = -s * e[j];
                    e[j] = c * e[j];
                }
            }
            continue;
        }
        if (std::fabs(d[q]) <= tol) {  // zero at the bottom: clear its column
            d[q] = 0.0;
            double f = e[q - 1];
            e[q - 1] = 0.0;
            for (int j = q - 1; j >= p && f != 0.0; --j) {
                const double r = rot_norm(d[j], f);
                const double ir = 1.0 / r;
                const double c = d[j] * ir, s = f * ir;
                d[j] = r;
                if (j > p) {
                    f = -s * e[j - 1];
                    e[j - 1] = c * e[j - 1];
                }
            }
            continue;
        }
        // Wilkinson shift: eigenvalue of the trailing 2x2 of B^T B nearer its last entry
        const double dm = d[q - 1], em = e[q - 1], dq = d[q];
        const double el = q - 1 > p ? e[q - 2] : 0.0;
        const double t11 = dm * dm + el * el, t12 = dm * em, t22 = dq * dq + em * em;
        const double h = 0.5 * (t11 - t22);
        const double den = h + (h >= 0.0 ? 1.0 : -1.0) * rot_norm(h, t12);
        const double mu = den != 0.0 ? t22 - t12 * t12 / den : t22;
        double y = d[p] * d[p] - mu, zz = d[p] * e[p];
        for (int k = p; k < q; ++k) {
            // right rotation on columns (k, k+1): zero zz against y
            double r = rot_norm(y, zz);
            double ir = r != 0.0 ? 1.0 / r : 0.0;
            double c = r != 0.0 ? y * ir : 1.0, s = -zz * ir;
            if (k > p) e[k - 1] = r;
            // [d_k e_k; 0 d_{k+1}] * [[c, s], [-s, c]] (the bulge below the diagonal)
            const double dk = d[k], ek = e[k], dk1 = d[k + 1];
            double a11 = c * dk - s * ek;
            double a12 = s * dk + c * ek;
            double a21 = -s * dk1;
            double a22 = c * dk1;
            // left rotation on rows (k, k+1): zero a21 against a11
            r = rot_norm(a11, a21);
            ir = r != 0.0 ? 1.0 / r : 0.0;
            c = r != 0.0 ? a11 * ir : 1.0;
            s = -a21 * ir;
            d[k] = r;
            // rows: [c -s; s c] * [[a11 a12 0], [a21 a22 e_{k+1}]]
            e[k] = c * a12 - s * a22;
            d[k + 1] = s * a12 + c * a22;
            if (k + 1 < q) {
                const double ek1 = e[k + 1];
                y = e[k];
                zz = -s * ek1;      // bulge at (k, k+2)
                e[k + 1] = c * ek1;
            }
        }
    }
    for (int i = 0; i < n; ++i) d[i] = std::fabs(d[i]);
    return true;
}

}  // namespace ed
