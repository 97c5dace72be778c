/*
 * hubbard_oracle.c — CPU restatement of the reference's Hubbard ED hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: only tests/, the
 * smoke() entry and bench.py's CPU-baseline / reference legs may load it.
 * The product library never links or calls it.
 *
 * What is restated here (citations are into the reference project
 * jeechul/Exact_Diagonalization_for_Fermionic_systems_with_GPU):
 *   - fixed-popcount basis in ascending-integer order and its rank table
 *       MBL_test/include/fermi_operator.h:44-53  (H_TBq::Labeling)
 *   - popcount and the Jordan-Wigner "particles strictly between" count
 *       MBL_test/include/fermi_operator.h:19-40  (count1, count1_bt_sites)
 *   - the per-spin ELL tables with z*Q+1 slots, slot-major, first-empty-slot
 *     stacking where 0.0 marks an empty slot
 *       MBL_test/include/fermi_operator.h:64-73   (stacking)
 *       MBL_test/include/fermi_operator.h:100-149 (Make_H, Make_J, Make_N)
 *   - the spin-split matvec y = (H_up (x) 1 + 1 (x) H_dn + U n_up n_dn) x,
 *     same term order (up slots, down slots, interaction) and FMA contraction
 *       MBL_test/include/HubMatrix_GPU.cuh:114-161 (Hubbard_mv_)
 *   - Lanczos three-term recurrence with the every-10-steps convergence test
 *     and the second-pass Ritz rebuild
 *       MBL_test/include/HubMatrix_GPU.cuh:541-613 (tridiagonal, eigen)
 *   - the continued-fraction correlator
 *       MBL_test/include/HubMatrix_GPU.cuh:820-849
 * The tridiagonal eigensolve (LAPACK dstedc behind LAPACKf77::dsted,
 * MBL_test/include/MAGMA_LAPACK.h:296-326) is replaced by this file's own
 * Sturm-bisection + inverse iteration for the lowest eigenpair; the Python
 * side cross-checks it with scipy.linalg.eigh_tridiagonal.
 *
 * Differences from the reference, all deliberate: 64-bit linear indices
 * (the reference's int gid overflows past 2^31 elements), a bounds check in
 * stacking (the reference writes past the table), explicit status returns.
 *
 * Parity pin: the tables are checked bit-for-bit against the reference's own
 * fermi_operator.h compiled by oracle/Makefile (oracle/_ref/ref_tables) and
 * stored as fixtures in tests/golden/.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_Z 10 /* slots per particle: fermi_operator.h:11 */

/* ---------------------------------------------------------------- basis -- */

static int popc64(uint64_t v) {
    int c = 0;
    while (v) { v &= v - 1; ++c; }
    return c;
}

/* fermi_operator.h:26-40: number of set bits strictly between the two sites */
static int count_between(uint64_t n, int i, int j) {
    int lo = i < j ? i : j, hi = i < j ? j : i;
    if (hi - lo <= 1) return 0;
    uint64_t mask = ((1ULL << (hi - lo - 1)) - 1ULL) << (lo + 1);
    return popc64(n & mask);
}

/* Number of N-bit words with popcount Q. */
int64_t orc_binom(int n, int k) {
    if (k < 0 || k > n) return 0;
    int64_t r = 1;
    for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
    return r;
}

/* fermi_operator.h:44-53: state[] lists the words with popcount Q in
 * ascending order; address[word] is its position (or -1). */
int orc_basis(int N, int Q, int64_t* state, int64_t* address) {
    if (N < 1 || N > 30) return -1;
    int64_t count = 0, dim = 1LL << N;
    for (int64_t n = 0; n < dim; ++n) {
        if (popc64((uint64_t)n) == Q) {
            state[count] = n;
            if (address) address[n] = count;
            ++count;
        } else if (address) {
            address[n] = -1;
        }
    }
    return (int)(count == orc_binom(N, Q) ? 0 : -2);
}

/* ---------------------------------------------------------------- tables -- */

typedef struct {
    int N, Q;
    int64_t count;   /* basis size */
    int nslots;      /* z*Q+1 */
    int64_t* state;
    int64_t* address;
    double* Ax;      /* Ax[slot*count + a] */
    int64_t* Aj;
    int overflow;    /* set when a row needed more than nslots slots */
} orc_tbq;

orc_tbq* orc_tbq_new(int N, int Q) {
    orc_tbq* h = (orc_tbq*)calloc(1, sizeof(orc_tbq));
    h->N = N; h->Q = Q;
    h->count = orc_binom(N, Q);
    h->nslots = ORC_Z * Q + 1;
    h->state = (int64_t*)malloc(sizeof(int64_t) * h->count);
    h->address = (int64_t*)malloc(sizeof(int64_t) * (1LL << N));
    h->Ax = (double*)calloc((size_t)h->count * h->nslots, sizeof(double));
    h->Aj = (int64_t*)calloc((size_t)h->count * h->nslots, sizeof(int64_t));
    orc_basis(N, Q, h->state, h->address);
    return h;
}

void orc_tbq_free(orc_tbq* h) {
    if (!h) return;
    free(h->state); free(h->address); free(h->Ax); free(h->Aj); free(h);
}

void orc_tbq_clear(orc_tbq* h) {
    memset(h->Ax, 0, sizeof(double) * h->count * h->nslots);
    memset(h->Aj, 0, sizeof(int64_t) * h->count * h->nslots);
    h->overflow = 0;
}

/* fermi_operator.h:64-73: put value into the first slot of row a whose
 * value is exactly 0.0 (the reference recurses slot by slot). */
static void stack_entry(orc_tbq* h, int64_t a, int64_t b, double value) {
    for (int s = 0; s < h->nslots; ++s) {
        size_t idx = (size_t)s * h->count + a;
        if (h->Ax[idx] == 0.0) {
            h->Ax[idx] += value;
            h->Aj[idx] = b;
            return;
        }
    }
    h->overflow = 1;
}

/* fermi_operator.h:100-115 (Make_H): t*(c+_i c_j + c+_j c_i) with sign
 * (-1)^(particles strictly between i and j). */
void orc_make_h(orc_tbq* h, int i, int j, double t) {
    for (int64_t a = 0; a < h->count; ++a) {
        uint64_t n = (uint64_t)h->state[a];
        int oi = (int)((n >> i) & 1ULL), oj = (int)((n >> j) & 1ULL);
        if (oi != oj) {
            uint64_t l = n ^ ((1ULL << i) | (1ULL << j));
            double sign = (count_between(n, i, j) & 1) ? -1.0 : 1.0;
            stack_entry(h, a, h->address[l], sign * t);
        }
    }
}

/* fermi_operator.h:117-138 (Make_J): +t when site i is empty and j full,
 * -t in the opposite case. */
void orc_make_j(orc_tbq* h, int i, int j, double t) {
    for (int64_t a = 0; a < h->count; ++a) {
        uint64_t n = (uint64_t)h->state[a];
        int oi = (int)((n >> i) & 1ULL), oj = (int)((n >> j) & 1ULL);
        if (oi == oj) continue;
        uint64_t l = n ^ ((1ULL << i) | (1ULL << j));
        double sign = (count_between(n, i, j) & 1) ? -1.0 : 1.0;
        stack_entry(h, a, h->address[l], (oi == 0 && oj == 1) ? sign * t : sign * (-t));
    }
}

/* fermi_operator.h:140-149 (Make_N): v*n_i, each call its own slot. */
void orc_make_n(orc_tbq* h, int i, double v) {
    for (int64_t a = 0; a < h->count; ++a) {
        uint64_t n = (uint64_t)h->state[a];
        if ((n >> i) & 1ULL) stack_entry(h, a, a, v);
    }
}

int orc_tbq_overflow(const orc_tbq* h) { return h->overflow; }
int64_t orc_tbq_count(const orc_tbq* h) { return h->count; }
int orc_tbq_nslots(const orc_tbq* h) { return h->nslots; }
const double* orc_tbq_ax(const orc_tbq* h) { return h->Ax; }
const int64_t* orc_tbq_aj(const orc_tbq* h) { return h->Aj; }
const int64_t* orc_tbq_state(const orc_tbq* h) { return h->state; }

/* ---------------------------------------------------------------- matvec -- */

/* HubMatrix_GPU.cuh:114-161, real vectors.  Term order and FMA use follow
 * the reference kernel: up slots (skipping empty ones), all down slots,
 * then U * popcount(up & dn & mask). */
void orc_matvec(const orc_tbq* up, const orc_tbq* dn, double U, uint64_t mask,
                const double* x, double* y) {
    const int64_t dimUP = up->count, dimDN = dn->count;
#pragma omp parallel for schedule(static)
    for (int64_t sv = 0; sv < dimUP; ++sv) {
        for (int64_t id = 0; id < dimDN; ++id) {
            double sum = 0.0;
            for (int s = 0; s < up->nslots; ++s) {
                double a = up->Ax[(size_t)s * dimUP + sv];
                if (a != 0.0) sum = fma(a, x[up->Aj[(size_t)s * dimUP + sv] * dimDN + id], sum);
            }
            for (int s = 0; s < dn->nslots; ++s) {
                double a = dn->Ax[(size_t)s * dimDN + id];
                sum = fma(a, x[sv * dimDN + dn->Aj[(size_t)s * dimDN + id]], sum);
            }
            if (U != 0.0) {
                uint64_t d = ((uint64_t)up->state[sv] & (uint64_t)dn->state[id]) & mask;
                sum = fma(U * (double)popc64(d), x[sv * dimDN + id], sum);
            }
            y[sv * dimDN + id] = sum;
        }
    }
}

/* Complex vectors (interleaved re,im), real tables: the M=complex
 * instantiation of the same kernel. */
void orc_matvec_z(const orc_tbq* up, const orc_tbq* dn, double U, uint64_t mask,
                  const double* x, double* y) {
    const int64_t dimUP = up->count, dimDN = dn->count;
#pragma omp parallel for schedule(static)
    for (int64_t sv = 0; sv < dimUP; ++sv) {
        for (int64_t id = 0; id < dimDN; ++id) {
            double sr = 0.0, si = 0.0;
            for (int s = 0; s < up->nslots; ++s) {
                double a = up->Ax[(size_t)s * dimUP + sv];
                if (a != 0.0) {
                    int64_t k = up->Aj[(size_t)s * dimUP + sv] * dimDN + id;
                    sr = fma(a, x[2 * k], sr); si = fma(a, x[2 * k + 1], si);
                }
            }
            for (int s = 0; s < dn->nslots; ++s) {
                double a = dn->Ax[(size_t)s * dimDN + id];
                int64_t k = sv * dimDN + dn->Aj[(size_t)s * dimDN + id];
                sr = fma(a, x[2 * k], sr); si = fma(a, x[2 * k + 1], si);
            }
            if (U != 0.0) {
                uint64_t d = ((uint64_t)up->state[sv] & (uint64_t)dn->state[id]) & mask;
                double e = U * (double)popc64(d);
                int64_t k = sv * dimDN + id;
                sr = fma(e, x[2 * k], sr); si = fma(e, x[2 * k + 1], si);
            }
            y[2 * (sv * dimDN + id)] = sr;
            y[2 * (sv * dimDN + id) + 1] = si;
        }
    }
}

/* ------------------------------------------------------- vector algebra -- */

/* Fixed chunks summed in order: the same result for any thread count (an
 * OpenMP reduction combines per-thread sums in an unspecified order, which
 * moves the last bits of a 200-step Lanczos from run to run). */
static double dot(const double* a, const double* b, int64_t n) {
    enum { kChunks = 256 };
    double part[kChunks];
    const int64_t chunk = (n + kChunks - 1) / kChunks;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < kChunks; ++k) {
        const int64_t lo = (int64_t)k * chunk;
        const int64_t hi = lo + chunk < n ? lo + chunk : n;
        double s = 0.0;
        for (int64_t i = lo; i < hi; ++i) s += a[i] * b[i];
        part[k] = s;
    }
    double s = 0.0;
    for (int k = 0; k < kChunks; ++k) s += part[k];
    return s;
}

/* --------------------------------------------- tridiagonal eigensolve -- */

/* Number of eigenvalues of the symmetric tridiagonal (a, b) below x, by the
 * Sturm sequence of LDL^T pivots.  b[k] couples rows k and k+1. */
static int sturm_count(int n, const double* a, const double* b, double x) {
    int c = 0;
    double q = a[0] - x;
    if (q < 0) ++c;
    for (int k = 1; k < n; ++k) {
        if (q == 0.0) q = 1e-300;
        q = (a[k] - x) - b[k - 1] * b[k - 1] / q;
        if (q < 0) ++c;
    }
    return c;
}

/* The k-th smallest eigenvalue (k = 0 is the lowest) by bisection on a
 * Gershgorin interval, to full double precision. */
double orc_tridiag_eigval(int n, const double* a, const double* b, int k) {
    double lo = a[0], hi = a[0];
    for (int i = 0; i < n; ++i) {
        double r = (i > 0 ? fabs(b[i - 1]) : 0.0) + (i < n - 1 ? fabs(b[i]) : 0.0);
        if (a[i] - r < lo) lo = a[i] - r;
        if (a[i] + r > hi) hi = a[i] + r;
    }
    for (int it = 0; it < 200; ++it) {
        double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;
        if (sturm_count(n, a, b, mid) > k) hi = mid; else lo = mid;
    }
    return 0.5 * (lo + hi);
}

/* Eigenvector of (a, b) for eigenvalue lam by inverse iteration with a
 * pivoted tridiagonal LU; z normalised, sign chosen so the largest-|.|
 * component is positive. */
void orc_tridiag_eigvec(int n, const double* a, const double* b, double lam, double* z) {
    if (n == 1) { z[0] = 1.0; return; }
    double scale = 0.0;
    for (int i = 0; i < n; ++i) scale = fmax(scale, fabs(a[i]) + (i < n - 1 ? fabs(b[i]) : 0.0));
    double pert = scale * 4e-16 + 1e-300;
    double* dl = (double*)malloc(sizeof(double) * n);
    double* dd = (double*)malloc(sizeof(double) * n);
    double* du = (double*)malloc(sizeof(double) * n);
    double* du2 = (double*)malloc(sizeof(double) * n);
    int* piv = (int*)malloc(sizeof(int) * n);
    /* LU of T - lam I with partial pivoting (rows k, k+1) */
    for (int i = 0; i < n; ++i) {
        dd[i] = a[i] - lam;
        du[i] = i < n - 1 ? b[i] : 0.0;
        dl[i] = i < n - 1 ? b[i] : 0.0;
        du2[i] = 0.0;
    }
    for (int k = 0; k < n - 1; ++k) {
        if (fabs(dd[k]) >= fabs(dl[k])) {
            piv[k] = 0;
            if (dd[k] == 0.0) dd[k] = pert;
            double m = dl[k] / dd[k];
            dl[k] = m;
            dd[k + 1] -= m * du[k];
        } else {
            piv[k] = 1;
            double m = dd[k] / dl[k];
            dd[k] = dl[k];
            dl[k] = m;
            double t = du[k];
            du[k] = dd[k + 1];
            dd[k + 1] = t - m * dd[k + 1];
            if (k < n - 2) { du2[k] = du[k + 1]; du[k + 1] = -m * du[k + 1]; }
        }
    }
    if (dd[n - 1] == 0.0) dd[n - 1] = pert;
    for (int i = 0; i < n; ++i) z[i] = 1.0 / sqrt((double)n);
    for (int iter = 0; iter < 4; ++iter) {
        /* forward: apply L^-1 with the recorded row swaps */
        for (int k = 0; k < n - 1; ++k) {
            if (piv[k]) { double t = z[k]; z[k] = z[k + 1]; z[k + 1] = t - dl[k] * z[k + 1]; }
            else z[k + 1] -= dl[k] * z[k];
        }
        /* back substitution with U (diag dd, super du, super-super du2) */
        z[n - 1] /= dd[n - 1];
        z[n - 2] = (z[n - 2] - du[n - 2] * z[n - 1]) / dd[n - 2];
        for (int k = n - 3; k >= 0; --k) z[k] = (z[k] - du[k] * z[k + 1] - du2[k] * z[k + 2]) / dd[k];
        double nrm = 0.0, big = 0.0; int ib = 0;
        for (int i = 0; i < n; ++i) { nrm += z[i] * z[i]; if (fabs(z[i]) > big) { big = fabs(z[i]); ib = i; } }
        nrm = sqrt(nrm);
        double sg = z[ib] < 0 ? -1.0 : 1.0;
        for (int i = 0; i < n; ++i) z[i] = sg * z[i] / nrm;
    }
    free(dl); free(dd); free(du); free(du2); free(piv);
}

/* --------------------------------------------------------------- Lanczos -- */

/* Operator callback over the oracle's tables. */
typedef struct {
    const orc_tbq *up, *dn;
    double U;
    uint64_t mask;
} orc_op;

/* HubMatrix_GPU.cuh:561-613 (Lanczos::eigen).
 * mode 0: reference — convergence test every 10 steps with
 *         tolconv = 0.01*sqrt(eps), anorm as in the reference, maxN steps.
 * mode 1: fixed  — exactly maxN steps.
 * reorth: 1 = full reorthogonalisation (classical Gram-Schmidt twice against
 *         all previous Lanczos vectors; requires storing them), 0 = none.
 * f (length D) is the start vector (need not be normalised; it is read only).
 * Outputs: alpha[0..n-1], beta[0..n] (beta[0] = |f|), *n_out = n, *e0,
 * evec (length D, normalised Ritz vector; may be NULL).
 * The Ritz vector is rebuilt by a second Lanczos pass exactly like the
 * reference (HubMatrix_GPU.cuh:600-612) when reorth == 0, and from the
 * stored basis when reorth == 1. */
int orc_lanczos(const orc_tbq* up, const orc_tbq* dn, double U, uint64_t mask,
                const double* f_in, int maxN, int mode, int reorth,
                double* alpha, double* beta, int* n_out, double* e0, double* evec) {
    const int64_t D = up->count * dn->count;
    double *f = (double*)malloc(sizeof(double) * D), *v0 = (double*)calloc(D, sizeof(double)),
           *v1 = (double*)malloc(sizeof(double) * D);
    double* basis = NULL;
    if (reorth) {
        basis = (double*)malloc(sizeof(double) * D * (size_t)(maxN + 1));
        if (!basis) { free(f); free(v0); free(v1); return -1; }
    }
    memcpy(f, f_in, sizeof(double) * D);
    const double eps = 2.220446049250313e-16;
    const double tolconv = 0.01 * sqrt(eps);
    double anorm = 0.0;
    double* z = (double*)malloc(sizeof(double) * (maxN + 1));
    beta[0] = sqrt(dot(f, f, D));
    int N;
    for (N = 0; N < maxN; ++N) {
        double inv = 1.0 / beta[N];
        for (int64_t i = 0; i < D; ++i) v1[i] = f[i] * inv;
        if (reorth) memcpy(basis + (size_t)N * D, v1, sizeof(double) * D);
        orc_matvec(up, dn, U, mask, v1, f);
        if (N != 0) for (int64_t i = 0; i < D; ++i) f[i] -= beta[N] * v0[i];
        alpha[N] = dot(v1, f, D);
        for (int64_t i = 0; i < D; ++i) f[i] -= alpha[N] * v1[i];
        if (reorth) {
            for (int pass = 0; pass < 2; ++pass) {
                for (int k = 0; k <= N; ++k) {
                    double c = dot(basis + (size_t)k * D, f, D);
                    for (int64_t i = 0; i < D; ++i) f[i] -= c * basis[(size_t)k * D + i];
                }
            }
        }
        beta[N + 1] = sqrt(dot(f, f, D));
        memcpy(v0, v1, sizeof(double) * D);
        if (N == 0) anorm = fabs(alpha[0] + beta[1]);
        else anorm = fmax(anorm, beta[N] + fabs(alpha[N] + beta[N + 1]));
        if (mode == 0 && N % 10 == 9) {
            double lam = orc_tridiag_eigval(N + 1, alpha, beta + 1, 0);
            orc_tridiag_eigvec(N + 1, alpha, beta + 1, lam, z);
            *e0 = lam;
            if (fabs(beta[N + 1] * z[N]) < tolconv * anorm && fabs(z[0]) > tolconv * anorm) break;
        }
    }
    int n = (N < maxN) ? N + 1 : maxN;
    *n_out = n;
    double lam = orc_tridiag_eigval(n, alpha, beta + 1, 0);
    orc_tridiag_eigvec(n, alpha, beta + 1, lam, z);
    *e0 = lam;
    if (evec) {
        memset(evec, 0, sizeof(double) * D);
        if (reorth) {
            for (int k = 0; k < n; ++k)
                for (int64_t i = 0; i < D; ++i) evec[i] += z[k] * basis[(size_t)k * D + i];
        } else {
            memcpy(f, f_in, sizeof(double) * D);
            memset(v0, 0, sizeof(double) * D);
            for (int k = 0; k < n; ++k) {
                double inv = 1.0 / beta[k];
                for (int64_t i = 0; i < D; ++i) v1[i] = f[i] * inv;
                orc_matvec(up, dn, U, mask, v1, f);
                if (k != 0) for (int64_t i = 0; i < D; ++i) f[i] -= beta[k] * v0[i];
                for (int64_t i = 0; i < D; ++i) f[i] -= alpha[k] * v1[i];
                memcpy(v0, v1, sizeof(double) * D);
                for (int64_t i = 0; i < D; ++i) evec[i] += z[k] * v1[i];
            }
        }
        double nrm = sqrt(dot(evec, evec, D));
        for (int64_t i = 0; i < D; ++i) evec[i] /= nrm;
    }
    free(f); free(v0); free(v1); free(z); free(basis);
    return 0;
}

/* HubMatrix_GPU.cuh:820-835: g(w) = |phi|^2 / (w + E - a0 - b1^2/(w + E - a1 - ...)),
 * evaluated bottom-up exactly like the reference.  w is complex (wr, wi);
 * a has n entries, b has n+1 (b[0] unused).  Output gr, gi. */
void orc_continued_fraction(int n, const double* a, const double* b, double norm2,
                            double energy, int nw, const double* wr, const double* wi,
                            double* gr, double* gi) {
    for (int idx = 0; idx < nw; ++idx) {
        /* gw = 1/(w + E - a[n-1]) */
        double zr = wr[idx] + energy - a[n - 1], zi = wi[idx];
        double den = zr * zr + zi * zi;
        double g_r = zr / den, g_i = -zi / den;
        for (int i = n - 2; i >= 0; --i) {
            double bb = b[i + 1] * b[i + 1];
            double tr = wr[idx] + energy - a[i] - g_r * bb, ti = wi[idx] - g_i * bb;
            den = tr * tr + ti * ti;
            g_r = tr / den; g_i = -ti / den;
        }
        gr[idx] = norm2 * g_r;
        gi[idx] = norm2 * g_i;
    }
}

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
