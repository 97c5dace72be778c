// ed_tridiag.cu — lowest eigenpair of the Lanczos tridiagonal T on the device.
//
// Replaces the reference's CPU LAPACK dstedc call (LAPACKf77::dsted,
// MBL_test/include/MAGMA_LAPACK.h:296-326, called from
// HubMatrix_GPU.cuh:591) for the eigenpair Lanczos uses: m[0] and the
// first eigenvector z.
//
// Eigenvalue: multisection over the whole GPU.  Each round evaluates the
// Sturm count (number of eigenvalues below x) at kPoints evenly spaced x in
// the current bracket and keeps the sub-bracket where the count first
// reaches 1; 5 rounds of 8192 points shrink any Gershgorin bracket to the
// last bits of an FP64 number.  The count uses the characteristic-polynomial
// recurrence p_k = (a_k - x) p_{k-1} - b_{k-1}^2 p_{k-2} (two FP64 products
// per step, no division — FP64 divides are long sequences on this GPU),
// with exact power-of-two rescaling to stay in range, and counts sign
// changes.
// Eigenvector: inverse iteration with a pivoted tridiagonal LU (one thread).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

namespace ed {

constexpr int kTriPoints = 8192;
constexpr int kTriRounds = 5;

struct TriState {
    double lo, hi, h;
    int idx;
    int n;
};

__device__ __forceinline__ int exp_field(double v) { return (int)((__double_as_longlong(v) >> 52) & 0x7FF); }

// Number of eigenvalues of T (diag a, squared off-diagonal b2) below x.
__device__ int sturm_count(int n, const double* __restrict__ a, const double* __restrict__ b2, double x) {
    double p0 = 1.0;
    double p1 = a[0] - x;
    int cnt = 0;
    if (p1 == 0.0) p1 = -1e-300;
    cnt += (p1 < 0.0);
    for (int k = 1; k < n; ++k) {
        double p2 = fma(a[k] - x, p1, -b2[k - 1] * p0);
        if (p2 == 0.0) p2 = (p1 < 0.0) ? 1e-300 : -1e-300;  // zero takes the sign opposite to its predecessor
        cnt += ((p2 < 0.0) != (p1 < 0.0));
        p0 = p1;
        p1 = p2;
        const int e0 = exp_field(p0), e1 = exp_field(p1);
        const int ex = e0 > e1 ? e0 : e1;
        if (ex > 1023 + 600 || ex < 1023 - 600) {
            // exact rescale of both terms by 2^(1023-ex): the larger becomes O(1)
            const double s = __longlong_as_double((long long)(2046 - ex) << 52);
            p0 *= s;
            p1 *= s;
        }
    }
    return cnt;
}

__global__ void k_tri_prep(const double* __restrict__ alpha, const double* __restrict__ off, int n,
                           double* __restrict__ b2, TriState* st) {
    __shared__ double smin[32], smax[32];
    double lo = 1e300, hi = -1e300;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double r = (i > 0 ? fabs(off[i - 1]) : 0.0) + (i < n - 1 ? fabs(off[i]) : 0.0);
        lo = fmin(lo, alpha[i] - r);
        hi = fmax(hi, alpha[i] + r);
        if (i < n - 1) b2[i] = off[i] * off[i];
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = fmin(lo, __shfl_down_sync(0xffffffffu, lo, o));
        hi = fmax(hi, __shfl_down_sync(0xffffffffu, hi, o));
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { smin[wid] = lo; smax[wid] = hi; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) { lo = fmin(lo, smin[w]); hi = fmax(hi, smax[w]); }
        // widen slightly so the bracket strictly contains the spectrum
        const double pad = 1e-12 * (fabs(lo) + fabs(hi)) + 1e-300;
        st->lo = lo - pad;
        st->hi = hi + pad;
        st->h = (st->hi - st->lo) / (kTriPoints + 1);
        st->idx = kTriPoints;
        st->n = n;
    }
}

__global__ void k_tri_round(const double* __restrict__ alpha, const double* __restrict__ b2, TriState* st) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= kTriPoints) return;
    const double x = st->lo + (double)(t + 1) * st->h;
    if (x >= st->hi) return;
    if (sturm_count(st->n, alpha, b2, x) >= 1) atomicMin(&st->idx, t);
}

__global__ void k_tri_update(TriState* st) {
    const int t = st->idx;
    const double lo = st->lo, h = st->h;
    double nhi = (t < kTriPoints) ? lo + (double)(t + 1) * h : st->hi;
    double nlo = (t == 0) ? lo : lo + (double)t * h;
    if (nhi > st->hi) nhi = st->hi;
    if (nlo < lo) nlo = lo;
    st->lo = nlo;
    st->hi = nhi;
    st->h = (nhi - nlo) / (kTriPoints + 1);
    st->idx = kTriPoints;
}

// Inverse iteration for the eigenvalue at the bracket midpoint; out[0] =
// eigenvalue, out[1..n] = unit eigenvector with its largest component
// positive.  Single thread; w holds 4n doubles + n ints of scratch.
__global__ void k_tri_vec(const double* __restrict__ alpha, const double* __restrict__ off, const TriState* st,
                          double* __restrict__ out, double* __restrict__ w) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int n = st->n;
    const double lam = 0.5 * (st->lo + st->hi);
    out[0] = lam;
    double* z = out + 1;
    if (n == 1) { z[0] = 1.0; return; }
    double* dl = w;
    double* dd = w + n;
    double* du = w + 2 * n;
    double* du2 = w + 3 * n;
    int* piv = reinterpret_cast<int*>(w + 4 * n);
    double scale = 0.0;
    for (int i = 0; i < n; ++i) scale = fmax(scale, fabs(alpha[i]) + (i < n - 1 ? fabs(off[i]) : 0.0));
    const double pert = scale * 4e-16 + 1e-300;
    for (int i = 0; i < n; ++i) {
        dd[i] = alpha[i] - lam;
        du[i] = i < n - 1 ? off[i] : 0.0;
        dl[i] = i < n - 1 ? off[i] : 0.0;
        du2[i] = 0.0;
    }
    for (int k = 0; k < n - 1; ++k) {
        if (fabs(dd[k]) >= fabs(dl[k])) {
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
            if (k < n - 2) { du2[k] = du[k + 1]; du[k + 1] = -m * du[k + 1]; }
        }
    }
    if (dd[n - 1] == 0.0) dd[n - 1] = pert;
    const double z0 = 1.0 / sqrt((double)n);
    for (int i = 0; i < n; ++i) z[i] = z0;
    for (int iter = 0; iter < 4; ++iter) {
        for (int k = 0; k < n - 1; ++k) {
            if (piv[k]) { const double t = z[k]; z[k] = z[k + 1]; z[k + 1] = t - dl[k] * z[k]; }
            else z[k + 1] -= dl[k] * z[k];
        }
        z[n - 1] /= dd[n - 1];
        z[n - 2] = (z[n - 2] - du[n - 2] * z[n - 1]) / dd[n - 2];
        for (int k = n - 3; k >= 0; --k) z[k] = (z[k] - du[k] * z[k + 1] - du2[k] * z[k + 2]) / dd[k];
        double nrm = 0.0, big = 0.0;
        int ib = 0;
        for (int i = 0; i < n; ++i) {
            nrm += z[i] * z[i];
            if (fabs(z[i]) > big) { big = fabs(z[i]); ib = i; }
        }
        const double inv = (z[ib] < 0.0 ? -1.0 : 1.0) / sqrt(nrm);
        for (int i = 0; i < n; ++i) z[i] *= inv;
    }
}

size_t tridiag_scratch_bytes(int n) {
    return 256 + sizeof(double) * (size_t)(5 * n + 8) + sizeof(int) * (size_t)(n + 8);
}

// alpha (n), off (n-1) on the device; out gets n+1 doubles.
cudaError_t launch_tridiag_lowest(int n, const double* alpha, const double* off, double* out, void* scratch,
                                  cudaStream_t s) {
    TriState* st = reinterpret_cast<TriState*>(scratch);
    double* b2 = reinterpret_cast<double*>(reinterpret_cast<char*>(scratch) + 256);
    double* w = b2 + n + 8;
    k_tri_prep<<<1, 256, 0, s>>>(alpha, off, n, b2, st);
    for (int r = 0; r < kTriRounds; ++r) {
        k_tri_round<<<kTriPoints / 64, 64, 0, s>>>(alpha, b2, st);
        k_tri_update<<<1, 1, 0, s>>>(st);
    }
    k_tri_vec<<<1, 32, 0, s>>>(alpha, off, st, out, w);
    return cudaGetLastError();
}

}  // namespace ed
