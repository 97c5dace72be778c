// The cost of the Lanczos tridiagonal's lowest eigenvalue on the device: the
// host's Sturm bisection (ed_tridiag.cpp) run by one device thread, and a
// 32-point multisection by one warp, on random n x n tridiagonals; each timed
// with CUDA events against the host solver, and the values compared with the
// host's.  Prints one line per (n, variant); exits 1 when the one-thread
// bisection does not reproduce the host value bit for bit.
#include <cuda_runtime.h>
#include <cstdio>
#include <cmath>
#include <vector>
#include <algorithm>
#include <limits>
#include <chrono>
#include "ed_tridiag.hpp"

__device__ int sturm(int n, const double* a, const double* b2, double pivmin, double x) {
    int c = 0;
    double q = __dsub_rn(a[0], x);
    if (fabs(q) < pivmin) q = -pivmin;
    c += q < 0.0;
    for (int k = 1; k < n; ++k) {
        q = __dsub_rn(__dsub_rn(a[k], x), __ddiv_rn(b2[k - 1], q));
        if (fabs(q) < pivmin) q = -pivmin;
        c += q < 0.0;
    }
    return c;
}

__global__ void k_bisect1(int n, const double* a, const double* b2, double lo, double hi, double pivmin, double* out, int* iters) {
    if (threadIdx.x != 0) return;
    int it = 0;
    for (; it < 2100; ++it) {
        const double mid = __dmul_rn(0.5, __dadd_rn(lo, hi));
        if (mid <= lo || mid >= hi) break;
        if (sturm(n, a, b2, pivmin, mid) >= 1) hi = mid; else lo = mid;
    }
    *out = __dmul_rn(0.5, __dadd_rn(lo, hi));
    *iters = it;
}

// 32 lanes: each round 31 interior points
__global__ void k_bisect32(int n, const double* a, const double* b2, double lo, double hi, double pivmin, double* out, int* iters) {
    const int l = threadIdx.x;
    int r = 0;
    for (; r < 200; ++r) {
        // points lo + (hi - lo) * k / 32, k = 1..31 (lane l evaluates k = l, lane 0 idle)
        const double w = __dsub_rn(hi, lo);
        double x = __dadd_rn(lo, __dmul_rn(w, (double)l / 32.0));
        if (!(x > lo && x < hi)) x = hi;  // collapsed points
        const int c = (l == 0) ? 0 : sturm(n, a, b2, pivmin, x);
        // first lane with count >= 1
        const unsigned m = __ballot_sync(0xffffffffu, l > 0 && c >= 1 && x < hi);
        const int k = m ? __ffs(m) - 1 : 32;
        const double nlo = __shfl_sync(0xffffffffu, k > 1 ? x : lo, k > 1 ? k - 1 : 0);
        const double nhi = k < 32 ? __shfl_sync(0xffffffffu, x, k) : hi;
        if (nlo == lo && nhi == hi) {
            // points collapsed: finish by plain bisection on lane 0
            break;
        }
        lo = nlo; hi = nhi;
        const double mid = __dmul_rn(0.5, __dadd_rn(lo, hi));
        if (mid <= lo || mid >= hi) break;
    }
    if (l == 0) {
        int it = 0;
        for (; it < 2100; ++it) {
            const double mid = __dmul_rn(0.5, __dadd_rn(lo, hi));
            if (mid <= lo || mid >= hi) break;
            if (sturm(n, a, b2, pivmin, mid) >= 1) hi = mid; else lo = mid;
        }
        *out = __dmul_rn(0.5, __dadd_rn(lo, hi));
        *iters = r * 100 + it;
    }
}

int main() {
    int bad = 0;
    for (int n : {50, 150, 300}) {
        std::vector<double> a(n), off(n - 1), b2(n - 1);
        unsigned long long s = 12345 + n;
        auto rnd = [&]() { s = s * 6364136223846793005ULL + 1442695040888963407ULL; return ((s >> 11) * (1.0 / 9007199254740992.0)); };
        for (int i = 0; i < n; ++i) a[i] = -30.0 + 60.0 * rnd();
        for (int i = 0; i < n - 1; ++i) { off[i] = 0.5 + 5.0 * rnd(); b2[i] = off[i] * off[i]; }
        double lo = 1e300, hi = -1e300, bmax = 0;
        for (int i = 0; i < n; ++i) {
            const double r = (i > 0 ? std::fabs(off[i - 1]) : 0.0) + (i < n - 1 ? std::fabs(off[i]) : 0.0);
            lo = std::min(lo, a[i] - r); hi = std::max(hi, a[i] + r);
            if (i < n - 1) bmax = std::max(bmax, b2[i]);
        }
        const double pad = 1e-12 * (std::fabs(lo) + std::fabs(hi)) + 1e-300;
        lo -= pad; hi += pad;
        const double pivmin = std::numeric_limits<double>::min() * std::max(1.0, bmax);
        auto t0 = std::chrono::steady_clock::now();
        const double host = ed::tridiag_lowest_host(n, a.data(), off.data(), nullptr);
        const double host_us = std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now() - t0).count();
        double *da, *db, *dout; int* dit;
        cudaMalloc(&da, 8 * n); cudaMalloc(&db, 8 * n); cudaMalloc(&dout, 8); cudaMalloc(&dit, 4);
        cudaMemcpy(da, a.data(), 8 * n, cudaMemcpyHostToDevice);
        cudaMemcpy(db, b2.data(), 8 * (n - 1), cudaMemcpyHostToDevice);
        cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
        for (int variant = 0; variant < 2; ++variant) {
            float ms = 0; double dv = 0; int its = 0;
            for (int rep = 0; rep < 3; ++rep) {
                cudaEventRecord(e0);
                if (variant == 0) k_bisect1<<<1, 32>>>(n, da, db, lo, hi, pivmin, dout, dit);
                else k_bisect32<<<1, 32>>>(n, da, db, lo, hi, pivmin, dout, dit);
                cudaEventRecord(e1);
                cudaEventSynchronize(e1);
                cudaEventElapsedTime(&ms, e0, e1);
            }
            cudaMemcpy(&dv, dout, 8, cudaMemcpyDeviceToHost);
            cudaMemcpy(&its, dit, 4, cudaMemcpyDeviceToHost);
            const cudaError_t ce = cudaGetLastError();
            printf("n=%d %s device %.1f us host %.1f us |device - host| = %.3g equal %d (%s)\n", n,
                   variant ? "warp32" : "thread1", ms * 1000.0, host_us, std::fabs(dv - host), dv == host,
                   cudaGetErrorString(ce));
            if (ce != cudaSuccess || (variant == 0 && dv != host)) bad = 1;
        }
    }
    return bad;
}
