// ed_lanczos.cu — device-resident FX Lanczos (HubMatrix_GPU.cuh:477-613).
//
// A run is either one persistent launch (ed_lanczos_fused.cu) or two
// launches per step:
//   k_matvec<OUT=1>  u = H w_j (exact), alpha_j, axpy coefficients
//   k_lz_axpy        w_{j+1} = a0 u + a1 w_j + a2 w_{j-1}, beta_{j+1}
// Scalars never leave the device during the recurrence.  The Ritz vector is
// a single weighted sum of the stored Krylov vectors (ED_RITZ_STORED: one
// int64 vector per step), or, when the basis does not fit, the reference's
// second Lanczos pass (ED_RITZ_RECOMPUTE), which regenerates the same
// vectors bit for bit and accumulates the sum as it goes.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <functional>
#include <thread>
#include <vector>

#include "ed_device.cuh"
#include "ed_internal.hpp"
#include "ed_lanczos.hpp"
#include "ed_lanczos_dev.cuh"
#include "ed_tridiag.hpp"

namespace ed {
using namespace dev;

cudaError_t launch_lz_fused(const ed_op* op, const LzFusedArgs& f, cudaStream_t s);
cudaError_t launch_lz_batch(const ed_op* op, const LzBatchArgs& f, cudaStream_t s);
cudaError_t launch_lz_multi(int device, int kinds, const LzMultiArgs& f, cudaStream_t s);

constexpr int kLzThreads = 256;

// Element-wise Lanczos kernels: about 8 elements per thread and at most five
// 256-thread CTAs per SM (all resident: these kernels take at most 48
// registers a thread), so each thread keeps several loads in flight and the
// last-block reduction has few partials.
static int lz_grid(int64_t n) {
    int64_t g = (n + 8 * kLzThreads - 1) / (8 * kLzThreads);
    if (g > 152 * 5) g = 152 * 5;
    return (int)(g < 1 ? 1 : g);
}

// ------------------------------------------------------------------ kernels --

__global__ void k_random(double* __restrict__ f, int64_t n, uint64_t seed) {
    for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b * 4 < n; b += (int64_t)gridDim.x * blockDim.x) {
        const Philox4 r = philox4x64_10((uint64_t)b, seed);
#pragma unroll
        for (int w = 0; w < 4; ++w) {
            const int64_t k = b * 4 + w;
            if (k < n) f[k] = uniform_pm1(r.v[w]);
        }
    }
}

template <typename Fin>
__device__ __forceinline__ void lz_reduce_tail(i128 ss, uint64_t mx, LzState* lz, int ctr, Fin fin) {
    __shared__ i128 s128[32];
    __shared__ uint64_t s64[32];
    const i128 bs = block_sum_i128(ss, s128);
    const uint64_t bm = block_max_u64(mx, s64);
    if (threadIdx.x == 0) {
        lz->part_lo[blockIdx.x] = (uint64_t)bs;
        lz->part_hi[blockIdx.x] = (uint64_t)((u128)bs >> 64);
        lz->part_max[blockIdx.x] = bm;
    }
    if (elect_last_block(&lz->counter[ctr])) {
        i128 s = 0;
        uint64_t m = 0;
        for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) {
            s += (i128)(((u128)__ldcg(lz->part_hi + i) << 64) | __ldcg(lz->part_lo + i));
            const uint64_t pm = __ldcg(lz->part_max + i);
            m = pm > m ? pm : m;
        }
        s = block_sum_i128(s, s128);
        m = block_max_u64(m, s64);
        if (threadIdx.x == 0) {
            fin(s, m);
            lz->counter[ctr] = 0;
        }
    }
}

// FP64 start vector -> FX slot 0, |f| and max|q|.
__global__ void __launch_bounds__(kLzThreads) k_lz_start(const double* __restrict__ f, int64_t n, const int* emax,
                                                         const int* flag, int64_t* __restrict__ q0, LzState* lz) {
    const int E = fx_exp_from_emax(*emax);
    i128 ss = 0;
    uint64_t mx = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t q = f64_to_fx(f[i], E);
        q0[i] = q;
        ss += mul_wide(q, q) >> 16;
        const uint64_t a = (uint64_t)(q < 0 ? -q : q);
        mx = a > mx ? a : mx;
    }
    lz_reduce_tail(ss, mx, lz, 2, [&](i128 s, uint64_t m) {
        lz->e[0] = E;
        lz->m[0] = m;
        lz->beta[0] = sqrt(i128_to_f64(s, 2 * E + 16));
        lz->min_bits = bitlen_u64(m);
        lz->status = (*flag) ? 6 : (m == 0 ? 7 : 0);
        lz->steps_done = 0;
    });
}

// w_{j+1} = round((at0 u + at1 x + at2 p) / 2^Fa)
__global__ void __launch_bounds__(kLzThreads) k_lz_axpy(const int64_t* __restrict__ uq, const int64_t* __restrict__ xq,
                                                        const int64_t* __restrict__ pq, int64_t* __restrict__ wq,
                                                        int64_t n, LzState* lz, int j) {
    const int64_t a0 = lz->at[0], a1 = lz->at[1], a2 = lz->at[2];
    const int Fa = lz->Fa;
    i128 ss = 0;
    uint64_t mx = 0;
    const int64_t npair = n >> 1;
    const longlong2* u2 = reinterpret_cast<const longlong2*>(uq);
    const longlong2* x2 = reinterpret_cast<const longlong2*>(xq);
    const longlong2* p2 = reinterpret_cast<const longlong2*>(pq);
    longlong2* w2 = reinterpret_cast<longlong2*>(wq);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < npair; i += (int64_t)gridDim.x * blockDim.x) {
        const longlong2 u = __ldg(u2 + i), x = __ldg(x2 + i), p = __ldg(p2 + i);
        longlong2 w;
        w.x = shr_round_i64(mul_wide(a0, u.x) + mul_wide(a1, x.x) + mul_wide(a2, p.x), Fa);
        w.y = shr_round_i64(mul_wide(a0, u.y) + mul_wide(a1, x.y) + mul_wide(a2, p.y), Fa);
        w2[i] = w;
        ss += (mul_wide(w.x, w.x) >> 16) + (mul_wide(w.y, w.y) >> 16);
        const uint64_t ax = (uint64_t)(w.x < 0 ? -w.x : w.x), ay = (uint64_t)(w.y < 0 ? -w.y : w.y);
        mx = ax > mx ? ax : mx;
        mx = ay > mx ? ay : mx;
    }
    if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
        const int64_t i = n - 1;
        const int64_t w = shr_round_i64(mul_wide(a0, uq[i]) + mul_wide(a1, xq[i]) + mul_wide(a2, pq[i]), Fa);
        wq[i] = w;
        ss += mul_wide(w, w) >> 16;
        const uint64_t a = (uint64_t)(w < 0 ? -w : w);
        mx = a > mx ? a : mx;
    }
    lz_reduce_tail(ss, mx, lz, 1, [&](i128 s, uint64_t m) { lz_after_axpy(lz, j, s, m); });
}

// |w|^2 and max|w| of slot j (after reorthogonalisation changed it).
__global__ void __launch_bounds__(kLzThreads) k_lz_stats(const int64_t* __restrict__ wq, int64_t n, LzState* lz, int j) {
    i128 ss = 0;
    uint64_t mx = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t w = wq[i];
        ss += mul_wide(w, w) >> 16;
        const uint64_t a = (uint64_t)(w < 0 ? -w : w);
        mx = a > mx ? a : mx;
    }
    lz_reduce_tail(ss, mx, lz, 3, [&](i128 s, uint64_t m) {
        const int e = lz->e[j];
        lz->m[j] = m;
        lz->beta[j] = sqrt(i128_to_f64(s, 2 * e + 16));
        const int bits = bitlen_u64(m);
        if (bits < lz->min_bits) lz->min_bits = bits;
        if (m == 0 && lz->status == 0) lz->status = 7;
    });
}

// partial[k * gridDim.y + c] = sum over chunk c of (q_k q_w) >> 24, exact.
__global__ void __launch_bounds__(kLzThreads) k_lz_dots(const int64_t* __restrict__ basis, int64_t n,
                                                        int64_t stride, const int64_t* __restrict__ w,
                                                        uint64_t* part_lo, uint64_t* part_hi) {
    const int k = blockIdx.x;
    const int c = blockIdx.y, nc = gridDim.y;
    const int64_t* q = basis + (int64_t)k * stride;
    i128 s = 0;
    for (int64_t i = (int64_t)c * blockDim.x + threadIdx.x; i < n; i += (int64_t)nc * blockDim.x)
        s += mul_wide(q[i], w[i]) >> 24;
    __shared__ i128 s128[32];
    s = block_sum_i128(s, s128);
    if (threadIdx.x == 0) {
        part_lo[k * nc + c] = (uint64_t)s;
        part_hi[k * nc + c] = (uint64_t)((u128)s >> 64);
    }
}

// Coefficient on q_k of one Gram-Schmidt pass, from the exact dot
// <w_k, w> = sum_c part[k][c] 2^(e_k + e_w + 24): <w_k, w> / beta_k^2 in units
// of w's exponent (the i128 total rounded once, as a host conversion of it
// would be; IEEE divide and exact scalings).
__device__ __forceinline__ double reorth_r(const uint64_t* lo, const uint64_t* hi, int k, int chunks, const int* e,
                                           const double* beta, int ew) {
    i128 acc = 0;
    for (int c = 0; c < chunks; ++c)
        acc += (i128)(((u128)hi[(size_t)k * chunks + c] << 64) | (u128)lo[(size_t)k * chunks + c]);
    const double dotv = i128_to_f64(acc, e[k] + ew + 24);
    return dotv / (beta[k] * beta[k]) * ldexp(1.0, e[k] - ew);
}

// One block: the integer coefficients (rt_k, rs_k) and common shift F of a
// Gram-Schmidt pass against w_0 .. w_{nk-1} (fx_coefs' rule: 62 - exponent
// bits per coefficient, less the guard bits of the sum of nk terms), so that
// no step of a reorthogonalised run waits for the host.
__global__ void __launch_bounds__(kLzThreads) k_reorth_coefs(const uint64_t* __restrict__ lo,
                                                             const uint64_t* __restrict__ hi, int nk, int chunks,
                                                             const int* __restrict__ e, const double* __restrict__ beta,
                                                             int64_t* __restrict__ rt, int* __restrict__ rs,
                                                             int* __restrict__ Fout) {
    __shared__ int sm[kLzThreads / 32];
    int extra = 0;
    while ((1 << (10 + extra)) < nk) ++extra;
    const int ew = e[nk];
    int fmin = 1 << 20;
    for (int k = threadIdx.x; k < nk; k += blockDim.x) {
        const double r = reorth_r(lo, hi, k, chunks, e, beta, ew);
        if (r != 0.0) {
            int ka;
            frexp(fabs(r), &ka);
            fmin = min(fmin, 62 - ka - extra);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) fmin = min(fmin, __shfl_xor_sync(0xffffffffu, fmin, o));
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = fmin;
    __syncthreads();
    int Fmin = 1 << 20;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) Fmin = min(Fmin, sm[w]);
    if (Fmin == (1 << 20)) Fmin = 0;
    for (int k = threadIdx.x; k < nk; k += blockDim.x) {
        const double r = reorth_r(lo, hi, k, chunks, e, beta, ew);
        int64_t t = 0;
        int sh = 0;
        if (r != 0.0) {
            int ka;
            frexp(fabs(r), &ka);
            const int F = 62 - ka - extra;
            if (F - Fmin < 120) {
                t = (int64_t)llrint(ldexp(r, F));
                sh = F - Fmin;
            }
        }
        rt[k] = t;
        rs[k] = sh;
    }
    if (threadIdx.x == 0) *Fout = Fmin;
}

// w <- w - round(sum_k (rt_k q_k >> rs_k) / 2^F)
// kReorthLanes lanes share an element: lane r of the group sums the terms
// k = r, r + kReorthLanes, ...; the exact 128-bit partials are combined by
// shuffles (the same total in any order) and the group's first lane writes.
constexpr int kReorthLanes = 4;

__global__ void __launch_bounds__(kLzThreads) k_lz_reorth(int64_t* __restrict__ w, const int64_t* __restrict__ basis,
                                                          int64_t n, int64_t stride, int nk,
                                                          const int64_t* __restrict__ rt, const int* __restrict__ rs,
                                                          const int* __restrict__ Fp) {
    const int F = *Fp;
    const int r = threadIdx.x % kReorthLanes;
    const int64_t groups = (int64_t)gridDim.x * (blockDim.x / kReorthLanes);
    const int64_t g0 = (int64_t)blockIdx.x * (blockDim.x / kReorthLanes) + threadIdx.x / kReorthLanes;
    // every lane of a warp runs the same number of iterations (the shuffles
    // need all 32): lanes past the end sum nothing and write nothing
    const int64_t iters = (n + groups - 1) / groups;
    for (int64_t t = 0; t < iters; ++t) {
        const int64_t i = g0 + t * groups;
        i128 acc = 0;
        if (i < n)
            for (int k = r; k < nk; k += kReorthLanes) acc += mul_wide(rt[k], basis[(int64_t)k * stride + i]) >> rs[k];
#pragma unroll
        for (int o = 1; o < kReorthLanes; o <<= 1) {
            const uint64_t lo = __shfl_xor_sync(0xffffffffu, (uint64_t)acc, o);
            const uint64_t hi = __shfl_xor_sync(0xffffffffu, (uint64_t)((u128)acc >> 64), o);
            acc += (i128)(((u128)hi << 64) | lo);
        }
        if (i < n && r == 0) w[i] -= (int64_t)shr_round(acc, F);
    }
}

// evec = sum_k (rt_k q_k >> rs_k) * 2^-F as FP64, plus |evec|^2 partials.
// A thread forms two adjacent elements from 16-byte loads of every slot
// (slots are 256-byte aligned), kRitzSlots slots per iteration with all their
// loads issued before the sums; the basis is read once.
constexpr int kRitzSlots = 16;

__global__ void __launch_bounds__(kLzThreads) k_ritz(const int64_t* __restrict__ basis, int64_t n, int64_t stride,
                                                     int nk, const int64_t* __restrict__ rt,
                                                     const int* __restrict__ rs, int F, double* __restrict__ out,
                                                     double* __restrict__ part, unsigned int* counter,
                                                     double* inv_norm) {
    double ss = 0.0;
    const int64_t npair = n >> 1;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < npair; i += (int64_t)gridDim.x * blockDim.x) {
        const longlong2* q = reinterpret_cast<const longlong2*>(basis) + i;
        const int64_t s2 = stride >> 1;
        i128 a0 = 0, a1 = 0;
        int k = 0;
        for (; k + kRitzSlots <= nk; k += kRitzSlots) {
            longlong2 v[kRitzSlots];
#pragma unroll
            for (int t = 0; t < kRitzSlots; ++t) v[t] = __ldg(q + (k + t) * s2);
#pragma unroll
            for (int t = 0; t < kRitzSlots; ++t) {
                const int64_t c = __ldg(rt + k + t);
                const int r = __ldg(rs + k + t);
                a0 += mul_wide(c, v[t].x) >> r;
                a1 += mul_wide(c, v[t].y) >> r;
            }
        }
        for (; k < nk; ++k) {
            const longlong2 v = __ldg(q + k * s2);
            const int64_t c = __ldg(rt + k);
            const int r = __ldg(rs + k);
            a0 += mul_wide(c, v.x) >> r;
            a1 += mul_wide(c, v.y) >> r;
        }
        const double x0 = i128_to_f64(a0, -F), x1 = i128_to_f64(a1, -F);
        out[2 * i] = x0;
        out[2 * i + 1] = x1;
        ss = fma(x0, x0, ss);
        ss = fma(x1, x1, ss);
    }
    if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
        const int64_t i = n - 1;
        i128 acc = 0;
        for (int k = 0; k < nk; ++k) acc += mul_wide(rt[k], basis[(int64_t)k * stride + i]) >> rs[k];
        const double v = i128_to_f64(acc, -F);
        out[i] = v;
        ss = fma(v, v, ss);
    }
    __shared__ double sd[32];
    const double bs = block_sum_f64(ss, sd);
    if (threadIdx.x == 0) part[blockIdx.x] = bs;
    if (elect_last_block(counter)) {
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int i = 0; i < (int)gridDim.x; ++i) t += __ldcg(part + i);
            *inv_norm = t > 0.0 ? 1.0 / sqrt(t) : 0.0;
            *counter = 0;
        }
    }
}

// Second-pass Ritz sum: acc (+)= (rt_k q_k >> rs_k) * 2^-F for the Lanczos
// vector q_k just produced (first: acc is overwritten).
__global__ void __launch_bounds__(kLzThreads) k_ritz_acc(double* __restrict__ acc, const int64_t* __restrict__ q,
                                                         int64_t n, const int64_t* __restrict__ rt,
                                                         const int* __restrict__ rs, int F, int k, int first) {
    const int64_t c = rt[k];
    const int r = rs[k];
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double t = i128_to_f64(mul_wide(c, q[i]) >> r, -F);
        acc[i] = first ? t : acc[i] + t;
    }
}

// *inv_norm = 1 / |v| (0 for a zero vector); block partials, last block sums.
__global__ void __launch_bounds__(kLzThreads) k_inv_norm(const double* __restrict__ v, int64_t n,
                                                         double* __restrict__ part, unsigned int* counter,
                                                         double* inv_norm) {
    double ss = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        ss = fma(v[i], v[i], ss);
    __shared__ double sd[32];
    const double bs = block_sum_f64(ss, sd);
    if (threadIdx.x == 0) part[blockIdx.x] = bs;
    if (elect_last_block(counter)) {
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int i = 0; i < (int)gridDim.x; ++i) t += __ldcg(part + i);
            *inv_norm = t > 0.0 ? 1.0 / sqrt(t) : 0.0;
            *counter = 0;
        }
    }
}

__global__ void k_scale(double* __restrict__ v, int64_t n, const double* __restrict__ s) {
    const double f = *s;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        v[i] *= f;
}

// ------------------------------------------------------------------- host --

cudaError_t launch_random(double* f, int64_t n, uint64_t seed, cudaStream_t s) {
    int64_t blocks = ((n + 3) / 4 + 255) / 256;
    if (blocks > 152 * 8) blocks = 152 * 8;
    if (blocks < 1) blocks = 1;
    k_random<<<(int)blocks, 256, 0, s>>>(f, n, seed);
    return cudaGetLastError();
}

namespace {

struct Workspace {
    int device = -1;
    size_t basis_slots = 0;
    int64_t DW = 0;
    int64_t stride = 0;  // slot stride in elements: DW rounded up to 32 (256-byte aligned slots)
    int max_steps = 0;
    int64_t* basis = nullptr;
    int64_t* u = nullptr;
    double* fbuf = nullptr;
    LzState* lz = nullptr;  // device struct
    LzState h;              // host mirror (pointers)
    int* emax = nullptr;
    int* flag = nullptr;
    uint64_t* dot_lo = nullptr;
    uint64_t* dot_hi = nullptr;
    int64_t* coef_rt = nullptr;
    int* coef_rs = nullptr;
    int* coef_F = nullptr;  // common shift of a device-computed Gram-Schmidt pass
    double* ritz_part = nullptr;
    unsigned int* ritz_ctr = nullptr;
    double* inv_norm = nullptr;
    unsigned int* gbar = nullptr;  // grid-barrier counter of the persistent kernel, then
                                   // its three reduction sets (kFusedSync bytes)
    unsigned long long* stamps = nullptr;  // phase timestamps (profile 2), kLzStamps per step
    uint64_t* fxbound = nullptr;           // 2^kFxBits - 1: the bound every Lanczos vector meets
    unsigned long long* cta_stamps = nullptr;  // per-CTA phase ends (profile 2)
    size_t cta_stamps_n = 0;
    std::vector<cudaEvent_t> events;  // profiling pool (pairs)
    // host-mapped mirror of alpha and beta for the reference mode's stop test
    unsigned char* mirror_base = nullptr;  // host address of the mapped block
    HostMirror* mirror_h = nullptr;        // host view of its header
    HostMirror* mirror_d = nullptr;        // device address of the header
    double* mirror_alpha = nullptr;        // host views of the arrays
    double* mirror_beta = nullptr;
    int mirror_cap = 0;
};

#define LZ_CK(x)                                    \
    do {                                            \
        cudaError_t e_ = (x);                       \
        if (e_ != cudaSuccess) {                    \
            op->last_error = cudaGetErrorString(e_); \
            return ED_ERR_CUDA;                     \
        }                                           \
    } while (0)

void free_ws(Workspace* w) {
    cudaFree(w->basis); cudaFree(w->u); cudaFree(w->fbuf); cudaFree(w->lz);
    cudaFree(w->h.e); cudaFree(w->h.m); cudaFree(w->h.beta); cudaFree(w->h.alpha);
    cudaFree(w->h.part_lo); cudaFree(w->h.part_hi); cudaFree(w->h.part_max); cudaFree(w->h.counter);
    cudaFree(w->emax); cudaFree(w->flag); 
    cudaFree(w->dot_lo); cudaFree(w->dot_hi); cudaFree(w->coef_rt); cudaFree(w->coef_rs); cudaFree(w->coef_F);
    cudaFree(w->ritz_part); cudaFree(w->ritz_ctr); cudaFree(w->inv_norm); cudaFree(w->gbar);
    cudaFree(w->stamps); cudaFree(w->fxbound); cudaFree(w->cta_stamps);
    for (cudaEvent_t e : w->events) cudaEventDestroy(e);
    if (w->mirror_base) cudaFreeHost(w->mirror_base);
    *w = Workspace();
}

// The host-mapped mirror for runs of up to max_steps steps (grow-only).
static cudaError_t ensure_mirror(Workspace* w, int max_steps) {
    const int cap = max_steps + 2;
    if (w->mirror_base && w->mirror_cap >= cap) return cudaSuccess;
    if (w->mirror_base) cudaFreeHost(w->mirror_base);
    w->mirror_base = nullptr;
    w->mirror_cap = 0;
    const size_t head = 64, bytes = head + 2 * sizeof(double) * (size_t)cap;
    cudaError_t e = cudaHostAlloc(reinterpret_cast<void**>(&w->mirror_base), bytes, cudaHostAllocMapped);
    if (e != cudaSuccess) return e;
    std::memset(w->mirror_base, 0, bytes);
    unsigned char* dbase = nullptr;
    e = cudaHostGetDevicePointer(reinterpret_cast<void**>(&dbase), w->mirror_base, 0);
    if (e != cudaSuccess) return e;
    w->mirror_h = reinterpret_cast<HostMirror*>(w->mirror_base);
    w->mirror_d = reinterpret_cast<HostMirror*>(dbase);
    w->mirror_alpha = reinterpret_cast<double*>(w->mirror_base + head);
    w->mirror_beta = w->mirror_alpha + cap;
    w->mirror_h->alpha = reinterpret_cast<double*>(dbase + head);  // device addresses, read by the kernel
    w->mirror_h->beta = w->mirror_h->alpha + cap;
    w->mirror_cap = cap;
    return cudaSuccess;
}

constexpr int kDotChunks = 64;
constexpr size_t kFusedSync = 192;  // barrier counter at 0, LzRedSet[4] at 32, row-queue counters at 160

ed_status ensure_ws(ed_op* op, Workspace* w, size_t slots, int64_t DW, int max_steps) {
    if (w->basis && w->basis_slots >= slots && w->DW == DW && w->max_steps >= max_steps) return ED_OK;
    free_ws(w);
    w->device = op->device;
    w->basis_slots = slots;
    w->DW = DW;
    w->stride = (DW + 31) / 32 * 32;
    w->max_steps = max_steps;
    const size_t ns = (size_t)max_steps + 2;
    // + 32 elements: the row engine's 16-byte-aligned row copies may read one past a slot's end
    LZ_CK(cudaMalloc(&w->basis, sizeof(int64_t) * (slots * (size_t)w->stride + 32)));
    LZ_CK(cudaMalloc(&w->u, sizeof(int64_t) * (size_t)DW));
    LZ_CK(cudaMalloc(&w->fbuf, sizeof(double) * (size_t)DW));
    LZ_CK(cudaMalloc(&w->lz, sizeof(LzState)));
    std::memset(&w->h, 0, sizeof(LzState));
    LZ_CK(cudaMalloc(&w->h.e, sizeof(int) * ns));
    LZ_CK(cudaMalloc(&w->h.m, sizeof(uint64_t) * ns));
    LZ_CK(cudaMalloc(&w->h.beta, sizeof(double) * ns));
    LZ_CK(cudaMalloc(&w->h.alpha, sizeof(double) * ns));
    LZ_CK(cudaMalloc(&w->h.part_lo, sizeof(uint64_t) * kLzMaxPartials));
    LZ_CK(cudaMalloc(&w->h.part_hi, sizeof(uint64_t) * kLzMaxPartials));
    LZ_CK(cudaMalloc(&w->h.part_max, sizeof(uint64_t) * kLzMaxPartials));
    LZ_CK(cudaMalloc(&w->h.counter, sizeof(unsigned int) * 4));
    LZ_CK(cudaMemset(w->h.counter, 0, sizeof(unsigned int) * 4));
    LZ_CK(cudaMalloc(&w->emax, sizeof(int)));
    LZ_CK(cudaMalloc(&w->flag, sizeof(int)));
    LZ_CK(cudaMalloc(&w->dot_lo, sizeof(uint64_t) * ns * kDotChunks));
    LZ_CK(cudaMalloc(&w->dot_hi, sizeof(uint64_t) * ns * kDotChunks));
    LZ_CK(cudaMalloc(&w->coef_rt, sizeof(int64_t) * ns));
    LZ_CK(cudaMalloc(&w->coef_rs, sizeof(int) * ns));
    LZ_CK(cudaMalloc(&w->coef_F, sizeof(int)));
    LZ_CK(cudaMalloc(&w->ritz_part, sizeof(double) * kLzMaxPartials));
    LZ_CK(cudaMalloc(&w->ritz_ctr, sizeof(unsigned int)));
    LZ_CK(cudaMemset(w->ritz_ctr, 0, sizeof(unsigned int)));
    LZ_CK(cudaMalloc(&w->inv_norm, sizeof(double)));
    LZ_CK(cudaMalloc(&w->gbar, kFusedSync));
    {
        const uint64_t bound = (1ULL << kFxBits) - 1;
        LZ_CK(cudaMalloc(&w->fxbound, sizeof(uint64_t)));
        LZ_CK(cudaMemcpy(w->fxbound, &bound, sizeof(uint64_t), cudaMemcpyHostToDevice));
    }
    LZ_CK(cudaMalloc(&w->stamps, sizeof(unsigned long long) * kLzStamps * ns));
    LZ_CK(cudaMemcpy(w->lz, &w->h, sizeof(LzState), cudaMemcpyHostToDevice));
    return ED_OK;
}

// Integer coefficients rt_k, shifts rs_k and common fractional bits F for
// sum_k r_k q_k with real r_k (|q_k| < 2^54, at most 2^10 terms per 2^126).
void fx_coefs(const std::vector<double>& r, std::vector<int64_t>* rt, std::vector<int>* rs, int* Fout) {
    const int nk = (int)r.size();
    int extra = 0;
    while ((1 << (10 + extra)) < nk) ++extra;
    std::vector<int> F(nk, 0);
    int Fmin = 1 << 20;
    for (int k = 0; k < nk; ++k) {
        if (r[k] == 0.0) continue;
        int ka;
        std::frexp(std::fabs(r[k]), &ka);
        F[k] = 62 - ka - extra;
        Fmin = std::min(Fmin, F[k]);
    }
    if (Fmin == (1 << 20)) Fmin = 0;
    rt->assign(nk, 0);
    rs->assign(nk, 0);
    for (int k = 0; k < nk; ++k) {
        if (r[k] == 0.0 || F[k] - Fmin >= 120) continue;
        (*rt)[k] = (int64_t)std::llrint(std::ldexp(r[k], F[k]));
        (*rs)[k] = F[k] - Fmin;
    }
    *Fout = Fmin;
}

}  // namespace

}  // namespace ed

namespace ed {
namespace {
// The workspace hangs off the op handle through an opaque pointer so the
// allocation survives across runs (no cudaMalloc inside a timed solve).
struct WsHolder {
    Workspace ws;
};
}  // namespace

void lanczos_free_ws(void* p) {
    if (!p) return;
    WsHolder* h = reinterpret_cast<WsHolder*>(p);
    free_ws(&h->ws);
    delete h;
}

void lanczos_basis(void* ws_slot, const int64_t** basis, int64_t* stride, const int** e_dev) {
    Workspace* w = &reinterpret_cast<WsHolder*>(ws_slot)->ws;
    *basis = w->basis;
    *stride = w->stride;
    *e_dev = w->h.e;
}

// stop_beta >= 0: Krylov use (time evolution): the run ends at the first
// beta_k < stop_beta * beta_0 (tested every ten steps like the reference
// mode's stop test) and T is k x k.
ed_status lanczos_run(ed_op* op, void** ws_slot, const ed_lanczos_cfg* cfg, const double* start, int start_mem,
                      double* evec, int evec_mem, double* alpha_h, double* beta_h, ed_lanczos_result* res,
                      cudaStream_t s, double stop_beta) {
    if (!cfg || cfg->max_steps < 1 || cfg->max_steps > 100000) return ED_ERR_ARG;
    const int W = op->cplx ? 2 : 1;
    const int64_t DW = op->D * W;
    const int max_steps = cfg->max_steps;
    // with reorthogonalisation the basis is stored anyway, and its Ritz sum
    // replaces the second pass
    const bool stored = cfg->ritz == ED_RITZ_STORED || cfg->reorth;
    const int ritz = (cfg->ritz == ED_RITZ_RECOMPUTE && cfg->reorth) ? ED_RITZ_STORED : cfg->ritz;
    const size_t slots = stored ? (size_t)max_steps + 1 : 3;
    if (!*ws_slot) *ws_slot = new WsHolder();
    Workspace* w = &reinterpret_cast<WsHolder*>(*ws_slot)->ws;
    ed_status st = ensure_ws(op, w, slots, DW, max_steps);
    if (st != ED_OK) return st;
    LzState* lz = w->lz;
    const LzState& H = w->h;
    int64_t launches = 0;
    const bool prof = cfg->profile == 1;     // per-step kernels timed with events
    const bool stamps = cfg->profile == 2;   // persistent kernel with phase timestamps
    const size_t need_ev = prof ? (size_t)4 * max_steps : (stamps ? (size_t)2 * (max_steps / 10 + 2) : 0);
    while (w->events.size() < need_ev) {
        cudaEvent_t e;
        LZ_CK(cudaEventCreate(&e));
        w->events.push_back(e);
    }
    auto slot = [&](int j) -> int64_t* { return w->basis + (size_t)(stored ? j : j % 3) * (size_t)w->stride; };

    // a failed earlier call may have left a last-block counter mid-count
    LZ_CK(cudaMemsetAsync(H.counter, 0, sizeof(unsigned int) * 4, s));
    LZ_CK(cudaMemsetAsync(w->ritz_ctr, 0, sizeof(unsigned int), s));
    // start vector
    if (cfg->start == ED_START_USER) {
        if (!start) return ED_ERR_ARG;
        LZ_CK(cudaMemcpyAsync(w->fbuf, start, sizeof(double) * DW,
                              start_mem == ED_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s));
    } else {
        LZ_CK(launch_random(w->fbuf, DW, cfg->seed, s));
        ++launches;
    }
    // the two-pass matvec works in its permuted down order: the start vector
    // is permuted into the u buffer (free until the first matvec)
    const double* start_vec = w->fbuf;
    if (op->striped) {
        LZ_CK(launch_permute_f64(op, w->fbuf, reinterpret_cast<double*>(w->u), 1, s));
        start_vec = reinterpret_cast<const double*>(w->u);
        ++launches;
    }
    LZ_CK(launch_emax(start_vec, DW, w->emax, w->flag, s));
    k_lz_start<<<lz_grid(DW), kLzThreads, 0, s>>>(start_vec, DW, w->emax, w->flag, slot(0), lz);
    LZ_CK(cudaGetLastError());
    launches += 2;

    const double eps = 2.220446049250313e-16;
    const double tolconv = 0.01 * std::sqrt(eps);
    std::vector<double> ha(max_steps + 2), hb(max_steps + 2);
    int n = max_steps;
    bool converged = false;
    double e0 = 0.0, resid = 0.0;
    std::vector<double> tri(max_steps + 2);
    int status_dev = 0;

    // The reference stop test on steps 0 .. nn-1 (HubMatrix_GPU.cuh:585-597):
    // the lowest Ritz pair of T_nn, converged when its residual estimate
    // |beta_nn z_{nn-1}| is below tolconv * anorm.
    auto ref_test = [&](int nn, const double* A, const double* Bv) -> bool {
        double anorm = std::fabs(A[0] + Bv[1]);
        for (int k = 1; k < nn; ++k) anorm = std::max(anorm, Bv[k] + std::fabs(A[k] + Bv[k + 1]));
        tri[0] = tridiag_lowest_host(nn, A, Bv + 1, tri.data() + 1);
        e0 = tri[0];
        return std::fabs(Bv[nn] * tri[nn]) < tolconv * anorm && std::fabs(tri[1]) > tolconv * anorm;
    };

    // Steps run in the persistent kernel for real single-class operators
    // whose down table fits shared memory as a gather schedule, unless
    // reorthogonalisation or per-step timing asks for the per-step kernels.
    // In the reference mode one launch runs every step while the host does
    // the stop test every ten steps on the alpha and beta the kernel mirrors
    // into mapped memory, and a host stop word ends the launch (a few steps
    // after the test passes; T and the Ritz vector use the first n only).
    // The tridiagonal eigensolve stays on the host: on this chip FP64 runs at
    // 1/64 of the FP32 rate, and one device thread's Sturm bisection of a
    // 300-step T takes milliseconds against ~0.1 ms on the host cores.  ED_LZ_FUSED=0 never uses it, ED_LZ_FUSED=1 also
    // for the other operators with a shared-memory plan (complex, several
    // classes), where the per-step kernels measured faster.
    const char* fz = std::getenv("ED_LZ_FUSED");
    const bool force = fz && fz[0] == '1', never = fz && fz[0] == '0';
    // ed_op_autotune's choice, when made, replaces the default rule
    const bool rule = fz ? (force || op->mv.dnSched != nullptr)
                         : (op->lz_mode == 2 || (op->lz_mode == 0 && op->mv.dnSched != nullptr));
    bool fused = op->tma_smem > 0 && !cfg->reorth && !prof && !never && rule;
    int steps_run = 0;
    int n_fused = 0;  // persistent launches
    int j = 0;
    while (j < max_steps) {
        if (fused) {
            const bool host_stop = cfg->mode == ED_LANCZOS_REFERENCE && stop_beta < 0.0 && j == 0;
            const int j1 = (!host_stop && (cfg->mode == ED_LANCZOS_REFERENCE || stop_beta >= 0.0))
                               ? std::min(max_steps, (j / 10 + 1) * 10)
                               : max_steps;
            LZ_CK(cudaMemsetAsync(w->gbar, 0, kFusedSync, s));
            if (host_stop) {
                LZ_CK(ensure_mirror(w, max_steps));
                w->mirror_h->done = 0;
                w->mirror_h->stop = 0;
                std::atomic_thread_fence(std::memory_order_seq_cst);
            }
            LzRedSet* red = reinterpret_cast<LzRedSet*>(reinterpret_cast<char*>(w->gbar) + 32);
            if (stamps) {
                const size_t need = (size_t)2 * max_steps * (op->lz_grid > 0 ? op->lz_grid : op->tma_grid);
                if (w->cta_stamps_n < need) {
                    cudaFree(w->cta_stamps);
                    w->cta_stamps = nullptr;
                    w->cta_stamps_n = 0;
                    LZ_CK(cudaMalloc(&w->cta_stamps, sizeof(unsigned long long) * need));
                    w->cta_stamps_n = need;
                }
            }
            unsigned int* taken = reinterpret_cast<unsigned int*>(reinterpret_cast<char*>(w->gbar) + 160);
            int* stop_word = reinterpret_cast<int*>(reinterpret_cast<char*>(w->gbar) + 176);
            LzFusedArgs fa{w->basis, w->stride, stored ? 1 : 0, j, j1, w->u, DW, lz, w->gbar, red, taken,
                           stamps ? w->stamps : nullptr, stamps ? w->cta_stamps : nullptr, grid_wait_limits(),
                           host_stop ? w->mirror_d : nullptr, host_stop ? stop_word : nullptr};
            if (stamps) LZ_CK(cudaEventRecord(w->events[2 * n_fused], s));
            const cudaError_t e = launch_lz_fused(op, fa, s);
            if (e == cudaSuccess && stamps) LZ_CK(cudaEventRecord(w->events[2 * n_fused + 1], s));
            if (e == cudaErrorNotSupported || e == cudaErrorCooperativeLaunchTooLarge) {
                cudaGetLastError();
                fused = false;  // this device cannot hold the grid: per-step kernels
                continue;
            }
            LZ_CK(e);
            ++launches;
            ++n_fused;
            if (host_stop) {
                // the stop test at every tenth step as the kernel's mirror
                // reaches it; the first test that passes stops the launch
                int checked = 0;
                bool ended = false;
                for (;;) {
                    const int done = __atomic_load_n(&w->mirror_h->done, __ATOMIC_ACQUIRE);
                    while (!converged && checked + 10 <= done && checked + 10 <= max_steps) {
                        checked += 10;
                        if (ref_test(checked, w->mirror_alpha, w->mirror_beta)) {
                            converged = true;
                            n = checked;
                            __atomic_store_n(&w->mirror_h->stop, checked, __ATOMIC_RELEASE);
                        }
                    }
                    if (converged || ended) break;
                    const cudaError_t q = cudaStreamQuery(s);
                    if (q == cudaSuccess) {
                        ended = true;  // one more pass over the final count
                        continue;
                    }
                    if (q != cudaErrorNotReady) LZ_CK(q);
                    std::this_thread::yield();
                }
                LZ_CK(cudaStreamSynchronize(s));
                steps_run = __atomic_load_n(&w->mirror_h->done, __ATOMIC_ACQUIRE);  // steps the launch ran
                j = max_steps;
                break;
            }
            j = j1;
        } else {
            if (prof) LZ_CK(cudaEventRecord(w->events[4 * j], s));
            // output shift from the |q| < 2^54 bound (as the persistent kernel
            // does), or from the exact max when reorthogonalisation may have
            // changed the vector
            LZ_CK(launch_matvec_lz(op, slot(j), w->u, lz, cfg->reorth ? H.m + j : w->fxbound, j, s));
            if (prof) LZ_CK(cudaEventRecord(w->events[4 * j + 1], s));
            const int64_t* pj = j > 0 ? slot(j - 1) : slot(j);
            if (prof) LZ_CK(cudaEventRecord(w->events[4 * j + 2], s));
            k_lz_axpy<<<lz_grid(DW), kLzThreads, 0, s>>>(w->u, slot(j), pj, slot(j + 1), DW, lz, j);
            LZ_CK(cudaGetLastError());
            if (prof) LZ_CK(cudaEventRecord(w->events[4 * j + 3], s));
            launches += 2;
            if (cfg->reorth) {
                // classical Gram-Schmidt, twice, against v_0..v_j
                const int nk = j + 1;
                // row chunks per dot: up to kDotChunks, ~2048 elements each
                // (exact integer sums: the split does not change them)
                const int chunks = (int)std::min<int64_t>(kDotChunks, std::max<int64_t>(1, (DW + 2047) / 2048));
                // the update sums nk basis vectors per element: four lanes
                // per element, so that small sectors still fill the GPU
                const int grr = (int)std::min<int64_t>(152 * 8, (DW * kReorthLanes + kLzThreads - 1) / kLzThreads);
                for (int pass = 0; pass < 2; ++pass) {
                    dim3 g(nk, chunks);
                    k_lz_dots<<<g, kLzThreads, 0, s>>>(w->basis, DW, w->stride, slot(j + 1), w->dot_lo, w->dot_hi);
                    LZ_CK(cudaGetLastError());
                    k_reorth_coefs<<<1, kLzThreads, 0, s>>>(w->dot_lo, w->dot_hi, nk, chunks, H.e, H.beta,
                                                            w->coef_rt, w->coef_rs, w->coef_F);
                    LZ_CK(cudaGetLastError());
                    k_lz_reorth<<<grr, kLzThreads, 0, s>>>(slot(j + 1), w->basis, DW, w->stride, nk,
                                                                   w->coef_rt, w->coef_rs, w->coef_F);
                    LZ_CK(cudaGetLastError());
                    launches += 1;
                    launches += 2;
                }
                k_lz_stats<<<lz_grid(DW), kLzThreads, 0, s>>>(slot(j + 1), DW, lz, j + 1);
                LZ_CK(cudaGetLastError());
                ++launches;
            }
            ++j;
        }
        steps_run = j;
        if (stop_beta >= 0.0 && j % 10 == 0 && j < max_steps) {
            LZ_CK(cudaMemcpyAsync(hb.data(), H.beta, sizeof(double) * (j + 1), cudaMemcpyDeviceToHost, s));
            LZ_CK(cudaMemcpyAsync(&status_dev, &lz->status, sizeof(int), cudaMemcpyDeviceToHost, s));
            LZ_CK(cudaStreamSynchronize(s));
            if (status_dev != 0) { n = j; break; }
            bool small = false;
            for (int k = 1; k <= j; ++k) small = small || hb[k] < stop_beta * hb[0];
            if (small) { n = j; break; }
        }
        if (cfg->mode == ED_LANCZOS_REFERENCE && j % 10 == 0) {
            const int nn = j;
            LZ_CK(cudaMemcpyAsync(ha.data(), H.alpha, sizeof(double) * nn, cudaMemcpyDeviceToHost, s));
            LZ_CK(cudaMemcpyAsync(hb.data(), H.beta, sizeof(double) * (nn + 1), cudaMemcpyDeviceToHost, s));
            LZ_CK(cudaMemcpyAsync(&status_dev, &lz->status, sizeof(int), cudaMemcpyDeviceToHost, s));
            LZ_CK(cudaStreamSynchronize(s));
            if (status_dev != 0) { n = nn; break; }
            if (ref_test(nn, ha.data(), hb.data())) {
                converged = true;
                n = nn;
                break;
            }
        }
    }

    // final T, status
    LzState hs;
    LZ_CK(cudaMemcpyAsync(&hs, lz, sizeof(LzState), cudaMemcpyDeviceToHost, s));
    LZ_CK(cudaMemcpyAsync(ha.data(), H.alpha, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    LZ_CK(cudaMemcpyAsync(hb.data(), H.beta, sizeof(double) * (n + 1), cudaMemcpyDeviceToHost, s));
    int err_flag = 0;
    LZ_CK(cudaMemcpyAsync(&err_flag, op->d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    LZ_CK(cudaStreamSynchronize(s));
    if (err_flag) {
        cudaMemset(op->d_err, 0, sizeof(int));
        return ED_ERR_TIMEOUT;
    }
    int status = hs.status;
    if (status == 7) {
        // breakdown: T is exact up to the first vanishing beta
        int nb = n;
        for (int k = 0; k < n; ++k)
            if (hb[k + 1] == 0.0) { nb = k + 1; break; }
        n = std::max(1, nb);
    } else if (status != 0) {
        return ED_ERR_NONFINITE;
    }
    if (stop_beta >= 0.0)
        for (int k = 1; k < n; ++k)
            if (hb[k] < stop_beta * hb[0]) { n = k; break; }
    tri[0] = tridiag_lowest_host(n, ha.data(), hb.data() + 1, tri.data() + 1);
    e0 = tri[0];
    resid = std::fabs(hb[n] * tri[n]);

    if (evec && ritz == ED_RITZ_STORED) {
        std::vector<int> ev(n);
        std::vector<uint64_t> mv(n);
        LZ_CK(cudaMemcpyAsync(ev.data(), H.e, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
        LZ_CK(cudaStreamSynchronize(s));
        std::vector<double> r(n);
        for (int k = 0; k < n; ++k) r[k] = tri[1 + k] / hb[k] * std::ldexp(1.0, ev[k]);
        std::vector<int64_t> rt;
        std::vector<int> rs;
        int F;
        fx_coefs(r, &rt, &rs, &F);
        LZ_CK(cudaMemcpyAsync(w->coef_rt, rt.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, s));
        LZ_CK(cudaMemcpyAsync(w->coef_rs, rs.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
        double* out = evec_mem == ED_MEM_DEVICE ? evec : w->fbuf;
        const int g = lz_grid(DW);
        // one pair of elements per thread where the grid allows
        int64_t gr = (DW / 2 + kLzThreads - 1) / kLzThreads;
        gr = std::max<int64_t>(1, std::min<int64_t>(gr, kLzMaxPartials));
        // in the two-pass matvec's permuted order the sum goes through u
        double* rv = op->striped ? reinterpret_cast<double*>(w->u) : out;
        k_ritz<<<(int)gr, kLzThreads, 0, s>>>(w->basis, DW, w->stride, n, w->coef_rt, w->coef_rs, F, rv, w->ritz_part,
                                        w->ritz_ctr, w->inv_norm);
        LZ_CK(cudaGetLastError());
        k_scale<<<g, kLzThreads, 0, s>>>(rv, DW, w->inv_norm);
        LZ_CK(cudaGetLastError());
        launches += 2;
        if (op->striped) {
            LZ_CK(launch_permute_f64(op, rv, out, 0, s));
            ++launches;
        }
        if (evec_mem != ED_MEM_DEVICE)
            LZ_CK(cudaMemcpyAsync(evec, out, sizeof(double) * DW, cudaMemcpyDeviceToHost, s));
        LZ_CK(cudaStreamSynchronize(s));
    }
    if (evec && ritz == ED_RITZ_RECOMPUTE) {
        // The reference's second pass (HubMatrix_GPU.cuh:600-612): the same
        // start vector and the same deterministic recurrence regenerate
        // w_0 .. w_{n-1} bit for bit; each is added to the Ritz sum with
        // weight z_k / beta_k as soon as it exists.
        std::vector<int> ev(n);
        LZ_CK(cudaMemcpyAsync(ev.data(), H.e, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
        LZ_CK(cudaStreamSynchronize(s));
        std::vector<double> r(n);
        for (int k = 0; k < n; ++k) r[k] = tri[1 + k] / hb[k] * std::ldexp(1.0, ev[k]);
        std::vector<int64_t> rt;
        std::vector<int> rs;
        int F;
        fx_coefs(r, &rt, &rs, &F);
        LZ_CK(cudaMemcpyAsync(w->coef_rt, rt.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, s));
        LZ_CK(cudaMemcpyAsync(w->coef_rs, rs.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
        LZ_CK(cudaMemsetAsync(H.counter, 0, sizeof(unsigned int) * 4, s));
        const double* sv = w->fbuf;
        if (op->striped) {
            LZ_CK(launch_permute_f64(op, w->fbuf, reinterpret_cast<double*>(w->u), 1, s));
            sv = reinterpret_cast<const double*>(w->u);
        }
        LZ_CK(launch_emax(sv, DW, w->emax, w->flag, s));
        k_lz_start<<<lz_grid(DW), kLzThreads, 0, s>>>(sv, DW, w->emax, w->flag, slot(0), lz);
        LZ_CK(cudaGetLastError());
        // the start vector in fbuf is consumed: fbuf can hold the sum
        double* out = evec_mem == ED_MEM_DEVICE ? evec : w->fbuf;
        const int g = lz_grid(DW);
        k_ritz_acc<<<g, kLzThreads, 0, s>>>(out, slot(0), DW, w->coef_rt, w->coef_rs, F, 0, 1);
        LZ_CK(cudaGetLastError());
        launches += 3;
        for (int k = 0; k + 1 < n; ++k) {
            LZ_CK(launch_matvec_lz(op, slot(k), w->u, lz, w->fxbound, k, s));
            const int64_t* pk = k > 0 ? slot(k - 1) : slot(k);
            k_lz_axpy<<<g, kLzThreads, 0, s>>>(w->u, slot(k), pk, slot(k + 1), DW, lz, k);
            LZ_CK(cudaGetLastError());
            k_ritz_acc<<<g, kLzThreads, 0, s>>>(out, slot(k + 1), DW, w->coef_rt, w->coef_rs, F, k + 1, 0);
            LZ_CK(cudaGetLastError());
            launches += 3;
        }
        k_inv_norm<<<g, kLzThreads, 0, s>>>(out, DW, w->ritz_part, w->ritz_ctr, w->inv_norm);
        LZ_CK(cudaGetLastError());
        k_scale<<<g, kLzThreads, 0, s>>>(out, DW, w->inv_norm);
        LZ_CK(cudaGetLastError());
        launches += 2;
        if (op->striped) {
            // back to the table order of the down index
            double* tmp = reinterpret_cast<double*>(w->u);
            LZ_CK(launch_permute_f64(op, out, tmp, 0, s));
            LZ_CK(cudaMemcpyAsync(out, tmp, sizeof(double) * DW, cudaMemcpyDeviceToDevice, s));
            ++launches;
        }
        if (evec_mem != ED_MEM_DEVICE)
            LZ_CK(cudaMemcpyAsync(evec, out, sizeof(double) * DW, cudaMemcpyDeviceToHost, s));
        int err2 = 0;
        LZ_CK(cudaMemcpyAsync(&err2, op->d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
        LZ_CK(cudaStreamSynchronize(s));
        if (err2) {
            cudaMemset(op->d_err, 0, sizeof(int));
            return ED_ERR_TIMEOUT;
        }
    }
    if (alpha_h) std::memcpy(alpha_h, ha.data(), sizeof(double) * n);
    if (beta_h) std::memcpy(beta_h, hb.data(), sizeof(double) * (n + 1));
    double mv_ms = 0.0, ax_ms = 0.0, rd_ms = 0.0, bar_ms = 0.0, sc_ms = 0.0, fz_ms = 0.0, rws_ms = 0.0, axs_ms = 0.0;
    if (prof) {
        LZ_CK(cudaStreamSynchronize(s));
        for (int j = 0; j < steps_run; ++j) {
            float a = 0.f, b = 0.f;
            LZ_CK(cudaEventElapsedTime(&a, w->events[4 * j], w->events[4 * j + 1]));
            LZ_CK(cudaEventElapsedTime(&b, w->events[4 * j + 2], w->events[4 * j + 3]));
            mv_ms += a;
            ax_ms += b;
        }
    } else if (stamps && n_fused > 0) {
        LZ_CK(cudaStreamSynchronize(s));
        for (int k = 0; k < n_fused; ++k) {
            float a = 0.f;
            LZ_CK(cudaEventElapsedTime(&a, w->events[2 * k], w->events[2 * k + 1]));
            fz_ms += a;
        }
        std::vector<unsigned long long> t((size_t)kLzStamps * steps_run);
        LZ_CK(cudaMemcpy(t.data(), w->stamps, sizeof(unsigned long long) * t.size(), cudaMemcpyDeviceToHost));
        auto ms = [](unsigned long long a, unsigned long long b) { return (double)(b - a) * 1e-6; };
        for (int j = 0; j < steps_run; ++j) {
            const unsigned long long* q = t.data() + (size_t)kLzStamps * j;
            mv_ms += ms(q[0], q[1]);
            ax_ms += ms(q[4], q[5]);
            rd_ms += ms(q[1], q[4]) + ms(q[5], q[8]);
            bar_ms += ms(q[2], q[3]) + ms(q[6], q[7]);
            sc_ms += ms(q[3], q[4]) + ms(q[7], q[8]);
        }
        const int G = op->lz_grid > 0 ? op->lz_grid : op->tma_grid;
        std::vector<unsigned long long> c((size_t)2 * steps_run * G);
        LZ_CK(cudaMemcpy(c.data(), w->cta_stamps, sizeof(unsigned long long) * c.size(), cudaMemcpyDeviceToHost));
        for (int j2 = 0; j2 < steps_run; ++j2)
            for (int ph = 0; ph < 2; ++ph) {
                const unsigned long long* q = c.data() + ((size_t)j2 * 2 + ph) * G;
                const auto mm = std::minmax_element(q, q + G);
                (ph ? axs_ms : rws_ms) += ms(*mm.first, *mm.second);
            }
    }
    if (res) {
        res->launches = launches;
        res->matvec_ms = mv_ms;
        res->axpy_ms = ax_ms;
        res->reduce_ms = rd_ms;
        res->barrier_ms = bar_ms;
        res->scalar_ms = sc_ms;
        res->fused_ms = fz_ms;
        res->rows_spread_ms = rws_ms;
        res->axpy_spread_ms = axs_ms;
        res->n_matvec = steps_run;
        res->e0 = e0;
        res->steps = n;
        res->converged = converged ? 1 : 0;
        res->status = status == 7 ? ED_ERR_BREAKDOWN : ED_OK;
        res->min_bits = hs.min_bits;
        res->residual = resid;
    }
    return ED_OK;
}


// Regenerate the vectors q_0 .. q_{n-1} of the last lanczos_run on this
// workspace (non-stored, per-step kernels: the same start vector, still in
// fbuf, and the same deterministic recurrence give them bit for bit) and
// hand each to visit(k, q_k) as soon as it exists (in the two-pass matvec's
// permuted down order for such operators).
ed_status lanczos_replay(ed_op* op, void* ws_slot, int n, const std::function<cudaError_t(int, const int64_t*)>& visit,
                         cudaStream_t s) {
    Workspace* w = &reinterpret_cast<WsHolder*>(ws_slot)->ws;
    if (n < 1 || n > w->max_steps || w->basis_slots < 3) return ED_ERR_ARG;
    const int64_t DW = w->DW;
    LzState* lz = w->lz;
    auto slot = [&](int j) -> int64_t* { return w->basis + (size_t)(j % 3) * (size_t)w->stride; };
    LZ_CK(cudaMemsetAsync(w->h.counter, 0, sizeof(unsigned int) * 4, s));
    const double* sv = w->fbuf;
    if (op->striped) {
        LZ_CK(launch_permute_f64(op, w->fbuf, reinterpret_cast<double*>(w->u), 1, s));
        sv = reinterpret_cast<const double*>(w->u);
    }
    LZ_CK(launch_emax(sv, DW, w->emax, w->flag, s));
    k_lz_start<<<lz_grid(DW), kLzThreads, 0, s>>>(sv, DW, w->emax, w->flag, slot(0), lz);
    LZ_CK(cudaGetLastError());
    LZ_CK(visit(0, slot(0)));
    for (int k = 0; k + 1 < n; ++k) {
        LZ_CK(launch_matvec_lz(op, slot(k), w->u, lz, w->fxbound, k, s));
        const int64_t* pk = k > 0 ? slot(k - 1) : slot(k);
        k_lz_axpy<<<lz_grid(DW), kLzThreads, 0, s>>>(w->u, slot(k), pk, slot(k + 1), DW, lz, k);
        LZ_CK(cudaGetLastError());
        LZ_CK(visit(k + 1, slot(k + 1)));
    }
    int err = 0;
    LZ_CK(cudaMemcpyAsync(&err, op->d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    LZ_CK(cudaStreamSynchronize(s));
    if (err) {
        cudaMemset(op->d_err, 0, sizeof(int));
        return ED_ERR_TIMEOUT;
    }
    return ED_OK;
}

// Row-engine variant of an operator's persistent Lanczos kernel.
static int lz_kind(const ed_op* o) {
    if (o->cplx) return o->mv_fast ? kKindCplxFast : (o->mv.upSegE ? kKindCplxSeg : kKindCplx);
    if (o->mv_fast) return o->mv.dnSched ? kKindRealSched : kKindRealFast;
    return o->mv.upSegE ? kKindRealSeg : kKindReal;
}

static bool same_tables(const ed_op* a, const ed_op* b) {
    return a->dimUP == b->dimUP && a->dimDN == b->dimDN && a->cplx == b->cplx && a->mask == b->mask &&
           a->tma_smem == b->tma_smem && lz_kind(a) == lz_kind(b) && a->tup.ent == b->tup.ent &&
           a->tup.len == b->tup.len && a->tup.npos == b->tup.npos && a->tdn.ent == b->tdn.ent &&
           a->tdn.len == b->tdn.len && a->tdn.npos == b->tdn.npos;
}

// B (<= kLzMultiMax) fixed-step Lanczos runs of operators of any sectors and
// kinds (each with a shared-memory plan, none on the two-pass matvec) in one
// persistent launch (k_lz_multi); starts, evecs, alpha and beta hold the
// instances one after another.  Then each run's T and Ritz vector as
// lanczos_run forms them from the stored basis.
static ed_status lanczos_multi_run(ed_op* const* ops, int B, const ed_lanczos_cfg* cfg, const double* starts,
                                   int start_mem, double* evecs, int evec_mem, double* alpha_h, double* beta_h,
                                   ed_lanczos_result* res, cudaStream_t s) {
    ed_op* op0 = ops[0];
    const int max_steps = cfg->max_steps;
    const bool want_ritz = cfg->ritz == ED_RITZ_STORED && evecs;
    std::vector<Workspace*> ws(B);
    std::vector<LzMultiInst> inst(B);
    std::vector<MvArgs> args(B);
    std::vector<int64_t> offs(B + 1, 0);
    int smem = 0;
    int64_t launches = 0;
    for (int b = 0; b < B; ++b) {
        ed_op* op = ops[b];
        if (op->tma_smem <= 0 || op->striped) return ED_ERR_NOT_BUILT;
        if (op->device != op0->device) return ED_ERR_ARG;
        const int64_t DW = op->D * (op->cplx ? 2 : 1);
        offs[b + 1] = offs[b] + DW;
        smem = std::max(smem, op->tma_smem);
        void** slot = lanczos_ws_slot(op);
        if (!*slot) *slot = new WsHolder();
        Workspace* w = &reinterpret_cast<WsHolder*>(*slot)->ws;
        ed_status st = ensure_ws(op, w, (size_t)max_steps + 1, DW, max_steps);
        if (st != ED_OK) return st;
        ws[b] = w;
        LZ_CK(cudaMemsetAsync(w->h.counter, 0, sizeof(unsigned int) * 4, s));
        LZ_CK(cudaMemsetAsync(w->ritz_ctr, 0, sizeof(unsigned int), s));
        if (cfg->start == ED_START_USER) {
            LZ_CK(cudaMemcpyAsync(w->fbuf, starts + offs[b], sizeof(double) * DW,
                                  start_mem == ED_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s));
        } else {
            LZ_CK(launch_random(w->fbuf, DW, cfg->seed + (uint64_t)b, s));
            ++launches;
        }
        LZ_CK(launch_emax(w->fbuf, DW, w->emax, w->flag, s));
        k_lz_start<<<lz_grid(DW), kLzThreads, 0, s>>>(w->fbuf, DW, w->emax, w->flag, w->basis, w->lz);
        LZ_CK(cudaGetLastError());
        launches += 2;
        int group = b;
        for (int c = 0; c < b; ++c)
            if (same_tables(ops[c], op)) { group = inst[c].group; break; }
        inst[b] = LzMultiInst{w->basis, w->u, w->lz, DW, w->stride, lz_kind(op), group, (int)op->dimUP, 0};
        args[b] = op->mv;
        args[b].err = op0->d_err;  // one error word for the launch
    }
    {
        const size_t sync_bytes = 128 + sizeof(unsigned int) * 2 * kLzMultiMax + sizeof(LzRedSet) * 4 * (size_t)B;
        unsigned char* sync = nullptr;
        LzMultiInst* dinst = nullptr;
        MvArgs* dargs = nullptr;
        if (cudaMallocAsync(&sync, sync_bytes, s) != cudaSuccess) return ED_ERR_ALLOC;
        if (cudaMallocAsync(&dinst, sizeof(LzMultiInst) * B, s) != cudaSuccess ||
            cudaMallocAsync(&dargs, sizeof(MvArgs) * B, s) != cudaSuccess) {
            cudaFreeAsync(sync, s);
            cudaFreeAsync(dinst, s);
            return ED_ERR_ALLOC;
        }
        cudaError_t le = cudaMemsetAsync(sync, 0, sync_bytes, s);
        if (le == cudaSuccess)
            le = cudaMemcpyAsync(dinst, inst.data(), sizeof(LzMultiInst) * B, cudaMemcpyHostToDevice, s);
        if (le == cudaSuccess) le = cudaMemcpyAsync(dargs, args.data(), sizeof(MvArgs) * B, cudaMemcpyHostToDevice, s);
        if (le == cudaSuccess) {
            // sync: barrier counter at 0, 2 * B queue counters at 128, then the reduction sets
            LzMultiArgs fa{dargs, dinst, B, 0, max_steps, smem, reinterpret_cast<unsigned int*>(sync),
                           reinterpret_cast<LzRedSet*>(sync + 128 + sizeof(unsigned int) * 2 * kLzMultiMax),
                           reinterpret_cast<unsigned int*>(sync + 128), grid_wait_limits()};
            int kinds = 0;
            for (int b = 0; b < B; ++b) kinds |= 1 << inst[b].kind;
            le = launch_lz_multi(op0->device, kinds, fa, s);
        }
        // the host copies of inst and args stay alive until the stream is synchronised below
        cudaFreeAsync(sync, s);
        cudaFreeAsync(dinst, s);
        cudaFreeAsync(dargs, s);
        if (le == cudaErrorNotSupported || le == cudaErrorCooperativeLaunchTooLarge) {
            cudaGetLastError();
            cudaStreamSynchronize(s);
            return ED_ERR_NOT_BUILT;
        }
        if (le != cudaSuccess) {
            cudaGetLastError();
            cudaStreamSynchronize(s);
            return ED_ERR_CUDA;
        }
        ++launches;
    }
    ed_status result = ED_OK;
    for (int b = 0; b < B && result == ED_OK; ++b) {
        Workspace* w = ws[b];
        const int64_t DW = offs[b + 1] - offs[b];
        const LzState& H = w->h;
        LzState hs;
        std::vector<double> ha(max_steps + 2), hb(max_steps + 2), tri(max_steps + 2);
        int n = max_steps, err_flag = 0;
        if (cudaMemcpyAsync(&hs, w->lz, sizeof(LzState), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaMemcpyAsync(ha.data(), H.alpha, sizeof(double) * n, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaMemcpyAsync(hb.data(), H.beta, sizeof(double) * (n + 1), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaMemcpyAsync(&err_flag, op0->d_err, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) {
            result = ED_ERR_CUDA;
            break;
        }
        if (err_flag) {
            cudaMemset(op0->d_err, 0, sizeof(int));
            result = ED_ERR_TIMEOUT;
            break;
        }
        if (hs.status == 7) {
            int nb = n;
            for (int k = 0; k < n; ++k)
                if (hb[k + 1] == 0.0) { nb = k + 1; break; }
            n = std::max(1, nb);
        } else if (hs.status != 0) {
            result = ED_ERR_NONFINITE;
            break;
        }
        tri[0] = tridiag_lowest_host(n, ha.data(), hb.data() + 1, tri.data() + 1);
        if (want_ritz) {
            std::vector<int> ev(n);
            if (cudaMemcpy(ev.data(), H.e, sizeof(int) * n, cudaMemcpyDeviceToHost) != cudaSuccess) {
                result = ED_ERR_CUDA;
                break;
            }
            std::vector<double> r(n);
            for (int k = 0; k < n; ++k) r[k] = tri[1 + k] / hb[k] * std::ldexp(1.0, ev[k]);
            std::vector<int64_t> rt;
            std::vector<int> rs;
            int F;
            fx_coefs(r, &rt, &rs, &F);
            double* out = evec_mem == ED_MEM_DEVICE ? evecs + offs[b] : w->fbuf;
            int64_t gr = (DW / 2 + kLzThreads - 1) / kLzThreads;
            gr = std::max<int64_t>(1, std::min<int64_t>(gr, kLzMaxPartials));
            if (cudaMemcpyAsync(w->coef_rt, rt.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, s) != cudaSuccess ||
                cudaMemcpyAsync(w->coef_rs, rs.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s) != cudaSuccess) {
                result = ED_ERR_CUDA;
                break;
            }
            k_ritz<<<(int)gr, kLzThreads, 0, s>>>(w->basis, DW, w->stride, n, w->coef_rt, w->coef_rs, F, out,
                                                  w->ritz_part, w->ritz_ctr, w->inv_norm);
            k_scale<<<lz_grid(DW), kLzThreads, 0, s>>>(out, DW, w->inv_norm);
            launches += 2;
            if (cudaGetLastError() != cudaSuccess) {
                result = ED_ERR_CUDA;
                break;
            }
            if (evec_mem != ED_MEM_DEVICE &&
                cudaMemcpyAsync(evecs + offs[b], out, sizeof(double) * DW, cudaMemcpyDeviceToHost, s) != cudaSuccess) {
                result = ED_ERR_CUDA;
                break;
            }
            if (cudaStreamSynchronize(s) != cudaSuccess) {
                result = ED_ERR_CUDA;
                break;
            }
        }
        if (alpha_h) std::memcpy(alpha_h + (size_t)b * max_steps, ha.data(), sizeof(double) * n);
        if (beta_h) std::memcpy(beta_h + (size_t)b * (max_steps + 1), hb.data(), sizeof(double) * (n + 1));
        if (res) {
            ed_lanczos_result& R = res[b];
            std::memset(&R, 0, sizeof(R));
            R.e0 = tri[0];
            R.steps = n;
            R.status = hs.status == 7 ? ED_ERR_BREAKDOWN : ED_OK;
            R.min_bits = hs.min_bits;
            R.residual = std::fabs(hb[n] * tri[n]);
            R.n_matvec = max_steps;
            R.launches = b == 0 ? launches : 0;
        }
    }
    cudaStreamSynchronize(s);
    return result;
}

// B fixed-step Lanczos runs in one persistent launch, each with its own
// workspace (the op's) and start vector; then each run's T and Ritz vector as
// lanczos_run forms them from the stored basis.  Operators that share their
// hopping tables (real, one class, gather schedule, B <= kLzBatchMax) run in
// k_lz_batch; any other mix of sectors and kinds in k_lz_multi
// (ED_LZ_BATCH=multi sends every batch there).
ed_status lanczos_batch_run(ed_op* const* ops, int B, const ed_lanczos_cfg* cfg, const double* starts, int start_mem,
                            double* evecs, int evec_mem, double* alpha_h, double* beta_h, ed_lanczos_result* res,
                            cudaStream_t s) {
    if (!ops || B < 1 || B > kLzMultiMax || !cfg || cfg->max_steps < 1 || cfg->max_steps > 100000) return ED_ERR_ARG;
    if (cfg->mode != ED_LANCZOS_FIXED || cfg->reorth || cfg->ritz == ED_RITZ_RECOMPUTE) return ED_ERR_ARG;
    if (cfg->start == ED_START_USER && !starts) return ED_ERR_ARG;
    ed_op* op0 = ops[0];
    for (int b = 0; b < B; ++b)
        if (!ops[b]) return ED_ERR_ARG;
    bool homogeneous = B <= kLzBatchMax;
    for (int b = 0; b < B && homogeneous; ++b) {
        const ed_op* o = ops[b];
        if (o->cplx || !o->mv_fast || !o->mv.dnSched || o->tma_smem <= 0 || o->striped || o->device != op0->device ||
            !same_tables(o, op0))
            homogeneous = false;
    }
    const char* force = std::getenv("ED_LZ_BATCH");
    if (!homogeneous || (force && std::strcmp(force, "multi") == 0))
        return lanczos_multi_run(ops, B, cfg, starts, start_mem, evecs, evec_mem, alpha_h, beta_h, res, s);
    const int64_t DW = op0->D;
    const int max_steps = cfg->max_steps;
    const bool want_ritz = cfg->ritz == ED_RITZ_STORED && evecs;
    std::vector<Workspace*> ws(B);
    std::vector<LzInst> inst(B);
    int64_t launches = 0;
    for (int b = 0; b < B; ++b) {
        ed_op* op = ops[b];
        void** slot = lanczos_ws_slot(op);
        if (!*slot) *slot = new WsHolder();
        Workspace* w = &reinterpret_cast<WsHolder*>(*slot)->ws;
        ed_status st = ensure_ws(op, w, (size_t)max_steps + 1, DW, max_steps);
        if (st != ED_OK) return st;
        ws[b] = w;
        LZ_CK(cudaMemsetAsync(w->h.counter, 0, sizeof(unsigned int) * 4, s));
        LZ_CK(cudaMemsetAsync(w->ritz_ctr, 0, sizeof(unsigned int), s));
        if (cfg->start == ED_START_USER) {
            LZ_CK(cudaMemcpyAsync(w->fbuf, starts + (size_t)b * DW, sizeof(double) * DW,
                                  start_mem == ED_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s));
        } else {
            LZ_CK(launch_random(w->fbuf, DW, cfg->seed + (uint64_t)b, s));
            ++launches;
        }
        LZ_CK(launch_emax(w->fbuf, DW, w->emax, w->flag, s));
        k_lz_start<<<lz_grid(DW), kLzThreads, 0, s>>>(w->fbuf, DW, w->emax, w->flag, w->basis, w->lz);
        LZ_CK(cudaGetLastError());
        launches += 2;
        const MvArgs& m = op->mv;
        inst[b] = LzInst{w->basis, w->u, w->lz, m.dUPq, m.dDNq, m.Uq, m.coefUP[0], m.coefDN[0], m.Fc,
                         m.unitUP, m.unitDN, m.mergeUD, m.nclsUP, m.nclsDN, m.bq_bits, 0};
    }
    // One persistent launch per range of instances; a range whose row
    // buffers do not fit shared memory is split in two.
    // Sync buffer: barrier counter at 0, item-queue counters at 64,
    // reduction sets at 128.
    std::function<ed_status(int, int)> run = [&](int b0, int b1) -> ed_status {
        const int Bn = b1 - b0;
        const size_t sync_bytes = 128 + sizeof(LzRedSet) * 4 * (size_t)Bn;
        unsigned char* sync = nullptr;
        LzInst* dinst = nullptr;
        if (cudaMallocAsync(&sync, sync_bytes, s) != cudaSuccess) return ED_ERR_ALLOC;
        if (cudaMallocAsync(&dinst, sizeof(LzInst) * Bn, s) != cudaSuccess) {
            cudaFreeAsync(sync, s);
            return ED_ERR_ALLOC;
        }
        cudaError_t le = cudaMemsetAsync(sync, 0, sync_bytes, s);
        if (le == cudaSuccess)
            le = cudaMemcpyAsync(dinst, inst.data() + b0, sizeof(LzInst) * Bn, cudaMemcpyHostToDevice, s);
        if (le == cudaSuccess) {
            LzBatchArgs fa{dinst, Bn, 0, max_steps, ws[0]->stride, DW, reinterpret_cast<unsigned int*>(sync),
                           reinterpret_cast<LzRedSet*>(sync + 128), reinterpret_cast<unsigned int*>(sync + 64),
                           grid_wait_limits()};
            le = launch_lz_batch(op0, fa, s);
        }
        cudaFreeAsync(sync, s);
        cudaFreeAsync(dinst, s);
        if (le == cudaSuccess) {
            ++launches;
            return ED_OK;
        }
        cudaGetLastError();
        if (le == cudaErrorNotSupported || le == cudaErrorCooperativeLaunchTooLarge) {
            if (Bn == 1) return ED_ERR_NOT_BUILT;
            const int mid = b0 + (Bn + 1) / 2;
            const ed_status st = run(b0, mid);
            return st != ED_OK ? st : run(mid, b1);
        }
        return ED_ERR_CUDA;
    };
    {
        const ed_status st = run(0, B);
        if (st != ED_OK) {
            cudaStreamSynchronize(s);
            return st;
        }
    }
    // every instance: T, status, Ritz vector
    ed_status result = ED_OK;
    for (int b = 0; b < B && result == ED_OK; ++b) {
        Workspace* w = ws[b];
        const LzState& H = w->h;
        LzState hs;
        std::vector<double> ha(max_steps + 2), hb(max_steps + 2), tri(max_steps + 2);
        int n = max_steps, err_flag = 0;
        if (cudaMemcpyAsync(&hs, w->lz, sizeof(LzState), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaMemcpyAsync(ha.data(), H.alpha, sizeof(double) * n, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaMemcpyAsync(hb.data(), H.beta, sizeof(double) * (n + 1), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaMemcpyAsync(&err_flag, op0->d_err, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) {
            result = ED_ERR_CUDA;
            break;
        }
        if (err_flag) {
            cudaMemset(op0->d_err, 0, sizeof(int));
            result = ED_ERR_TIMEOUT;
            break;
        }
        if (hs.status == 7) {
            int nb = n;
            for (int k = 0; k < n; ++k)
                if (hb[k + 1] == 0.0) { nb = k + 1; break; }
            n = std::max(1, nb);
        } else if (hs.status != 0) {
            result = ED_ERR_NONFINITE;
            break;
        }
        tri[0] = tridiag_lowest_host(n, ha.data(), hb.data() + 1, tri.data() + 1);
        if (want_ritz) {
            std::vector<int> ev(n);
            if (cudaMemcpy(ev.data(), H.e, sizeof(int) * n, cudaMemcpyDeviceToHost) != cudaSuccess) {
                result = ED_ERR_CUDA;
                break;
            }
            std::vector<double> r(n);
            for (int k = 0; k < n; ++k) r[k] = tri[1 + k] / hb[k] * std::ldexp(1.0, ev[k]);
            std::vector<int64_t> rt;
            std::vector<int> rs;
            int F;
            fx_coefs(r, &rt, &rs, &F);
            double* out = evec_mem == ED_MEM_DEVICE ? evecs + (size_t)b * DW : w->fbuf;
            int64_t gr = (DW / 2 + kLzThreads - 1) / kLzThreads;
            gr = std::max<int64_t>(1, std::min<int64_t>(gr, kLzMaxPartials));
            if (cudaMemcpyAsync(w->coef_rt, rt.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, s) != cudaSuccess ||
                cudaMemcpyAsync(w->coef_rs, rs.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s) != cudaSuccess) {
                result = ED_ERR_CUDA;
                break;
            }
            k_ritz<<<(int)gr, kLzThreads, 0, s>>>(w->basis, DW, w->stride, n, w->coef_rt, w->coef_rs, F, out,
                                                  w->ritz_part, w->ritz_ctr, w->inv_norm);
            k_scale<<<lz_grid(DW), kLzThreads, 0, s>>>(out, DW, w->inv_norm);
            launches += 2;
            if (cudaGetLastError() != cudaSuccess) {
                result = ED_ERR_CUDA;
                break;
            }
            if (evec_mem != ED_MEM_DEVICE &&
                cudaMemcpyAsync(evecs + (size_t)b * DW, out, sizeof(double) * DW, cudaMemcpyDeviceToHost, s) != cudaSuccess) {
                result = ED_ERR_CUDA;
                break;
            }
            if (cudaStreamSynchronize(s) != cudaSuccess) {
                result = ED_ERR_CUDA;
                break;
            }
        }
        if (alpha_h) std::memcpy(alpha_h + (size_t)b * max_steps, ha.data(), sizeof(double) * n);
        if (beta_h) std::memcpy(beta_h + (size_t)b * (max_steps + 1), hb.data(), sizeof(double) * (n + 1));
        if (res) {
            ed_lanczos_result& R = res[b];
            std::memset(&R, 0, sizeof(R));
            R.e0 = tri[0];
            R.steps = n;
            R.status = hs.status == 7 ? ED_ERR_BREAKDOWN : ED_OK;
            R.min_bits = hs.min_bits;
            R.residual = std::fabs(hb[n] * tri[n]);
            R.n_matvec = max_steps;
            R.launches = b == 0 ? launches : 0;
        }
    }
    cudaStreamSynchronize(s);
    return result;
}

}  // namespace ed
