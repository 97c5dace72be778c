// ed_matvec_striped.cu — two-pass matvec for sectors whose down rows do not
// fit in shared memory (Lieb18 9+9: 48,620 x 48,620, 18.9 GB per vector), for
// real operators with one coefficient class per spin.
//
// Inside this path the down index is in reverse Cuthill-McKee order (the
// vectors are permuted on the way in and out), so the down hops of column c
// stay within +-B of c (B = the order's bandwidth, 8,875 at Lieb18 after the
// hop-count sort below).
//
// Pass D (k_mv_down): row-major.  A work item is (row u, chunk of C columns);
//   the CTA copies the window x[u, c0-B .. c0+C+B) of the row into shared
//   memory with one bulk copy (consecutive chunks overlap, so most of it
//   comes from L2) and every column of the chunk sums its down-hop entries
//   from the window through a gather schedule (16-bit words: offset in the
//   chunk's window | sign << 15; at most two targets per bank pair in a
//   step, idle lanes on a zero slot; the columns are ordered by hop count
//   within blocks of 256 so that a warp's lanes have similar step counts; the
//   schedule is the same for every row and is read from L2, eight steps of
//   a column packed in one 16-byte load; a step adds the window value xor-ed
//   with its sign mask, and a column's count of negative entries is added
//   once).  Output: the exact int64 down sums S_dn.
// Pass U (k_mv_up): column stripes of kStripe columns, stripe-major over all
//   rows so that the stripe of x (dim_up x kStripe x 8 B) stays in L2 while
//   every row's up neighbours gather from it; a warp computes one row of a
//   stripe (two column pairs per lane, 16-byte loads), adds S_dn and the diagonal,
//   rounds once, and writes u (FX, Lanczos) or y (FP64, permuted order; the
//   operator apply keeps the table-order kernels).
// HBM traffic per matvec: pass D reads x and writes S_dn, pass U reads x,
// S_dn and writes the result: 5 x 8 B per element (vs 2 x 8 B ideal, and
// ~14 x 8 B when every up neighbour row is re-read from HBM).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "ed_device.cuh"
#include "ed_internal.hpp"
#include "ed_matvec_common.cuh"
#include "ed_matvec_tma.cuh"

namespace ed {
using namespace dev;

constexpr int kStripe = 128;       // columns of a pass-U stripe (32 lanes x 4)
constexpr int kDownThreads = 1024;
constexpr int kUpThreads = 896;    // 28 warps (71 registers a thread): 28 rows of a stripe per item

// One schedule word holds two steps (16 bits each: window offset in bits
// 0..14, sign in bit 15; the even step in the low half).  A step adds
// (v ^ m) with m = 0 or -1 from its sign bit; the -m parts of a column, the
// number of its negative entries, are added once per column (g.negcnt).
// Byte offsets come out of a word in two operations and the sign mask in one
// (prmt replicating bit 15 or bit 31 over the word).
__device__ __forceinline__ uint32_t off_lo(uint32_t w) { return (w << 3) & 0x3FFF8u; }
__device__ __forceinline__ uint32_t off_hi(uint32_t w) { return (w >> 13) & 0x3FFF8u; }
__device__ __forceinline__ uint32_t sgn_lo(uint32_t w) {
    uint32_t m;
    asm("prmt.b32 %0, %1, 0, 0x9999;" : "=r"(m) : "r"(w));
    return m;
}
__device__ __forceinline__ uint32_t sgn_hi(uint32_t w) { return (uint32_t)((int32_t)w >> 31); }

// v ^ (m, m): the 64-bit term of one step
__device__ __forceinline__ uint64_t dterm(const unsigned char* winb, uint32_t off, uint32_t m) {
    const uint64_t v = *reinterpret_cast<const uint64_t*>(winb + off);
    uint64_t mm;
    asm("mov.b64 %0, {%1, %1};" : "=l"(mm) : "r"(m));
    return v ^ mm;
}

// The eight steps of one lane-packed 16-byte schedule group.
__device__ __forceinline__ uint64_t dgroup8(const unsigned char* winb, const uint4 w) {
    const uint64_t a = dterm(winb, off_lo(w.x), sgn_lo(w.x)) + dterm(winb, off_hi(w.x), sgn_hi(w.x));
    const uint64_t b = dterm(winb, off_lo(w.y), sgn_lo(w.y)) + dterm(winb, off_hi(w.y), sgn_hi(w.y));
    const uint64_t c = dterm(winb, off_lo(w.z), sgn_lo(w.z)) + dterm(winb, off_hi(w.z), sgn_hi(w.z));
    const uint64_t d = dterm(winb, off_lo(w.w), sgn_lo(w.w)) + dterm(winb, off_hi(w.w), sgn_hi(w.w));
    return (a + b) + (c + d);
}

// The first rem (0..7) steps of a group: one jump into the unrolled steps
// (rem is the same for the 32 lanes of a warp).
__device__ __forceinline__ uint64_t dtail(const unsigned char* winb, const uint4 w, int rem) {
    uint64_t acc = 0;
    switch (rem) {
        case 7: acc += dterm(winb, off_lo(w.w), sgn_lo(w.w)); [[fallthrough]];
        case 6: acc += dterm(winb, off_hi(w.z), sgn_hi(w.z)); [[fallthrough]];
        case 5: acc += dterm(winb, off_lo(w.z), sgn_lo(w.z)); [[fallthrough]];
        case 4: acc += dterm(winb, off_hi(w.y), sgn_hi(w.y)); [[fallthrough]];
        case 3: acc += dterm(winb, off_lo(w.y), sgn_lo(w.y)); [[fallthrough]];
        case 2: acc += dterm(winb, off_hi(w.x), sgn_hi(w.x)); [[fallthrough]];
        case 1: acc += dterm(winb, off_lo(w.x), sgn_lo(w.x)); [[fallthrough]];
        default: break;
    }
    return acc;
}

// ---------------------------------------------------------------- pass D --
__global__ void __launch_bounds__(kDownThreads, 1) k_mv_down(const StripedArgs g) {
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ int give_up;
    int64_t* win = reinterpret_cast<int64_t*>(sm);
    const int64_t dimDN = g.dimDN;
    const int64_t nchunk = (dimDN + g.chunk - 1) / g.chunk;
    const int64_t nitems = g.dimUP * nchunk;
    const int tid = threadIdx.x;
    if (tid == 0) {
        tma::mbar_init(&bar, 1);
        tma::fence_mbar_init();
        give_up = 0;
    }
    if (tid < 16) win[g.zbase + tid] = 0;  // never written by a window copy
    __syncthreads();
    uint32_t phase = 0;
    for (int64_t it = blockIdx.x; it < nitems; it += gridDim.x, phase ^= 1) {
        const int64_t u = it / nchunk, k = it - u * nchunk;
        const int64_t c0 = k * g.chunk, c1 = min(c0 + (int64_t)g.chunk, dimDN);
        const int64_t w0 = max((int64_t)0, c0 - g.bw) & ~(int64_t)15;
        int64_t w1 = min(dimDN, c1 + g.bw);
        w1 = (w1 + 1) & ~(int64_t)1;  // dim_dn is even: 16-byte copy sizes
        if (tid == 0) {
            tma::fence_proxy_async_smem();
            const uint32_t bytes = (uint32_t)((w1 - w0) * 8);
            tma::expect_tx(&bar, bytes);
            tma::bulk_g2s(win, g.xq + u * dimDN + w0, bytes, &bar);
        }
        if (!tma::mbar_wait(&bar, phase)) {
            if (tid == 0) atomicExch(g.err, 1);
            give_up = 1;
        }
        __syncthreads();
        if (give_up) {
            // the window copy (the only one in flight) must land before the
            // CTA leaves: wait for it once more (bounded)
            if (tid == 0) tma::mbar_wait(&bar, phase);
            return;
        }
        if (tid == 32 && it + gridDim.x < nitems) {
            // the next item's window into L2 while this one is summed, so
            // that its copy into shared memory does not wait on HBM
            const int64_t itn = it + gridDim.x, un = itn / nchunk, kn = itn - un * nchunk;
            const int64_t c0n = kn * g.chunk, c1n = min(c0n + (int64_t)g.chunk, dimDN);
            const int64_t w0n = max((int64_t)0, c0n - g.bw) & ~(int64_t)15;
            int64_t w1n = min(dimDN, c1n + g.bw);
            w1n = (w1n + 1) & ~(int64_t)1;
            asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(g.xq + un * dimDN + w0n),
                         "r"((uint32_t)((w1n - w0n) * 8))
                         : "memory");
        }
        // one column per iteration: its step count, negative-entry count and
        // first two schedule groups are loaded together, each later group one
        // group ahead of its use
        const unsigned char* winb = sm;
        const uint4* sched = reinterpret_cast<const uint4*>(g.sched16);
        for (int64_t c = c0 + tid; c < c1; c += kDownThreads) {
            const uint4* sp = sched + (size_t)(c >> 5) * (size_t)g.s8 * 32 + (c & 31);
            const int n = __ldg(g.steps32 + (c >> 5));
            uint64_t acc = __ldg(g.negcnt + c);
            uint4 cur = __ldg(sp), nxt = make_uint4(0u, 0u, 0u, 0u);
            if (g.s8 > 1) nxt = __ldg(sp + 32);
            const int full = n >> 3;
            for (int q = 0; q < full; ++q) {
                acc += dgroup8(winb, cur);
                cur = nxt;
                if (q + 2 < g.s8) nxt = __ldg(sp + 32 * (q + 2));
            }
            acc += dtail(winb, cur, n & 7);
            g.sdn[u * dimDN + c] = (int64_t)acc;
        }
        __syncthreads();  // the window is free for the next copy
    }
}

// ---------------------------------------------------------------- pass U --
// Column-stripe-major items: item = stripe * dim_up + row, one warp each;
// warp w of CTA b takes items b * 28 + w, + 28 * gridDim.x, ...  A lane
// holds two column pairs 64 columns apart (c, c + 1 and c + 64, c + 65), so
// each 16-byte load instruction of the warp reads one contiguous 512-byte
// segment; the second pair is absent past the end of the row.  Row offsets
// are 32-bit element offsets (a vector has < 2^32 elements).
template <int OUT>
__global__ void __launch_bounds__(kUpThreads, 1) k_mv_up(const MvArgs a, const StripedArgs g) {
    const int64_t dimUP = g.dimUP, dimDN = g.dimDN;
    const uint32_t dn32 = (uint32_t)dimDN;
    const int64_t nstripe = (dimDN + kStripe - 1) / kStripe;
    const int64_t nitems = nstripe * dimUP;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t nwarps = (int64_t)gridDim.x * (kUpThreads / 32);
    const int64_t* __restrict__ xq = g.xq;
    int E_out = 0, s_u = 0;
    if (OUT == 0) {
        E_out = fx_exp_from_emax(*a.p_emax) - a.Fc;
    } else {
        const int b = a.bq_bits + bitlen_u64(*a.p_mx) - 62;
        s_u = b > 0 ? b : 0;
    }
    const bool merge = a.mergeUD != 0;
    const bool unitU = a.unitUP != 0 && a.nclsUP == 1;
    const bool unitD = a.unitDN != 0 && a.nclsDN == 1;
    i128 dot = 0;
    uint64_t mx = 0;
    for (int64_t it = (int64_t)blockIdx.x * (kUpThreads / 32) + warp; it < nitems; it += nwarps) {
        const int64_t st = it / dimUP, u = it - st * dimUP;
        const uint32_t c = (uint32_t)(st * kStripe) + 2u * (uint32_t)lane;  // dim_dn is even
        if (c >= dn32) continue;
        const bool two = c + 64u < dn32;  // the second pair of columns exists
        const uint32_t rowu = (uint32_t)u * dn32 + c;
        // the row's down sums (streamed from HBM) are prefetched into L2 by one
        // bulk prefetch now and read after the gathers, with the row's own
        // values (in the L2-resident stripe): no registers held across the
        // gathers for them, which leaves room for 28 warps per SM
        if (lane == 0) {
            const uint32_t c0 = (uint32_t)(st * kStripe);
            const uint32_t nb = ((dn32 - c0 < (uint32_t)kStripe ? dn32 - c0 : (uint32_t)kStripe) * 8u) & ~15u;
            if (nb)
                asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(g.sdn + (uint32_t)u * dn32 + c0),
                             "r"(nb)
                             : "memory");
        }
        const uint32_t p0 = __ldg(a.upPtr + u), len = __ldg(a.upPtr + u + 1) - p0;
        const int npos = (int)__ldg(a.upNpos + u);
        int64_t sp[4] = {0, 0, 0, 0};  // + neighbours added, - neighbours subtracted
        int k = 0;
#pragma unroll 4
        for (; k < npos; ++k) {
            const uint32_t o = (__ldg(a.upEntC + p0 + k) & kColMask) * dn32 + c;
            const longlong2 v0 = __ldcg(reinterpret_cast<const longlong2*>(xq + o));
            const longlong2 v1 = two ? __ldcg(reinterpret_cast<const longlong2*>(xq + o + 64u)) : make_longlong2(0, 0);
            sp[0] += v0.x;
            sp[1] += v0.y;
            sp[2] += v1.x;
            sp[3] += v1.y;
        }
#pragma unroll 4
        for (; k < (int)len; ++k) {
            const uint32_t o = (__ldg(a.upEntC + p0 + k) & kColMask) * dn32 + c;
            const longlong2 v0 = __ldcg(reinterpret_cast<const longlong2*>(xq + o));
            const longlong2 v1 = two ? __ldcg(reinterpret_cast<const longlong2*>(xq + o + 64u)) : make_longlong2(0, 0);
            sp[0] -= v0.x;
            sp[1] -= v0.y;
            sp[2] -= v1.x;
            sp[3] -= v1.y;
        }
        longlong2 dsv[2], xs[2];
        dsv[0] = __ldcs(reinterpret_cast<const longlong2*>(g.sdn + rowu));
        xs[0] = __ldcg(reinterpret_cast<const longlong2*>(xq + rowu));
        if (two) {
            dsv[1] = __ldcs(reinterpret_cast<const longlong2*>(g.sdn + rowu + 64u));
            xs[1] = __ldcg(reinterpret_cast<const longlong2*>(xq + rowu + 64u));
        } else {
            dsv[1] = make_longlong2(0, 0);
            xs[1] = dsv[1];
        }
        const uint64_t stu = __ldg(a.stUP + u);
        const int64_t du = __ldg(a.dUPq + u);
        // the two column pairs one after the other, each stored at once
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (h == 1 && !two) break;
            int64_t oq[2];
            double of[2];
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int q = 2 * h + e;
                const int64_t dn_sum = e ? dsv[h].y : dsv[h].x;
                const int64_t xv = e ? xs[h].y : xs[h].x;
                i128 ar = 0, ai = 0;
                if (merge) {
                    apply_class<false>(ar, ai, sp[q] + dn_sum, 0, a.coefUP, 0, unitU, a.Fc);
                } else {
                    if (len) apply_class<false>(ar, ai, sp[q], 0, a.coefUP, 0, unitU, a.Fc);
                    if (a.nclsDN) apply_class<false>(ar, ai, dn_sum, 0, a.coefDN, 0, unitD, a.Fc);
                }
                const uint32_t cq = c + 64u * h + e;
                const int64_t dq = du + __ldg(g.dDNq + cq) + a.Uq * (int64_t)__popcll(stu & __ldg(g.stDN + cq) & a.mask);
                ar += mul_wide(dq, xv);
                if (OUT == 0) {
                    of[e] = i128_to_f64(ar, E_out);
                } else {
                    oq[e] = shr_round_i64(ar, s_u);
                    dot += mul_wide(xv, oq[e]) >> 24;
                    const uint64_t aq = (uint64_t)(oq[e] < 0 ? -oq[e] : oq[e]);
                    mx = aq > mx ? aq : mx;
                }
            }
            if (OUT == 0) {
                // the FP64 result overwrites S_dn in place (permuted order)
                *reinterpret_cast<double2*>(g.sdn + rowu + 64u * h) = make_double2(of[0], of[1]);
            } else {
                __stcs(reinterpret_cast<longlong2*>(a.uq + rowu + 64u * h), make_longlong2(oq[0], oq[1]));
            }
        }
    }
    if (OUT == 1) mv_lanczos_epilogue(a, dot, mx, s_u);
}

// ---------------------------------------------------- down-index permutes --
// out[u, c'] = in[u, perm[c']] (forward: table order -> permuted order) or
// out[u, perm[c']] = in[u, c'] (back).  Grid-stride over elements, so each
// row's random reads or writes stay within one L2-resident row.
template <typename T>
__global__ void k_permute_rows(const T* __restrict__ in, T* __restrict__ out, int64_t dimUP, int64_t dimDN,
                               const uint32_t* __restrict__ perm, int forward) {
    const int64_t D = dimUP * dimDN;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t u = i / dimDN, c = i - u * dimDN;
        const int64_t p = u * dimDN + __ldg(perm + c);
        if (forward) out[i] = in[p];
        else out[p] = in[i];
    }
}

// xq[u, c'] = FX(x[u, perm[c']]) at the exponent of d_emax
__global__ void k_to_fx_perm(const double* __restrict__ x, int64_t dimUP, int64_t dimDN,
                             const uint32_t* __restrict__ perm, const int* __restrict__ emax, int64_t* __restrict__ xq) {
    const int E = fx_exp_from_emax(*emax);
    const int64_t D = dimUP * dimDN;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t u = i / dimDN, c = i - u * dimDN;
        xq[i] = f64_to_fx(x[u * dimDN + __ldg(perm + c)], E);
    }
}

static int grid_of(int64_t n) {
    int64_t g = (n + 255) / 256;
    return (int)std::max<int64_t>(1, std::min<int64_t>(g, 152 * 16));
}

cudaError_t launch_striped_down(const ed_op* op, const StripedArgs& g, cudaStream_t s) {
    const int smem = op->st_win * 8;
    cudaError_t e = cudaFuncSetAttribute(k_mv_down, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    k_mv_down<<<op->st_grid, kDownThreads, smem, s>>>(g);
    return cudaGetLastError();
}

cudaError_t launch_striped_up(const ed_op* op, const MvArgs& a, const StripedArgs& g, int out, cudaStream_t s) {
    if (out == 0) k_mv_up<0><<<op->st_grid, kUpThreads, 0, s>>>(a, g);
    else k_mv_up<1><<<op->st_grid, kUpThreads, 0, s>>>(a, g);
    return cudaGetLastError();
}

cudaError_t launch_permute_f64(const ed_op* op, const double* in, double* out, int forward, cudaStream_t s) {
    k_permute_rows<double><<<grid_of(op->D), 256, 0, s>>>(in, out, op->dimUP, op->dimDN, op->d_permDN, forward);
    return cudaGetLastError();
}

cudaError_t launch_permute_i64(const ed_op* op, const int64_t* in, int64_t* out, int forward, cudaStream_t s) {
    k_permute_rows<int64_t><<<grid_of(op->D), 256, 0, s>>>(in, out, op->dimUP, op->dimDN, op->d_permDN, forward);
    return cudaGetLastError();
}

cudaError_t launch_to_fx_perm(const ed_op* op, const double* x, const int* d_emax, int64_t* xq, cudaStream_t s) {
    k_to_fx_perm<<<grid_of(op->D), 256, 0, s>>>(x, op->dimUP, op->dimDN, op->d_permDN, d_emax, xq);
    return cudaGetLastError();
}

}  // namespace ed
