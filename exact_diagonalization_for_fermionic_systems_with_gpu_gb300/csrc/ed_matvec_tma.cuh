// ed_matvec_tma.cuh — the shared-memory row engine of the matvec, used by the
// one-launch matvec (ed_matvec_tma.cu) and by the persistent Lanczos kernel
// (ed_lanczos_fused.cu).
//
// A CTA of kTmaThreads threads
//  * holds the whole down-spin operator (CSR entries, row pointers, npos,
//    folded diagonal, bitstrings) in shared memory, moved there by TMA bulk
//    copies (cp.async.bulk global->shared, completion counted on an mbarrier);
//  * walks the up-rows u = blockIdx.x, + gridDim.x, ... with x[u, :] double
//    buffered by bulk copies: row u+gridDim.x streams in while row u is
//    computed;
//  * computes the down term entirely from shared memory and the up term with
//    coalesced L2 loads, two output columns per thread so at least eight
//    up-term loads are in flight per thread.
// Every mbarrier wait is bounded: after kMaxSpin polls the CTA records an
// error in *err, waits (bounded) for its copies in flight and stops.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "ed_device.cuh"
#include "ed_internal.hpp"
#include "ed_matvec_common.cuh"

namespace ed {
using namespace dev;

constexpr int kTmaThreads = 512;
constexpr int kTmaUpStage = 256;  // longest up-row held in the static offset arrays
constexpr long long kMaxSpin = 1LL << 22;

namespace tma {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// generic-proxy accesses of shared memory before async-proxy writes into it
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// generic-proxy writes of global memory (observed by this thread) before
// async-proxy reads of it
__device__ __forceinline__ void fence_proxy_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }

__device__ __forceinline__ void expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// dst, src 16-byte aligned; bytes a multiple of 16
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// Bounded wait for the phase with the given parity; false when it gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    const uint32_t addr = smem_u32(bar);
    for (long long it = 0; it < kMaxSpin; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(addr), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__host__ __device__ constexpr uint32_t round16(uint32_t b) { return (b + 15u) / 16u * 16u; }

}  // namespace tma

// Shared-memory views: the dynamic area follows the byte offsets in MvArgs
// (barriers at 0: [0], [1] row buffers, [2] down tables); the up-row offsets
// and the give-up word are static arrays of the kernel.
struct TmaSmem {
    uint64_t* bar;
    int64_t* row0;
    int64_t* row1;
    uint32_t* dptr;
    uint32_t* dent;
    uint8_t* dnpos;
    int64_t* ddq;
    uint64_t* dst;
    uint16_t* sched;  // gather schedule (when a.dnSched)
    uint8_t* steps;
    uint32_t* uoff;
    uint32_t* uent;
    int* give_up;
};

__device__ __forceinline__ TmaSmem tma_view(const MvArgs& a, unsigned char* sm, uint32_t* uoff, uint32_t* uent,
                                            int* give_up) {
    TmaSmem S;
    S.bar = reinterpret_cast<uint64_t*>(sm);
    S.row0 = reinterpret_cast<int64_t*>(sm + a.sm_row0);
    S.row1 = reinterpret_cast<int64_t*>(sm + a.sm_row1);
    S.dptr = reinterpret_cast<uint32_t*>(sm + a.sm_dnptr);
    S.dent = reinterpret_cast<uint32_t*>(sm + a.sm_dnent);
    S.dnpos = sm + a.sm_dnnpos;
    S.ddq = reinterpret_cast<int64_t*>(sm + a.sm_ddnq);
    S.dst = reinterpret_cast<uint64_t*>(sm + a.sm_stdn);
    S.sched = reinterpret_cast<uint16_t*>(sm + a.sm_sched);
    S.steps = sm + a.sm_steps;
    S.uoff = uoff;
    S.uent = uent;
    S.give_up = give_up;
    return S;
}

// Thread 0: initialise the three barriers.
__device__ __forceinline__ void tma_init(const TmaSmem& S) {
    for (int k = 0; k < 3; ++k) tma::mbar_init(&S.bar[k], 1);
    tma::fence_mbar_init();
    *S.give_up = 0;
}

// Thread 0: start the copies of the down-spin tables (completion on bar[2]).
// The device tables are allocated in multiples of 16 bytes and the shared
// regions in multiples of 128, so every copy is rounded up to 16 bytes.
__device__ __forceinline__ void tma_issue_tables(const MvArgs& a, const TmaSmem& S) {
    const uint32_t dimDN = (uint32_t)a.dimDN;
    if (a.dnSched) {
        const uint32_t b_sc = tma::round16((uint32_t)a.schedSteps * (uint32_t)a.dimDNp * 2u),
                       b_stp = tma::round16((uint32_t)a.dimDNp / 32u), b_dq = tma::round16(dimDN * 8u);
        tma::expect_tx(&S.bar[2], b_sc + b_stp + 2 * b_dq);
        if (b_sc) tma::bulk_g2s(S.sched, a.dnSched, b_sc, &S.bar[2]);
        tma::bulk_g2s(S.steps, a.dnSteps, b_stp, &S.bar[2]);
        tma::bulk_g2s(S.ddq, a.dDNq, b_dq, &S.bar[2]);
        tma::bulk_g2s(S.dst, a.stDN, b_dq, &S.bar[2]);
        return;
    }
    const uint32_t b_ptr = tma::round16((dimDN + 1) * 4u), b_ent = tma::round16(a.dnNnz * 4u),
                   b_pos = tma::round16(dimDN), b_dq = tma::round16(dimDN * 8u), b_st = b_dq;
    tma::expect_tx(&S.bar[2], b_ptr + b_ent + b_pos + b_dq + b_st);
    tma::bulk_g2s(S.dptr, a.dnPtr, b_ptr, &S.bar[2]);
    if (b_ent) tma::bulk_g2s(S.dent, a.dnEntC, b_ent, &S.bar[2]);  // no down hops: nothing to copy
    tma::bulk_g2s(S.dnpos, a.dnNpos, b_pos, &S.bar[2]);
    tma::bulk_g2s(S.ddq, a.dDNq, b_dq, &S.bar[2]);
    tma::bulk_g2s(S.dst, a.stDN, b_st, &S.bar[2]);
}

// The 16 zeros of both row buffers that idle lanes of the gather schedule
// read (the bulk copies only ever write [0, dimDN)).
__device__ __forceinline__ void tma_zero_slots(const MvArgs& a, const TmaSmem& S) {
    if (threadIdx.x < 17) {  // 16 zeros after [x | -x] at either row offset
        S.row0[2 * a.schedNeg + threadIdx.x] = 0;
        S.row1[2 * a.schedNeg + threadIdx.x] = 0;
    }
}

// Offset (0 or 1 element) of row u inside its row buffer: a bulk copy starts
// on a 16-byte boundary, so with an odd dim_dn (real vectors) every other
// row is copied from the element before it.
template <bool CPLX>
__device__ __forceinline__ uint32_t tma_row_off(const MvArgs& a, uint32_t u) {
    return CPLX ? 0u : (uint32_t)(((uint64_t)u * (uint64_t)a.dimDN) & 1u);
}

// Thread 0: start the copy of row u of x into row buffer `buf`: the
// 16-byte-aligned run of whole 16-byte words around the row (one element
// before it when it starts at an odd index, one after it to round up; the
// vectors carry two elements of padding), the row at tma_row_off.
template <bool CPLX>
__device__ __forceinline__ void tma_issue_row(const MvArgs& a, const TmaSmem& S, const int64_t* xq, uint32_t u,
                                              int buf) {
    constexpr int W = CPLX ? 2 : 1;
    const uint32_t off = tma_row_off<CPLX>(a, u);
    const uint32_t n = CPLX ? (uint32_t)a.dimDN * 2u : (((uint32_t)a.dimDN + off + 1u) & ~1u);
    const uint32_t bytes = n * 8u;
    tma::expect_tx(&S.bar[buf], bytes);
    tma::bulk_g2s(buf ? S.row1 : S.row0, xq + (size_t)u * a.dimDN * W - off, bytes, &S.bar[buf]);
}

// Up-term element load: read-only path for a one-launch matvec, L2
// (coherent) loads when x was written earlier in the same launch.
template <bool CPLX, bool COH>
__device__ __forceinline__ void up_load(const int64_t* __restrict__ xq, uint32_t idx, int64_t& r, int64_t& i) {
    if (CPLX) {
        const longlong2* p = reinterpret_cast<const longlong2*>(xq) + idx;
        const longlong2 v = COH ? __ldcg(p) : __ldg(p);
        r = v.x;
        i = v.y;
    } else {
        r = COH ? __ldcg(xq + idx) : __ldg(xq + idx);
        i = 0;
    }
}

template <bool CPLX, bool COH>
__device__ __forceinline__ void acc_up(const int64_t* __restrict__ xq, uint32_t idx, int64_t& r, int64_t& i) {
    int64_t vr, vi;
    up_load<CPLX, COH>(xq, idx, vr, vi);
    r += vr;
    if (CPLX) i += vi;
}

// Element col of a staged row: one 16-byte shared load for a complex
// element (row buffers are 16-byte aligned and complex rows start at
// offset 0), one 8-byte load for a real one.
template <bool CPLX>
__device__ __forceinline__ void row_elem(const int64_t* xrow, uint32_t col, int64_t& r, int64_t& i) {
    if (CPLX) {
        const longlong2 v = *reinterpret_cast<const longlong2*>(xrow + col);
        r = v.x;
        i = v.y;
    } else {
        r = xrow[col];
        i = 0;
    }
}

// First row of this CTA (rowList[rowStart[b]]); false when it has none.
__device__ __forceinline__ bool tma_first_row(const MvArgs& a, uint32_t* u) {
    const uint32_t r0 = __ldg(a.rowStart + blockIdx.x);
    if (r0 >= __ldg(a.rowStart + blockIdx.x + 1)) return false;
    *u = __ldg(a.rowList + r0);
    return true;
}

// The rows of this CTA: u = H x (OUT 0: FP64 y with exponent E_out; OUT 1:
// FX uq >> s_u with the <x,u> and max|u| partials in dot, mx).
// On entry thread 0 has issued the copy of the CTA's first row into buffer
// rc & 1 (when it has rows) and the tables are in shared memory; rc counts
// the rows this CTA has streamed so far (it fixes buffer and barrier phase)
// and is advanced past the rows done.  On a give-up *S.give_up is set, the
// copy in flight has been waited for and the function returns early.
// Rows of the CTA.  Static: the host plan rowList[rowStart[b] ..).  Dynamic
// (taken != null): CTA b starts at rowQueue[b] and takes each further row as
// rowQueue[gridDim.x + atomicAdd(taken, 1)] while it computes the current
// one, so CTAs that finish early take more rows (the queue is in decreasing
// order of cost).  *snext is a shared word for the index taken.
// SPLIT: the unit queue (a.unitQueue), whose last entries are column ranges
// of rows (low 24 bits: the row).
template <bool SPLIT = false>
__device__ __forceinline__ bool tma_first_row_dyn(const MvArgs& a, uint32_t* u) {
    if (blockIdx.x >= (SPLIT ? a.nunits : (uint32_t)a.dimUP)) return false;
    *u = SPLIT ? (__ldg(a.unitQueue + blockIdx.x) & 0xFFFFFFu) : __ldg(a.rowQueue + blockIdx.x);
    return true;
}

// GDIAG: the folded down diagonal is read from a.dDNq in global memory
// instead of the staged copy (instances that share staged tables but not
// their on-site terms, k_lz_multi).
template <bool CPLX, int OUT, bool FAST, bool COH, bool SCHED, bool DYN, bool SEG = false, bool GDIAG = false,
          bool SPLIT = false>
__device__ __forceinline__ void tma_rows(const MvArgs& a, const TmaSmem& S, const int64_t* __restrict__ xq,
                                         int64_t* __restrict__ uq, double* __restrict__ y, uint32_t& rc, int E_out,
                                         int s_u, i128& dot, uint64_t& mx, unsigned int* taken = nullptr,
                                         uint32_t* snext = nullptr) {
    constexpr int W = CPLX ? 2 : 1;
    const uint32_t dimDN = (uint32_t)a.dimDN;
    const int tid = threadIdx.x, T = blockDim.x;
    const bool merge = a.mergeUD != 0;
    const bool unitU = a.unitUP != 0 && a.nclsUP == 1;
    const bool unitD = a.unitDN != 0 && a.nclsDN == 1;
    const uint32_t nq = SPLIT ? a.nunits : (uint32_t)a.dimUP;
    const uint32_t* const queue = SPLIT ? a.unitQueue : a.rowQueue;

    // The next row is taken and its copy issued by the last thread (with
    // rows shorter than 2T it has the fewest columns) after the barrier below:
    // the queue atomic, issued at the row start, and the row-index lookup
    // then keep no thread from that barrier.
    const int qt = T - 1;
    const uint32_t r1 = DYN ? nq : __ldg(a.rowStart + blockIdx.x + 1);
    for (uint32_t r = DYN ? blockIdx.x : __ldg(a.rowStart + blockIdx.x); r < r1; ++rc) {
        const uint32_t qe = DYN ? __ldg(queue + r) : __ldg(a.rowList + r);
        const uint32_t u = SPLIT ? (qe & 0xFFFFFFu) : qe;
        // the unit's columns: the whole row, or a range of a multiple of 32
        // columns (the lanes keep their columns mod 32)
        uint32_t lo = 0, hi = dimDN;
        if (SPLIT && (qe >> 24)) {
            const uint32_t P = 1u << (qe >> 28), ch = ((dimDN + P - 1) / P + 31u) & ~31u;
            lo = ((qe >> 24) & 0xFu) * ch;
            hi = min(dimDN, lo + ch);
        }
        const int buf = rc & 1;
        const uint32_t parity = (rc >> 1) & 1;
        uint32_t taken_at = 0;
        if (DYN && tid == qt) taken_at = atomicAdd(taken, 1u);  // consumed after the barrier
        const uint32_t p0 = __ldg(a.upPtr + u), lenU = __ldg(a.upPtr + u + 1) - p0;
        const int nposU = FAST ? (int)__ldg(a.upNpos + u) : 0;
        for (uint32_t k = tid; k < lenU; k += T) {
            const uint32_t e = __ldg(a.upEntC + p0 + k);
            S.uoff[k] = (e & kColMask) * dimDN;
            S.uent[k] = e;
        }
        if (!tma::mbar_wait(&S.bar[buf], parity)) {
            if (tid == 0) atomicExch(a.err, 1);
            *S.give_up = 1;
        } else if (SCHED) {
            // -x beside x, so that a schedule index carries the sign
            int64_t* xb = (buf ? S.row1 : S.row0) + tma_row_off<CPLX>(a, u);
            for (uint32_t i = tid; i < dimDN; i += T) xb[a.schedNeg + i] = -xb[i];
        }
        __syncthreads();
        if (*S.give_up) {
            // the current row's copy (the wait that gave up) is the only one
            // counted on a barrier: it must land before the CTA leaves and its
            // shared memory is reassigned (bounded; if it gives up again the
            // rows are undefined)
            if (tid == 0) tma::mbar_wait(&S.bar[buf], parity);
            return;
        }
        // prefetch the next row into the other buffer (its readers finished
        // at the barrier that closed the previous iteration)
        if (tid == qt) {
            const uint32_t rn = DYN ? gridDim.x + taken_at : r + 1;
            if (DYN) *snext = rn;
            if (rn < r1) {
                const uint32_t un = DYN ? (__ldg(queue + rn) & (SPLIT ? 0xFFFFFFu : 0xFFFFFFFFu)) : __ldg(a.rowList + rn);
                tma::fence_proxy_async_smem();
                tma_issue_row<CPLX>(a, S, xq, un, buf ^ 1);
            }
        }
        const int64_t* xrow = (buf ? S.row1 : S.row0) + tma_row_off<CPLX>(a, u);
        const uint32_t ubase = u * dimDN;

        // two columns (d0, d0 + T) per iteration; one in the class-segmented
        // path, which takes its columns one after the other anyway (fewer
        // live 128-bit accumulators)
        for (uint32_t d0 = lo + tid; d0 < hi; d0 += (SEG ? 1u : 2u) * T) {
            const uint32_t d1 = d0 + T;
            const bool v1 = !SEG && d1 < hi;
            const uint32_t d1c = v1 ? d1 : d0;  // clamp: the second column repeats d0 and is not stored
            i128 ar0 = 0, ai0 = 0, ar1 = 0, ai1 = 0;
            if (FAST) {
                int64_t upr0 = 0, upi0 = 0, unr0 = 0, uni0 = 0, upr1 = 0, upi1 = 0, unr1 = 0, uni1 = 0;
                int k = 0;
                if (v1) {
#pragma unroll 4
                    for (; k < nposU; ++k) {
                        const uint32_t o = S.uoff[k];
                        acc_up<CPLX, COH>(xq, o + d0, upr0, upi0);
                        acc_up<CPLX, COH>(xq, o + d1, upr1, upi1);
                    }
#pragma unroll 4
                    for (; k < (int)lenU; ++k) {
                        const uint32_t o = S.uoff[k];
                        acc_up<CPLX, COH>(xq, o + d0, unr0, uni0);
                        acc_up<CPLX, COH>(xq, o + d1, unr1, uni1);
                    }
                } else {
#pragma unroll 4
                    for (; k < nposU; ++k) acc_up<CPLX, COH>(xq, S.uoff[k] + d0, upr0, upi0);
#pragma unroll 4
                    for (; k < (int)lenU; ++k) acc_up<CPLX, COH>(xq, S.uoff[k] + d0, unr0, uni0);
                }
                int64_t dr0 = 0, di0 = 0, dr1 = 0, di1 = 0;
                if (SCHED) {
                    // conflict-free schedule: in every step the 16 lanes of a
                    // half warp read 16 different bank pairs of [x | -x | 0]
                    const uint32_t dp = (uint32_t)a.dimDNp;
                    const uint16_t* sc0 = S.sched + d0;
                    const int n0 = S.steps[d0 >> 5];
#pragma unroll 4
                    for (int s = 0; s < n0; ++s) dr0 += xrow[sc0[s * dp]];
                    if (v1) {
                        const uint16_t* sc1 = S.sched + d1;
                        const int n1 = S.steps[d1 >> 5];
#pragma unroll 4
                        for (int s = 0; s < n1; ++s) dr1 += xrow[sc1[s * dp]];
                    }
                } else {
#pragma unroll
                for (int c = 0; c < 2; ++c) {
                    const uint32_t d = c ? d1c : d0;
                    const uint32_t q0 = S.dptr[d], q1 = S.dptr[d + 1], qp = q0 + S.dnpos[d];
                    int64_t pr = 0, pi = 0, nr = 0, ni = 0;
                    for (uint32_t q = q0; q < qp; ++q) {
                        const uint32_t col = (S.dent[q] & kColMask) * W;
                        int64_t vr, vi;
                        row_elem<CPLX>(xrow, col, vr, vi);
                        pr += vr;
                        if (CPLX) pi += vi;
                    }
                    for (uint32_t q = qp; q < q1; ++q) {
                        const uint32_t col = (S.dent[q] & kColMask) * W;
                        int64_t vr, vi;
                        row_elem<CPLX>(xrow, col, vr, vi);
                        nr += vr;
                        if (CPLX) ni += vi;
                    }
                    if (c) {
                        dr1 = pr - nr;
                        di1 = pi - ni;
                    } else {
                        dr0 = pr - nr;
                        di0 = pi - ni;
                    }
                }
                }
                if (merge) {
                    apply_class<CPLX>(ar0, ai0, (upr0 - unr0) + dr0, (upi0 - uni0) + di0, a.coefUP, 0, unitU, a.Fc);
                    apply_class<CPLX>(ar1, ai1, (upr1 - unr1) + dr1, (upi1 - uni1) + di1, a.coefUP, 0, unitU, a.Fc);
                } else {
                    if (lenU) {
                        apply_class<CPLX>(ar0, ai0, upr0 - unr0, upi0 - uni0, a.coefUP, 0, unitU, a.Fc);
                        apply_class<CPLX>(ar1, ai1, upr1 - unr1, upi1 - uni1, a.coefUP, 0, unitU, a.Fc);
                    }
                    if (a.nclsDN) {
                        apply_class<CPLX>(ar0, ai0, dr0, di0, a.coefDN, 0, unitD, a.Fc);
                        apply_class<CPLX>(ar1, ai1, dr1, di1, a.coefDN, 0, unitD, a.Fc);
                    }
                }
            } else if (SEG) {
                // at most kSegCls classes: class by class over segments taken
                // from the rows' class-end bytes (+ entries first), the same
                // loop bounds for every lane in the up row; with equal class
                // lists the up and down sums of a class share one product.
                const uint32_t se_u = __ldg(a.upSegE + u), sp_u = __ldg(a.upSegP + u);
                const int ncl = max(a.nclsUP, a.nclsDN);
#pragma unroll 1
                for (int cc = 0; cc < (v1 ? 2 : 1); ++cc) {
                    const uint32_t d = cc ? d1c : d0;
                    // this column's accumulators, stored into ar0/ai0 or
                    // ar1/ai1 at the end (not a reference chosen at run time,
                    // which would put all four in local memory)
                    i128 ar = 0, ai = 0;
                    const uint32_t se = __ldg(a.dnSegE + d), sp = __ldg(a.dnSegP + d);
                    const uint32_t q0 = S.dptr[d];
                    uint32_t ub = 0, b = 0;
                    for (int c = 0; c < ncl; ++c) {
                        int64_t r = 0, i = 0;
                        if (c < a.nclsUP) {
                            const uint32_t up = (sp_u >> (8 * c)) & 0xFFu, ue = (se_u >> (8 * c)) & 0xFFu;
                            for (uint32_t k = ub; k < up; ++k) acc_up<CPLX, COH>(xq, S.uoff[k] + d, r, i);
                            for (uint32_t k = up; k < ue; ++k) {
                                int64_t vr, vi;
                                up_load<CPLX, COH>(xq, S.uoff[k] + d, vr, vi);
                                r -= vr;
                                i -= vi;
                            }
                            ub = ue;
                            if (!a.mergeMC) {
                                apply_class<CPLX>(ar, ai, r, i, a.coefUP, c, unitU, a.Fc);
                                r = 0;
                                i = 0;
                            }
                        }
                        if (c < a.nclsDN) {
                            const uint32_t pc = (sp >> (8 * c)) & 0xFFu, ec = (se >> (8 * c)) & 0xFFu;
                            for (uint32_t q = q0 + b; q < q0 + pc; ++q) {
                                const uint32_t col = (S.dent[q] & kColMask) * W;
                                int64_t vr, vi;
                                row_elem<CPLX>(xrow, col, vr, vi);
                                r += vr;
                                if (CPLX) i += vi;
                            }
                            for (uint32_t q = q0 + pc; q < q0 + ec; ++q) {
                                const uint32_t col = (S.dent[q] & kColMask) * W;
                                int64_t vr, vi;
                                row_elem<CPLX>(xrow, col, vr, vi);
                                r -= vr;
                                if (CPLX) i -= vi;
                            }
                            b = ec;
                            apply_class<CPLX>(ar, ai, r, i, a.coefDN, c, unitD, a.Fc);
                        } else if (a.mergeMC) {
                            apply_class<CPLX>(ar, ai, r, i, a.coefUP, c, unitU, a.Fc);
                        }
                    }
                    if (cc) {
                        ar1 = ar;
                        ai1 = ai;
                    } else {
                        ar0 = ar;
                        ai0 = ai;
                    }
                }
            } else {
#pragma unroll
                for (int c = 0; c < 2; ++c) {
                    const uint32_t d = c ? d1c : d0;
                    i128& ar = c ? ar1 : ar0;
                    i128& ai = c ? ai1 : ai0;
                    {
                        int cur = -1;
                        int64_t sr = 0, si = 0;
                        for (uint32_t k = 0; k < lenU; ++k) {
                            const uint32_t e = S.uent[k];
                            const int cl = (int)((e >> kClassShift) & kClassMask);
                            if (cl != cur) {
                                if (cur >= 0) apply_class<CPLX>(ar, ai, sr, si, a.coefUP, cur, unitU, a.Fc);
                                sr = 0;
                                si = 0;
                                cur = cl;
                            }
                            int64_t r, i;
                            up_load<CPLX, COH>(xq, S.uoff[k] + d, r, i);
                            sr += apply_sign(r, e);
                            if (CPLX) si += apply_sign(i, e);
                        }
                        if (cur >= 0) apply_class<CPLX>(ar, ai, sr, si, a.coefUP, cur, unitU, a.Fc);
                    }
                    {
                        int cur = -1;
                        int64_t sr = 0, si = 0;
                        for (uint32_t q = S.dptr[d]; q < S.dptr[d + 1]; ++q) {
                            const uint32_t e = S.dent[q];
                            const int cl = (int)((e >> kClassShift) & kClassMask);
                            if (cl != cur) {
                                if (cur >= 0) apply_class<CPLX>(ar, ai, sr, si, a.coefDN, cur, unitD, a.Fc);
                                sr = 0;
                                si = 0;
                                cur = cl;
                            }
                            const uint32_t col = (e & kColMask) * W;
                            int64_t vr, vi;
                            row_elem<CPLX>(xrow, col, vr, vi);
                            sr += apply_sign(vr, e);
                            if (CPLX) si += apply_sign(vi, e);
                        }
                        if (cur >= 0) apply_class<CPLX>(ar, ai, sr, si, a.coefDN, cur, unitD, a.Fc);
                    }
                }
            }
            // the row's diagonal terms, read here rather than held across the sums
            const uint64_t stu = __ldg(a.stUP + u);
            const int64_t du = __ldg(a.dUPq + u);
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                if (c == 1 && !v1) break;
                const uint32_t d = c ? d1 : d0;
                i128& ar = c ? ar1 : ar0;
                i128& ai = c ? ai1 : ai0;
                int64_t xr, xi;
                row_elem<CPLX>(xrow, d * W, xr, xi);
                const int64_t ddn = GDIAG ? __ldg(a.dDNq + d) : S.ddq[d];
                const int64_t dq = du + ddn + a.Uq * (int64_t)__popcll(stu & S.dst[d] & a.mask);
                ar += mul_wide(dq, xr);
                if (CPLX) ai += mul_wide(dq, xi);
                const size_t o = (size_t)(ubase + d) * W;
                if (OUT == 0) {
                    y[o] = i128_to_f64(ar, E_out);
                    if (CPLX) y[o + 1] = i128_to_f64(ai, E_out);
                } else {
                    const int64_t qr = shr_round_i64(ar, s_u);
                    uq[o] = qr;
                    dot += mul_wide(xr, qr) >> 24;
                    uint64_t aq = (uint64_t)(qr < 0 ? -qr : qr);
                    mx = aq > mx ? aq : mx;
                    if (CPLX) {
                        const int64_t qi = shr_round_i64(ai, s_u);
                        uq[o + 1] = qi;
                        dot += mul_wide(xi, qi) >> 24;
                        aq = (uint64_t)(qi < 0 ? -qi : qi);
                        mx = aq > mx ? aq : mx;
                    }
                }
            }
        }
        __syncthreads();  // row buffer and uoff are free for the next iteration; *snext is written
        r = DYN ? *snext : r + 1;
    }
}

}  // namespace ed
