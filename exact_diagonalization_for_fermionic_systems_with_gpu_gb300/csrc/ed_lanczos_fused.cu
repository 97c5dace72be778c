// ed_lanczos_fused.cu — a run of FX Lanczos steps in one persistent
// cooperative launch (HubMatrix_GPU.cuh:561-590, the recurrence of eigen()).
//
// The per-step path costs two launches per step, and the matvec launch
// re-stages the down-spin tables into every CTA's shared memory each time.
// Here each CTA (two per SM, all co-resident) stages the tables once and then
// loops over the steps:
//   phase M  u = H w_j with the shared-memory row engine, rows handed out
//            through a queue (heaviest first, taken with an atomic counter),
//            then <w_j, u> and max|u|                           -> grid barrier
//            every CTA derives alpha_j and the axpy coefficients (identical
//            in every CTA: same integers, same scalar code)
//   phase A  w_{j+1} = (a0 u + a1 w_j + a2 w_{j-1}) >> Fa on a grid-stride
//            slice, then |w_{j+1}|^2 and max|w_{j+1}|           -> grid barrier
//            (a data barrier: beta_{j+1} is read with the next step's sums)
// The matvec's output shift uses the bound |q| < 2^54 that every Lanczos
// vector meets by construction, so no step waits for a norm before its
// matvec; the per-step kernels use the same bound when they run without
// reorthogonalisation.
// Grid reductions: each CTA reduces its values in shared memory and thread 0
// adds them to a global accumulator set with integer atomics — the 128-bit
// sum split into three 42-bit limbs, so the total is exact and independent of
// the order of arrival — and takes the max with atomicMax, before it arrives
// at the barrier.  After the barrier one read of four words gives every CTA
// the grid totals.  Four accumulator sets rotate: set r % 4 serves reduction
// r (two per step), which is read after barrier r or r+1; block 0 zeroes the
// set of reduction r-2 once barrier r has completed (all its readers have
// passed barrier r), and its next user adds only after barrier r+1, which
// block 0 reaches after the zeroing.
// The integer totals and the scalar arithmetic are those of the per-step
// kernels, so the Lanczos coefficients are bit-identical to the per-step path.
// Vectors written during the launch are read back with L2 (coherent) loads,
// and before the bulk copies of a row written by another CTA the issuing
// thread orders them behind the grid barrier with a proxy fence.
// Grid barriers are bounded (poll count and %globaltimer, limits in
// GridWait): a CTA that gives up sets *err and leaves; the host then reports
// ED_ERR_TIMEOUT.  No bulk copy is in flight at a grid barrier (a CTA's row
// copies all land before its rows are done), so leaving there is safe.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include "ed_lanczos.hpp"
#include "ed_lanczos_dev.cuh"
#include "ed_matvec_tma.cuh"

namespace ed {
using namespace dev;

namespace {

constexpr uint64_t kLimb = (1ULL << 42) - 1;

__device__ __forceinline__ unsigned int ld_relaxed_gpu(const unsigned int* p) {
    unsigned int v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void red_release_gpu_add(unsigned int* p, unsigned int v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

// A word of host-mapped memory written by the host (system scope).
__device__ __forceinline__ int ld_relaxed_sys(const int* p) {
    int v;
    asm volatile("ld.relaxed.sys.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Block 0: slot k of the host mirror complete (alpha[k-1], beta[k]), the
// data before the count (system-scope fence).
__device__ __forceinline__ void mirror_slot(HostMirror* hm, const LzState* lz, int k) {
    if (k > 0) hm->alpha[k - 1] = lz->alpha[k - 1];
    hm->beta[k] = lz->beta[k];
    __threadfence_system();
    *(volatile int*)&hm->done = k;
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Thread 0: add a CTA's sum and max to an accumulator set.
__device__ __forceinline__ void red_push(LzRedSet* r, i128 v, uint64_t m) {
    const u128 uv = (u128)v;
    atomicAdd(&r->l0, (unsigned long long)(uv & kLimb));
    atomicAdd(&r->l1, (unsigned long long)((uv >> 42) & kLimb));
    atomicAdd(&r->l2, (unsigned long long)(int64_t)(v >> 84));
    atomicMax(&r->mx, (unsigned long long)m);
}

// Thread 0, after the barrier: the grid totals.
__device__ __forceinline__ void red_pull(const LzRedSet* r, i128& v, uint64_t& m) {
    const unsigned long long l0 = __ldcg(&r->l0), l1 = __ldcg(&r->l1), l2 = __ldcg(&r->l2);
    m = __ldcg(&r->mx);
    v = (i128)((u128)l0 + ((u128)l1 << 42) + ((u128)(i128)(int64_t)l2 << 84));
}

// Grid-wide barrier on a monotone arrival counter: the k-th barrier of the
// launch completes when k * gridDim.x CTAs have arrived.  Writes and atomics
// before it (by any thread of any CTA) are visible after it.  False when the
// wait gave up; *give_up is then set for the whole CTA.
__device__ __forceinline__ bool grid_sync(unsigned int* gbar, unsigned int& target, int* give_up, int* err,
                                          const GridWait& lim) {
    __syncthreads();
    if (threadIdx.x == 0) {
        target += gridDim.x;
        // release: this CTA's writes and atomics (ordered before this thread
        // by the CTA barrier above) before the arrival
        red_release_gpu_add(gbar, 1u);
        const unsigned long long t0 = global_ns();
        const unsigned int want = target + lim.extra;
        long long it = 0;
        while (ld_relaxed_gpu(gbar) < want) {
            if (++it > lim.spin || global_ns() - t0 > lim.ns) {
                atomicExch(err, 1);
                *give_up = 1;
                break;
            }
        }
        fence_acq_rel_gpu();  // acquire: everything released before the last arrival
    }
    __syncthreads();
    return *give_up == 0;
}

__device__ __forceinline__ unsigned long long* stamps_at(const LzFusedArgs& f, int j) {
    return f.stamps ? f.stamps + kLzStamps * (size_t)j : nullptr;
}

// Timestamps (block 0, thread 0) per step: 0 start, 1 rows done, 2 block
// sums done, 3 barrier passed, 4 coefficients done, 5 axpy done, 6 block sums
// done, 7 barrier passed, 8 scalars done.

struct SlotScalars {
    int e;
    uint64_t m;
    double beta;
    double ib;  // 1 / beta (0 when beta is 0)
};

// Thread 0: slot k (= w_k) is complete with exponent e, exact sum of
// (q q) >> 16 and max |q|: beta_k, breakdown and precision bookkeeping
// (lz_after_axpy's), shift the slot scalars, block 0 stores them.
__device__ __forceinline__ void slot_done(LzState* lz, int k, int e, i128 ss, uint64_t m, SlotScalars& sX,
                                          SlotScalars& sP, int& status, int& min_bits, bool store) {
    const double beta = lz_beta(ss, e);
    const int bits = bitlen_u64(m);
    if (bits < min_bits) min_bits = bits;
    if (m == 0 && status == 0) status = 7;  // breakdown
    if (store) {
        lz->e[k] = e;
        lz->m[k] = m;
        lz->beta[k] = beta;
        lz->min_bits = min_bits;
        lz->status = status;
        lz->steps_done = k;
    }
    sP = sX;
    sX = {e, m, beta, lz_inv(beta)};
}

}  // namespace

template <bool CPLX, bool FAST, bool SCHED, bool SEG = false>
__global__ void __launch_bounds__(kTmaThreads, 2) k_lz_fused(const MvArgs a, const LzFusedArgs f) {
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ uint32_t uoff[kTmaUpStage];
    __shared__ uint32_t uent[kTmaUpStage];
    __shared__ int give_up;
    __shared__ i128 s128[32];
    __shared__ uint64_t s64[32];
    __shared__ SlotScalars sX, sP;  // slots j and j-1
    __shared__ int s_status, s_min_bits;
    __shared__ LzCoefs s_coef;
    const TmaSmem S = tma_view(a, sm, uoff, uent, &give_up);
    LzState* lz = f.lz;
    const int tid = threadIdx.x;
    __shared__ uint32_t s_next;  // row-queue index taken by thread 0
    uint32_t u0 = 0;
    // real runs take the unit queue (its last rows split into column ranges,
    // which narrows the CTAs' finishing spread); complex runs the row queue
    const bool has_row = tma_first_row_dyn<!CPLX>(a, &u0);
    const uint32_t G = gridDim.x;

    if (tid == 0) {
        tma_init(S);
        tma_issue_tables(a, S);
        const int j = f.j0;
        sX = {lz->e[j], lz->m[j], lz->beta[j], lz_inv(lz->beta[j])};
        if (j > 0) sP = {lz->e[j - 1], lz->m[j - 1], lz->beta[j - 1], lz_inv(lz->beta[j - 1])};
        else sP = {0, 0, 0.0, 0.0};
        s_status = lz->status;
        s_min_bits = lz->min_bits;
        if (f.mirror && blockIdx.x == 0 && j == 0) mirror_slot(f.mirror, lz, 0);
    }
    if (SCHED) tma_zero_slots(a, S);
    __syncthreads();
    if (!tma::mbar_wait(&S.bar[2], 0)) {
        if (tid == 0) atomicExch(a.err, 1);
        give_up = 1;
    }
    __syncthreads();
    if (give_up) {
        // the table copy is the only one in flight (rows are issued in the
        // step loop): wait for it once more (bounded) before leaving
        if (tid == 0) tma::mbar_wait(&S.bar[2], 0);
        return;
    }

    auto slot = [&](int j) -> int64_t* {
        return f.basis + (size_t)(f.stored ? j : j % 3) * (size_t)f.stride;
    };

    uint32_t rc = 0;          // rows streamed through the row buffers
    unsigned int target = 0;  // grid-barrier arrivals expected so far
    // every Lanczos vector has |q| < 2^54 (start vector by its FX exponent,
    // later ones by the axpy bound), so the matvec shift needs no reduction
    const int sb = a.bq_bits + kFxBits - 62;
    const int s_u = sb > 0 ? sb : 0;
    for (int j = f.j0; j < f.j1; ++j) {
        const int64_t* xq = slot(j);
        const int64_t* pq = j > 0 ? slot(j - 1) : slot(j);
        int64_t* wq = slot(j + 1);
        const bool stamp = f.stamps && blockIdx.x == 0 && tid == 0;
        unsigned long long* st = stamps_at(f, j);
        if (stamp) st[0] = global_ns();
        const int rM = 2 * (j - f.j0), rA = rM + 1;  // reductions (and barriers) of this step

        // ---- phase M: u = H w_j -------------------------------------------
        if (tid == 0 && has_row) {
            tma::fence_proxy_async_global();
            tma::fence_proxy_async_smem();
            tma_issue_row<CPLX>(a, S, xq, u0, rc & 1);
        }
        if (tid == kTmaThreads - 32 && j > f.j0) {
            // slot j from the previous step's axpy reduction, while the first
            // row copy is in flight (read at the scalar update after the next
            // barrier); the last warp, whose second column is past the end
            // of a row when dim_dn < 2 * kTmaThreads - 32
            i128 ss;
            uint64_t mw;
            red_pull(&f.red[(rM - 1) % 4], ss, mw);
            slot_done(lz, j, s_coef.e_w, ss, mw, sX, sP, s_status, s_min_bits, blockIdx.x == 0);
            if (f.mirror && blockIdx.x == 0) mirror_slot(f.mirror, lz, j);
        }
        {
            i128 dot = 0;
            uint64_t mx = 0;
            tma_rows<CPLX, 1, FAST, true, SCHED, true, SEG, false, !CPLX>(a, S, xq, f.u, nullptr, rc, 0, s_u, dot, mx,
                                                       f.taken + (j & 1), &s_next);
            if (give_up) return;
            if (stamp) st[1] = global_ns();
            if (f.cta_stamps && tid == 0) f.cta_stamps[(size_t)j * 2 * G + blockIdx.x] = global_ns();
            block_sum_max(dot, mx, s128, s64);
            if (tid == 0) red_push(&f.red[rM % 4], dot, mx);
            if (stamp) st[2] = global_ns();
        }
        if (!grid_sync(f.gbar, target, &give_up, a.err, f.wait)) return;
        // block 0 reads the host's stop word now and passes it on before the
        // step's last barrier (the load's latency hides behind the axpy)
        int host_stop = 0;
        if (f.mirror && blockIdx.x == 0 && tid == 0) host_stop = ld_relaxed_sys(&f.mirror->stop);
        if (tid == 0) {
            if (stamp) st[3] = global_ns();
            i128 s;
            uint64_t m;
            red_pull(&f.red[rM % 4], s, m);
            if (blockIdx.x == 0) {
                if (rM >= 2) f.red[(rM - 2) % 4] = LzRedSet{0, 0, 0, 0};
                // the other queue counter was last taken from in step j-1 and
                // is next taken from in step j+1, after the next barrier
                f.taken[(j + 1) & 1] = 0;
            }
            const int e_u = sX.e - a.Fc + s_u;
            s_coef = lz_coefs(j, s, e_u, m, sX.e, sX.m, sX.beta, sX.ib, sP.e, sP.m, sP.ib, s_status);
            if (blockIdx.x == 0) {
                lz->s_u = s_u;
                lz->e_u = e_u;
                lz->m_u = m;
                lz->alpha[j] = s_coef.alpha;
                for (int k = 0; k < 3; ++k) {
                    lz->at[k] = s_coef.at[k];
                    lz->sh[k] = 0;
                }
                lz->Fa = s_coef.Fa;
                lz->e_w = s_coef.e_w;
            }
            if (stamp) st[4] = global_ns();
        }
        __syncthreads();

        // ---- phase A: w_{j+1} = (a0 u + a1 w_j + a2 w_{j-1}) >> Fa ---------
        {
            const int64_t a0 = s_coef.at[0], a1 = s_coef.at[1], a2 = s_coef.at[2];
            const int Fa = s_coef.Fa;
            i128 ss = 0;
            uint64_t mw = 0;
            const int64_t npair = f.n >> 1;
            const longlong2* u2 = reinterpret_cast<const longlong2*>(f.u);
            const longlong2* x2 = reinterpret_cast<const longlong2*>(xq);
            const longlong2* p2 = reinterpret_cast<const longlong2*>(pq);
            longlong2* w2 = reinterpret_cast<longlong2*>(wq);
            for (int64_t i = (int64_t)blockIdx.x * blockDim.x + tid; i < npair; i += (int64_t)G * blockDim.x) {
                const longlong2 uu = __ldcg(u2 + i), xx = __ldcg(x2 + i), pp = __ldcg(p2 + i);
                longlong2 w;
                w.x = shr_round_i64(mul_wide(a0, uu.x) + mul_wide(a1, xx.x) + mul_wide(a2, pp.x), Fa);
                w.y = shr_round_i64(mul_wide(a0, uu.y) + mul_wide(a1, xx.y) + mul_wide(a2, pp.y), Fa);
                w2[i] = w;
                ss += (mul_wide(w.x, w.x) >> 16) + (mul_wide(w.y, w.y) >> 16);
                const uint64_t ax = (uint64_t)(w.x < 0 ? -w.x : w.x), ay = (uint64_t)(w.y < 0 ? -w.y : w.y);
                mw = ax > mw ? ax : mw;
                mw = ay > mw ? ay : mw;
            }
            if ((f.n & 1) && blockIdx.x == 0 && tid == 0) {
                const int64_t i = f.n - 1;
                const int64_t w = shr_round_i64(
                    mul_wide(a0, __ldcg(f.u + i)) + mul_wide(a1, __ldcg(xq + i)) + mul_wide(a2, __ldcg(pq + i)), Fa);
                wq[i] = w;
                ss += mul_wide(w, w) >> 16;
                const uint64_t aw = (uint64_t)(w < 0 ? -w : w);
                mw = aw > mw ? aw : mw;
            }
            if (stamp) st[5] = global_ns();
            if (f.cta_stamps) {
                __syncthreads();
                if (tid == 0) f.cta_stamps[((size_t)j * 2 + 1) * G + blockIdx.x] = global_ns();
            }
            block_sum_max(ss, mw, s128, s64);
            if (tid == 0) red_push(&f.red[rA % 4], ss, mw);
            if (f.mirror && blockIdx.x == 0 && tid == 0) *(volatile int*)f.stop_word = host_stop;
            if (stamp) st[6] = global_ns();
        }
        // a data barrier: the next matvec gathers w_{j+1} from every CTA; the
        // norm and max of w_{j+1} are read at the next step's reduction
        if (!grid_sync(f.gbar, target, &give_up, a.err, f.wait)) return;
        // the same stop decision in every CTA: the word block 0 wrote before the barrier
        const int stop_at = f.mirror ? *(volatile int*)f.stop_word : 0;
        const bool last = j + 1 == f.j1 || (stop_at > 0 && j + 1 >= stop_at);
        if (tid == 0) {
            if (blockIdx.x == 0 && rA >= 2) f.red[(rA - 2) % 4] = LzRedSet{0, 0, 0, 0};
            if (stamp) st[7] = st[8] = global_ns();
            if (last && blockIdx.x == 0) {
                // the last slot of this launch: block 0 stores its scalars
                i128 ss;
                uint64_t mw;
                red_pull(&f.red[rA % 4], ss, mw);
                slot_done(lz, j + 1, s_coef.e_w, ss, mw, sX, sP, s_status, s_min_bits, true);
                if (f.mirror) mirror_slot(f.mirror, lz, j + 1);
            }
        }
        __syncthreads();
        if (last) break;
    }
}

// ---------------------------------------------------------------- batch --
// B Lanczos runs in lockstep in one persistent launch (k_lz_batch): the
// instances share the first operator's hopping tables (in shared memory, as
// in k_lz_fused) and differ in their diagonals and scalars (LzInst).  The
// work items of a matvec phase are (instance, row) pairs, instance-major,
// handed out through a queue like k_lz_fused's rows; a CTA keeps the
// instance's <x, u> and max|u| partials in registers while consecutive items
// belong to it and every warp adds them to per-instance shared limb sums
// when the instance changes (and its norm partials after each instance's
// axpy slice).  The barriers, the four rotating reduction sets (B sets each)
// and the scalar update (thread b of every CTA for instance b) are
// k_lz_fused's, so every instance's coefficients are bit-identical to its own
// single run; what the batch saves is the per-step barrier and scalar time
// of B - 1 runs.  Real operators with one hopping class and a gather
// schedule.

// A warp's (v, m) into per-instance shared limb sums (all 32 lanes call it).
__device__ __forceinline__ void batch_flush(i128 v, uint64_t m, unsigned long long* accl, unsigned long long* accm) {
    v = warp_sum_i128(v);
    m = warp_max_u64(m);
    if ((threadIdx.x & 31) == 0) {
        const u128 uv = (u128)v;
        atomicAdd(&accl[0], (unsigned long long)(uv & kLimb));
        atomicAdd(&accl[1], (unsigned long long)((uv >> 42) & kLimb));
        atomicAdd(&accl[2], (unsigned long long)(int64_t)(v >> 84));
        atomicMax(accm, (unsigned long long)m);
    }
}

__device__ __forceinline__ i128 batch_total(const unsigned long long* accl) {
    return (i128)((u128)accl[0] + ((u128)accl[1] << 42) + ((u128)(i128)(int64_t)accl[2] << 84));
}

__device__ __forceinline__ void class_add(i128& ar, int64_t s, int64_t coef, bool unit, int Fc) {
    ar += unit ? (((i128)s) << Fc) : mul_wide(s, coef);
}

__global__ void __launch_bounds__(kTmaThreads, 2) k_lz_batch(const MvArgs a, const LzBatchArgs f) {
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ uint32_t uoff[kTmaUpStage];
    __shared__ uint32_t uent[kTmaUpStage];
    __shared__ int give_up;
    __shared__ uint32_t s_next;
    __shared__ SlotScalars sX[kLzBatchMax], sP[kLzBatchMax];
    __shared__ int s_status[kLzBatchMax], s_min_bits[kLzBatchMax], s_ew[kLzBatchMax];
    __shared__ LzCoefs s_coef[kLzBatchMax];
    __shared__ unsigned long long accl[kLzBatchMax][3], accm[kLzBatchMax];
    const TmaSmem S = tma_view(a, sm, uoff, uent, &give_up);
    const int tid = threadIdx.x, T = blockDim.x;
    const int B = f.B;
    const uint32_t nq = (uint32_t)a.dimUP, dimDN = (uint32_t)a.dimDN;
    const uint32_t nitems = (uint32_t)B * nq;
    const uint32_t G = gridDim.x;
    const bool has_item = blockIdx.x < nitems;

    if (tid == 0) {
        tma_init(S);
        tma_issue_tables(a, S);
    }
    if (tid < B) {
        const LzState* lz = f.inst[tid].lz;
        const int j = f.j0;
        sX[tid] = {lz->e[j], lz->m[j], lz->beta[j], lz_inv(lz->beta[j])};
        if (j > 0) sP[tid] = {lz->e[j - 1], lz->m[j - 1], lz->beta[j - 1], lz_inv(lz->beta[j - 1])};
        else sP[tid] = {0, 0, 0.0, 0.0};
        s_status[tid] = lz->status;
        s_min_bits[tid] = lz->min_bits;
        s_ew[tid] = 0;
        accl[tid][0] = accl[tid][1] = accl[tid][2] = 0;
        accm[tid] = 0;
    }
    tma_zero_slots(a, S);
    __syncthreads();
    if (!tma::mbar_wait(&S.bar[2], 0)) {
        if (tid == 0) atomicExch(a.err, 1);
        give_up = 1;
    }
    __syncthreads();
    if (give_up) {
        // the table copy is the only one in flight (rows are issued in the
        // step loop): wait for it once more (bounded) before leaving
        if (tid == 0) tma::mbar_wait(&S.bar[2], 0);
        return;
    }

    uint32_t rc = 0;          // rows streamed through the row buffers
    unsigned int target = 0;  // grid-barrier arrivals expected so far
    for (int j = f.j0; j < f.j1; ++j) {
        const int rM = 2 * (j - f.j0), rA = rM + 1;
        // ---- phase M: u_b = H_b w_j of every instance, item by item --------
        uint32_t it = blockIdx.x;
        if (tid == 0 && has_item) {
            tma::fence_proxy_async_global();
            tma::fence_proxy_async_smem();
            const uint32_t b0 = it / nq;
            tma_issue_row<false>(a, S, f.inst[b0].basis + (size_t)j * f.stride, __ldg(a.rowQueue + (it - b0 * nq)),
                                 rc & 1);
        }
        if (tid >= kTmaThreads - 32 && tid < kTmaThreads - 32 + B && j > f.j0) {
            // slot j of instance b from the previous step's axpy reduction,
            // while the first row copy is in flight (the last warp)
            const int b = tid - (kTmaThreads - 32);
            i128 ss;
            uint64_t mw;
            red_pull(&f.red[((rM - 1) % 4) * B + b], ss, mw);
            slot_done(f.inst[b].lz, j, s_ew[b], ss, mw, sX[b], sP[b], s_status[b], s_min_bits[b], blockIdx.x == 0);
        }
        {
            i128 dot = 0;
            uint64_t mx = 0;
            int cur = has_item ? (int)(it / nq) : -1;
            while (it < nitems) {
                const uint32_t b = it / nq;
                const uint32_t u = __ldg(a.rowQueue + (it - b * nq));
                const LzInst& I = f.inst[b];
                const int64_t* xq = I.basis + (size_t)j * f.stride;
                const int buf = rc & 1;
                const uint32_t parity = (rc >> 1) & 1;
                bool issued_next = false;
                if (tid == 0) {
                    const uint32_t rn = G + atomicAdd(f.taken + (j & 1), 1u);
                    s_next = rn;
                    if (rn < nitems) {
                        const uint32_t bn = rn / nq;
                        tma::fence_proxy_async_smem();
                        tma_issue_row<false>(a, S, f.inst[bn].basis + (size_t)j * f.stride,
                                             __ldg(a.rowQueue + (rn - bn * nq)), buf ^ 1);
                        issued_next = true;
                    }
                }
                const uint32_t p0 = __ldg(a.upPtr + u), lenU = __ldg(a.upPtr + u + 1) - p0;
                const int nposU = (int)__ldg(a.upNpos + u);
                for (uint32_t k = tid; k < lenU; k += T) S.uoff[k] = (__ldg(a.upEntC + p0 + k) & kColMask) * dimDN;
                if (!tma::mbar_wait(&S.bar[buf], parity)) {
                    if (tid == 0) atomicExch(a.err, 1);
                    give_up = 1;
                } else {
                    int64_t* xb = (buf ? S.row1 : S.row0) + tma_row_off<false>(a, u);
                    for (uint32_t i = tid; i < dimDN; i += T) xb[a.schedNeg + i] = -xb[i];
                }
                __syncthreads();
                if (give_up) {
                    // this item's copy (once more) and the next item's must
                    // land before the CTA leaves (bounded waits)
                    if (tid == 0) {
                        tma::mbar_wait(&S.bar[buf], parity);
                        if (issued_next) tma::mbar_wait(&S.bar[buf ^ 1], ((rc + 1) >> 1) & 1);
                    }
                    return;
                }
                const uint32_t r_next = s_next;
                const int64_t* xrow = (buf ? S.row1 : S.row0) + tma_row_off<false>(a, u);
                const uint64_t stu = __ldg(a.stUP + u);
                const int64_t du = __ldg(I.dUPq + u);
                const int64_t* ddq = I.dDNq;
                const int64_t Uq = I.Uq, cU = I.coefUP, cD = I.coefDN;
                const int Fc = I.Fc;
                const uint32_t ubase = u * dimDN;
                const int sb = I.bq_bits + kFxBits - 62;
                const int s_u = sb > 0 ? sb : 0;
                const bool unitU = I.unitUP != 0 && I.nclsUP == 1;
                const bool unitD = I.unitDN != 0 && I.nclsDN == 1;
                const bool merge = I.mergeUD != 0, hasD = I.nclsDN != 0;
                int64_t* uq = I.u;
                const uint32_t dp = (uint32_t)a.dimDNp;
                for (uint32_t d0 = tid; d0 < dimDN; d0 += 2 * T) {
                    const uint32_t d1 = d0 + T;
                    const bool v1 = d1 < dimDN;
                    int64_t up0 = 0, un0 = 0, up1 = 0, un1 = 0;
                    int k = 0;
                    if (v1) {
#pragma unroll 4
                        for (; k < nposU; ++k) {
                            const uint32_t o = S.uoff[k];
                            up0 += __ldcg(xq + o + d0);
                            up1 += __ldcg(xq + o + d1);
                        }
#pragma unroll 4
                        for (; k < (int)lenU; ++k) {
                            const uint32_t o = S.uoff[k];
                            un0 += __ldcg(xq + o + d0);
                            un1 += __ldcg(xq + o + d1);
                        }
                    } else {
#pragma unroll 4
                        for (; k < nposU; ++k) up0 += __ldcg(xq + S.uoff[k] + d0);
#pragma unroll 4
                        for (; k < (int)lenU; ++k) un0 += __ldcg(xq + S.uoff[k] + d0);
                    }
                    int64_t dr0 = 0, dr1 = 0;
                    {
                        const uint16_t* sc0 = S.sched + d0;
                        const int n0 = S.steps[d0 >> 5];
#pragma unroll 4
                        for (int s = 0; s < n0; ++s) dr0 += xrow[sc0[s * dp]];
                    }
                    if (v1) {
                        const uint16_t* sc1 = S.sched + d1;
                        const int n1 = S.steps[d1 >> 5];
#pragma unroll 4
                        for (int s = 0; s < n1; ++s) dr1 += xrow[sc1[s * dp]];
                    }
#pragma unroll
                    for (int c = 0; c < 2; ++c) {
                        if (c == 1 && !v1) break;
                        const uint32_t d = c ? d1 : d0;
                        const int64_t su = c ? up1 - un1 : up0 - un0;
                        const int64_t sd = c ? dr1 : dr0;
                        i128 ar = 0;
                        if (merge) {
                            class_add(ar, su + sd, cU, unitU, Fc);
                        } else {
                            if (lenU) class_add(ar, su, cU, unitU, Fc);
                            if (hasD) class_add(ar, sd, cD, unitD, Fc);
                        }
                        const int64_t xr = xrow[d];
                        const int64_t dq = du + __ldg(ddq + d) + Uq * (int64_t)__popcll(stu & S.dst[d] & a.mask);
                        ar += mul_wide(dq, xr);
                        const int64_t qr = shr_round_i64(ar, s_u);
                        uq[(size_t)ubase + d] = qr;
                        dot += mul_wide(xr, qr) >> 24;
                        const uint64_t aq = (uint64_t)(qr < 0 ? -qr : qr);
                        mx = aq > mx ? aq : mx;
                    }
                }
                __syncthreads();  // row buffer and uoff are free for the next item
                ++rc;
                it = r_next;
                const int nb = it < nitems ? (int)(it / nq) : -1;
                if (nb != cur) {
                    batch_flush(dot, mx, accl[cur], &accm[cur]);
                    dot = 0;
                    mx = 0;
                    cur = nb;
                }
            }
        }
        __syncthreads();
        if (tid < B) {
            red_push(&f.red[(rM % 4) * B + tid], batch_total(accl[tid]), accm[tid]);
            accl[tid][0] = accl[tid][1] = accl[tid][2] = 0;
            accm[tid] = 0;
        }
        if (!grid_sync(f.gbar, target, &give_up, a.err, f.wait)) return;
        if (tid < B) {
            const int b = tid;
            LzState* lz = f.inst[b].lz;
            i128 s;
            uint64_t m;
            red_pull(&f.red[(rM % 4) * B + b], s, m);
            if (blockIdx.x == 0) {
                if (rM >= 2) f.red[((rM - 2) % 4) * B + b] = LzRedSet{0, 0, 0, 0};
                if (b == 0) f.taken[(j + 1) & 1] = 0;
            }
            const LzInst& I = f.inst[b];
            const int sb = I.bq_bits + kFxBits - 62;
            const int s_u = sb > 0 ? sb : 0;
            const int e_u = sX[b].e - I.Fc + s_u;
            s_coef[b] = lz_coefs(j, s, e_u, m, sX[b].e, sX[b].m, sX[b].beta, sX[b].ib, sP[b].e, sP[b].m, sP[b].ib,
                                 s_status[b]);
            s_ew[b] = s_coef[b].e_w;
            if (blockIdx.x == 0) {
                lz->s_u = s_u;
                lz->e_u = e_u;
                lz->m_u = m;
                lz->alpha[j] = s_coef[b].alpha;
                for (int k = 0; k < 3; ++k) {
                    lz->at[k] = s_coef[b].at[k];
                    lz->sh[k] = 0;
                }
                lz->Fa = s_coef[b].Fa;
                lz->e_w = s_coef[b].e_w;
            }
        }
        __syncthreads();

        // ---- phase A: w_{j+1} of every instance ----------------------------
        // last instance first: the rows phase ended on it, so its u and w_j
        // are the vectors still in L2, and the next rows phase starts on
        // instance 0, whose w_{j+1} this phase writes last
        for (int b = B - 1; b >= 0; --b) {
            const LzInst& I = f.inst[b];
            const int64_t* xq = I.basis + (size_t)j * f.stride;
            const int64_t* pq = j > 0 ? I.basis + (size_t)(j - 1) * f.stride : xq;
            int64_t* wq = I.basis + (size_t)(j + 1) * f.stride;
            const int64_t a0 = s_coef[b].at[0], a1 = s_coef[b].at[1], a2 = s_coef[b].at[2];
            const int Fa = s_coef[b].Fa;
            i128 ss = 0;
            uint64_t mw = 0;
            const int64_t npair = f.n >> 1;
            const longlong2* u2 = reinterpret_cast<const longlong2*>(I.u);
            const longlong2* x2 = reinterpret_cast<const longlong2*>(xq);
            const longlong2* p2 = reinterpret_cast<const longlong2*>(pq);
            longlong2* w2 = reinterpret_cast<longlong2*>(wq);
            for (int64_t i = (int64_t)blockIdx.x * blockDim.x + tid; i < npair; i += (int64_t)G * blockDim.x) {
                const longlong2 uu = __ldcg(u2 + i), xx = __ldcg(x2 + i), pp = __ldcg(p2 + i);
                longlong2 w;
                w.x = shr_round_i64(mul_wide(a0, uu.x) + mul_wide(a1, xx.x) + mul_wide(a2, pp.x), Fa);
                w.y = shr_round_i64(mul_wide(a0, uu.y) + mul_wide(a1, xx.y) + mul_wide(a2, pp.y), Fa);
                w2[i] = w;
                ss += (mul_wide(w.x, w.x) >> 16) + (mul_wide(w.y, w.y) >> 16);
                const uint64_t ax = (uint64_t)(w.x < 0 ? -w.x : w.x), ay = (uint64_t)(w.y < 0 ? -w.y : w.y);
                mw = ax > mw ? ax : mw;
                mw = ay > mw ? ay : mw;
            }
            if ((f.n & 1) && blockIdx.x == 0 && tid == 0) {
                const int64_t i = f.n - 1;
                const int64_t w = shr_round_i64(
                    mul_wide(a0, __ldcg(I.u + i)) + mul_wide(a1, __ldcg(xq + i)) + mul_wide(a2, __ldcg(pq + i)), Fa);
                wq[i] = w;
                ss += mul_wide(w, w) >> 16;
                const uint64_t aw = (uint64_t)(w < 0 ? -w : w);
                mw = aw > mw ? aw : mw;
            }
            batch_flush(ss, mw, accl[b], &accm[b]);
        }
        __syncthreads();
        if (tid < B) {
            red_push(&f.red[(rA % 4) * B + tid], batch_total(accl[tid]), accm[tid]);
            accl[tid][0] = accl[tid][1] = accl[tid][2] = 0;
            accm[tid] = 0;
        }
        if (!grid_sync(f.gbar, target, &give_up, a.err, f.wait)) return;
        if (tid < B && blockIdx.x == 0) {
            const int b = tid;
            if (rA >= 2) f.red[((rA - 2) % 4) * B + b] = LzRedSet{0, 0, 0, 0};
            if (j + 1 == f.j1) {
                i128 ss;
                uint64_t mw;
                red_pull(&f.red[(rA % 4) * B + b], ss, mw);
                slot_done(f.inst[b].lz, j + 1, s_coef[b].e_w, ss, mw, sX[b], sP[b], s_status[b], s_min_bits[b], true);
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------- multi --
// B Lanczos runs of any sectors, real or complex, in lockstep in one
// persistent launch (k_lz_multi).  Each step walks the instances in order:
// for instance b every CTA takes rows from b's own queue (its first row at
// blockIdx.x, the rest by an atomic counter, heaviest first) with the row
// engine variant of b's operator, and moves on to b + 1 as soon as b's queue
// is empty, so the CTAs' finishing spread is paid once per step, not per
// instance.  A CTA copies b's operator arguments into shared memory when it
// reaches b, and re-stages the down-spin tables when b's group (sector and
// hopping terms) differs from the staged one; the folded down diagonal, which
// instances of one group need not share, is read from global memory.  The
// <x, u> and max|u| partials of every instance go through per-instance shared
// limb sums, the barriers, reduction sets and per-instance scalar updates are
// k_lz_batch's, so every run's coefficients equal its own single run's bit
// for bit (the matvec sums are exact integers whatever the variant).

template <bool CPLX>
__device__ __forceinline__ void multi_first_row(const MvArgs& a, const TmaSmem& S, const int64_t* xq, uint32_t rc) {
    tma::fence_proxy_async_global();
    tma::fence_proxy_async_smem();
    tma_issue_row<CPLX>(a, S, xq, __ldg(a.rowQueue + blockIdx.x), rc & 1);
}

// The row-engine variant of instance kind `kind`; KINDS (a bit per LzKind)
// lists the variants this instantiation of k_lz_multi carries, so that a
// batch of one or two kinds does not pay the registers of all seven.
template <int KINDS>
__device__ __forceinline__ void multi_rows(int kind, const MvArgs& a, const TmaSmem& S, const int64_t* xq, int64_t* uq,
                                           uint32_t& rc, int s_u, i128& dot, uint64_t& mx, unsigned int* taken,
                                           uint32_t* snext) {
#define ED_MULTI_CASE(K, C, F, SC, SG)                                                                              \
    if (((KINDS >> K) & 1) && kind == K) {                                                                          \
        tma_rows<C, 1, F, true, SC, true, SG, true>(a, S, xq, uq, nullptr, rc, 0, s_u, dot, mx, taken, snext);     \
        return;                                                                                                     \
    }
    ED_MULTI_CASE(kKindRealSched, false, true, true, false)
    ED_MULTI_CASE(kKindRealFast, false, true, false, false)
    ED_MULTI_CASE(kKindRealSeg, false, false, false, true)
    ED_MULTI_CASE(kKindReal, false, false, false, false)
    ED_MULTI_CASE(kKindCplxFast, true, true, false, false)
    ED_MULTI_CASE(kKindCplxSeg, true, false, false, true)
    ED_MULTI_CASE(kKindCplx, true, false, false, false)
#undef ED_MULTI_CASE
}

template <int KINDS>
__global__ void __launch_bounds__(kTmaThreads, 2) k_lz_multi(const LzMultiArgs f) {
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ uint32_t uoff[kTmaUpStage];
    __shared__ uint32_t uent[kTmaUpStage];
    __shared__ int give_up;
    __shared__ uint32_t s_next;
    __shared__ __align__(16) MvArgs s_args;
    __shared__ SlotScalars sX[kLzMultiMax], sP[kLzMultiMax];
    __shared__ int s_status[kLzMultiMax], s_min_bits[kLzMultiMax], s_ew[kLzMultiMax];
    __shared__ LzCoefs s_coef[kLzMultiMax];
    __shared__ unsigned long long accl[kLzMultiMax][3], accm[kLzMultiMax];
    const int tid = threadIdx.x;
    const int B = f.B;
    const uint32_t G = gridDim.x;

    if (tid == 0) {
        TmaSmem S0;
        S0.bar = reinterpret_cast<uint64_t*>(sm);
        S0.give_up = &give_up;
        tma_init(S0);
    }
    if (tid < B) {
        const LzState* lz = f.inst[tid].lz;
        const int j = f.j0;
        sX[tid] = {lz->e[j], lz->m[j], lz->beta[j], lz_inv(lz->beta[j])};
        if (j > 0) sP[tid] = {lz->e[j - 1], lz->m[j - 1], lz->beta[j - 1], lz_inv(lz->beta[j - 1])};
        else sP[tid] = {0, 0, 0.0, 0.0};
        s_status[tid] = lz->status;
        s_min_bits[tid] = lz->min_bits;
        s_ew[tid] = 0;
        accl[tid][0] = accl[tid][1] = accl[tid][2] = 0;
        accm[tid] = 0;
    }
    __syncthreads();

    uint32_t rc = 0;          // rows streamed through the row buffers
    uint32_t tc = 0;          // table stagings (phases of bar[2])
    int cur = -1, staged = -1;
    unsigned int target = 0;  // grid-barrier arrivals expected so far
    for (int j = f.j0; j < f.j1; ++j) {
        const int rM = 2 * (j - f.j0), rA = rM + 1;
        if (tid >= kTmaThreads - 32 && tid < kTmaThreads - 32 + B && j > f.j0) {
            // slot j of instance b from the previous step's axpy reduction
            const int b = tid - (kTmaThreads - 32);
            i128 ss;
            uint64_t mw;
            red_pull(&f.red[((rM - 1) % 4) * B + b], ss, mw);
            slot_done(f.inst[b].lz, j, s_ew[b], ss, mw, sX[b], sP[b], s_status[b], s_min_bits[b], blockIdx.x == 0);
        }
        // ---- phase M: u_b = H_b w_j of every instance, instance by instance
        for (int b = 0; b < B; ++b) {
            const LzMultiInst I = f.inst[b];
            if (b != cur) {
                __syncthreads();  // the previous instance's rows and arguments are done with
                const uint64_t* src = reinterpret_cast<const uint64_t*>(f.args + b);
                uint64_t* dst = reinterpret_cast<uint64_t*>(&s_args);
                for (int k = tid; k < (int)(sizeof(MvArgs) / 8); k += blockDim.x) dst[k] = __ldg(src + k);
                __syncthreads();
                cur = b;
            }
            const TmaSmem S = tma_view(s_args, sm, uoff, uent, &give_up);
            if (I.group != staged) {
                if (tid == 0) {
                    tma::fence_proxy_async_smem();
                    tma_issue_tables(s_args, S);
                }
                if (I.kind == kKindRealSched) tma_zero_slots(s_args, S);
                if (!tma::mbar_wait(&S.bar[2], tc & 1)) {
                    if (tid == 0) atomicExch(s_args.err, 1);
                    give_up = 1;
                }
                __syncthreads();
                if (give_up) {
                    if (tid == 0) tma::mbar_wait(&S.bar[2], tc & 1);  // the table copy lands before the CTA leaves
                    return;
                }
                ++tc;
                staged = I.group;
            }
            const int sb = s_args.bq_bits + kFxBits - 62;
            const int s_u = sb > 0 ? sb : 0;
            const int64_t* xq = I.basis + (size_t)j * (size_t)I.stride;
            const bool cplx = I.kind >= kKindCplxFast;
            if (tid == 0 && blockIdx.x < (uint32_t)I.dimUP) {
                if (cplx) multi_first_row<true>(s_args, S, xq, rc);
                else multi_first_row<false>(s_args, S, xq, rc);
            }
            i128 dot = 0;
            uint64_t mx = 0;
            multi_rows<KINDS>(I.kind, s_args, S, xq, I.u, rc, s_u, dot, mx, f.taken + (j & 1) * B + b, &s_next);
            if (give_up) return;
            batch_flush(dot, mx, accl[b], &accm[b]);
        }
        __syncthreads();
        if (tid < B) {
            red_push(&f.red[(rM % 4) * B + tid], batch_total(accl[tid]), accm[tid]);
            accl[tid][0] = accl[tid][1] = accl[tid][2] = 0;
            accm[tid] = 0;
        }
        if (!grid_sync(f.gbar, target, &give_up, f.args[0].err, f.wait)) return;
        if (tid < B) {
            const int b = tid;
            LzState* lz = f.inst[b].lz;
            const MvArgs& ab = f.args[b];
            i128 s;
            uint64_t m;
            red_pull(&f.red[(rM % 4) * B + b], s, m);
            if (blockIdx.x == 0) {
                if (rM >= 2) f.red[((rM - 2) % 4) * B + b] = LzRedSet{0, 0, 0, 0};
                // the other parity's queue counters are next taken from after the next barrier
                f.taken[((j + 1) & 1) * B + b] = 0;
            }
            const int sb = ab.bq_bits + kFxBits - 62;
            const int s_u = sb > 0 ? sb : 0;
            const int e_u = sX[b].e - ab.Fc + s_u;
            s_coef[b] = lz_coefs(j, s, e_u, m, sX[b].e, sX[b].m, sX[b].beta, sX[b].ib, sP[b].e, sP[b].m, sP[b].ib,
                                 s_status[b]);
            s_ew[b] = s_coef[b].e_w;
            if (blockIdx.x == 0) {
                lz->s_u = s_u;
                lz->e_u = e_u;
                lz->m_u = m;
                lz->alpha[j] = s_coef[b].alpha;
                for (int k = 0; k < 3; ++k) {
                    lz->at[k] = s_coef[b].at[k];
                    lz->sh[k] = 0;
                }
                lz->Fa = s_coef[b].Fa;
                lz->e_w = s_coef[b].e_w;
            }
        }
        __syncthreads();

        // ---- phase A: w_{j+1} of every instance, last instance first ------
        for (int b = B - 1; b >= 0; --b) {
            const LzMultiInst I = f.inst[b];
            const int64_t* xq = I.basis + (size_t)j * (size_t)I.stride;
            const int64_t* pq = j > 0 ? I.basis + (size_t)(j - 1) * (size_t)I.stride : xq;
            int64_t* wq = I.basis + (size_t)(j + 1) * (size_t)I.stride;
            const int64_t a0 = s_coef[b].at[0], a1 = s_coef[b].at[1], a2 = s_coef[b].at[2];
            const int Fa = s_coef[b].Fa;
            i128 ss = 0;
            uint64_t mw = 0;
            const int64_t npair = I.n >> 1;
            const longlong2* u2 = reinterpret_cast<const longlong2*>(I.u);
            const longlong2* x2 = reinterpret_cast<const longlong2*>(xq);
            const longlong2* p2 = reinterpret_cast<const longlong2*>(pq);
            longlong2* w2 = reinterpret_cast<longlong2*>(wq);
            for (int64_t i = (int64_t)blockIdx.x * blockDim.x + tid; i < npair; i += (int64_t)G * blockDim.x) {
                const longlong2 uu = __ldcg(u2 + i), xx = __ldcg(x2 + i), pp = __ldcg(p2 + i);
                longlong2 w;
                w.x = shr_round_i64(mul_wide(a0, uu.x) + mul_wide(a1, xx.x) + mul_wide(a2, pp.x), Fa);
                w.y = shr_round_i64(mul_wide(a0, uu.y) + mul_wide(a1, xx.y) + mul_wide(a2, pp.y), Fa);
                w2[i] = w;
                ss += (mul_wide(w.x, w.x) >> 16) + (mul_wide(w.y, w.y) >> 16);
                const uint64_t ax = (uint64_t)(w.x < 0 ? -w.x : w.x), ay = (uint64_t)(w.y < 0 ? -w.y : w.y);
                mw = ax > mw ? ax : mw;
                mw = ay > mw ? ay : mw;
            }
            if ((I.n & 1) && blockIdx.x == 0 && tid == 0) {
                const int64_t i = I.n - 1;
                const int64_t w = shr_round_i64(
                    mul_wide(a0, __ldcg(I.u + i)) + mul_wide(a1, __ldcg(xq + i)) + mul_wide(a2, __ldcg(pq + i)), Fa);
                wq[i] = w;
                ss += mul_wide(w, w) >> 16;
                const uint64_t aw = (uint64_t)(w < 0 ? -w : w);
                mw = aw > mw ? aw : mw;
            }
            batch_flush(ss, mw, accl[b], &accm[b]);
        }
        __syncthreads();
        if (tid < B) {
            red_push(&f.red[(rA % 4) * B + tid], batch_total(accl[tid]), accm[tid]);
            accl[tid][0] = accl[tid][1] = accl[tid][2] = 0;
            accm[tid] = 0;
        }
        if (!grid_sync(f.gbar, target, &give_up, f.args[0].err, f.wait)) return;
        if (tid < B && blockIdx.x == 0) {
            const int b = tid;
            if (rA >= 2) f.red[((rA - 2) % 4) * B + b] = LzRedSet{0, 0, 0, 0};
            if (j + 1 == f.j1) {
                i128 ss;
                uint64_t mw;
                red_pull(&f.red[(rA % 4) * B + b], ss, mw);
                slot_done(f.inst[b].lz, j + 1, s_coef[b].e_w, ss, mw, sX[b], sP[b], s_status[b], s_min_bits[b], true);
            }
        }
        __syncthreads();
    }
}

// Cooperative launch of a heterogeneous batch: f.smem dynamic bytes (the
// largest plan of its operators), as many CTAs as are co-resident (one or
// two per SM; the row queues take any grid).
cudaError_t launch_lz_multi(int device, int kinds, const LzMultiArgs& f, cudaStream_t s) {
    constexpr int kRS = 1 << kKindRealSched, kCS = 1 << kKindCplxSeg, kAll = (1 << 7) - 1;
    const void* fn = (kinds & ~kRS) == 0          ? (const void*)k_lz_multi<kRS>
                     : (kinds & ~kCS) == 0        ? (const void*)k_lz_multi<kCS>
                     : (kinds & ~(kRS | kCS)) == 0 ? (const void*)k_lz_multi<kRS | kCS>
                                                   : (const void*)k_lz_multi<kAll>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, f.smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0, sms = 0, coop = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kTmaThreads, f.smem)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device)) != cudaSuccess) return e;
    if (!coop || per_sm < 1) return cudaErrorNotSupported;
    per_sm = per_sm > 2 ? 2 : per_sm;
    LzMultiArgs fv = f;
    void* args[] = {&fv};
    return cudaLaunchCooperativeKernel(fn, dim3((unsigned)(per_sm * sms)), dim3(kTmaThreads), args, (size_t)f.smem, s);
}

// Cooperative launch of the batch: grid and shared memory of the first
// operator's plan.
cudaError_t launch_lz_batch(const ed_op* op, const LzBatchArgs& f, cudaStream_t s) {
    if (op->tma_smem <= 0 || op->cplx || !op->mv_fast || !op->mv.dnSched) return cudaErrorNotSupported;
    const void* fn = (const void*)k_lz_batch;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, op->tma_smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0, sms = 0, coop = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kTmaThreads, op->tma_smem)) != cudaSuccess)
        return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, op->device)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, op->device)) != cudaSuccess) return e;
    if (!coop || (int64_t)per_sm * sms < op->tma_grid) return cudaErrorNotSupported;
    MvArgs av = op->mv;
    LzBatchArgs fv = f;
    void* args[] = {&av, &fv};
    return cudaLaunchCooperativeKernel(fn, dim3((unsigned)op->tma_grid), dim3(kTmaThreads), args,
                                       (size_t)op->tma_smem, s);
}

GridWait grid_wait_limits() {
    GridWait w{1LL << 26, 4000000000ULL, 0u};
    if (const char* v = std::getenv("ED_GRID_WAIT")) {
        unsigned long long ns = 0;
        unsigned int extra = 0;
        if (std::sscanf(v, "%llu,%u", &ns, &extra) >= 1 && ns > 0) {
            w.ns = ns;
            w.extra = extra;
        }
    }
    return w;
}

// Cooperative launch of steps j0 .. j1-1; cudaErrorNotSupported when the
// operator has no shared-memory plan, or the grid cannot be co-resident.
// f.gbar and the four sets at f.red must be zero.
cudaError_t launch_lz_fused(const ed_op* op, const LzFusedArgs& f, cudaStream_t s) {
    if (op->tma_smem <= 0) return cudaErrorNotSupported;
    const void* fn;
    if (op->cplx)
        fn = op->mv_fast ? (const void*)k_lz_fused<true, true, false>
             : op->mv.upSegE ? (const void*)k_lz_fused<true, false, false, true>
                             : (const void*)k_lz_fused<true, false, false>;
    else if (!op->mv_fast)
        fn = op->mv.upSegE ? (const void*)k_lz_fused<false, false, false, true>
                           : (const void*)k_lz_fused<false, false, false>;
    else
        fn = op->mv.dnSched ? (const void*)k_lz_fused<false, true, true> : (const void*)k_lz_fused<false, true, false>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, op->tma_smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0, sms = 0, coop = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kTmaThreads, op->tma_smem)) != cudaSuccess)
        return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, op->device)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, op->device)) != cudaSuccess) return e;
    // the work queue takes any grid; every CTA must be resident
    const int64_t g = op->lz_grid > 0 ? op->lz_grid : op->tma_grid;
    if (!coop || (int64_t)per_sm * sms < g) return cudaErrorNotSupported;
    MvArgs av = op->mv;
    LzFusedArgs fv = f;
    void* args[] = {&av, &fv};
    return cudaLaunchCooperativeKernel(fn, dim3((unsigned)g), dim3(kTmaThreads), args, (size_t)op->tma_smem, s);
}

}  // namespace ed
