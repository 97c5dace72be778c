// ed_matvec_tma.cu — matvec for spin sectors whose down-spin tables fit in
// shared memory (dim_dn up to a few thousand: chains and clusters up to
// ~14 sites, Kagome/Lieb 12).
//
// Persistent CTAs walk up-rows u = blockIdx.x, + gridDim.x, ...  Each CTA
//  * copies the whole down-spin operator (CSR entries, folded diagonal,
//    bitstrings) into shared memory once per launch;
//  * double-buffers the rows x[u, :] in shared memory with TMA bulk copies
//    (cp.async.bulk global->shared, completion counted on an mbarrier):
//    row u+gridDim.x streams in while row u is computed;
//  * computes the down term entirely from shared memory and the up term
//    with coalesced L2 loads, two output columns per thread so at least
//    eight up-term loads are in flight per thread.
// Every mbarrier wait is bounded: after kMaxSpin polls the CTA records an
// error in *err, stops issuing copies and skips the rest of its rows.
#include <cuda_runtime.h>

#include <cstdint>

#include "ed_device.cuh"
#include "ed_internal.hpp"
#include "ed_matvec_common.cuh"

namespace ed {
using namespace dev;

constexpr int kTmaThreads = 512;
constexpr int kTmaUpStage = 256;
constexpr long long kMaxSpin = 1LL << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// One thread: announce `bytes` of transaction on the barrier and start the
// bulk copy that will complete them.  src, dst 16-byte aligned, bytes % 16 == 0.
__device__ __forceinline__ void tma_row_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
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

template <bool CPLX>
__device__ __forceinline__ void acc_up(const int64_t* __restrict__ xq, uint32_t idx, int64_t& r, int64_t& i) {
    int64_t vr, vi;
    load_x<CPLX>(xq, idx, vr, vi);
    r += vr;
    if (CPLX) i += vi;
}

template <bool CPLX, int OUT, bool FAST>
__global__ void __launch_bounds__(kTmaThreads, 2) k_matvec_tma(const MvArgs a) {
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ uint32_t uoff[kTmaUpStage];
    __shared__ uint32_t uent[kTmaUpStage];
    __shared__ int give_up;
    constexpr int W = CPLX ? 2 : 1;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm);
    int64_t* const row0 = reinterpret_cast<int64_t*>(sm + a.sm_row0);
    int64_t* const row1 = reinterpret_cast<int64_t*>(sm + a.sm_row1);
    uint32_t* dptr = reinterpret_cast<uint32_t*>(sm + a.sm_dnptr);
    uint32_t* dent = reinterpret_cast<uint32_t*>(sm + a.sm_dnent);
    uint8_t* dnpos = sm + a.sm_dnnpos;
    int64_t* ddq = reinterpret_cast<int64_t*>(sm + a.sm_ddnq);
    uint64_t* dst_ = reinterpret_cast<uint64_t*>(sm + a.sm_stdn);

    const uint32_t dimUP = (uint32_t)a.dimUP, dimDN = (uint32_t)a.dimDN;
    const uint32_t row_bytes = dimDN * W * 8u;
    const int64_t* __restrict__ xq = a.xq;
    const int tid = threadIdx.x, T = blockDim.x;

    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
        give_up = 0;
        if (blockIdx.x < dimUP)
            tma_row_load(row0, xq + (size_t)blockIdx.x * dimDN * W, row_bytes, &bar[0]);
    }
    // down-spin operator into shared memory (overlaps the first row copy);
    // 16-byte loads, several in flight per thread
    const uint32_t nnz = a.dnNnz;
    {
        const uint32_t n4 = nnz / 4;
        const uint4* s4 = reinterpret_cast<const uint4*>(a.dnEntC);
        uint4* d4 = reinterpret_cast<uint4*>(dent);
#pragma unroll 4
        for (uint32_t i = tid; i < n4; i += T) d4[i] = __ldg(s4 + i);
        for (uint32_t i = 4 * n4 + tid; i < nnz; i += T) dent[i] = __ldg(a.dnEntC + i);
    }
    for (uint32_t i = tid; i <= dimDN; i += T) dptr[i] = __ldg(a.dnPtr + i);
#pragma unroll 2
    for (uint32_t i = tid; i < dimDN; i += T) {
        dnpos[i] = FAST ? __ldg(a.dnNpos + i) : 0;
        ddq[i] = __ldg(a.dDNq + i);
        dst_[i] = __ldg(a.stDN + i);
    }
    __syncthreads();

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

    int it = 0;
    bool issued_next = false;  // thread 0: a copy for row u+gridDim.x is in flight
    for (uint32_t u = blockIdx.x; u < dimUP; u += gridDim.x, ++it) {
        const int buf = it & 1;
        const uint32_t parity = (uint32_t)((it >> 1) & 1);
        // prefetch the next row into the other buffer (its readers finished
        // at the barrier that closed the previous iteration)
        const uint32_t un = u + gridDim.x;
        issued_next = false;
        if (tid == 0 && un < dimUP && !give_up) {
            fence_proxy_async();
            tma_row_load(buf ? row0 : row1, xq + (size_t)un * dimDN * W, row_bytes, buf ? &bar[0] : &bar[1]);
            issued_next = true;
        }
        const uint32_t p0 = __ldg(a.upPtr + u), lenU = __ldg(a.upPtr + u + 1) - p0;
        const int nposU = FAST ? (int)__ldg(a.upNpos + u) : 0;
        for (uint32_t k = tid; k < lenU; k += T) {
            const uint32_t e = __ldg(a.upEntC + p0 + k);
            uoff[k] = (e & kColMask) * dimDN;
            uent[k] = e;
        }
        if (!mbar_wait(buf ? &bar[1] : &bar[0], parity)) {
            if (tid == 0) atomicExch(a.err, 1);
            give_up = 1;
        }
        __syncthreads();
        if (give_up) break;
        const int64_t* xrow = buf ? row1 : row0;
        const uint64_t stu = __ldg(a.stUP + u);
        const int64_t du = __ldg(a.dUPq + u);
        const uint32_t ubase = u * dimDN;

        for (uint32_t d0 = tid; d0 < dimDN; d0 += 2 * T) {
            const uint32_t d1 = d0 + T;
            const bool v1 = d1 < dimDN;
            const uint32_t d1c = v1 ? d1 : d0;  // clamp: the second column repeats d0 and is not stored
            i128 ar0 = 0, ai0 = 0, ar1 = 0, ai1 = 0;
            if (FAST) {
                int64_t upr0 = 0, upi0 = 0, unr0 = 0, uni0 = 0, upr1 = 0, upi1 = 0, unr1 = 0, uni1 = 0;
                int k = 0;
#pragma unroll 4
                for (; k < nposU; ++k) {
                    const uint32_t o = uoff[k];
                    acc_up<CPLX>(xq, o + d0, upr0, upi0);
                    acc_up<CPLX>(xq, o + d1c, upr1, upi1);
                }
#pragma unroll 4
                for (; k < (int)lenU; ++k) {
                    const uint32_t o = uoff[k];
                    acc_up<CPLX>(xq, o + d0, unr0, uni0);
                    acc_up<CPLX>(xq, o + d1c, unr1, uni1);
                }
                int64_t dr[2] = {0, 0}, di[2] = {0, 0};
#pragma unroll
                for (int c = 0; c < 2; ++c) {
                    const uint32_t d = c ? d1c : d0;
                    const uint32_t q0 = dptr[d], q1 = dptr[d + 1], qp = q0 + dnpos[d];
                    int64_t pr = 0, pi = 0, nr = 0, ni = 0;
                    for (uint32_t q = q0; q < qp; ++q) {
                        const uint32_t col = (dent[q] & kColMask) * W;
                        pr += xrow[col];
                        if (CPLX) pi += xrow[col + 1];
                    }
                    for (uint32_t q = qp; q < q1; ++q) {
                        const uint32_t col = (dent[q] & kColMask) * W;
                        nr += xrow[col];
                        if (CPLX) ni += xrow[col + 1];
                    }
                    dr[c] = pr - nr;
                    di[c] = pi - ni;
                }
                if (merge) {
                    apply_class<CPLX>(ar0, ai0, (upr0 - unr0) + dr[0], (upi0 - uni0) + di[0], a.coefUP, 0, unitU, a.Fc);
                    apply_class<CPLX>(ar1, ai1, (upr1 - unr1) + dr[1], (upi1 - uni1) + di[1], a.coefUP, 0, unitU, a.Fc);
                } else {
                    if (lenU) {
                        apply_class<CPLX>(ar0, ai0, upr0 - unr0, upi0 - uni0, a.coefUP, 0, unitU, a.Fc);
                        apply_class<CPLX>(ar1, ai1, upr1 - unr1, upi1 - uni1, a.coefUP, 0, unitU, a.Fc);
                    }
                    if (a.nclsDN) {
                        apply_class<CPLX>(ar0, ai0, dr[0], di[0], a.coefDN, 0, unitD, a.Fc);
                        apply_class<CPLX>(ar1, ai1, dr[1], di[1], a.coefDN, 0, unitD, a.Fc);
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
                            const uint32_t e = uent[k];
                            const int cl = (int)((e >> kClassShift) & kClassMask);
                            if (cl != cur) {
                                if (cur >= 0) apply_class<CPLX>(ar, ai, sr, si, a.coefUP, cur, unitU, a.Fc);
                                sr = 0; si = 0; cur = cl;
                            }
                            int64_t r, i;
                            load_x<CPLX>(xq, uoff[k] + d, r, i);
                            sr += apply_sign(r, e);
                            if (CPLX) si += apply_sign(i, e);
                        }
                        if (cur >= 0) apply_class<CPLX>(ar, ai, sr, si, a.coefUP, cur, unitU, a.Fc);
                    }
                    {
                        int cur = -1;
                        int64_t sr = 0, si = 0;
                        for (uint32_t q = dptr[d]; q < dptr[d + 1]; ++q) {
                            const uint32_t e = dent[q];
                            const int cl = (int)((e >> kClassShift) & kClassMask);
                            if (cl != cur) {
                                if (cur >= 0) apply_class<CPLX>(ar, ai, sr, si, a.coefDN, cur, unitD, a.Fc);
                                sr = 0; si = 0; cur = cl;
                            }
                            const uint32_t col = (e & kColMask) * W;
                            sr += apply_sign(xrow[col], e);
                            if (CPLX) si += apply_sign(xrow[col + 1], e);
                        }
                        if (cur >= 0) apply_class<CPLX>(ar, ai, sr, si, a.coefDN, cur, unitD, a.Fc);
                    }
                }
            }
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                if (c == 1 && !v1) break;
                const uint32_t d = c ? d1 : d0;
                i128& ar = c ? ar1 : ar0;
                i128& ai = c ? ai1 : ai0;
                const int64_t xr = xrow[d * W];
                const int64_t xi = CPLX ? xrow[d * W + 1] : 0;
                const int64_t dq = du + ddq[d] + a.Uq * (int64_t)__popcll(stu & dst_[d] & a.mask);
                ar += mul_wide(dq, xr);
                if (CPLX) ai += mul_wide(dq, xi);
                const size_t o = (size_t)(ubase + d) * W;
                if (OUT == 0) {
                    a.y[o] = i128_to_f64(ar, E_out);
                    if (CPLX) a.y[o + 1] = i128_to_f64(ai, E_out);
                } else {
                    const int64_t qr = shr_round_i64(ar, s_u);
                    a.uq[o] = qr;
                    dot += mul_wide(xr, qr) >> 24;
                    uint64_t aq = (uint64_t)(qr < 0 ? -qr : qr);
                    mx = aq > mx ? aq : mx;
                    if (CPLX) {
                        const int64_t qi = shr_round_i64(ai, s_u);
                        a.uq[o + 1] = qi;
                        dot += mul_wide(xi, qi) >> 24;
                        aq = (uint64_t)(qi < 0 ? -qi : qi);
                        mx = aq > mx ? aq : mx;
                    }
                }
            }
        }
        __syncthreads();  // row buffer and uoff are free for the next iteration
    }
    // a copy issued for a row this CTA will not reach can only exist after a
    // give-up; wait for it (bounded) so no transfer outlives the CTA
    if (give_up && tid == 0 && issued_next) {
        const int bufn = it & 1;
        mbar_wait(bufn ? &bar[0] : &bar[1], (uint32_t)(((it + 1) >> 1) & 1));
    }
    if (OUT == 1) mv_lanczos_epilogue(a, dot, mx, s_u);
}

// Shared-memory plan: returns the dynamic bytes (0 when the sector does not
// fit or rows are not 16-byte multiples).
int tma_plan(const ed_op* op, MvArgs* a) {
    const int W = op->cplx ? 2 : 1;
    const int64_t dimDN = op->dimDN;
    const int64_t row_bytes = dimDN * W * 8;
    if (row_bytes % 16 != 0) return 0;
    auto up16 = [](int64_t v) { return (v + 127) / 128 * 128; };
    int64_t off = 128;  // two mbarriers
    a->sm_row0 = (int)off;
    off += up16(row_bytes);
    a->sm_row1 = (int)off;
    off += up16(row_bytes);
    a->sm_dnptr = (int)off;
    off += up16((dimDN + 1) * 4);
    a->sm_dnent = (int)off;
    off += up16(op->tdn.nnz * 4);
    a->sm_dnnpos = (int)off;
    off += up16(dimDN);
    a->sm_ddnq = (int)off;
    off += up16(dimDN * 8);
    a->sm_stdn = (int)off;
    off += up16(dimDN * 8);
    const int64_t static_bytes = 2 * kTmaUpStage * 4 + 64 + 8 * 64;  // uoff, uent, reduction scratch
    if (off + static_bytes > 227 * 1024) return 0;
    return (int)off;
}

template <bool CPLX, int OUT, bool FAST>
static cudaError_t launch_tma3(const ed_op* op, const MvArgs& a, cudaStream_t s) {
    auto kern = k_matvec_tma<CPLX, OUT, FAST>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, op->tma_smem);
    if (e != cudaSuccess) return e;
    kern<<<op->tma_grid, kTmaThreads, op->tma_smem, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_matvec_tma(const ed_op* op, const MvArgs& a, int out, cudaStream_t s) {
    if (op->cplx) {
        if (out == 0) return op->mv_fast ? launch_tma3<true, 0, true>(op, a, s) : launch_tma3<true, 0, false>(op, a, s);
        return op->mv_fast ? launch_tma3<true, 1, true>(op, a, s) : launch_tma3<true, 1, false>(op, a, s);
    }
    if (out == 0) return op->mv_fast ? launch_tma3<false, 0, true>(op, a, s) : launch_tma3<false, 0, false>(op, a, s);
    return op->mv_fast ? launch_tma3<false, 1, true>(op, a, s) : launch_tma3<false, 1, false>(op, a, s);
}

int tma_grid(const ed_op* op) {
    int per_sm = 0;
    const void* f = op->mv_fast ? (const void*)k_matvec_tma<false, 1, true> : (const void*)k_matvec_tma<false, 1, false>;
    if (op->cplx) f = op->mv_fast ? (const void*)k_matvec_tma<true, 1, true> : (const void*)k_matvec_tma<true, 1, false>;
    cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, op->tma_smem);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, kTmaThreads, op->tma_smem) != cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, op->device);
    int64_t g = (int64_t)sms * per_sm;
    if (g > op->dimUP) g = op->dimUP;
    return (int)(g < 1 ? 1 : g);
}

}  // namespace ed
