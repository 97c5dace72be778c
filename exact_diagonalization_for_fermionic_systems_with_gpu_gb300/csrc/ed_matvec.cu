// ed_matvec.cu — the spin-split Hubbard matvec on sm_103a.
//
// y[u, d] = sum_k c_up(u,k) x[j_up(u,k), d]          (H_up (x) 1)
//         + sum_k c_dn(d,k) x[u, j_dn(d,k)]          (1 (x) H_dn)
//         + (eps_up[u] + eps_dn[d] + U popc(s_up[u] & s_dn[d] & mask)) x[u, d]
// (the reference kernel Hubbard_mv_, MBL_test/include/HubMatrix_GPU.cuh:114-161).
//
// Work decomposition: one CTA per up-row u (grid-stride), threads over the
// down index d.  The CTA stages row u of x (and the row's up-table entries)
// in shared memory; the down term then gathers from shared memory, the up
// term reads rows j_up(u,k) of x with loads coalesced over d.  Each +-x is an
// exact int64 add; each distinct coefficient (a "class") multiplies its
// partial sum once, 64x64->128 bits, so the only rounding is the final one.
#include <cuda_runtime.h>

#include "ed_device.cuh"
#include "ed_internal.hpp"
#include "ed_lanczos.hpp"
#include "ed_lanczos_dev.cuh"

namespace ed {
using namespace dev;

constexpr int kMvThreads = 256;
constexpr int kUpStage = 256;  // up-table entries staged per row (max row length 255)

// --------------------------------------------------------------- FX input --

__global__ void k_emax(const double* __restrict__ x, int64_t n, int* emax, int* flag) {
    int local = 0, bad = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int be = f64_biased_exp(x[i]);
        bad |= (be == 2047);
        local = be > local ? be : local;
    }
    __shared__ int scratch[32];
    int r = block_max_int(local, scratch);
    if (threadIdx.x == 0) atomicMax(emax, r);
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1);
}

__global__ void k_to_fx(const double* __restrict__ x, int64_t n, const int* __restrict__ emax,
                        int64_t* __restrict__ xq) {
    const int E = fx_exp_from_emax(*emax);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        xq[i] = f64_to_fx(x[i], E);
}

static int elementwise_grid(int64_t n) {
    int64_t g = (n + 255) / 256;
    if (g > 152 * 16) g = 152 * 16;
    return (int)(g < 1 ? 1 : g);
}

cudaError_t launch_emax(const double* x, int64_t n, int* d_emax, int* d_flag, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(d_emax, 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(d_flag, 0, sizeof(int), s)) != cudaSuccess) return e;
    k_emax<<<elementwise_grid(n), 256, 0, s>>>(x, n, d_emax, d_flag);
    return cudaGetLastError();
}

cudaError_t launch_to_fx(const double* x, int64_t n, const int* d_emax, int64_t* xq, cudaStream_t s) {
    k_to_fx<<<elementwise_grid(n), 256, 0, s>>>(x, n, d_emax, xq);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ matvec --

__device__ __forceinline__ int64_t apply_sign(int64_t v, uint32_t e) {
    int64_t m = (int64_t)((int32_t)e >> 31);  // 0 or -1
    return (v ^ m) - m;
}

template <bool CPLX>
__device__ __forceinline__ void apply_class(i128& ar, i128& ai, int64_t sr, int64_t si,
                                            const int64_t* __restrict__ coef, int c, bool unit, int Fc) {
    if (unit) {
        ar += ((i128)sr) << Fc;
        if (CPLX) ai += ((i128)si) << Fc;
        return;
    }
    const int64_t cr = coef[2 * c];
    ar += mul_wide(sr, cr);
    if (CPLX) {
        const int64_t ci = coef[2 * c + 1];
        ai += mul_wide(si, cr);
        if (ci != 0) {
            ar -= mul_wide(si, ci);
            ai += mul_wide(sr, ci);
        }
    }
}

// OUT = 0: FP64 y (operator apply); OUT = 1: FX u with the Lanczos epilogue.
template <bool CPLX, bool STAGE, int OUT>
__global__ void __launch_bounds__(kMvThreads) k_matvec(const MvArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int W = CPLX ? 2 : 1;
    uint32_t* ups = reinterpret_cast<uint32_t*>(smem_raw);                 // kUpStage entries
    int64_t* xs = reinterpret_cast<int64_t*>(smem_raw + kUpStage * sizeof(uint32_t));  // staged row

    const int64_t dimUP = a.dimUP, dimDN = a.dimDN;
    int E_out = 0, s_u = 0;
    if (OUT == 0) {
        E_out = fx_exp_from_emax(*a.p_emax) - a.Fc;
    } else {
        int b = a.bq_bits + bitlen_u64(*a.p_mx) - 62;
        s_u = b > 0 ? b : 0;
    }
    i128 dot = 0;
    uint64_t mx = 0;
    const bool merge = a.mergeUD != 0;
    const bool unitU = a.unitUP != 0 && a.nclsUP == 1;
    const bool unitD = a.unitDN != 0 && a.nclsDN == 1;

    for (int64_t u = blockIdx.x; u < dimUP; u += gridDim.x) {
        const int lenU = a.upLen[u];
        __syncthreads();  // the previous row's staged data is no longer read
        for (int k = threadIdx.x; k < lenU; k += blockDim.x) ups[k] = a.upEnt[(int64_t)k * dimUP + u];
        const int64_t* xrow = a.xq + u * dimDN * W;
        if (STAGE) {
            const int64_t nrow = dimDN * W;
            if ((nrow & 1) == 0) {
                const longlong2* src = reinterpret_cast<const longlong2*>(xrow);
                longlong2* dst = reinterpret_cast<longlong2*>(xs);
                for (int64_t i = threadIdx.x; i < nrow / 2; i += blockDim.x) dst[i] = src[i];
            } else {
                for (int64_t i = threadIdx.x; i < nrow; i += blockDim.x) xs[i] = xrow[i];
            }
            xrow = xs;
        }
        __syncthreads();
        const uint64_t stu = a.stUP[u];
        const int64_t du = a.dUPq[u];

        for (int64_t d = threadIdx.x; d < dimDN; d += blockDim.x) {
            i128 ar = 0, ai = 0;
            const int lenD = a.dnLen[d];
            if (merge) {
                int64_t sr = 0, si = 0;
                for (int k = 0; k < lenU; ++k) {
                    const uint32_t e = ups[k];
                    const int64_t idx = ((int64_t)(e & kColMask) * dimDN + d) * W;
                    if (CPLX) {
                        const longlong2 v = *reinterpret_cast<const longlong2*>(a.xq + idx);
                        sr += apply_sign(v.x, e);
                        si += apply_sign(v.y, e);
                    } else {
                        sr += apply_sign(a.xq[idx], e);
                    }
                }
                for (int k = 0; k < lenD; ++k) {
                    const uint32_t e = a.dnEnt[(int64_t)k * dimDN + d];
                    const int64_t c = (int64_t)(e & kColMask) * W;
                    sr += apply_sign(xrow[c], e);
                    if (CPLX) si += apply_sign(xrow[c + 1], e);
                }
                apply_class<CPLX>(ar, ai, sr, si, a.coefUP, 0, unitU, a.Fc);
            } else {
                // up term, entries sorted by class
                {
                    int cur = -1;
                    int64_t sr = 0, si = 0;
                    for (int k = 0; k < lenU; ++k) {
                        const uint32_t e = ups[k];
                        const int c = (int)((e >> kClassShift) & kClassMask);
                        if (c != cur) {
                            if (cur >= 0) apply_class<CPLX>(ar, ai, sr, si, a.coefUP, cur, unitU, a.Fc);
                            sr = 0; si = 0; cur = c;
                        }
                        const int64_t idx = ((int64_t)(e & kColMask) * dimDN + d) * W;
                        if (CPLX) {
                            const longlong2 v = *reinterpret_cast<const longlong2*>(a.xq + idx);
                            sr += apply_sign(v.x, e);
                            si += apply_sign(v.y, e);
                        } else {
                            sr += apply_sign(a.xq[idx], e);
                        }
                    }
                    if (cur >= 0) apply_class<CPLX>(ar, ai, sr, si, a.coefUP, cur, unitU, a.Fc);
                }
                // down term
                {
                    int cur = -1;
                    int64_t sr = 0, si = 0;
                    for (int k = 0; k < lenD; ++k) {
                        const uint32_t e = a.dnEnt[(int64_t)k * dimDN + d];
                        const int c = (int)((e >> kClassShift) & kClassMask);
                        if (c != cur) {
                            if (cur >= 0) apply_class<CPLX>(ar, ai, sr, si, a.coefDN, cur, unitD, a.Fc);
                            sr = 0; si = 0; cur = c;
                        }
                        const int64_t col = (int64_t)(e & kColMask) * W;
                        sr += apply_sign(xrow[col], e);
                        if (CPLX) si += apply_sign(xrow[col + 1], e);
                    }
                    if (cur >= 0) apply_class<CPLX>(ar, ai, sr, si, a.coefDN, cur, unitD, a.Fc);
                }
            }
            // diagonal: folded site potentials + U * double occupancy
            const int64_t xr = xrow[d * W];
            const int64_t xi = CPLX ? xrow[d * W + 1] : 0;
            const int64_t dq = du + a.dDNq[d] + a.Uq * (int64_t)__popcll(stu & a.stDN[d] & a.mask);
            ar += mul_wide(dq, xr);
            if (CPLX) ai += mul_wide(dq, xi);

            const int64_t o = (u * dimDN + d) * W;
            if (OUT == 0) {
                a.y[o] = i128_to_f64(ar, E_out);
                if (CPLX) a.y[o + 1] = i128_to_f64(ai, E_out);
            } else {
                const int64_t qr = (int64_t)shr_round(ar, s_u);
                a.uq[o] = qr;
                dot += mul_wide(xr, qr) >> 24;
                uint64_t aq = (uint64_t)(qr < 0 ? -qr : qr);
                mx = aq > mx ? aq : mx;
                if (CPLX) {
                    const int64_t qi = (int64_t)shr_round(ai, s_u);
                    a.uq[o + 1] = qi;
                    dot += mul_wide(xi, qi) >> 24;
                    aq = (uint64_t)(qi < 0 ? -qi : qi);
                    mx = aq > mx ? aq : mx;
                }
            }
        }
    }

    if (OUT == 1) {
        __shared__ i128 s128[32];
        __shared__ uint64_t s64[32];
        LzState* lz = reinterpret_cast<LzState*>(a.lz);
        const i128 bs = block_sum_i128(dot, s128);
        const uint64_t bm = block_max_u64(mx, s64);
        if (threadIdx.x == 0) {
            lz->part_lo[blockIdx.x] = (uint64_t)bs;
            lz->part_hi[blockIdx.x] = (uint64_t)((u128)bs >> 64);
            lz->part_max[blockIdx.x] = bm;
        }
        if (elect_last_block(&lz->counter[0])) {
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
                lz_after_matvec(lz, a.step, s, m, s_u, a.Fc);
                lz->counter[0] = 0;
            }
        }
    }
}

// ------------------------------------------------------------------ launch --

int matvec_grid(const ed_op* op) {
    int64_t g = op->dimUP;
    const int64_t cap = 152 * 8;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

template <bool CPLX, int OUT>
static cudaError_t launch_mv(const ed_op* op, const MvArgs& a, cudaStream_t s) {
    const int smem = kUpStage * (int)sizeof(uint32_t) + op->stage_smem;
    if (op->stage_smem > 0) {
        auto kern = k_matvec<CPLX, true, OUT>;
        if (smem > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            if (e != cudaSuccess) return e;
        }
        kern<<<op->grid, kMvThreads, smem, s>>>(a);
    } else {
        k_matvec<CPLX, false, OUT><<<op->grid, kMvThreads, smem, s>>>(a);
    }
    return cudaGetLastError();
}

cudaError_t launch_matvec_f64(const ed_op* op, const int64_t* xq, const int* d_emax, double* y,
                              cudaStream_t s) {
    MvArgs a = op->mv;
    a.xq = xq;
    a.p_emax = d_emax;
    a.y = y;
    return op->cplx ? launch_mv<true, 0>(op, a, s) : launch_mv<false, 0>(op, a, s);
}

cudaError_t launch_matvec_lz(const ed_op* op, const int64_t* xq, int64_t* uq, void* lz,
                             const uint64_t* d_mx, int step, cudaStream_t s) {
    MvArgs a = op->mv;
    a.xq = xq;
    a.uq = uq;
    a.lz = lz;
    a.step = step;
    a.p_mx = d_mx;
    return op->cplx ? launch_mv<true, 1>(op, a, s) : launch_mv<false, 1>(op, a, s);
}

}  // namespace ed
