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

#include <cmath>

#include "ed_device.cuh"
#include "ed_internal.hpp"
#include "ed_lanczos.hpp"
#include "ed_lanczos_dev.cuh"
#include "ed_matvec_common.cuh"

namespace ed {
using namespace dev;

constexpr int kMvMaxThreads = 512;
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

// OUT = 0: FP64 y (operator apply); OUT = 1: FX u with the Lanczos epilogue.
// FAST: at most one coefficient class per spin; each row's entries are
// ordered positive-then-negative, so a hop is one load and one 64-bit add.
template <bool CPLX, bool STAGE, int OUT, bool FAST>
__global__ void __launch_bounds__(kMvMaxThreads) k_matvec(const MvArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int W = CPLX ? 2 : 1;
    uint32_t* uoff = reinterpret_cast<uint32_t*>(smem_raw);                          // kUpStage
    uint32_t* uent = uoff + kUpStage;                                                  // kUpStage
    int64_t* xs = reinterpret_cast<int64_t*>(smem_raw + 2 * kUpStage * sizeof(uint32_t));  // staged row

    const uint32_t dimUP = (uint32_t)a.dimUP, dimDN = (uint32_t)a.dimDN;
    const int64_t* __restrict__ xq = a.xq;
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

    for (uint32_t u = blockIdx.x; u < dimUP; u += gridDim.x) {
        const int lenU = a.upLen[u];
        const int nposU = FAST ? (int)a.upNpos[u] : 0;
        __syncthreads();  // the previous row's staged data is no longer read
        for (int k = threadIdx.x; k < lenU; k += blockDim.x) {
            const uint32_t e = a.upEnt[(size_t)k * dimUP + u];
            uoff[k] = (e & kColMask) * dimDN;
            if (!FAST) uent[k] = e;
        }
        const int64_t* xrow = xq + (size_t)u * dimDN * W;
        if (STAGE) {
            const uint32_t nrow = dimDN * W;
            if ((nrow & 1) == 0) {
                const longlong2* src = reinterpret_cast<const longlong2*>(xrow);
                longlong2* dst = reinterpret_cast<longlong2*>(xs);
                for (uint32_t i = threadIdx.x; i < nrow / 2; i += blockDim.x) dst[i] = __ldg(src + i);
            } else {
                for (uint32_t i = threadIdx.x; i < nrow; i += blockDim.x) xs[i] = __ldg(xrow + i);
            }
            xrow = xs;
        }
        __syncthreads();
        const uint64_t stu = a.stUP[u];
        const int64_t du = a.dUPq[u];
        const uint32_t ubase = u * dimDN;

        for (uint32_t d = threadIdx.x; d < dimDN; d += blockDim.x) {
            i128 ar = 0, ai = 0;
            const int lenD = a.dnLen[d];
            const uint32_t* __restrict__ de = a.dnEnt + d;
            if (FAST) {
                int64_t upr = 0, upi = 0, unr = 0, uni = 0;  // up term, + and - entries
                int k = 0;
#pragma unroll 4
                for (; k < nposU; ++k) {
                    int64_t r, i;
                    load_x<CPLX>(xq, uoff[k] + d, r, i);
                    upr += r;
                    if (CPLX) upi += i;
                }
#pragma unroll 4
                for (; k < lenU; ++k) {
                    int64_t r, i;
                    load_x<CPLX>(xq, uoff[k] + d, r, i);
                    unr += r;
                    if (CPLX) uni += i;
                }
                int64_t dpr = 0, dpi = 0, dnr = 0, dni = 0;  // down term
                const int nposD = a.dnNpos[d];
                int kk = 0;
#pragma unroll 4
                for (; kk < nposD; ++kk) {
                    const uint32_t c = (__ldg(de + (size_t)kk * dimDN) & kColMask) * W;
                    dpr += xrow[c];
                    if (CPLX) dpi += xrow[c + 1];
                }
#pragma unroll 4
                for (; kk < lenD; ++kk) {
                    const uint32_t c = (__ldg(de + (size_t)kk * dimDN) & kColMask) * W;
                    dnr += xrow[c];
                    if (CPLX) dni += xrow[c + 1];
                }
                if (merge) {
                    apply_class<CPLX>(ar, ai, (upr + dpr) - (unr + dnr), (upi + dpi) - (uni + dni), a.coefUP, 0,
                                      unitU, a.Fc);
                } else {
                    if (lenU) apply_class<CPLX>(ar, ai, upr - unr, upi - uni, a.coefUP, 0, unitU, a.Fc);
                    if (lenD) apply_class<CPLX>(ar, ai, dpr - dnr, dpi - dni, a.coefDN, 0, unitD, a.Fc);
                }
            } else {
                // general tables: entries sorted by class, sign per entry
                {
                    int cur = -1;
                    int64_t sr = 0, si = 0;
                    for (int k = 0; k < lenU; ++k) {
                        const uint32_t e = uent[k];
                        const int c = (int)((e >> kClassShift) & kClassMask);
                        if (c != cur) {
                            if (cur >= 0) apply_class<CPLX>(ar, ai, sr, si, a.coefUP, cur, unitU, a.Fc);
                            sr = 0; si = 0; cur = c;
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
                    for (int k = 0; k < lenD; ++k) {
                        const uint32_t e = __ldg(de + (size_t)k * dimDN);
                        const int c = (int)((e >> kClassShift) & kClassMask);
                        if (c != cur) {
                            if (cur >= 0) apply_class<CPLX>(ar, ai, sr, si, a.coefDN, cur, unitD, a.Fc);
                            sr = 0; si = 0; cur = c;
                        }
                        const uint32_t col = (e & kColMask) * W;
                        sr += apply_sign(xrow[col], e);
                        if (CPLX) si += apply_sign(xrow[col + 1], e);
                    }
                    if (cur >= 0) apply_class<CPLX>(ar, ai, sr, si, a.coefDN, cur, unitD, a.Fc);
                }
            }
            // diagonal: folded site potentials + U * double occupancy
            const int64_t xr = xrow[d * W];
            const int64_t xi = CPLX ? xrow[d * W + 1] : 0;
            const int64_t dq = du + __ldg(a.dDNq + d) + a.Uq * (int64_t)__popcll(stu & __ldg(a.stDN + d) & a.mask);
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

    if (OUT == 1) mv_lanczos_epilogue(a, dot, mx, s_u);
}

// ------------------------------------------------------------------ launch --

int matvec_grid(const ed_op* op) {
    int64_t g = op->dimUP;
    const int64_t cap = 152 * 8;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

// Threads per CTA: a multiple of 32 in [128, 512] that covers the down index
// in as few passes as possible with little idle tail.
int matvec_threads(int64_t dimDN) {
    int best = 256;
    double best_eff = 0.0;
    for (int t = 128; t <= kMvMaxThreads; t += 32) {
        const int64_t passes = (dimDN + t - 1) / t;
        const double eff = (double)dimDN / (double)(passes * t);
        if (eff > best_eff + 1e-9 || (std::fabs(eff - best_eff) < 1e-9 && t > best)) {
            best_eff = eff;
            best = t;
        }
    }
    return best;
}

template <bool CPLX, int OUT, bool FAST>
static cudaError_t launch_mv3(const ed_op* op, const MvArgs& a, cudaStream_t s) {
    const int smem = 2 * kUpStage * (int)sizeof(uint32_t) + op->stage_smem;
    if (op->stage_smem > 0) {
        auto kern = k_matvec<CPLX, true, OUT, FAST>;
        if (smem > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            if (e != cudaSuccess) return e;
        }
        kern<<<op->grid, op->mv_threads, smem, s>>>(a);
    } else {
        k_matvec<CPLX, false, OUT, FAST><<<op->grid, op->mv_threads, smem, s>>>(a);
    }
    return cudaGetLastError();
}

template <bool CPLX, int OUT>
static cudaError_t launch_mv(const ed_op* op, const MvArgs& a, cudaStream_t s) {
    return op->mv_fast ? launch_mv3<CPLX, OUT, true>(op, a, s) : launch_mv3<CPLX, OUT, false>(op, a, s);
}

cudaError_t striped_args(ed_op* op, const int64_t* xq, StripedArgs* g) {
    if (!op->d_sdn) {
        cudaError_t e = cudaMalloc(&op->d_sdn, sizeof(int64_t) * (size_t)op->D);
        if (e != cudaSuccess) return e;
    }
    g->xq = xq;
    g->sdn = op->d_sdn;
    g->dimUP = op->dimUP;
    g->dimDN = op->dimDN;
    g->sched16 = op->d_sched16;
    g->steps32 = op->d_steps32;
    g->negcnt = op->d_negDN;
    g->cpad = op->st_cpad;
    g->s8 = op->st_s8;
    g->bw = op->st_bw;
    g->chunk = op->st_chunk;
    g->zbase = op->st_zbase;

    g->dDNq = op->d_dDNqP;
    g->stDN = op->d_stDNp;
    g->err = op->d_err;
    return cudaSuccess;
}

cudaError_t launch_matvec_f64(const ed_op* op, const int64_t* xq, const int* d_emax, double* y,
                              cudaStream_t s) {
    MvArgs a = op->mv;
    a.xq = xq;
    a.p_emax = d_emax;
    a.y = y;
    // the FP64 apply stays in table order: for one product the two-pass
    // matvec's permutations in and out cost more than they save (the
    // Lanczos path, which permutes once per solve, uses it)
    if (op->tma_smem > 0) return launch_matvec_tma(op, a, 0, s);
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
    if (op->striped) {
        StripedArgs g;
        cudaError_t e = striped_args(const_cast<ed_op*>(op), xq, &g);
        if (e == cudaSuccess) e = launch_striped_down(op, g, s);
        if (e == cudaSuccess) e = launch_striped_up(op, a, g, 1, s);
        return e;
    }
    if (op->tma_smem > 0) return launch_matvec_tma(op, a, 1, s);
    return op->cplx ? launch_mv<true, 1>(op, a, s) : launch_mv<false, 1>(op, a, s);
}

}  // namespace ed
