// ed_krylov.cu — Krylov time evolution psi(t) = exp(-i H t) psi0.
//
// The reference (Krylov<C>, MBL_test/include/HubMatrix_GPU.cuh:619-728)
// builds the tridiagonal T of psi0 with up to 1000 Lanczos steps, stopping
// at b < 1e-10, diagonalises it with LAPACK dsted, and for every time step
// regenerates the Krylov vectors with one Hubbard_mv each while adding
// (sum_j e^{-i m_j t} z_j[0] z_j[i]) v_i into phi.
//
// Here the recurrence is the Lanczos run of ed_lanczos.cu (the persistent
// kernel where the operator has one), its basis kept in device memory in the
// FX format (v_k = q_k 2^e_k / beta_k); T's propagator column
// exp(-i T t) e_0 comes from the host QR solver (ed_tridiag.cpp); and one
// kernel forms psi(t) = beta_0 sum_k c_k(t) v_k for up to kKrTimes times per
// pass over the basis.  Each time costs one read of the basis instead of
// the reference's n matvecs.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/ed_hubbard.h"
#include "ed_internal.hpp"
#include "ed_tridiag.hpp"

namespace ed {
namespace {

constexpr int kKrThreads = 256;
constexpr int kKrTimes = 8;  // times formed per pass over the basis
constexpr int kKrBlocks = 152 * 8;

int kr_grid(int64_t n) {
    int64_t g = (n + kKrThreads - 1) / kKrThreads;
    return (int)std::max<int64_t>(1, std::min<int64_t>(g, kKrBlocks));
}

// per block: sum of squares of the real and of the imaginary parts
__global__ void k_part_norms(const double* __restrict__ z, int64_t n, double* __restrict__ part) {
    double s0 = 0.0, s1 = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double2 v = reinterpret_cast<const double2*>(z)[i];
        s0 = fma(v.x, v.x, s0);
        s1 = fma(v.y, v.y, s1);
    }
    __shared__ double r0[kKrThreads], r1[kKrThreads];
    r0[threadIdx.x] = s0;
    r1[threadIdx.x] = s1;
    __syncthreads();
    for (int w = kKrThreads / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            r0[threadIdx.x] += r0[threadIdx.x + w];
            r1[threadIdx.x] += r1[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = r0[0];
        part[2 * blockIdx.x + 1] = r1[0];
    }
}

// real vector of part p (0: re, 1: im) of n complex values
__global__ void k_part(const double* __restrict__ z, int64_t n, int p, double* __restrict__ out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = z[2 * i + p];
}

// out[t] = (accumulate ? out[t] : 0) + f * sum_k coef[t][k] q_k for t < nt,
// f = i when times_i, else 1; q_k real (CPLX false) or complex.
template <bool CPLX>
__global__ void __launch_bounds__(kKrThreads) k_krylov_combine(const int64_t* __restrict__ basis, int64_t stride,
                                                               int64_t n, int nk, const double2* __restrict__ coef,
                                                               int nt, double2* __restrict__ out, int64_t out_stride,
                                                               int accumulate, int times_i) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double2 acc[kKrTimes];
#pragma unroll
        for (int t = 0; t < kKrTimes; ++t) acc[t] = make_double2(0.0, 0.0);
        for (int k = 0; k < nk; ++k) {
            double wr, wi = 0.0;
            if (CPLX) {
                const longlong2 q = __ldg(reinterpret_cast<const longlong2*>(basis + (size_t)k * stride) + i);
                wr = (double)q.x;
                wi = (double)q.y;
            } else {
                wr = (double)__ldg(basis + (size_t)k * stride + i);
            }
#pragma unroll
            for (int t = 0; t < kKrTimes; ++t) {
                if (t < nt) {
                    const double2 c = __ldg(coef + (size_t)t * nk + k);
                    acc[t].x = fma(c.x, wr, fma(-c.y, wi, acc[t].x));
                    acc[t].y = fma(c.x, wi, fma(c.y, wr, acc[t].y));
                }
            }
        }
#pragma unroll
        for (int t = 0; t < kKrTimes; ++t) {
            if (t < nt) {
                double2 v = times_i ? make_double2(-acc[t].y, acc[t].x) : acc[t];
                double2* o = out + (size_t)t * out_stride + i;
                if (accumulate) {
                    const double2 p = *o;
                    v.x += p.x;
                    v.y += p.y;
                }
                *o = v;
            }
        }
    }
}

// Two-pass-matvec operators (the basis is not kept): out[t][p(i)] +=
// f * coef[t] q[i] for the regenerated real vector q in the permuted down
// order, p(i) = u * dim_dn + perm[c] its table-order position, f = i when
// times_i; every position is touched by one thread.
__global__ void __launch_bounds__(kKrThreads) k_krylov_acc_perm(const int64_t* __restrict__ q, int64_t dimUP,
                                                               int64_t dimDN, const uint32_t* __restrict__ perm,
                                                               const double2* __restrict__ coef, int nt,
                                                               double2* __restrict__ out, int64_t out_stride,
                                                               int times_i) {
    const int64_t D = dimUP * dimDN;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t u = i / dimDN, c = i - u * dimDN;
        const int64_t p = u * dimDN + __ldg(perm + c);
        const double w = (double)__ldg(q + i);
        for (int t = 0; t < nt; ++t) {
            const double2 cf = __ldg(coef + t);
            double2* o = out + (size_t)t * out_stride + p;
            double2 v = *o;
            if (times_i) {
                v.x -= cf.y * w;
                v.y += cf.x * w;
            } else {
                v.x += cf.x * w;
                v.y += cf.y * w;
            }
            *o = v;
        }
    }
}

}  // namespace
}  // namespace ed

extern "C" {

ed_status ed_krylov_evolve(ed_op* op, const ed_krylov_cfg* cfg, const double* psi0, int psi0_mem, int n_times,
                           const double* times, double* psi_out, int out_mem, ed_krylov_result* res,
                           void* stream) {
    using namespace ed;
    if (!op || !cfg || !psi0 || n_times < 0 || (n_times > 0 && (!times || !psi_out))) return ED_ERR_ARG;
    if (cfg->max_steps < 1 || cfg->max_steps > 100000 || !(cfg->tol >= 0.0)) return ED_ERR_ARG;
    if (psi0_mem != ED_MEM_HOST && psi0_mem != ED_MEM_DEVICE) return ED_ERR_ARG;
    if (out_mem != ED_MEM_HOST && out_mem != ED_MEM_DEVICE) return ED_ERR_ARG;
    for (int t = 0; t < n_times; ++t)
        if (!std::isfinite(times[t])) return ED_ERR_ARG;
    if (cudaSetDevice(op->device) != cudaSuccess) return ED_ERR_CUDA;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const int64_t D = op->D;
    int64_t launches = 0;
    ed_status st = ED_OK;

    double *d0 = nullptr, *dout = nullptr, *tmp = nullptr, *part = nullptr;
    double2* dcoef = nullptr;
    auto release = [&]() {
        if (psi0_mem == ED_MEM_HOST) cudaFreeAsync(d0, s);
        if (out_mem == ED_MEM_HOST) cudaFreeAsync(dout, s);
        cudaFreeAsync(tmp, s);
        cudaFreeAsync(part, s);
        cudaFreeAsync(dcoef, s);
        cudaStreamSynchronize(s);
    };
#define KR_CK(x)                            \
    do {                                    \
        if ((x) != cudaSuccess) {           \
            release();                      \
            return ED_ERR_CUDA;             \
        }                                   \
    } while (0)

    const size_t vbytes = sizeof(double) * 2 * (size_t)D;
    if (psi0_mem == ED_MEM_HOST) {
        if (cudaMallocAsync(&d0, vbytes, s) != cudaSuccess) return ED_ERR_ALLOC;
        KR_CK(cudaMemcpyAsync(d0, psi0, vbytes, cudaMemcpyHostToDevice, s));
    } else {
        d0 = const_cast<double*>(psi0);
    }
    const bool acc = cfg->accumulate != 0;
    if (out_mem == ED_MEM_HOST) {
        if (n_times > 0 && cudaMallocAsync(&dout, vbytes * n_times, s) != cudaSuccess) { release(); return ED_ERR_ALLOC; }
        if (n_times > 0 && acc) KR_CK(cudaMemcpyAsync(dout, psi_out, vbytes * n_times, cudaMemcpyHostToDevice, s));
    } else {
        dout = psi_out;
    }
    // |re psi0|^2, |im psi0|^2 (block partials summed in order on the host)
    const int g = kr_grid(D);
    if (cudaMallocAsync(&part, sizeof(double) * 2 * g, s) != cudaSuccess) { release(); return ED_ERR_ALLOC; }
    k_part_norms<<<g, kKrThreads, 0, s>>>(d0, D, part);
    KR_CK(cudaGetLastError());
    ++launches;
    std::vector<double> hp(2 * g);
    KR_CK(cudaMemcpyAsync(hp.data(), part, sizeof(double) * 2 * g, cudaMemcpyDeviceToHost, s));
    KR_CK(cudaStreamSynchronize(s));
    double n2[2] = {0.0, 0.0};
    for (int b = 0; b < g; ++b) {
        n2[0] += hp[2 * b];
        n2[1] += hp[2 * b + 1];
    }
    if (!std::isfinite(n2[0]) || !std::isfinite(n2[1])) { release(); return ED_ERR_NONFINITE; }

    // one recurrence for a complex operator; one per nonzero part for a real one
    struct Run { const double* start; int part; };
    std::vector<Run> runs;
    if (op->cplx) {
        if (n2[0] + n2[1] > 0.0) runs.push_back({d0, -1});
    } else {
        if (D > 0 && cudaMallocAsync(&tmp, sizeof(double) * (size_t)D, s) != cudaSuccess) { release(); return ED_ERR_ALLOC; }
        for (int p = 0; p < 2; ++p)
            if (n2[p] > 0.0) runs.push_back({tmp, p});
    }
    if ((runs.empty() || op->striped) && n_times > 0 && !acc) KR_CK(cudaMemsetAsync(dout, 0, vbytes * n_times, s));

    ed_lanczos_cfg lc{};
    lc.max_steps = cfg->max_steps;
    lc.mode = ED_LANCZOS_FIXED;
    lc.reorth = cfg->reorth;
    // the two-pass matvec's sectors keep three vectors and regenerate the basis
    lc.ritz = op->striped ? ED_RITZ_NONE : ED_RITZ_STORED;
    lc.start = ED_START_USER;
    std::vector<double> alpha(cfg->max_steps + 2), beta(cfg->max_steps + 2);
    int max_n = 0;
    double err = 0.0;
    bool written = acc;
    if (n_times > 0 && cudaMallocAsync(&dcoef, sizeof(double2) * (size_t)n_times * (cfg->max_steps + 1), s) != cudaSuccess) {
        release();
        return ED_ERR_ALLOC;
    }
    for (const Run& r : runs) {
        if (r.part >= 0) {
            k_part<<<kr_grid(D), kKrThreads, 0, s>>>(d0, D, r.part, tmp);
            KR_CK(cudaGetLastError());
            ++launches;
        }
        ed_lanczos_result lr{};
        st = lanczos_run(op, lanczos_ws_slot(op), &lc, r.start, ED_MEM_DEVICE, nullptr, ED_MEM_DEVICE, alpha.data(),
                         beta.data(), &lr, s, cfg->tol);
        if (st != ED_OK) { release(); return st; }
        launches += lr.launches;
        const int n = lr.steps;
        max_n = std::max(max_n, n);
        if (n_times == 0) continue;
        std::vector<double> c((size_t)2 * n * n_times);
        if (!tridiag_expm_e0(n, alpha.data(), beta.data() + 1, n_times, times, c.data())) {
            release();
            return ED_ERR_BREAKDOWN;
        }
        const int64_t* basis;
        int64_t stride;
        const int* e_dev;
        lanczos_basis(*lanczos_ws_slot(op), &basis, &stride, &e_dev);
        std::vector<int> e(n);
        KR_CK(cudaMemcpyAsync(e.data(), e_dev, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
        KR_CK(cudaStreamSynchronize(s));
        // psi(t) = beta_0 sum_k c_k(t) v_k,  v_k = q_k 2^e_k / beta_k
        std::vector<double2> coef((size_t)n * n_times);
        for (int t = 0; t < n_times; ++t) {
            for (int k = 0; k < n; ++k) {
                const double f = beta[0] * std::ldexp(1.0, e[k]) / beta[k];
                coef[(size_t)t * n + k] = make_double2(f * c[(size_t)2 * n * t + 2 * k], f * c[(size_t)2 * n * t + 2 * k + 1]);
            }
            const double* cl = c.data() + (size_t)2 * n * t + 2 * (n - 1);
            err = std::max(err, beta[n] * std::hypot(cl[0], cl[1]) * beta[0]);
        }
        if (op->striped) {
            // coefficients time-major per vector: coefk[k][t]
            std::vector<double2> coefk((size_t)n * n_times);
            for (int t = 0; t < n_times; ++t)
                for (int k = 0; k < n; ++k) coefk[(size_t)k * n_times + t] = coef[(size_t)t * n + k];
            KR_CK(cudaMemcpyAsync(dcoef, coefk.data(), sizeof(double2) * coefk.size(), cudaMemcpyHostToDevice, s));
            const int cg = kr_grid(D);
            const int ti = r.part == 1 ? 1 : 0;
            double2* o = reinterpret_cast<double2*>(dout);
            st = lanczos_replay(op, *lanczos_ws_slot(op), n, [&](int k, const int64_t* qk) -> cudaError_t {
                k_krylov_acc_perm<<<cg, kKrThreads, 0, s>>>(qk, op->dimUP, op->dimDN, op->d_permDN,
                                                             dcoef + (size_t)k * n_times, n_times, o, D, ti);
                ++launches;
                return cudaGetLastError();
            }, s);
            if (st != ED_OK) { release(); return st; }
            KR_CK(cudaStreamSynchronize(s));
            written = true;
            continue;
        }
        KR_CK(cudaMemcpyAsync(dcoef, coef.data(), sizeof(double2) * coef.size(), cudaMemcpyHostToDevice, s));
        const int cg = kr_grid(D);
        for (int t0 = 0; t0 < n_times; t0 += kKrTimes) {
            const int nt = std::min(kKrTimes, n_times - t0);
            double2* o = reinterpret_cast<double2*>(dout) + (size_t)t0 * D;
            const double2* cf = dcoef + (size_t)t0 * n;
            if (op->cplx)
                k_krylov_combine<true><<<cg, kKrThreads, 0, s>>>(basis, stride, D, n, cf, nt, o, D, written ? 1 : 0,
                                                                 r.part == 1 ? 1 : 0);
            else
                k_krylov_combine<false><<<cg, kKrThreads, 0, s>>>(basis, stride, D, n, cf, nt, o, D, written ? 1 : 0,
                                                                  r.part == 1 ? 1 : 0);
            KR_CK(cudaGetLastError());
            ++launches;
        }
        // the next run overwrites the basis and the coefficients
        KR_CK(cudaStreamSynchronize(s));
        written = true;
    }
    if (out_mem == ED_MEM_HOST && n_times > 0)
        KR_CK(cudaMemcpyAsync(psi_out, dout, vbytes * n_times, cudaMemcpyDeviceToHost, s));
    KR_CK(cudaStreamSynchronize(s));
#undef KR_CK
    release();
    if (res) {
        res->steps = max_n;
        res->runs = (int)runs.size();
        res->norm = std::sqrt(n2[0] + n2[1]);
        res->err_est = err;
        res->launches = launches;
    }
    return ED_OK;
}

}  // extern "C"
