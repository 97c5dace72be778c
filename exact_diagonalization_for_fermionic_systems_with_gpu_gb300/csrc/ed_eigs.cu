// ed_eigs.cu — the nev lowest eigenpairs of a real operator: thick-restart
// Lanczos with full reorthogonalisation, all vectors in device memory.
//
// The reference gets them from Spectra::SymEigsSolver on the host
// (TotalSpin/src/TotalSpinExcited_Lieb_randomHop.cu:133-143: nev pairs,
// ncv = 4 (nev + 1), SmallestAlge, maxit 1000, tol 1e-10), an implicitly
// restarted Lanczos method (its GPU copy: TotalSpin/include/SymEigsSolver.cuh
// :89-121 restart, :125-140 convergence test, :143-168 restart size) whose
// operator moves every vector between host and device
// (HubMatrix_TotalSpin.cuh:282-311).
//
// Here: implicit restarting with the ncv - k unwanted Ritz values as exact
// shifts keeps span{the k wanted Ritz vectors, the residual}, so the restart
// is done as a thick restart (Wu & Simon, SIAM J. Matrix Anal. Appl. 22
// (2000) 602): the k Ritz vectors V Z[:, i] and the normalised residual become
// the new first k + 1 basis vectors and the recurrence continues from there.
// Every new vector is orthogonalised twice against the whole basis (classical
// Gram-Schmidt, "twice is enough"), so the projected matrix T = V^T H V is
// read off the Gram-Schmidt coefficients; its eigenpairs come from a cyclic
// Jacobi solve on the host (T is ncv x ncv).  Convergence and the restart
// size follow Spectra's rules (the ARPACK dsaup2 adjustment).  One cycle of
// ncv - k steps is launched without a host synchronisation: the
// coefficients are reduced on the device in a fixed order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <limits>
#include <vector>

#include "../../include/ed_hubbard.h"
#include "ed_internal.hpp"

namespace ed {
cudaError_t launch_random(double* f, int64_t n, uint64_t seed, cudaStream_t s);

namespace {

constexpr int kEgThreads = 256;
constexpr int kEgChunks = 152 * 2;  // row chunks of a dot product (fixed: determinism)
constexpr int kEgOut = 8;           // vectors formed per pass of the combination kernel

__device__ __forceinline__ double block_sum(double v, double* sh) {
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int w = kEgThreads / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}

// part[k * gridDim.x + chunk] = sum over the chunk's rows of V_k[i] * w[i]
__global__ void __launch_bounds__(kEgThreads) k_mdot(const double* __restrict__ V, int64_t stride,
                                                     const double* __restrict__ w, int64_t n, double* __restrict__ part) {
    __shared__ double sh[kEgThreads];
    const int k = blockIdx.y;
    const double* v = V + (size_t)k * stride;
    double s = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * kEgThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kEgThreads)
        s = fma(v[i], w[i], s);
    s = block_sum(s, sh);
    if (threadIdx.x == 0) part[(size_t)k * gridDim.x + blockIdx.x] = s;
}

// coef[k] = sum_c part[k][c] (fixed order); tcol[k] = (acc ? tcol[k] : 0) + coef[k]
__global__ void __launch_bounds__(kEgThreads) k_reduce(const double* __restrict__ part, int chunks,
                                                       double* __restrict__ coef, double* __restrict__ tcol, int acc) {
    __shared__ double sh[kEgThreads];
    const int k = blockIdx.x;
    double s = 0.0;
    for (int c = threadIdx.x; c < chunks; c += kEgThreads) s += part[(size_t)k * chunks + c];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) {
        coef[k] = s;
        if (tcol) tcol[k] = (acc ? tcol[k] : 0.0) + s;
    }
}

// w[i] -= sum_k coef[k] V_k[i]
__global__ void __launch_bounds__(kEgThreads) k_maxpy(double* __restrict__ w, const double* __restrict__ V,
                                                      int64_t stride, int nk, const double* __restrict__ coef,
                                                      int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * kEgThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kEgThreads) {
        double s = w[i];
        for (int k = 0; k < nk; ++k) s = fma(-__ldg(coef + k), __ldg(V + (size_t)k * stride + i), s);
        w[i] = s;
    }
}

// v = w / beta, beta = sqrt(*ss) (v = 0 when beta = 0); beta_out = beta
__global__ void __launch_bounds__(kEgThreads) k_scale(double* __restrict__ v, const double* __restrict__ w,
                                                      const double* __restrict__ ss, int64_t n,
                                                      double* __restrict__ beta_out) {
    const double b = sqrt(*ss);
    const double r = b > 0.0 ? 1.0 / b : 0.0;
    if (blockIdx.x == 0 && threadIdx.x == 0) *beta_out = b;
    for (int64_t i = (int64_t)blockIdx.x * kEgThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kEgThreads)
        v[i] = w[i] * r;
}

// out_t[i] = sum_k coef[t * nk + k] V_k[i] for t < nt
__global__ void __launch_bounds__(kEgThreads) k_combine(const double* __restrict__ V, int64_t stride, int64_t n, int nk,
                                                        const double* __restrict__ coef, int nt,
                                                        double* __restrict__ out, int64_t out_stride) {
    for (int64_t i = (int64_t)blockIdx.x * kEgThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kEgThreads) {
        double acc[kEgOut];
#pragma unroll
        for (int t = 0; t < kEgOut; ++t) acc[t] = 0.0;
        for (int k = 0; k < nk; ++k) {
            const double v = __ldg(V + (size_t)k * stride + i);
#pragma unroll
            for (int t = 0; t < kEgOut; ++t)
                if (t < nt) acc[t] = fma(__ldg(coef + (size_t)t * nk + k), v, acc[t]);
        }
#pragma unroll
        for (int t = 0; t < kEgOut; ++t)
            if (t < nt) out[(size_t)t * out_stride + i] = acc[t];
    }
}

int eg_grid(int64_t n) {
    const int64_t g = (n + kEgThreads - 1) / kEgThreads;
    return (int)std::max<int64_t>(1, std::min<int64_t>(g, 152 * 8));
}

}  // namespace

// Eigenpairs of a dense symmetric n x n matrix (column-major, destroyed):
// cyclic-by-row Jacobi with the symmetric Schur rotation (Golub & Van Loan,
// Matrix Computations, 4th ed., Algorithms 8.5.1 and 8.5.3), sweeps until the
// off-diagonal norm is below eps * |A|_F.  w ascending; Z column j the unit
// eigenvector of w[j].  False when 100 sweeps did not converge.
bool sym_eigen_jacobi(int n, double* A, double* w, double* Z) {
    std::vector<double> V((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) V[(size_t)i * n + i] = 1.0;
    auto a = [&](int i, int j) -> double& { return A[(size_t)j * n + i]; };
    double fro = 0.0;
    for (size_t i = 0; i < (size_t)n * n; ++i) fro += A[i] * A[i];
    fro = std::sqrt(fro);
    const double eps = std::numeric_limits<double>::epsilon();
    bool ok = false;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0;
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < j; ++i) off += 2.0 * a(i, j) * a(i, j);
        if (std::sqrt(off) <= eps * fro) {
            ok = true;
            break;
        }
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = a(p, q);
                if (apq == 0.0) continue;
                // symmetric Schur: c, s with [c s; -s c]^T A_pq [c s; -s c] diagonal
                const double tau = (a(q, q) - a(p, p)) / (2.0 * apq);
                const double t = (tau >= 0.0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
                const double c = 1.0 / std::sqrt(1.0 + t * t), s = t * c;
                for (int k = 0; k < n; ++k) {  // A <- A J (columns p, q)
                    const double akp = a(k, p), akq = a(k, q);
                    a(k, p) = c * akp - s * akq;
                    a(k, q) = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {  // A <- J^T A (rows p, q)
                    const double apk = a(p, k), aqk = a(q, k);
                    a(p, k) = c * apk - s * aqk;
                    a(q, k) = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {  // V <- V J
                    double* vp = &V[(size_t)p * n + k];
                    double* vq = &V[(size_t)q * n + k];
                    const double x = *vp, y = *vq;
                    *vp = c * x - s * y;
                    *vq = s * x + c * y;
                }
            }
    }
    std::vector<int> ord(n);
    for (int i = 0; i < n; ++i) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return a(x, x) < a(y, y); });
    for (int j = 0; j < n; ++j) {
        w[j] = a(ord[j], ord[j]);
        for (int k = 0; k < n; ++k) Z[(size_t)j * n + k] = V[(size_t)ord[j] * n + k];
    }
    return ok;
}

}  // namespace ed

extern "C" {

ed_status ed_dense_sym_eigen(int n, const double* a, double* w, double* z) {
    if (n < 1 || !a || !w) return ED_ERR_ARG;
    std::vector<double> A(a, a + (size_t)n * n), Z((size_t)n * n);
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < j; ++i) A[(size_t)j * n + i] = A[(size_t)i * n + j] = 0.5 * (A[(size_t)j * n + i] + A[(size_t)i * n + j]);
    if (!ed::sym_eigen_jacobi(n, A.data(), w, Z.data())) return ED_ERR_NOT_CONVERGED;
    if (z) std::copy(Z.begin(), Z.end(), z);
    return ED_OK;
}

ed_status ed_eigs_lowest(ed_op* op, const ed_eigs_cfg* cfg, const double* start, int start_mem, double* evals,
                         double* evecs, int evec_mem, double* resid, ed_eigs_result* res, void* stream) {
    using namespace ed;
    if (!op || !cfg || !evals) return ED_ERR_ARG;
    if (op->cplx) return ED_ERR_NOT_BUILT;
    const int64_t n = op->D;
    const int nev = cfg->nev;
    int ncv = cfg->ncv;
    if (nev < 1 || (int64_t)nev >= n || ncv <= nev || cfg->max_restarts < 1 || !(cfg->tol > 0.0)) return ED_ERR_ARG;
    if ((int64_t)ncv > n) ncv = (int)n;
    if (cfg->start == ED_START_USER && !start) return ED_ERR_ARG;
    if (evecs && evec_mem != ED_MEM_HOST && evec_mem != ED_MEM_DEVICE) return ED_ERR_ARG;
    if (cudaSetDevice(op->device) != cudaSuccess) return ED_ERR_CUDA;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const int64_t stride = (n + 31) / 32 * 32;
    const int m = ncv;

    double *V = nullptr, *Vn = nullptr, *w = nullptr, *part = nullptr, *coef = nullptr, *Tdev = nullptr,
           *beta = nullptr, *zc = nullptr;
    auto release = [&]() {
        cudaFree(V); cudaFree(Vn); cudaFree(w); cudaFree(part); cudaFree(coef); cudaFree(Tdev); cudaFree(beta);
        cudaFree(zc);
    };
    if (cudaMalloc(&V, sizeof(double) * (size_t)(m + 1) * stride) != cudaSuccess ||
        cudaMalloc(&Vn, sizeof(double) * (size_t)(m + 1) * stride) != cudaSuccess ||
        cudaMalloc(&w, sizeof(double) * (size_t)stride) != cudaSuccess ||
        cudaMalloc(&part, sizeof(double) * (size_t)(m + 1) * kEgChunks) != cudaSuccess ||
        cudaMalloc(&coef, sizeof(double) * (m + 1)) != cudaSuccess ||
        cudaMalloc(&Tdev, sizeof(double) * (size_t)m * m) != cudaSuccess ||
        cudaMalloc(&beta, sizeof(double) * (m + 1)) != cudaSuccess ||
        cudaMalloc(&zc, sizeof(double) * (size_t)m * (m + 1)) != cudaSuccess) {
        release();
        return ED_ERR_ALLOC;
    }
#define EG_CK(x)                      \
    do {                              \
        if ((x) != cudaSuccess) {     \
            release();                \
            return ED_ERR_CUDA;       \
        }                             \
    } while (0)
    int64_t launches = 0, n_mv = 0;
    const int g = eg_grid(n);
    // v_0 = start / |start|
    if (cfg->start == ED_START_USER) {
        EG_CK(cudaMemcpyAsync(w, start, sizeof(double) * n,
                              start_mem == ED_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s));
    } else {
        EG_CK(launch_random(w, n, cfg->seed, s));
        ++launches;
    }
    auto norm_into = [&](double* dst, int bidx) -> cudaError_t {
        k_mdot<<<dim3(kEgChunks, 1), kEgThreads, 0, s>>>(w, stride, w, n, part);
        k_reduce<<<1, kEgThreads, 0, s>>>(part, kEgChunks, coef, nullptr, 0);
        k_scale<<<g, kEgThreads, 0, s>>>(dst, w, coef, n, beta + bidx);
        launches += 3;
        return cudaGetLastError();
    };
    EG_CK(norm_into(V, 0));

    std::vector<double> T((size_t)m * m, 0.0), Tc((size_t)m * m), theta(m), Z((size_t)m * m), hb(m + 1);
    const double eps = std::numeric_limits<double>::epsilon();
    const double eps23 = std::pow(eps, 2.0 / 3.0);
    int k0 = 0, restarts = 0, nconv = 0;
    std::vector<double> rest(m, 0.0);
    int msize = m;  // size of T in the final cycle (smaller after an invariant subspace)
    ed_status st = ED_OK;
    for (;;) {
        // steps k0 .. m-1 of the cycle
        for (int j = k0; j < m; ++j) {
            const ed_status ps = ed_op_perform(op, V + (size_t)j * stride, w, ED_MEM_DEVICE, stream);
            if (ps != ED_OK) { release(); return ps; }
            launches += 3;
            ++n_mv;
            for (int pass = 0; pass < 2; ++pass) {
                k_mdot<<<dim3(kEgChunks, j + 1), kEgThreads, 0, s>>>(V, stride, w, n, part);
                k_reduce<<<j + 1, kEgThreads, 0, s>>>(part, kEgChunks, coef, Tdev + (size_t)j * m, pass);
                k_maxpy<<<g, kEgThreads, 0, s>>>(w, V, stride, j + 1, coef, n);
                launches += 3;
            }
            EG_CK(norm_into(V + (size_t)(j + 1) * stride, j + 1));
        }
        EG_CK(cudaMemcpyAsync(Tc.data(), Tdev, sizeof(double) * (size_t)m * m, cudaMemcpyDeviceToHost, s));
        EG_CK(cudaMemcpyAsync(hb.data(), beta, sizeof(double) * (m + 1), cudaMemcpyDeviceToHost, s));
        EG_CK(cudaStreamSynchronize(s));
        int err_flag = 0;
        EG_CK(cudaMemcpy(&err_flag, op->d_err, sizeof(int), cudaMemcpyDeviceToHost));
        if (err_flag) {
            cudaMemset(op->d_err, 0, sizeof(int));
            release();
            return ED_ERR_TIMEOUT;
        }
        // T: the kept block diag(theta), the new columns from the coefficients
        for (int j = k0; j < m; ++j)
            for (int i = 0; i <= j; ++i) T[(size_t)j * m + i] = T[(size_t)i * m + j] = Tc[(size_t)j * m + i];
        double tnorm = 0.0;
        for (double v : T) tnorm = std::max(tnorm, std::fabs(v));
        for (double v : T)
            if (!std::isfinite(v)) { release(); return ED_ERR_NONFINITE; }
        // an invariant subspace: the first vanishing beta ends the basis
        msize = m;
        for (int j = k0 + 1; j <= m; ++j)
            if (hb[j] <= 64.0 * eps * std::max(tnorm, 1e-300)) { msize = j; break; }
        std::vector<double> Tm((size_t)msize * msize);
        for (int j = 0; j < msize; ++j)
            for (int i = 0; i < msize; ++i) Tm[(size_t)j * msize + i] = T[(size_t)j * m + i];
        std::vector<double> th(msize), Zm((size_t)msize * msize);
        if (!sym_eigen_jacobi(msize, Tm.data(), th.data(), Zm.data())) { release(); return ED_ERR_NOT_CONVERGED; }
        const double fnorm = msize < m ? 0.0 : hb[m];
        // Spectra's test: |last component| * |f| < tol * max(eps^(2/3), |theta|)
        nconv = 0;
        for (int i = 0; i < std::min(nev, msize); ++i) {
            rest[i] = std::fabs(Zm[(size_t)i * msize + msize - 1]) * fnorm;
            if (rest[i] < cfg->tol * std::max(eps23, std::fabs(th[i]))) ++nconv;
        }
        if (msize < nev) { release(); return ED_ERR_BREAKDOWN; }
        if (nconv >= nev || restarts >= cfg->max_restarts || msize < m) {
            theta.assign(th.begin(), th.end());
            Z.assign(Zm.begin(), Zm.end());
            break;
        }
        // restart size (SymEigsSolver.cuh:143-168, ARPACK dsaup2)
        int k = nev;
        for (int i = nev; i < m; ++i)
            if (std::fabs(Zm[(size_t)i * m + m - 1]) < eps) ++k;
        k += std::min(nconv, (m - k) / 2);
        if (k == 1 && m >= 6) k = m / 2;
        else if (k == 1 && m > 2) k = 2;
        k = std::min(k, m - 1);
        // thick restart: Vn[0..k-1] = V Z[:, 0..k-1], Vn[k] = V[m]
        std::vector<double> zc_h((size_t)k * m);
        for (int t = 0; t < k; ++t)
            for (int q = 0; q < m; ++q) zc_h[(size_t)t * m + q] = Zm[(size_t)t * m + q];
        EG_CK(cudaMemcpyAsync(zc, zc_h.data(), sizeof(double) * zc_h.size(), cudaMemcpyHostToDevice, s));
        for (int t0 = 0; t0 < k; t0 += kEgOut) {
            const int nt = std::min(kEgOut, k - t0);
            k_combine<<<g, kEgThreads, 0, s>>>(V, stride, n, m, zc + (size_t)t0 * m, nt, Vn + (size_t)t0 * stride, stride);
            ++launches;
        }
        EG_CK(cudaGetLastError());
        EG_CK(cudaMemcpyAsync(Vn + (size_t)k * stride, V + (size_t)m * stride, sizeof(double) * n,
                              cudaMemcpyDeviceToDevice, s));
        EG_CK(cudaStreamSynchronize(s));  // zc_h is released at the end of this scope
        std::swap(V, Vn);
        std::fill(T.begin(), T.end(), 0.0);
        for (int i = 0; i < k; ++i) T[(size_t)i * m + i] = th[i];
        k0 = k;
        ++restarts;
    }
    if (nconv < nev) st = ED_ERR_NOT_CONVERGED;  // the pairs are still returned
    for (int i = 0; i < nev; ++i) evals[i] = theta[i];
    if (resid)
        for (int i = 0; i < nev; ++i) resid[i] = rest[i];
    if (evecs) {
        std::vector<double> zc_h((size_t)nev * msize);
        for (int t = 0; t < nev; ++t)
            for (int q = 0; q < msize; ++q) zc_h[(size_t)t * msize + q] = Z[(size_t)t * msize + q];
        EG_CK(cudaMemcpyAsync(zc, zc_h.data(), sizeof(double) * zc_h.size(), cudaMemcpyHostToDevice, s));
        double* out = evec_mem == ED_MEM_DEVICE ? evecs : Vn;  // Vn is free here
        for (int t0 = 0; t0 < nev; t0 += kEgOut) {
            const int nt = std::min(kEgOut, nev - t0);
            k_combine<<<g, kEgThreads, 0, s>>>(V, stride, n, msize, zc + (size_t)t0 * msize, nt,
                                               out + (size_t)t0 * (evec_mem == ED_MEM_DEVICE ? n : stride),
                                               evec_mem == ED_MEM_DEVICE ? n : stride);
            ++launches;
        }
        EG_CK(cudaGetLastError());
        if (evec_mem == ED_MEM_HOST)
            for (int t = 0; t < nev; ++t)
                EG_CK(cudaMemcpyAsync(evecs + (size_t)t * n, Vn + (size_t)t * stride, sizeof(double) * n,
                                      cudaMemcpyDeviceToHost, s));
        EG_CK(cudaStreamSynchronize(s));
    }
#undef EG_CK
    release();
    if (res) {
        res->nconv = std::min(nconv, nev);
        res->restarts = restarts;
        res->n_matvec = n_mv;
        res->launches = launches;
        double mr = 0.0;
        for (int i = 0; i < nev; ++i) mr = std::max(mr, rest[i]);
        res->max_resid = mr;
    }
    return st;
}

}  // extern "C"
