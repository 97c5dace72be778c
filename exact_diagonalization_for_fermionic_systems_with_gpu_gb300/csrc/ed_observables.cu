// ed_observables.cu — what the drivers compute from a ground state:
// dot products, expectation values, site densities and double occupancies
// (Hellmann-Feynman derivatives), the continued-fraction correlator and the
// Kubo Drude weight (HubMatrix_GPU.cuh:820-849,
// drude_v2_cal_Kagome_randomHop.cu:183-220), the second-order flux response
// by a Lanczos solve of the linear-response equation, and the half-system
// entanglement entropy (entangle_entropy.h:22-44,177-197; block singular
// values in ed_ee_bidiag.cu, cusolverDnDgesvd for blocks beyond it).
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/ed_hubbard.h"
#include "ed_device.cuh"
#include "ed_internal.hpp"

namespace ed {
using namespace dev;

constexpr int kObThreads = 256;
constexpr int kObBlocks = 152 * 2;

// ----------------------------------------------------------------- dots --
// Deterministic FP64 dot: fixed grid, per-block sums in fixed order, then
// one block sums the block results in index order.
__global__ void k_dot(const double* __restrict__ x, const double* __restrict__ y, int64_t n, int conj_pairs,
                      double* part) {
    double re = 0.0, im = 0.0;
    if (conj_pairs) {
        for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
            const double xr = x[2 * k], xi = x[2 * k + 1], yr = y[2 * k], yi = y[2 * k + 1];
            re = fma(xr, yr, fma(xi, yi, re));
            im = fma(xr, yi, fma(-xi, yr, im));
        }
    } else {
        for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
            re = fma(x[k], y[k], re);
    }
    __shared__ double sd[32];
    const double br = block_sum_f64(re, sd);
    const double bi = block_sum_f64(im, sd);
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = br;
        part[2 * blockIdx.x + 1] = bi;
    }
}

__global__ void k_dot_final(const double* part, int nb, double* out) {
    if (threadIdx.x == 0) {
        double r = 0.0, i = 0.0;
        for (int b = 0; b < nb; ++b) { r += part[2 * b]; i += part[2 * b + 1]; }
        out[0] = r;
        out[1] = i;
    }
}

// ------------------------------------------------------------------ S^2 --
// y = S_xy x with S_xy = (S+S- + S-S+)/2 on the (N_up, N_dn) product basis
// (TotalSpin/include/HubMatrix_TotalSpin.cuh:20-66):
//   S_xy = 1/2 sum_i [n_i,up (1 - n_i,dn) + n_i,dn (1 - n_i,up)]
//          - sum_{i<j} (c+_j,up c_i,up c+_i,dn c_j,dn + h.c.)
// A spin exchange moves an up particle and a down particle between two
// singly occupied sites of opposite spin; its fermion sign is (-1)^(number of
// up and down particles strictly between the two sites), and the term enters
// as -x for an even count, +x for an odd one.  One thread per element: the
// exchange partners come from bit operations on the two words and their
// ranks from the CNS binomial tables (bt[p * kdim + k] = C(p, k)).
__device__ __forceinline__ int64_t cns_rank_dev(uint64_t w, const int64_t* __restrict__ bt, int kdim) {
    int64_t r = 0;
    int k = 0;
    while (w) {
        const int p = __ffsll((long long)w) - 1;
        r += bt[p * kdim + k + 1];
        ++k;
        w &= w - 1;
    }
    return r;
}

__global__ void k_sxy(const double* __restrict__ x, double* __restrict__ y, int64_t dimUP, int64_t dimDN, int W,
                      const uint64_t* __restrict__ stUP, const uint64_t* __restrict__ stDN,
                      const int64_t* __restrict__ btU, int kdU, const int64_t* __restrict__ btD, int kdD) {
    const int64_t D = dimUP * dimDN;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < D; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t u = k / dimDN, d = k - u * dimDN;
        const uint64_t up = stUP[u], dn = stDN[d];
        const uint64_t single = up ^ dn;
        const double half = 0.5 * (double)__popcll(single);
        double sr = half * x[k * W], si = W == 2 ? half * x[k * W + 1] : 0.0;
        for (uint64_t a = single & up; a; a &= a - 1) {
            const int p = __ffsll((long long)a) - 1;
            for (uint64_t b = single & dn; b; b &= b - 1) {
                const int q = __ffsll((long long)b) - 1;
                const uint64_t ex = (1ULL << p) | (1ULL << q);
                const uint64_t up2 = up ^ ex, dn2 = dn ^ ex;
                const int i = p < q ? p : q, j = p < q ? q : p;
                const uint64_t between = ((1ULL << j) - 1ULL) & ~((2ULL << i) - 1ULL);
                const int nsign = __popcll(up2 & between) + __popcll(dn2 & between);
                const int64_t kk = cns_rank_dev(up2, btU, kdU) * dimDN + cns_rank_dev(dn2, btD, kdD);
                const double vr = x[kk * W];
                sr += (nsign & 1) ? vr : -vr;
                if (W == 2) {
                    const double vi = x[kk * W + 1];
                    si += (nsign & 1) ? vi : -vi;
                }
            }
        }
        y[k * W] = sr;
        if (W == 2) y[k * W + 1] = si;
    }
}

// y = x - c * p (complex pairs when cplx), c = (cr, ci)
__global__ void k_project(const double* __restrict__ x, const double* __restrict__ p, const double* __restrict__ c,
                          int64_t n, int cplx, double* __restrict__ y) {
    const double cr = c[0], ci = c[1];
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        if (cplx) {
            const double pr = p[2 * k], pi = p[2 * k + 1];
            y[2 * k] = x[2 * k] - (cr * pr - ci * pi);
            y[2 * k + 1] = x[2 * k + 1] - (cr * pi + ci * pr);
        } else {
            y[k] = x[k] - cr * p[k];
        }
    }
}

// ------------------------------------------------------ site densities --
// |psi|^2 in 2^-60 fixed point; P_up[u] (row sums, block-exact), P_dn[d]
// (column sums) and per-site double occupancy as exact int64 atomics, so the
// result does not depend on scheduling.
__global__ void k_densities(const double* __restrict__ psi, int64_t dimUP, int64_t dimDN, int cplx,
                            const uint64_t* __restrict__ stUP, const uint64_t* __restrict__ stDN,
                            unsigned long long* __restrict__ pup, unsigned long long* __restrict__ pdn,
                            unsigned long long* __restrict__ docc) {
    __shared__ unsigned long long sdocc[64];
    __shared__ unsigned long long srow[32];
    for (int i = threadIdx.x; i < 64; i += blockDim.x) sdocc[i] = 0;
    __syncthreads();
    for (int64_t u = blockIdx.x; u < dimUP; u += gridDim.x) {
        const uint64_t su = stUP[u];
        unsigned long long rsum = 0;
        for (int64_t d = threadIdx.x; d < dimDN; d += blockDim.x) {
            const int64_t k = u * dimDN + d;
            double w;
            if (cplx) w = fma(psi[2 * k], psi[2 * k], psi[2 * k + 1] * psi[2 * k + 1]);
            else w = psi[k] * psi[k];
            const unsigned long long q = (unsigned long long)f64_to_fx(w, -60);
            rsum += q;
            atomicAdd(pdn + d, q);
            uint64_t both = su & stDN[d];
            while (both) {
                const int i = __ffsll((long long)both) - 1;
                atomicAdd(sdocc + i, q);
                both &= both - 1;
            }
        }
        // exact block sum of the row
        for (int off = 16; off > 0; off >>= 1) rsum += __shfl_down_sync(0xffffffffu, rsum, off);
        if ((threadIdx.x & 31) == 0) srow[threadIdx.x >> 5] = rsum;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long t = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += srow[w];
            pup[u] = t;
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < 64; i += blockDim.x)
        if (sdocc[i]) atomicAdd(docc + i, sdocc[i]);
}

// ------------------------------------------------- continued fraction --
// g(w) = norm2 / (w + E - a0 - b1^2 / (w + E - a1 - ...)), evaluated from
// the bottom like HubMatrix_GPU.cuh:830-834; one thread per frequency.
__global__ void k_cfrac(int n, const double* __restrict__ a, const double* __restrict__ b, double norm2, double energy,
                        int nw, const double* __restrict__ w, double* __restrict__ g) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nw) return;
    const double wr = w[2 * idx], wi = w[2 * idx + 1];
    double zr = wr + energy - a[n - 1], zi = wi;
    double den = zr * zr + zi * zi;
    double gr = zr / den, gi = -zi / den;
    for (int i = n - 2; i >= 0; --i) {
        const double bb = b[i + 1] * b[i + 1];
        const double tr = wr + energy - a[i] - gr * bb, ti = wi - gi * bb;
        den = tr * tr + ti * ti;
        gr = tr / den;
        gi = -ti / den;
    }
    g[2 * idx] = norm2 * gr;
    g[2 * idx + 1] = norm2 * gi;
}

// ------------------------------------------------- entanglement matrix --
// psi[u, d] -> block s = (nA_up(u), nA_dn(d)), stored column-major with the
// larger dimension as rows (gesvd needs m >= n).
struct EeMeta {
    const int32_t* nA_up;   // per up state: particles in A
    const int32_t* ia_up;   // rank of its A part among A parts with that count
    const int32_t* ib_up;   // rank of its B part
    const int32_t* nA_dn;
    const int32_t* ia_dn;
    const int32_t* ib_dn;
    const int64_t* blk_off;  // [(QA_up+1)*(QA_dn+1)] element offset of block
    const int32_t* blk_rowsA;  // rows of the A side (rA)
    const int32_t* blk_colsB;  // cols of the B side (cB)
    const int32_t* dimA_dn;    // A-part count of the down spin for each nA_dn
    const int32_t* dimB_dn;    // B-part count of the down spin for each nA_dn
    int nqd;                   // QA_dn + 1 (stride of the block table)
};

__global__ void k_ee_scatter(const double* __restrict__ psi, int64_t dimUP, int64_t dimDN, EeMeta m,
                             double* __restrict__ blocks) {
    const int64_t n = dimUP * dimDN;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t u = k / dimDN, d = k - u * dimDN;
        const int au = m.nA_up[u], ad = m.nA_dn[d];
        const int s = au * m.nqd + ad;
        const int64_t rA = m.blk_rowsA[s], cB = m.blk_colsB[s];
        const int64_t row = (int64_t)m.ia_up[u] * m.dimA_dn[ad] + m.ia_dn[d];
        const int64_t col = (int64_t)m.ib_up[u] * m.dimB_dn[ad] + m.ib_dn[d];
        int64_t pos;
        if (rA >= cB) pos = col * rA + row;  // column-major rA x cB
        else pos = row * cB + col;           // column-major cB x rA (the transpose)
        blocks[m.blk_off[s] + pos] = psi[k];
    }
}

cudaError_t launch_random(double* f, int64_t n, uint64_t seed, cudaStream_t s);

}  // namespace ed

namespace {

using ed::kObBlocks;
using ed::kObThreads;

// Block SVDs by cusolverDnDgesvd, for the blocks the cluster kernel leaves
// (or every block with ED_EE_METHOD=gesvd).  One call runs a block at one
// SM's FP64 rate, so the blocks run concurrently: a per-device pool of
// workers, each a host thread with its own stream, cuSOLVER handle and
// workspace (created on first use, kept for the life of the process), takes
// the blocks largest-first to the least-loaded worker.
struct EeWorker {
    cudaStream_t st = nullptr;
    cusolverDnHandle_t h = nullptr;
    double* work = nullptr;
    int lwork = 0;
    double* rwork = nullptr;
    int rwork_n = 0;
    int* info = nullptr;
    cudaEvent_t done = nullptr;
};

struct EePool {
    std::mutex mu;
    std::vector<EeWorker> w;
};

// One worker by default: with several concurrent workers the gesvd results
// differed (1e-9 .. 3e-6 in the entropy) in rare runs after earlier calls
// had used the pool, a cause not found; the cluster bidiagonalisation takes
// every block of the sectors run here, so this path is a fallback.
// ED_EE_STREAMS=k (<= 32) sets k workers.
int ee_workers() {
    const char* e = std::getenv("ED_EE_STREAMS");
    const int k = e ? std::atoi(e) : 1;
    return std::max(1, std::min(k, 32));
}

EePool* ee_pool(int device) {
    static std::mutex mu;
    static std::vector<EePool*> pools;
    std::lock_guard<std::mutex> g(mu);
    if ((int)pools.size() <= device) pools.resize(device + 1, nullptr);
    if (!pools[device]) pools[device] = new EePool();
    return pools[device];
}

ed_status ee_block_svd(int device, cudaStream_t s, double* blocks, const std::vector<int64_t>& off,
                       const std::vector<int>& mm, const std::vector<int>& nn, const std::vector<int64_t>& svo,
                       double* sv_all, const std::vector<char>& skip) {
    EePool* pool = ee_pool(device);
    std::lock_guard<std::mutex> g(pool->mu);
    const int K = ee_workers();
    while ((int)pool->w.size() < K) {
        EeWorker w;
        // a blocking stream: it orders itself with the legacy default stream,
        // which cuSOLVER may use inside a call
        if (cudaStreamCreate(&w.st) != cudaSuccess) return ED_ERR_CUDA;
        if (cusolverDnCreate(&w.h) != CUSOLVER_STATUS_SUCCESS) return ED_ERR_CUDA;
        cusolverDnSetStream(w.h, w.st);
        if (cudaMalloc(&w.info, sizeof(int)) != cudaSuccess) return ED_ERR_ALLOC;
        if (cudaEventCreateWithFlags(&w.done, cudaEventDisableTiming) != cudaSuccess) return ED_ERR_CUDA;
        pool->w.push_back(w);
    }
    // largest first, each to the least-loaded worker (cost ~ m n^2)
    std::vector<int> order;
    for (size_t k = 0; k < off.size(); ++k)
        if (nn[k] > 0 && !skip[k]) order.push_back((int)k);
    if (order.empty()) return ED_OK;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return (double)mm[a] * nn[a] * nn[a] > (double)mm[b] * nn[b] * nn[b];
    });
    std::vector<std::vector<int>> part(K);
    std::vector<double> load(K, 0.0);
    for (int k : order) {
        const int q = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        part[q].push_back(k);
        load[q] += (double)mm[k] * nn[k] * nn[k] + 2e5;  // + a per-call overhead
    }
    cudaEvent_t ready;
    if (cudaEventCreateWithFlags(&ready, cudaEventDisableTiming) != cudaSuccess) return ED_ERR_CUDA;
    cudaEventRecord(ready, s);
    std::vector<ed_status> res(K, ED_OK);
    auto run = [&](int q) {
        EeWorker& w = pool->w[q];
        if (cudaSetDevice(device) != cudaSuccess) {
            res[q] = ED_ERR_CUDA;
            return;
        }
        // workspace for the largest of this worker's blocks, sized before any
        // of them is queued (the stream is idle: its last call was waited for)
        int lw_max = 0, n_max = 0;
        for (int k : part[q]) {
            int lw = 0;
            if (cusolverDnDgesvd_bufferSize(w.h, mm[k], nn[k], &lw) != CUSOLVER_STATUS_SUCCESS) { res[q] = ED_ERR_CUDA; return; }
            lw_max = std::max(lw_max, lw);
            n_max = std::max(n_max, nn[k]);
        }
        if (cudaStreamSynchronize(w.st) != cudaSuccess) { res[q] = ED_ERR_CUDA; return; }
        if (lw_max > w.lwork) {
            cudaFree(w.work);
            w.work = nullptr;
            w.lwork = 0;
            if (cudaMalloc(&w.work, sizeof(double) * lw_max) != cudaSuccess) { res[q] = ED_ERR_ALLOC; return; }
            w.lwork = lw_max;
        }
        if (n_max > w.rwork_n) {
            cudaFree(w.rwork);
            w.rwork = nullptr;
            w.rwork_n = 0;
            if (cudaMalloc(&w.rwork, sizeof(double) * n_max) != cudaSuccess) { res[q] = ED_ERR_ALLOC; return; }
            w.rwork_n = n_max;
        }
        if (cudaStreamWaitEvent(w.st, ready, 0) != cudaSuccess) {
            res[q] = ED_ERR_CUDA;
            return;
        }
        for (int k : part[q]) {
            if (cusolverDnDgesvd(w.h, 'N', 'N', mm[k], nn[k], blocks + off[k], mm[k], sv_all + svo[k], nullptr,
                                 mm[k], nullptr, nn[k], w.work, w.lwork, w.rwork, w.info) != CUSOLVER_STATUS_SUCCESS) {
                res[q] = ED_ERR_CUDA;
                return;
            }
        }
        if (cudaEventRecord(w.done, w.st) != cudaSuccess) res[q] = ED_ERR_CUDA;
    };
    std::vector<std::thread> th;
    for (int q = 1; q < K; ++q)
        if (!part[q].empty()) th.emplace_back(run, q);
    if (!part[0].empty()) run(0);
    for (std::thread& t : th) t.join();
    cudaEventDestroy(ready);
    ed_status st = ED_OK;
    for (int q = 0; q < K; ++q) {
        if (res[q] != ED_OK) st = res[q];
        if (!part[q].empty() && res[q] == ED_OK && cudaStreamWaitEvent(s, pool->w[q].done, 0) != cudaSuccess)
            st = ED_ERR_CUDA;
    }
    return st;
}

struct ObScratch {
    double* part = nullptr;
    double* out = nullptr;
};

int ob_grid(int64_t n) {
    int64_t g = (n + kObThreads - 1) / kObThreads;
    if (g > kObBlocks) g = kObBlocks;
    return (int)(g < 1 ? 1 : g);
}

// dot into a host pair (re, im); x, y device
ed_status dev_dot(const double* x, const double* y, int64_t n, bool cplx, double* out2, cudaStream_t s) {
    double *part = nullptr, *res = nullptr;
    const int g = ob_grid(n);
    if (cudaMallocAsync(&part, sizeof(double) * 2 * g, s) != cudaSuccess) return ED_ERR_ALLOC;
    if (cudaMallocAsync(&res, sizeof(double) * 2, s) != cudaSuccess) { cudaFreeAsync(part, s); return ED_ERR_ALLOC; }
    ed::k_dot<<<g, kObThreads, 0, s>>>(x, y, n, cplx ? 1 : 0, part);
    ed::k_dot_final<<<1, 32, 0, s>>>(part, g, res);
    cudaError_t e = cudaMemcpyAsync(out2, res, sizeof(double) * 2, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFreeAsync(part, s);
    cudaFreeAsync(res, s);
    return e == cudaSuccess ? ED_OK : ED_ERR_CUDA;
}

// Copy a vector to the device when it lives on the host; *dev is the
// device pointer to use, *owned the buffer to free.
ed_status to_device(const double* p, int64_t nd, int mem, const double** dev, double** owned, cudaStream_t s) {
    *owned = nullptr;
    if (mem == ED_MEM_DEVICE) { *dev = p; return ED_OK; }
    if (cudaMallocAsync(owned, sizeof(double) * nd, s) != cudaSuccess) return ED_ERR_ALLOC;
    if (cudaMemcpyAsync(*owned, p, sizeof(double) * nd, cudaMemcpyHostToDevice, s) != cudaSuccess) return ED_ERR_CUDA;
    *dev = *owned;
    return ED_OK;
}

int64_t binom_i(int n, int k) { return ed::binom(n, k); }

uint64_t pext64(uint64_t x, uint64_t mask) {
    uint64_t r = 0;
    int k = 0;
    while (mask) {
        const int p = __builtin_ctzll(mask);
        if ((x >> p) & 1ULL) r |= 1ULL << k;
        ++k;
        mask &= mask - 1;
    }
    return r;
}

int64_t cns_rank(uint64_t w) {
    int64_t r = 0;
    int k = 0;
    while (w) {
        const int p = __builtin_ctzll(w);
        r += ed::binom(p, k + 1);
        ++k;
        w &= w - 1;
    }
    return r;
}

}  // namespace

extern "C" {

ed_status ed_vec_dot(int64_t n, const double* x, const double* y, int mem, double* out, void* stream) {
    if (n < 0 || !out || (n && (!x || !y)) || (mem != ED_MEM_HOST && mem != ED_MEM_DEVICE)) return ED_ERR_ARG;
    if (mem == ED_MEM_HOST) {
        double s = 0.0;
        for (int64_t k = 0; k < n; ++k) s = std::fma(x[k], y[k], s);
        *out = s;
        return ED_OK;
    }
    double r[2];
    ed_status st = dev_dot(x, y, n, false, r, reinterpret_cast<cudaStream_t>(stream));
    if (st == ED_OK) *out = r[0];
    return st;
}

ed_status ed_vec_zdot(int64_t n, const double* x, const double* y, int mem, double* out, void* stream) {
    if (n < 0 || !out || (n && (!x || !y)) || (mem != ED_MEM_HOST && mem != ED_MEM_DEVICE)) return ED_ERR_ARG;
    if (mem == ED_MEM_HOST) {
        double re = 0.0, im = 0.0;
        for (int64_t k = 0; k < n; ++k) {
            re = std::fma(x[2 * k], y[2 * k], std::fma(x[2 * k + 1], y[2 * k + 1], re));
            im = std::fma(x[2 * k], y[2 * k + 1], std::fma(-x[2 * k + 1], y[2 * k], im));
        }
        out[0] = re;
        out[1] = im;
        return ED_OK;
    }
    return dev_dot(x, y, n, true, out, reinterpret_cast<cudaStream_t>(stream));
}

namespace {

// y = S_xy x, both on the device
ed_status sxy_device(const ed_op* op, const double* x, double* y, cudaStream_t s) {
    auto table = [](int n, int q, std::vector<int64_t>* bt) {
        const int kdim = q + 2;
        bt->assign((size_t)(n + 1) * kdim, 0);
        for (int p = 0; p <= n; ++p)
            for (int k = 0; k < kdim; ++k) (*bt)[(size_t)p * kdim + k] = ed::binom(p, k);
        return kdim;
    };
    std::vector<int64_t> tu, td;
    const int kdU = table(op->n_sites, op->n_up, &tu), kdD = table(op->n_sites, op->n_dn, &td);
    int64_t* d_bt = nullptr;
    if (cudaMallocAsync(&d_bt, sizeof(int64_t) * (tu.size() + td.size()), s) != cudaSuccess) return ED_ERR_ALLOC;
    cudaMemcpyAsync(d_bt, tu.data(), sizeof(int64_t) * tu.size(), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_bt + tu.size(), td.data(), sizeof(int64_t) * td.size(), cudaMemcpyHostToDevice, s);
    int64_t blocks = (op->D + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    ed::k_sxy<<<(int)std::max<int64_t>(blocks, 1), 256, 0, s>>>(x, y, op->dimUP, op->dimDN, op->cplx ? 2 : 1,
                                                               op->d_stUP, op->d_stDN, d_bt, kdU,
                                                               d_bt + tu.size(), kdD);
    const cudaError_t e = cudaGetLastError();
    cudaFreeAsync(d_bt, s);
    return e == cudaSuccess ? ED_OK : ED_ERR_CUDA;
}

}  // namespace

ed_status ed_s2_apply(ed_op* op, const double* x, double* y, int mem, void* stream) {
    if (!op || !x || !y || (mem != ED_MEM_HOST && mem != ED_MEM_DEVICE)) return ED_ERR_ARG;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const int64_t nd = op->D * (op->cplx ? 2 : 1);
    if (mem == ED_MEM_DEVICE) return sxy_device(op, x, y, s);
    const double* dx;
    double* owned;
    ed_status st = to_device(x, nd, mem, &dx, &owned, s);
    double* dy = nullptr;
    if (st == ED_OK && cudaMallocAsync(&dy, sizeof(double) * nd, s) != cudaSuccess) st = ED_ERR_ALLOC;
    if (st == ED_OK) st = sxy_device(op, dx, dy, s);
    if (st == ED_OK && cudaMemcpyAsync(y, dy, sizeof(double) * nd, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        st = ED_ERR_CUDA;
    if (dy) cudaFreeAsync(dy, s);
    if (owned) cudaFreeAsync(owned, s);
    if (cudaStreamSynchronize(s) != cudaSuccess && st == ED_OK) st = ED_ERR_CUDA;
    return st;
}

ed_status ed_s2_expect(ed_op* op, const double* psi, int mem, double* out, void* stream) {
    if (!op || !psi || !out || (mem != ED_MEM_HOST && mem != ED_MEM_DEVICE)) return ED_ERR_ARG;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const int64_t nd = op->D * (op->cplx ? 2 : 1);
    const double* dpsi;
    double* owned;
    ed_status st = to_device(psi, nd, mem, &dpsi, &owned, s);
    double* spsi = nullptr;
    if (st == ED_OK && cudaMallocAsync(&spsi, sizeof(double) * nd, s) != cudaSuccess) st = ED_ERR_ALLOC;
    if (st == ED_OK) st = sxy_device(op, dpsi, spsi, s);
    double r[2] = {0.0, 0.0};
    if (st == ED_OK) st = dev_dot(dpsi, spsi, op->D, op->cplx, r, s);
    if (spsi) cudaFreeAsync(spsi, s);
    if (owned) cudaFreeAsync(owned, s);
    cudaStreamSynchronize(s);
    if (st == ED_OK) {
        const double sz = 0.5 * (op->n_up - op->n_dn);
        out[0] = r[0];
        out[1] = sz * sz + r[0];
    }
    return st;
}

ed_status ed_op_expect(ed_op* op, const double* psi, int mem, double* out, void* stream) {
    if (!op || !psi || !out) return ED_ERR_ARG;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const int W = op->cplx ? 2 : 1;
    const int64_t nd = op->D * W;
    const double* dpsi;
    double* owned;
    ed_status st = to_device(psi, nd, mem, &dpsi, &owned, s);
    double* hpsi = nullptr;
    if (st == ED_OK && cudaMallocAsync(&hpsi, sizeof(double) * nd, s) != cudaSuccess) st = ED_ERR_ALLOC;
    if (st == ED_OK) st = ed_op_perform(op, dpsi, hpsi, ED_MEM_DEVICE, stream);
    double r[2] = {0.0, 0.0};
    if (st == ED_OK) st = dev_dot(dpsi, hpsi, op->D, op->cplx, r, s);
    if (!op->cplx) r[1] = 0.0;
    if (hpsi) cudaFreeAsync(hpsi, s);
    if (owned) cudaFreeAsync(owned, s);
    cudaStreamSynchronize(s);
    if (st == ED_OK) {
        out[0] = r[0];
        out[1] = r[1];
    }
    return st;
}

ed_status ed_site_densities(ed_op* op, const double* psi, int mem, double* n_up, double* n_dn, double* docc,
                            void* stream) {
    if (!op || !psi) return ED_ERR_ARG;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const int W = op->cplx ? 2 : 1;
    const int64_t nd = op->D * W;
    const double* dpsi;
    double* owned;
    ed_status st = to_device(psi, nd, mem, &dpsi, &owned, s);
    if (st != ED_OK) return st;
    unsigned long long* acc = nullptr;
    const size_t nacc = (size_t)op->dimUP + (size_t)op->dimDN + 64;
    if (cudaMallocAsync(&acc, sizeof(unsigned long long) * nacc, s) != cudaSuccess) {
        if (owned) cudaFreeAsync(owned, s);
        return ED_ERR_ALLOC;
    }
    cudaMemsetAsync(acc, 0, sizeof(unsigned long long) * nacc, s);
    int64_t g = op->dimUP < kObBlocks * 4 ? op->dimUP : kObBlocks * 4;
    ed::k_densities<<<(int)g, kObThreads, 0, s>>>(dpsi, op->dimUP, op->dimDN, op->cplx ? 1 : 0, op->d_stUP,
                                                  op->d_stDN, acc, acc + op->dimUP, acc + op->dimUP + op->dimDN);
    std::vector<unsigned long long> h(nacc);
    cudaError_t e = cudaMemcpyAsync(h.data(), acc, sizeof(unsigned long long) * nacc, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFreeAsync(acc, s);
    if (owned) cudaFreeAsync(owned, s);
    if (e != cudaSuccess) return ED_ERR_CUDA;
    const int N = op->n_sites;
    const double scale = std::ldexp(1.0, -60);
    std::vector<long double> nu(N, 0.0L), ndn(N, 0.0L);
    for (int64_t u = 0; u < op->dimUP; ++u) {
        uint64_t w = op->bup.state[u];
        while (w) {
            const int i = __builtin_ctzll(w);
            nu[i] += (long double)h[u];
            w &= w - 1;
        }
    }
    for (int64_t d = 0; d < op->dimDN; ++d) {
        uint64_t w = op->bdn.state[d];
        while (w) {
            const int i = __builtin_ctzll(w);
            ndn[i] += (long double)h[op->dimUP + d];
            w &= w - 1;
        }
    }
    for (int i = 0; i < N; ++i) {
        if (n_up) n_up[i] = (double)(nu[i] * scale);
        if (n_dn) n_dn[i] = (double)(ndn[i] * scale);
        if (docc) docc[i] = (double)h[op->dimUP + op->dimDN + i] * scale;
    }
    return ED_OK;
}

ed_status ed_continued_fraction(int n, const double* alpha, const double* beta, double norm2, double energy, int nw,
                                const double* omega, double* g) {
    if (n < 1 || nw < 0 || !alpha || !beta || (nw && (!omega || !g))) return ED_ERR_ARG;
    if (nw == 0) return ED_OK;
    double *d = nullptr;
    const size_t tot = (size_t)n + (size_t)n + 1 + 4 * (size_t)nw;
    if (cudaMalloc(&d, sizeof(double) * tot) != cudaSuccess) return ED_ERR_ALLOC;
    double *da = d, *db = d + n, *dw = d + 2 * n + 1, *dg = dw + 2 * nw;
    cudaMemcpy(da, alpha, sizeof(double) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(db, beta, sizeof(double) * (n + 1), cudaMemcpyHostToDevice);
    cudaMemcpy(dw, omega, sizeof(double) * 2 * nw, cudaMemcpyHostToDevice);
    ed::k_cfrac<<<(nw + 127) / 128, 128>>>(n, da, db, norm2, energy, nw, dw, dg);
    cudaError_t e = cudaMemcpy(g, dg, sizeof(double) * 2 * nw, cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e == cudaSuccess ? ED_OK : ED_ERR_CUDA;
}

ed_status ed_drude_kubo(ed_op* H, ed_op* J, ed_op* K, const double* psi, double e0, const ed_kubo_cfg* cfg,
                        ed_kubo_result* res, double* sigma_out, void* stream) {
    if (!H || !J || !K || !psi || !cfg || !res || cfg->lanczos_steps < 1 || cfg->n_omega < 1) return ED_ERR_ARG;
    if (H->cplx || J->cplx || K->cplx || H->D != J->D || H->D != K->D) return ED_ERR_ARG;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const int64_t D = H->D;
    double* phi = nullptr;
    if (cudaMallocAsync(&phi, sizeof(double) * D, s) != cudaSuccess) return ED_ERR_ALLOC;
    // phi = J|psi> (compute_sigma_omega, HubMatrix_GPU.cuh:838-846)
    ed_status st = ed_op_perform(J, psi, phi, ED_MEM_DEVICE, stream);
    // Lanczos::tridiagonal from phi/|phi| (fixed steps, no Ritz vector)
    const int n = cfg->lanczos_steps;
    std::vector<double> a(n), b(n + 1);
    ed_lanczos_result lr;
    if (st == ED_OK) {
        ed_lanczos_cfg lc;
        std::memset(&lc, 0, sizeof(lc));
        lc.max_steps = n;
        lc.mode = ED_LANCZOS_FIXED;
        lc.ritz = ED_RITZ_NONE;
        lc.start = ED_START_USER;
        st = ed_lanczos_run(H, &lc, phi, ED_MEM_DEVICE, nullptr, ED_MEM_DEVICE, a.data(), b.data(), &lr, stream);
    }
    if (st == ED_OK) {
        const int m = lr.steps;
        const double norm2 = b[0] * b[0];  // |phi|^2 (lanctri.norm returns the squared norm)
        std::vector<double> w(2 * cfg->n_omega), g(2 * cfg->n_omega);
        for (int i = 0; i < cfg->n_omega; ++i) {
            w[2 * i] = cfg->omega_step * (double)(i + 1);
            w[2 * i + 1] = cfg->delta;
        }
        std::vector<double> bb(m + 1);
        for (int i = 0; i <= m; ++i) bb[i] = b[i];
        st = ed_continued_fraction(m, a.data(), bb.data(), norm2, e0, cfg->n_omega, w.data(), g.data());
        if (st == ED_OK) {
            double vertex = 0.0;
            for (int i = 0; i < cfg->n_omega; ++i) {
                const double sigma = -1.0 / (M_PI * w[2 * i]) * g[2 * i + 1];
                if (sigma_out) sigma_out[i] = sigma;
                if (w[2 * i] > cfg->omega_cutoff) vertex += sigma * cfg->omega_step;
            }
            double kin[2];
            st = ed_op_expect(K, psi, ED_MEM_DEVICE, kin, stream);
            if (st == ED_OK) {
                res->kinetic = kin[0];
                res->vertex = vertex;
                res->drude = (-kin[0] - 2.0 * vertex) / cfg->volume;
            }
        }
    }
    cudaFreeAsync(phi, s);
    cudaStreamSynchronize(s);
    return st;
}

}  // extern "C"

namespace {

// <x|(H - E0)^-1|x> for a device vector x orthogonal to the ground level:
// -|x|^2 g(0), with g from the continued fraction of a `steps`-step Lanczos
// run of H started at x, at w = 0 without broadening:
// g(0) = 1/(E0 - a0 - b1^2/(E0 - a1 - ...)).
ed_status resolvent_form(ed_op* H, const double* x, double e0, int steps, double* out, cudaStream_t s) {
    std::vector<double> a(steps), bt(steps + 1);
    ed_lanczos_cfg lc;
    std::memset(&lc, 0, sizeof(lc));
    lc.max_steps = steps;
    lc.mode = ED_LANCZOS_FIXED;
    lc.ritz = ED_RITZ_NONE;
    lc.start = ED_START_USER;
    ed_lanczos_result lr;
    const ed_status st = ed_lanczos_run(H, &lc, x, ED_MEM_DEVICE, nullptr, ED_MEM_DEVICE, a.data(), bt.data(), &lr, s);
    if (st != ED_OK) return st;
    const int m = lr.steps;
    long double gz = 1.0L / ((long double)e0 - a[m - 1]);
    for (int i = m - 2; i >= 0; --i) gz = 1.0L / ((long double)e0 - a[i] - gz * (long double)bt[i + 1] * bt[i + 1]);
    *out = -(double)((long double)bt[0] * bt[0] * gz);
    return ED_OK;
}

}  // namespace

extern "C" {

ed_status ed_response(ed_op* H, ed_op* dH, ed_op* d2H, const double* psi, double e0, int steps, double* first,
                      double* second, void* stream) {
    if (!H || !dH || !psi || steps < 1 || (second && !d2H)) return ED_ERR_ARG;
    if (dH->D != H->D || dH->cplx != H->cplx || (d2H && (d2H->D != H->D || d2H->cplx != H->cplx))) return ED_ERR_ARG;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const bool cplx = H->cplx;
    const int64_t nd = H->D * (cplx ? 2 : 1);
    double *phi = nullptr, *b = nullptr, *coef = nullptr;
    if (cudaMallocAsync(&phi, sizeof(double) * nd, s) != cudaSuccess ||
        cudaMallocAsync(&b, sizeof(double) * nd, s) != cudaSuccess ||
        cudaMallocAsync(&coef, sizeof(double) * 2, s) != cudaSuccess)
        return ED_ERR_ALLOC;
    ed_status st = ed_op_perform(dH, psi, phi, ED_MEM_DEVICE, stream);
    double ov[2] = {0.0, 0.0}, nn[2] = {0.0, 0.0};
    if (st == ED_OK) st = dev_dot(psi, phi, H->D, cplx, ov, s);  // <psi|dH psi>
    if (st == ED_OK) st = dev_dot(psi, psi, H->D, cplx, nn, s);
    if (st == ED_OK && first) *first = ov[0] / nn[0];
    if (st == ED_OK && second) {
        // b = Q dH psi = dH psi - psi <psi|dH psi>/<psi|psi>
        double c[2] = {ov[0] / nn[0], cplx ? ov[1] / nn[0] : 0.0};
        cudaMemcpyAsync(coef, c, sizeof(double) * 2, cudaMemcpyHostToDevice, s);
        ed::k_project<<<ob_grid(H->D), kObThreads, 0, s>>>(phi, psi, coef, H->D, cplx ? 1 : 0, b);
        double resp = 0.0;
        st = resolvent_form(H, b, e0, steps, &resp, s);
        if (st == ED_OK) {
            resp /= nn[0];
            double d2[2] = {0.0, 0.0};
            st = ed_op_expect(d2H, psi, ED_MEM_DEVICE, d2, stream);
            if (st == ED_OK) *second = d2[0] / nn[0] - 2.0 * resp;
        }
    }
    cudaFreeAsync(phi, s);
    cudaFreeAsync(b, s);
    cudaFreeAsync(coef, s);
    cudaStreamSynchronize(s);
    return st;
}

ed_status ed_response_batch(ed_op* const* H, ed_op* const* dH, ed_op* const* d2H, int n, const double* psis,
                            const double* e0, int steps, double* first, double* second, void* stream) {
    if (!H || !dH || !psis || !e0 || !first || n < 1 || n > 16 || steps < 1 || (second && !d2H)) return ED_ERR_ARG;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    std::vector<int64_t> off(n + 1, 0);
    for (int i = 0; i < n; ++i) {
        if (!H[i] || !dH[i] || (second && !d2H[i])) return ED_ERR_ARG;
        if (dH[i]->D != H[i]->D || dH[i]->cplx != H[i]->cplx ||
            (second && (d2H[i]->D != H[i]->D || d2H[i]->cplx != H[i]->cplx)))
            return ED_ERR_ARG;
        off[i + 1] = off[i] + H[i]->D * (H[i]->cplx ? 2 : 1);
    }
    double *phi = nullptr, *b = nullptr, *coef = nullptr;
    if (cudaMallocAsync(&phi, sizeof(double) * off[n], s) != cudaSuccess ||
        cudaMallocAsync(&b, sizeof(double) * off[n], s) != cudaSuccess ||
        cudaMallocAsync(&coef, sizeof(double) * 2, s) != cudaSuccess) {
        cudaFreeAsync(phi, s);
        cudaFreeAsync(b, s);
        return ED_ERR_ALLOC;
    }
    std::vector<double> nn(n, 0.0);
    ed_status st = ED_OK;
    // b_i = Q dH_i psi_i, first_i = <psi_i|dH_i|psi_i> / <psi_i|psi_i>
    for (int i = 0; i < n && st == ED_OK; ++i) {
        const bool cplx = H[i]->cplx;
        const double* psi = psis + off[i];
        st = ed_op_perform(dH[i], psi, phi + off[i], ED_MEM_DEVICE, stream);
        double ov[2] = {0.0, 0.0}, n2[2] = {0.0, 0.0};
        if (st == ED_OK) st = dev_dot(psi, phi + off[i], H[i]->D, cplx, ov, s);
        if (st == ED_OK) st = dev_dot(psi, psi, H[i]->D, cplx, n2, s);
        if (st != ED_OK) break;
        nn[i] = n2[0];
        first[i] = ov[0] / n2[0];
        if (second) {
            const double c[2] = {ov[0] / n2[0], cplx ? ov[1] / n2[0] : 0.0};
            if (cudaMemcpyAsync(coef, c, sizeof(double) * 2, cudaMemcpyHostToDevice, s) != cudaSuccess) {
                st = ED_ERR_CUDA;
                break;
            }
            ed::k_project<<<ob_grid(H[i]->D), kObThreads, 0, s>>>(phi + off[i], psi, coef, H[i]->D, cplx ? 1 : 0,
                                                                 b + off[i]);
        }
    }
    if (st == ED_OK && second) {
        // every resolvent form from one batched Lanczos launch started at the b_i
        std::vector<double> a((size_t)n * steps), bt((size_t)n * (steps + 1));
        std::vector<ed_lanczos_result> lr(n);
        ed_lanczos_cfg lc;
        std::memset(&lc, 0, sizeof(lc));
        lc.max_steps = steps;
        lc.mode = ED_LANCZOS_FIXED;
        lc.ritz = ED_RITZ_NONE;
        lc.start = ED_START_USER;
        st = ed::lanczos_batch_run(H, n, &lc, b, ED_MEM_DEVICE, nullptr, ED_MEM_DEVICE, a.data(), bt.data(), lr.data(),
                                   s);
        if (st == ED_ERR_NOT_BUILT) {
            // no persistent plan for these operators: one run each
            st = ED_OK;
            for (int i = 0; i < n && st == ED_OK; ++i) {
                double r = 0.0, d2[2] = {0.0, 0.0};
                st = resolvent_form(H[i], b + off[i], e0[i], steps, &r, s);
                if (st == ED_OK) st = ed_op_expect(d2H[i], psis + off[i], ED_MEM_DEVICE, d2, stream);
                if (st == ED_OK) second[i] = d2[0] / nn[i] - 2.0 * r / nn[i];
            }
        } else {
            for (int i = 0; i < n && st == ED_OK; ++i) {
                const double* ai = a.data() + (size_t)i * steps;
                const double* bi = bt.data() + (size_t)i * (steps + 1);
                const int m = lr[i].steps;
                long double gz = 1.0L / ((long double)e0[i] - ai[m - 1]);
                for (int k = m - 2; k >= 0; --k)
                    gz = 1.0L / ((long double)e0[i] - ai[k] - gz * (long double)bi[k + 1] * bi[k + 1]);
                const double resp = -(double)((long double)bi[0] * bi[0] * gz) / nn[i];
                double d2[2] = {0.0, 0.0};
                st = ed_op_expect(d2H[i], psis + off[i], ED_MEM_DEVICE, d2, stream);
                if (st == ED_OK) second[i] = d2[0] / nn[i] - 2.0 * resp;
            }
        }
    }
    cudaFreeAsync(phi, s);
    cudaFreeAsync(b, s);
    cudaFreeAsync(coef, s);
    cudaStreamSynchronize(s);
    return st;
}

ed_status ed_response_subspace(ed_op* H, ed_op* dH, ed_op* d2H, const double* psis, int g, double e0, int steps,
                               double* d1, double* d2m, void* stream) {
    if (!H || !dH || !d2H || !psis || !d1 || !d2m || g < 1 || g > 4 || steps < 1) return ED_ERR_ARG;
    if (dH->D != H->D || dH->cplx != H->cplx || d2H->D != H->D || d2H->cplx != H->cplx) return ED_ERR_ARG;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const bool cplx = H->cplx;
    const int64_t n = H->D, nd = n * (cplx ? 2 : 1);
    auto col = [&](const double* base, int i) { return base + (size_t)i * (size_t)nd; };
    auto wcol = [&](double* base, int i) { return base + (size_t)i * (size_t)nd; };
    double *sv = nullptr, *phi = nullptr, *bv = nullptr, *x = nullptr, *coef = nullptr;
    if (cudaMallocAsync(&sv, sizeof(double) * nd * g, s) != cudaSuccess ||
        cudaMallocAsync(&phi, sizeof(double) * nd * g, s) != cudaSuccess ||
        cudaMallocAsync(&bv, sizeof(double) * nd * g, s) != cudaSuccess ||
        cudaMallocAsync(&x, sizeof(double) * nd, s) != cudaSuccess ||
        cudaMallocAsync(&coef, sizeof(double) * 2, s) != cudaSuccess) {
        cudaFreeAsync(sv, s);
        cudaFreeAsync(phi, s);
        cudaFreeAsync(bv, s);
        cudaFreeAsync(x, s);
        return ED_ERR_ALLOC;
    }
    std::vector<double> D1(2 * g * g, 0.0), E2(2 * g * g, 0.0), R(2 * g * g, 0.0), Rd(g, 0.0);
    ed_status st = ED_OK;
    // the states, orthonormalised in order (classical Gram-Schmidt, twice)
    if (cudaMemcpyAsync(sv, psis, sizeof(double) * nd * g, cudaMemcpyDeviceToDevice, s) != cudaSuccess) st = ED_ERR_CUDA;
    for (int i = 0; i < g && st == ED_OK; ++i) {
        for (int pass = 0; pass < 2 && st == ED_OK; ++pass)
            for (int k = 0; k < i && st == ED_OK; ++k) {
                double c[2] = {0.0, 0.0};
                st = dev_dot(col(sv, k), col(sv, i), n, cplx, c, s);
                if (st != ED_OK) break;
                if (!cplx) c[1] = 0.0;
                if (cudaMemcpyAsync(coef, c, sizeof(double) * 2, cudaMemcpyHostToDevice, s) != cudaSuccess) {
                    st = ED_ERR_CUDA;
                    break;
                }
                ed::k_project<<<ob_grid(n), kObThreads, 0, s>>>(col(sv, i), col(sv, k), coef, n, cplx ? 1 : 0,
                                                               wcol(sv, i));
            }
        double nn[2] = {0.0, 0.0};
        if (st == ED_OK) st = dev_dot(col(sv, i), col(sv, i), n, cplx, nn, s);
        if (st == ED_OK && !(nn[0] > 0.0)) st = ED_ERR_ARG;  // the states are not independent
        if (st == ED_OK) {
            const double c[2] = {1.0 - 1.0 / std::sqrt(nn[0]), 0.0};  // y = x - c x = x / |x|
            if (cudaMemcpyAsync(coef, c, sizeof(double) * 2, cudaMemcpyHostToDevice, s) != cudaSuccess) st = ED_ERR_CUDA;
            ed::k_project<<<ob_grid(n), kObThreads, 0, s>>>(col(sv, i), col(sv, i), coef, n, cplx ? 1 : 0,
                                                           wcol(sv, i));
        }
    }
    psis = sv;
    // phi_j = dH psi_j, D1_ij = <psi_i|phi_j>
    for (int j = 0; j < g && st == ED_OK; ++j) st = ed_op_perform(dH, col(psis, j), wcol(phi, j), ED_MEM_DEVICE, s);
    for (int i = 0; i < g && st == ED_OK; ++i)
        for (int j = 0; j < g && st == ED_OK; ++j) st = dev_dot(col(psis, i), col(phi, j), n, cplx, &D1[2 * (i * g + j)], s);
    // b_j = phi_j - sum_i psi_i D1_ij (the ground subspace projected out);
    // each coefficient is copied in stream order before the kernel using it
    for (int j = 0; j < g && st == ED_OK; ++j) {
        if (cudaMemcpyAsync(wcol(bv, j), col(phi, j), sizeof(double) * nd, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
            st = ED_ERR_CUDA;
        for (int i = 0; i < g && st == ED_OK; ++i) {
            const double c[2] = {D1[2 * (i * g + j)], cplx ? D1[2 * (i * g + j) + 1] : 0.0};
            if (cudaMemcpyAsync(coef, c, sizeof(double) * 2, cudaMemcpyHostToDevice, s) != cudaSuccess) {
                st = ED_ERR_CUDA;
                break;
            }
            ed::k_project<<<ob_grid(n), kObThreads, 0, s>>>(col(bv, j), col(psis, i), coef, n, cplx ? 1 : 0,
                                                           wcol(bv, j));
        }
    }
    // E2_ij = <psi_i|d2H|psi_j> (phi reused as d2H psi_j)
    for (int j = 0; j < g && st == ED_OK; ++j) st = ed_op_perform(d2H, col(psis, j), wcol(phi, j), ED_MEM_DEVICE, s);
    for (int i = 0; i < g && st == ED_OK; ++i)
        for (int j = 0; j < g && st == ED_OK; ++j) st = dev_dot(col(psis, i), col(phi, j), n, cplx, &E2[2 * (i * g + j)], s);
    // resolvent forms: R(b_i) on the diagonal; off the diagonal by
    // polarisation, Re R_ij = (R(b_i + b_j) - R(b_i) - R(b_j)) / 2 and
    // Im R_ij = -(R(b_i + i b_j) - R(b_i) - R(b_j)) / 2
    for (int i = 0; i < g && st == ED_OK; ++i) st = resolvent_form(H, col(bv, i), e0, steps, &Rd[i], s);
    for (int i = 0; i < g && st == ED_OK; ++i) {
        R[2 * (i * g + i)] = Rd[i];
        for (int j = i + 1; j < g && st == ED_OK; ++j) {
            for (int part = 0; part < (cplx ? 2 : 1) && st == ED_OK; ++part) {
                // x = b_i - c b_j with c = -1 (sum) or -i (b_i + i b_j)
                const double c[2] = {part ? 0.0 : -1.0, part ? -1.0 : 0.0};
                if (cudaMemcpyAsync(coef, c, sizeof(double) * 2, cudaMemcpyHostToDevice, s) != cudaSuccess) {
                    st = ED_ERR_CUDA;
                    break;
                }
                ed::k_project<<<ob_grid(n), kObThreads, 0, s>>>(col(bv, i), col(bv, j), coef, n, cplx ? 1 : 0, x);
                double r = 0.0;
                st = resolvent_form(H, x, e0, steps, &r, s);
                const double v = 0.5 * (r - Rd[i] - Rd[j]);
                if (part == 0) {
                    R[2 * (i * g + j)] = v;
                    R[2 * (j * g + i)] = v;
                } else {
                    R[2 * (i * g + j) + 1] = -v;
                    R[2 * (j * g + i) + 1] = v;
                }
            }
        }
    }
    if (st == ED_OK) {
        for (int k = 0; k < 2 * g * g; ++k) {
            d1[k] = D1[k];
            d2m[k] = E2[k] - 2.0 * R[k];
        }
        if (!cplx)
            for (int k = 0; k < g * g; ++k) d1[2 * k + 1] = d2m[2 * k + 1] = 0.0;
    }
    cudaFreeAsync(sv, s);
    cudaFreeAsync(phi, s);
    cudaFreeAsync(bv, s);
    cudaFreeAsync(x, s);
    cudaFreeAsync(coef, s);
    cudaStreamSynchronize(s);
    return st;
}

// The entropies of n_states states of op's sector (psi: n_states x rows,
// row-major): every state's blocks go through the same bidiagonalisation
// launches and host SVD pool, so a batch fills the GPU where one state's
// blocks leave SMs idle.  Each state's result equals its own one-state call
// bit for bit (the same blocks, cluster sizes and summation order).
static ed_status ee_states(ed_op* op, int n_states, const double* psi, int mem, uint64_t a_mask, double* s_vn,
                           double* s_ref, void* stream) {
    if (!op || !psi || n_states < 1) return ED_ERR_ARG;
    if (op->cplx) return ED_ERR_NOT_BUILT;
    const int N = op->n_sites;
    const uint64_t all = (N >= 64) ? ~0ULL : ((1ULL << N) - 1ULL);
    a_mask &= all;
    const uint64_t b_mask = all ^ a_mask;
    const int nA = __builtin_popcountll(a_mask), nB = N - nA;
    const int Qu = op->n_up, Qd = op->n_dn;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    // labels per spin state (entangle_entropy.h:22-44, with per-sector ranks)
    auto labels = [&](const ed::SpinBasis& bs, std::vector<int32_t>* na, std::vector<int32_t>* ia,
                      std::vector<int32_t>* ib) {
        na->resize(bs.count);
        ia->resize(bs.count);
        ib->resize(bs.count);
        for (int64_t r = 0; r < bs.count; ++r) {
            const uint64_t w = bs.state[r];
            const uint64_t pa = pext64(w, a_mask), pb = pext64(w, b_mask);
            (*na)[r] = __builtin_popcountll(pa);
            (*ia)[r] = (int32_t)cns_rank(pa);
            (*ib)[r] = (int32_t)cns_rank(pb);
        }
    };
    std::vector<int32_t> nau, iau, ibu, nad, iad, ibd;
    labels(op->bup, &nau, &iau, &ibu);
    labels(op->bdn, &nad, &iad, &ibd);
    const int nqu = std::min(Qu, nA) + 1, nqd = std::min(Qd, nA) + 1;
    const int nblk = nqu * nqd;
    std::vector<int64_t> off(nblk, 0);
    std::vector<int32_t> rA(nblk, 0), cB(nblk, 0), dimA_dn(nqd), dimB_dn(nqd);
    int64_t total = 0;
    for (int kd = 0; kd < nqd; ++kd) {
        dimA_dn[kd] = (int32_t)binom_i(nA, kd);
        dimB_dn[kd] = (int32_t)binom_i(nB, Qd - kd);
    }
    for (int ku = 0; ku < nqu; ++ku)
        for (int kd = 0; kd < nqd; ++kd) {
            const int sidx = ku * nqd + kd;
            rA[sidx] = (int32_t)(binom_i(nA, ku) * binom_i(nA, kd));
            cB[sidx] = (int32_t)(binom_i(nB, Qu - ku) * binom_i(nB, Qd - kd));
            off[sidx] = total;
            total += (int64_t)rA[sidx] * cB[sidx];
        }
    // device copies
    const double* dpsi;
    double* owned;
    ed_status st = to_device(psi, op->D * n_states, mem, &dpsi, &owned, s);
    if (st != ED_OK) return st;
    std::vector<int32_t> meta_i;
    auto push = [&](const std::vector<int32_t>& v) { meta_i.insert(meta_i.end(), v.begin(), v.end()); };
    push(nau); push(iau); push(ibu); push(nad); push(iad); push(ibd); push(rA); push(cB); push(dimA_dn); push(dimB_dn);
    int32_t* dmi = nullptr;
    int64_t* doff = nullptr;
    double* blocks = nullptr;
    const int64_t nall = std::max<int64_t>(total * n_states, 1);
    if (cudaMalloc(&dmi, sizeof(int32_t) * meta_i.size()) != cudaSuccess ||
        cudaMalloc(&doff, sizeof(int64_t) * off.size()) != cudaSuccess ||
        cudaMalloc(&blocks, sizeof(double) * nall) != cudaSuccess) {
        cudaFree(dmi); cudaFree(doff);
        if (owned) cudaFreeAsync(owned, s);
        return ED_ERR_ALLOC;
    }
    cudaMemcpyAsync(dmi, meta_i.data(), sizeof(int32_t) * meta_i.size(), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(doff, off.data(), sizeof(int64_t) * off.size(), cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(blocks, 0, sizeof(double) * nall, s);
    ed::EeMeta m;
    size_t p = 0;
    m.nA_up = dmi + p; p += nau.size();
    m.ia_up = dmi + p; p += iau.size();
    m.ib_up = dmi + p; p += ibu.size();
    m.nA_dn = dmi + p; p += nad.size();
    m.ia_dn = dmi + p; p += iad.size();
    m.ib_dn = dmi + p; p += ibd.size();
    m.blk_rowsA = dmi + p; p += rA.size();
    m.blk_colsB = dmi + p; p += cB.size();
    m.dimA_dn = dmi + p; p += dimA_dn.size();
    m.dimB_dn = dmi + p; p += dimB_dn.size();
    m.blk_off = doff;
    m.nqd = nqd;
    for (int b = 0; b < n_states; ++b)
        ed::k_ee_scatter<<<ob_grid(op->D), kObThreads, 0, s>>>(dpsi + (size_t)b * op->D, op->dimUP, op->dimDN, m,
                                                               blocks + (size_t)b * total);
    // every state's blocks in one list: singular values of every block;
    // cusolverDnDgesvd (jobu = jobvt = 'N', as entangle_entropy.h:231-291) on
    // the device's worker streams for the blocks the cluster
    // bidiagonalisation does not take
    const size_t nk = (size_t)nblk * n_states;
    std::vector<int64_t> offs(nk);
    std::vector<int> mmv(nk), nnv(nk);
    std::vector<int64_t> svo(nk + 1, 0);
    for (size_t k = 0; k < nk; ++k) {
        const size_t kb = k % nblk, b = k / nblk;
        offs[k] = off[kb] + (int64_t)b * total;
        mmv[k] = std::max(rA[kb], cB[kb]);
        nnv[k] = std::min(rA[kb], cB[kb]);
        svo[k + 1] = svo[k] + nnv[k];
    }
    // blocks that fit a thread-block cluster: Householder bidiagonalisation
    // on the device + bidiagonal SVD on the host; the rest through cuSOLVER
    std::vector<double> hs(std::max<int64_t>(svo.back(), 1), 0.0);
    std::vector<char> done;
    if (st == ED_OK) st = ed::ee_bidiag_blocks(op->device, s, blocks, offs, mmv, nnv, svo, &hs, &done);
    bool rest = false;
    for (size_t k = 0; k < nk; ++k) rest = rest || (!done.empty() && !done[k] && nnv[k] > 0);
    double* sv_all = nullptr;
    if (st == ED_OK && rest) {
        if (cudaMalloc(&sv_all, sizeof(double) * std::max<int64_t>(svo.back(), 1)) != cudaSuccess) st = ED_ERR_ALLOC;
        if (st == ED_OK) st = ee_block_svd(op->device, s, blocks, offs, mmv, nnv, svo, sv_all, done);
        std::vector<double> hg(std::max<int64_t>(svo.back(), 1));
        if (st == ED_OK &&
            (cudaMemcpyAsync(hg.data(), sv_all, sizeof(double) * svo.back(), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
             cudaStreamSynchronize(s) != cudaSuccess))
            st = ED_ERR_CUDA;
        for (size_t k = 0; st == ED_OK && k < nk; ++k)
            if (!done[k]) std::copy(hg.begin() + svo[k], hg.begin() + svo[k + 1], hs.begin() + svo[k]);
    }
    for (int b = 0; st == ED_OK && b < n_states; ++b) {
        double svn = 0.0, sref = 0.0;
        // block by block, each in descending order: a fixed summation order
        for (int64_t i = svo[(size_t)b * nblk]; i < svo[(size_t)(b + 1) * nblk]; ++i) {
            const double x = hs[i];
            if (x > 0.0) {
                sref += -x * std::log(x);
                const double q = x * x;
                if (q > 0.0) svn += -q * std::log(q);
            }
        }
        if (s_vn) s_vn[b] = svn;
        if (s_ref) s_ref[b] = sref;
    }
    cudaFree(sv_all);
    cudaFree(blocks); cudaFree(dmi); cudaFree(doff);
    if (owned) cudaFreeAsync(owned, s);
    cudaStreamSynchronize(s);
    return st;
}

ed_status ed_entanglement_entropy(ed_op* op, const double* psi, int mem, uint64_t a_mask, double* s_vn, double* s_ref,
                                  void* stream) {
    return ee_states(op, 1, psi, mem, a_mask, s_vn, s_ref, stream);
}

ed_status ed_entanglement_entropy_batch(ed_op* op, int n_states, const double* psis, int mem, uint64_t a_mask,
                                        double* s_vn, double* s_ref, void* stream) {
    return ee_states(op, n_states, psis, mem, a_mask, s_vn, s_ref, stream);
}

}  // extern "C"
