// ed_ee_bidiag.cu — singular values of the entanglement-matrix blocks:
// Householder bidiagonalisation on the device, one thread-block cluster per
// block, then the Golub-Kahan bidiagonal SVD on the host.
//
// cusolverDnDgesvd runs a block of a few hundred rows at one SM's FP64 rate
// (a 400 x 400 block: 8.5e7 FMA, 26 ms on GB300, where FP64 issues at 1/64
// of FP32).  Here the rows of a block are spread over the CTAs of a cluster
// (up to 16 SMs), each CTA holding its slab of rows in shared memory for the
// whole reduction; a step k of the alternating reflections (Golub & Van
// Loan, Matrix Computations, 4th ed., Algorithm 5.4.2) needs two cluster
// barriers: one after every CTA has written its partial column norm and its
// partial w' = A[k+1:, k]^T A[k+1:, k+1:] (summed by every CTA in rank order
// through distributed shared memory, so all CTAs hold identical reflectors),
// one after the owner of row k has formed the right reflector.  The right
// reflector's update is local to each CTA's rows.  Output: the bidiagonal
// (d, e) of every block; its singular values are those of the block up to
// eps |block| (the backward error of the reflections), the accuracy gesvd has.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/ed_hubbard.h"
#include "ed_internal.hpp"
#include "ed_tridiag.hpp"

namespace cg = cooperative_groups;

namespace ed {
namespace {

constexpr int kBdThreads = 512;
constexpr int kBdWarps = kBdThreads / 32;

struct EeJob {
    int64_t off;  // block: column-major m x n (m >= n) at blocks + off
    int32_t m, n;
    int64_t de;   // d at dd + de (n values), e at ee + de (n - 1 values)
};

// dynamic shared memory (doubles) of a CTA holding R rows of an n-column block
size_t bd_smem_doubles(int R, int n) { return (size_t)R * n + 5 * (size_t)n + 2 + R + 2; }

// LAPACK dlarfg convention: H = I - tau v v^T, v_0 = 1, H [alpha; x] = [beta; 0]
__device__ __forceinline__ void bd_reflector(double alpha, double xnorm2, double* beta, double* tau, double* scale) {
    if (xnorm2 == 0.0) {
        *beta = alpha;
        *tau = 0.0;
        *scale = 0.0;
        return;
    }
    const double b = -copysign(sqrt(fma(alpha, alpha, xnorm2)), alpha);
    *beta = b;
    *tau = (b - alpha) / b;
    *scale = 1.0 / (alpha - b);
}

__global__ void __launch_bounds__(kBdThreads, 1) k_ee_bidiag(const EeJob* __restrict__ jobs,
                                                             const double* __restrict__ blocks,
                                                             double* __restrict__ dd, double* __restrict__ ee) {
    cg::cluster_group cl = cg::this_cluster();
    const int CS = (int)cl.num_blocks();
    const int rank = (int)cl.block_rank();
    const EeJob J = jobs[blockIdx.x / CS];
    const int m = J.m, n = J.n;
    const int R = (m + CS - 1) / CS;
    const int r0 = min(m, rank * R), r1 = min(m, r0 + R);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    extern __shared__ double sm[];
    double* slab = sm;                    // own rows, row-major, stride n
    double* part = slab + (size_t)R * n;  // [j] = sum over own rows i > k of A_ik A_ij, j >= k
    double* rowk = part + n + 1;          // row k (columns >= k), written by its owner
    double* wv = rowk + n;                // w_j of the left reflector
    double* ubuf = wv + n;                // right reflector u_j (j > k), tau' at [n]
    double* uu = ubuf + n + 1;            // local copy of u
    double* zz = uu + n;                  // v_i of the left reflector, then z_i of the right one
    double* sc = zz + R;                  // tau, scale of the left reflector
    const double* src = blocks + J.off;
    for (int64_t idx = tid; idx < (int64_t)(r1 - r0) * n; idx += kBdThreads) {
        const int i = (int)(idx % (r1 - r0)), j = (int)(idx / (r1 - r0));
        slab[(size_t)i * n + j] = src[(size_t)j * m + r0 + i];
    }
    __syncthreads();
    for (int k = 0; k < n; ++k) {
        const int owner = k / R;
        const int ilo = max(r0, k + 1);
        // (1) partials over own rows below k; part[k] is the column's sigma'
        for (int j = k + tid; j < n; j += kBdThreads) {
            double w = 0.0;
            for (int i = ilo; i < r1; ++i) w = fma(slab[(size_t)(i - r0) * n + k], slab[(size_t)(i - r0) * n + j], w);
            part[j] = w;
        }
        if (rank == owner)
            for (int j = k + tid; j < n; j += kBdThreads) rowk[j] = slab[(size_t)(k - r0) * n + j];
        cl.sync();  // A: partials and row k visible cluster-wide
        const double* rk = cl.map_shared_rank(rowk, owner);
        // (2) one warp forms the left reflector (a fixed shuffle tree over the
        // ranks, the same in every CTA)
        if (warp == 0) {
            double sg = lane < CS ? cl.map_shared_rank(part, lane)[k] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) sg += __shfl_xor_sync(0xffffffffu, sg, o);
            if (lane == 0) {
                double beta, tau, scale;
                bd_reflector(rk[k], sg, &beta, &tau, &scale);
                sc[0] = tau;
                sc[1] = scale;
                if (rank == owner) dd[J.de + k] = beta;
            }
        }
        __syncthreads();
        const double tau = sc[0], scale = sc[1];
        for (int j = k + 1 + tid; j < n; j += kBdThreads) {
            double w = 0.0;
#pragma unroll 4
            for (int r = 0; r < CS; ++r) w += cl.map_shared_rank(part, r)[j];
            wv[j] = fma(scale, w, rk[j]);
        }
        const int il = max(r0, k);
        for (int i = il + tid; i < r1; i += kBdThreads)
            zz[i - r0] = (i == k) ? 1.0 : slab[(size_t)(i - r0) * n + k] * scale;
        __syncthreads();
        // (3) left update of own rows i >= k: A_ij -= tau v_i w_j
        if (tau != 0.0) {
            for (int j = k + 1 + tid; j < n; j += kBdThreads) {
                const double tw = tau * wv[j];
                for (int i = il; i < r1; ++i)
                    slab[(size_t)(i - r0) * n + j] = fma(-tw, zz[i - r0], slab[(size_t)(i - r0) * n + j]);
            }
        }
        __syncthreads();
        if (k + 1 >= n) break;
        // (4) one warp of the owner of row k forms the right reflector of A[k, k+1:]
        if (rank == owner && warp == 0) {
            const double* ak = slab + (size_t)(k - r0) * n;
            double x2 = 0.0;
            for (int j = k + 2 + lane; j < n; j += 32) x2 = fma(ak[j], ak[j], x2);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x2 += __shfl_xor_sync(0xffffffffu, x2, o);
            double b2, t2, s2;
            bd_reflector(ak[k + 1], x2, &b2, &t2, &s2);
            for (int j = k + 2 + lane; j < n; j += 32) ubuf[j] = ak[j] * s2;
            if (lane == 0) {
                ubuf[k + 1] = 1.0;
                ubuf[n] = t2;
                ee[J.de + k] = b2;
            }
        }
        cl.sync();  // B: the right reflector visible cluster-wide
        // (5) right update of own rows below k: z_i = A[i, k+1:] u, A -= tau' z u^T
        const double* ur = cl.map_shared_rank(ubuf, owner);
        const double tau2 = ur[n];
        for (int j = k + 1 + tid; j < n; j += kBdThreads) uu[j] = ur[j];
        __syncthreads();
        if (tau2 != 0.0) {
            for (int i = ilo + warp; i < r1; i += kBdWarps) {
                const double* ai = slab + (size_t)(i - r0) * n;
                double z = 0.0;
                for (int j = k + 1 + lane; j < n; j += 32) z = fma(ai[j], uu[j], z);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) z += __shfl_xor_sync(0xffffffffu, z, o);
                if (lane == 0) zz[i - r0] = z;
            }
            __syncthreads();
            for (int j = k + 1 + tid; j < n; j += kBdThreads) {
                const double tu = tau2 * uu[j];
                for (int i = ilo; i < r1; ++i)
                    slab[(size_t)(i - r0) * n + j] = fma(-tu, zz[i - r0], slab[(size_t)(i - r0) * n + j]);
            }
        }
        __syncthreads();
    }
    cl.sync();  // no CTA leaves while another may still read its shared memory
}

// Launch one cluster of cs CTAs per job; false when this device cannot run it.
bool launch_bidiag(const std::vector<EeJob>& jobs, int cs, const double* blocks, double* dd, double* ee,
                   cudaStream_t s, EeJob* djobs, size_t smem_bytes) {
    if (jobs.empty()) return true;
    if (cudaFuncSetAttribute(k_ee_bidiag, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes) != cudaSuccess)
        return false;
    if (cs > 8 && cudaFuncSetAttribute(k_ee_bidiag, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
        return false;
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3((unsigned)(jobs.size() * cs), 1, 1);
    lc.blockDim = dim3(kBdThreads, 1, 1);
    lc.dynamicSmemBytes = smem_bytes;
    lc.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cs;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    lc.attrs = at;
    lc.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, k_ee_bidiag, &lc) != cudaSuccess || nclusters < 1) {
        cudaGetLastError();
        return false;
    }
    if (cudaLaunchKernelEx(&lc, k_ee_bidiag, (const EeJob*)djobs, blocks, dd, ee) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return true;
}

}  // namespace

// Streams for the per-cluster-size launches (created once per device).
cudaStream_t bd_stream(int device, int i) {
    static std::mutex mu;
    static std::vector<std::vector<cudaStream_t>> st;
    std::lock_guard<std::mutex> g(mu);
    if ((int)st.size() <= device) st.resize(device + 1);
    while ((int)st[device].size() <= i) {
        cudaStream_t x = nullptr;
        if (cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
        st[device].push_back(x);
    }
    return st[device][i];
}

// Singular values of the blocks that fit the cluster kernel: handled[k] = 1
// and their values (descending) in sv_host[svo[k] ..).  The others are left
// for the cuSOLVER path.  Cluster size per block in proportion to its work
// (m n^2), the largest block on 16 CTAs, so that all clusters run in one
// wave and finish together; one launch per cluster size, on its own stream.
ed_status ee_bidiag_blocks(int device, cudaStream_t s, const double* blocks, const std::vector<int64_t>& off,
                           const std::vector<int>& mm, const std::vector<int>& nn, const std::vector<int64_t>& svo,
                           std::vector<double>* sv_host, std::vector<char>* handled) {
    const char* env = std::getenv("ED_EE_METHOD");
    handled->assign(off.size(), 0);
    if (env && std::string(env) == "gesvd") return ED_OK;
    int max_smem = 0;
    cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    const size_t cap = (size_t)max_smem / sizeof(double);
    double wmax = 0.0;
    for (size_t k = 0; k < off.size(); ++k) wmax = std::max(wmax, (double)mm[k] * nn[k] * nn[k]);
    constexpr int kSizes = 5;  // cluster sizes 1, 2, 4, 8, 16
    std::vector<EeJob> group[kSizes];
    size_t smem[kSizes] = {0, 0, 0, 0, 0};
    std::vector<int> tag(off.size(), -1);
    for (size_t k = 0; k < off.size(); ++k) {
        const int m = mm[k], n = nn[k];
        if (n <= 0) { (*handled)[k] = 1; continue; }
        const double want = 16.0 * (double)m * n * n / wmax;
        int g = 0;
        while (g < kSizes - 1 && (double)(1 << g) < want) ++g;
        while (g < kSizes && bd_smem_doubles((m + (1 << g) - 1) >> g, n) > cap) ++g;
        if (g >= kSizes) continue;  // too large for a cluster: cuSOLVER
        tag[k] = g;
        group[g].push_back(EeJob{off[k], m, n, svo[k]});
        smem[g] = std::max(smem[g], bd_smem_doubles((m + (1 << g) - 1) >> g, n));
    }
    size_t njobs = 0;
    for (int g = 0; g < kSizes; ++g) njobs += group[g].size();
    if (njobs == 0) return ED_OK;
    const int64_t total = svo.back();
    double *dd = nullptr, *ee = nullptr;
    EeJob* djobs = nullptr;
    if (cudaMalloc(&dd, sizeof(double) * std::max<int64_t>(total, 1)) != cudaSuccess ||
        cudaMalloc(&ee, sizeof(double) * std::max<int64_t>(total, 1)) != cudaSuccess ||
        cudaMalloc(&djobs, sizeof(EeJob) * njobs) != cudaSuccess) {
        cudaFree(dd); cudaFree(ee); cudaFree(djobs);
        return ED_ERR_ALLOC;
    }
    std::vector<EeJob> all;
    size_t first[kSizes];
    for (int g = kSizes - 1; g >= 0; --g) {
        first[g] = all.size();
        all.insert(all.end(), group[g].begin(), group[g].end());
    }
    ed_status st = ED_OK;
    if (cudaMemcpyAsync(djobs, all.data(), sizeof(EeJob) * njobs, cudaMemcpyHostToDevice, s) != cudaSuccess)
        st = ED_ERR_CUDA;
    cudaEvent_t ready = nullptr;
    if (st == ED_OK && (cudaEventCreateWithFlags(&ready, cudaEventDisableTiming) != cudaSuccess ||
                        cudaEventRecord(ready, s) != cudaSuccess))
        st = ED_ERR_CUDA;
    bool ok[kSizes] = {true, true, true, true, true};
    std::vector<cudaEvent_t> done_ev;
    for (int g = kSizes - 1; st == ED_OK && g >= 0; --g) {
        if (group[g].empty()) continue;
        cudaStream_t gs = bd_stream(device, g);
        cudaEvent_t ev = nullptr;
        if (!gs || cudaStreamWaitEvent(gs, ready, 0) != cudaSuccess ||
            cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
            st = ED_ERR_CUDA;
            break;
        }
        ok[g] = launch_bidiag(group[g], 1 << g, blocks, dd, ee, gs, djobs + first[g], smem[g] * sizeof(double));
        cudaEventRecord(ev, gs);
        cudaStreamWaitEvent(s, ev, 0);
        done_ev.push_back(ev);
    }
    std::vector<double> hd(std::max<int64_t>(total, 1)), he(std::max<int64_t>(total, 1));
    if (st == ED_OK && (cudaMemcpyAsync(hd.data(), dd, sizeof(double) * total, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                        cudaMemcpyAsync(he.data(), ee, sizeof(double) * total, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                        cudaStreamSynchronize(s) != cudaSuccess))
        st = ED_ERR_CUDA;
    for (cudaEvent_t ev : done_ev) cudaEventDestroy(ev);
    if (ready) cudaEventDestroy(ready);
    cudaFree(dd); cudaFree(ee); cudaFree(djobs);
    if (st != ED_OK) return st;
    // the bidiagonal SVDs on host threads, largest first
    std::vector<int> todo;
    for (size_t k = 0; k < off.size(); ++k)
        if (tag[k] >= 0 && ok[tag[k]]) todo.push_back((int)k);
    std::stable_sort(todo.begin(), todo.end(), [&](int a, int b) { return nn[a] > nn[b]; });
    std::vector<char> fail(off.size(), 0);
    const int nth = std::max(1, std::min<int>((int)todo.size(), (int)std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    std::atomic<int> next(0);
    auto work = [&]() {
        for (;;) {
            const int t = next.fetch_add(1);
            if (t >= (int)todo.size()) return;
            const int k = todo[t];
            double* d = hd.data() + svo[k];
            double* e = he.data() + svo[k];
            if (!bidiag_singular_values(nn[k], d, e)) { fail[k] = 1; continue; }
            std::sort(d, d + nn[k], [](double x, double y) { return x > y; });
            std::copy(d, d + nn[k], sv_host->data() + svo[k]);
        }
    };
    for (int i = 1; i < nth; ++i) th.emplace_back(work);
    work();
    for (std::thread& t : th) t.join();
    for (int k : todo)
        if (!fail[k]) (*handled)[k] = 1;
    return ED_OK;
}

}  // namespace ed
