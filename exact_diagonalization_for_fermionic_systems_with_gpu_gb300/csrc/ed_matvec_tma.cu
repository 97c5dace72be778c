// ed_matvec_tma.cu — one-launch matvec for spin sectors whose down-spin
// tables fit in shared memory (dim_dn up to a few thousand: chains and
// clusters up to ~14 sites, Kagome/Lieb 12).  The row engine lives in
// ed_matvec_tma.cuh; this file adds the kernel around it, the shared-memory
// plan and the launchers.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <functional>
#include <queue>
#include <vector>

#include "ed_matvec_tma.cuh"

namespace ed {
using namespace dev;

constexpr double kRowCostUp = 0.8;  // up-term share of a row's cost at the mean up-row length

template <bool CPLX, int OUT, bool FAST, bool SCHED, bool SEG = false>
__global__ void __launch_bounds__(kTmaThreads, 2) k_matvec_tma(const MvArgs a) {
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ uint32_t uoff[kTmaUpStage];
    __shared__ uint32_t uent[kTmaUpStage];
    __shared__ int give_up;
    const TmaSmem S = tma_view(a, sm, uoff, uent, &give_up);
    uint32_t u0 = 0;
    const bool has_row = tma_first_row(a, &u0);
    if (threadIdx.x == 0) {
        tma_init(S);
        tma_issue_tables(a, S);
        if (has_row) tma_issue_row<CPLX>(a, S, a.xq, u0, 0);
    }
    if (SCHED) tma_zero_slots(a, S);
    __syncthreads();
    if (!tma::mbar_wait(&S.bar[2], 0)) {
        if (threadIdx.x == 0) atomicExch(a.err, 1);
        give_up = 1;
    }
    __syncthreads();

    int E_out = 0, s_u = 0;
    if (OUT == 0) {
        E_out = fx_exp_from_emax(*a.p_emax) - a.Fc;
    } else {
        const int b = a.bq_bits + bitlen_u64(*a.p_mx) - 62;
        s_u = b > 0 ? b : 0;
    }
    i128 dot = 0;
    uint64_t mx = 0;
    uint32_t rc = 0;
    if (!give_up) {
        tma_rows<CPLX, OUT, FAST, false, SCHED, false, SEG>(a, S, a.xq, a.uq, a.y, rc, E_out, s_u, dot, mx);
    } else if (threadIdx.x == 0) {
        // the table copy (the wait that gave up, once more) and the first row
        // copy must land before the CTA exits (bounded waits)
        tma::mbar_wait(&S.bar[2], 0);
        if (has_row) tma::mbar_wait(&S.bar[0], 0);
    }
    if (OUT == 1) mv_lanczos_epilogue(a, dot, mx, s_u);
}

// Shared-memory plan: returns the dynamic bytes (0 when the sector does not
// fit or rows are not 16-byte multiples).
int tma_plan(const ed_op* op, MvArgs* a) {
    const int W = op->cplx ? 2 : 1;
    const int64_t dimDN = op->dimDN;
    // an odd real row is copied with one element before or after it
    const int64_t row_bytes = ((dimDN * W + 2) & ~(int64_t)1) * 8;
    // the gather schedule serves the single-class real kernel only
    if (op->cplx || !op->mv_fast) {
        a->dnSched = nullptr;
        a->dnSteps = nullptr;
    }
    auto up128 = [](int64_t v) { return (v + 127) / 128 * 128; };
    // with the schedule a row buffer holds [x | -x | 16 zeros]
    const int64_t buf_bytes = a->dnSched ? ((int64_t)2 * a->schedNeg + 18) * 8 : row_bytes;
    int64_t off = 128;  // mbarriers
    a->sm_row0 = (int)off;
    off += up128(buf_bytes);
    a->sm_row1 = (int)off;
    off += up128(buf_bytes);
    if (a->dnSched) {
        a->sm_sched = (int)off;
        off += up128((int64_t)a->schedSteps * a->dimDNp * 2);
        a->sm_steps = (int)off;
        off += up128(a->dimDNp / 32);
    } else {
        a->sm_dnptr = (int)off;
        off += up128((dimDN + 1) * 4);
        a->sm_dnent = (int)off;
        off += up128(op->tdn.nnz * 4);
        a->sm_dnnpos = (int)off;
        off += up128(dimDN);
    }
    a->sm_ddnq = (int)off;
    off += up128(dimDN * 8);
    a->sm_stdn = (int)off;
    off += up128(dimDN * 8);
    const int64_t static_bytes = 2 * kTmaUpStage * 4 + 64 + 24 * 64;  // uoff, uent, reduction scratch
    if (off + static_bytes > 227 * 1024) return 0;
    return (int)off;
}

template <bool CPLX, int OUT, bool FAST, bool SCHED, bool SEG = false>
static cudaError_t launch_tma4(const ed_op* op, const MvArgs& a, cudaStream_t s) {
    auto kern = k_matvec_tma<CPLX, OUT, FAST, SCHED, SEG>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, op->tma_smem);
    if (e != cudaSuccess) return e;
    kern<<<op->tma_grid, kTmaThreads, op->tma_smem, s>>>(a);
    return cudaGetLastError();
}

template <int OUT>
static cudaError_t launch_tma_out(const ed_op* op, const MvArgs& a, cudaStream_t s) {
    if (op->cplx) {
        if (op->mv_fast) return launch_tma4<true, OUT, true, false>(op, a, s);
        return a.upSegE ? launch_tma4<true, OUT, false, false, true>(op, a, s) : launch_tma4<true, OUT, false, false>(op, a, s);
    }
    if (!op->mv_fast)
        return a.upSegE ? launch_tma4<false, OUT, false, false, true>(op, a, s) : launch_tma4<false, OUT, false, false>(op, a, s);
    return a.dnSched ? launch_tma4<false, OUT, true, true>(op, a, s) : launch_tma4<false, OUT, true, false>(op, a, s);
}

cudaError_t launch_matvec_tma(const ed_op* op, const MvArgs& a, int out, cudaStream_t s) {
    return out == 0 ? launch_tma_out<0>(op, a, s) : launch_tma_out<1>(op, a, s);
}

int tma_grid(const ed_op* op) {
    int per_sm = 0;
    const void* f;
    if (op->cplx)
        f = op->mv_fast ? (const void*)k_matvec_tma<true, 1, true, false>
            : op->mv.upSegE ? (const void*)k_matvec_tma<true, 1, false, false, true>
                            : (const void*)k_matvec_tma<true, 1, false, false>;
    else if (!op->mv_fast)
        f = op->mv.upSegE ? (const void*)k_matvec_tma<false, 1, false, false, true>
                          : (const void*)k_matvec_tma<false, 1, false, false>;
    else
        f = op->mv.dnSched ? (const void*)k_matvec_tma<false, 1, true, true> : (const void*)k_matvec_tma<false, 1, true, false>;
    cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, op->tma_smem);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, kTmaThreads, op->tma_smem) != cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    if (per_sm > 2) per_sm = 2;
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, op->device);
    // every CTA is resident at once (the persistent Lanczos kernel relies on
    // it); rows are spread over them by row_plan, some CTAs may have none
    return sms * per_sm;
}

void row_plan(const SpinTable& up, int G, std::vector<uint32_t>* start, std::vector<uint32_t>* list,
              std::vector<uint32_t>* queue, double w) {
    const int64_t n = up.count;
    if (w < 0.0) {
        w = kRowCostUp;
        if (const char* e = std::getenv("ED_ROW_COST_UP")) w = std::atof(e);
    }
    double mean = 0.0;
    for (int64_t u = 0; u < n; ++u) mean += up.len[u];
    mean = n ? mean / (double)n : 0.0;
    std::vector<double> cost(n);
    for (int64_t u = 0; u < n; ++u) cost[u] = 1.0 + (mean > 0.0 ? w * up.len[u] / mean : 0.0);
    std::vector<uint32_t> order(n);
    for (int64_t u = 0; u < n; ++u) order[u] = (uint32_t)u;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) { return cost[x] > cost[y]; });
    *queue = order;
    // least-loaded CTA first; ties to the lowest index
    using Slot = std::pair<double, int>;
    std::priority_queue<Slot, std::vector<Slot>, std::greater<Slot>> heap;
    for (int b = 0; b < G; ++b) heap.push({0.0, b});
    std::vector<std::vector<uint32_t>> rows(G);
    for (uint32_t u : order) {
        Slot sl = heap.top();
        heap.pop();
        rows[sl.second].push_back(u);
        sl.first += cost[u];
        heap.push(sl);
    }
    start->assign(G + 1, 0);
    list->clear();
    list->reserve(n);
    for (int b = 0; b < G; ++b) {
        std::sort(rows[b].begin(), rows[b].end());
        (*start)[b] = (uint32_t)list->size();
        list->insert(list->end(), rows[b].begin(), rows[b].end());
    }
    (*start)[G] = (uint32_t)list->size();
}

}  // namespace ed
