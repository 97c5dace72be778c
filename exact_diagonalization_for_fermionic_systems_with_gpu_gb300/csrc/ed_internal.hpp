// ed_internal.hpp — the operator handle and the launchers behind the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <functional>
#include <string>
#include <vector>

#include "../../include/ed_hubbard.h"
#include "ed_tables.hpp"

namespace ed {

constexpr int kMaxCls = kMaxClasses;
constexpr int kSegCls = 4;  // classes a segmented row table describes (one byte each)

// Everything the matvec kernel needs, passed by value (< 4 KB).
struct MvArgs {
    const int64_t* xq;  // FX input, interleaved re,im when complex
    int64_t dimUP, dimDN;
    const uint32_t* upEnt;
    const uint8_t* upLen;
    const uint8_t* upNpos;
    const uint32_t* dnEnt;
    const uint8_t* dnLen;
    const uint8_t* dnNpos;
    const int64_t* dUPq;  // folded diagonals, scale 2^-Fc
    const int64_t* dDNq;
    const uint64_t* stUP;
    const uint64_t* stDN;
    uint64_t mask;
    int64_t Uq;           // U * 2^Fc
    int Fc;
    int nclsUP, nclsDN;
    int unitUP, unitDN;   // single class with |coef| == 1 (coef_q == 2^Fc)
    int mergeUD;          // single class each, equal coefficients
    int bq_bits;          // bitlen of the per-unit row bound (acc <= 2^bq_bits * max|x_q|)
    // CSR copies of the tables (shared-memory kernel)
    const uint32_t* upPtr;
    const uint32_t* upEntC;
    const uint32_t* dnPtr;
    const uint32_t* dnEntC;
    uint32_t dnNnz;
    // conflict-free gather schedule of the down term (real single-class
    // operators; null otherwise): entries [schedSteps][dimDNp], steps per
    // 32-column block
    const uint16_t* dnSched;
    const uint8_t* dnSteps;
    int schedSteps;
    int dimDNp;
    int schedNeg;         // index of -x[0] in the row buffer; zeros at 2 * schedNeg
    // rows of each CTA of the shared-memory kernels (balanced on the host):
    // CTA b computes rows rowList[rowStart[b] .. rowStart[b+1])
    const uint32_t* rowStart;
    const uint32_t* rowList;
    const uint32_t* rowQueue;  // all rows in decreasing order of cost (dynamic distribution)
    // The single-run persistent kernel's queue: rowQueue with its last rows
    // (those past the last full wave of CTAs) split into column ranges.  An
    // entry is a row, or row | part << 24 | log2(parts) << 28 for a range.
    const uint32_t* unitQueue;
    uint32_t nunits;           // entries of unitQueue
    int* err;             // device word set when a bounded wait gives up
    // shared-memory plan of the TMA kernel (byte offsets)
    int sm_row0, sm_row1, sm_dnptr, sm_dnent, sm_dnnpos, sm_ddnq, sm_stdn;
    int sm_sched, sm_steps;  // schedule layout (instead of dnptr/dnent/dnnpos)
    // output
    double* y;            // FP64 output (perform path)
    const int* p_emax;    // device: max biased exponent of the FP64 input
    int64_t* uq;          // FX output (Lanczos path)
    const uint64_t* p_mx; // device: max |x_q| of the FX input (Lanczos path)
    // Lanczos per-step reduction outputs
    void* lz;             // LzState* (device)
    int step;
    // class segments of every row (tables with at most kSegCls classes,
    // entries sorted by class, + before -): byte c of segE[r] is the end of
    // class c's entries in row r, byte c of segP[r] the end of its + entries
    // (both relative to the row start); null for tables with more classes
    const uint32_t* upSegE;
    const uint32_t* upSegP;
    const uint32_t* dnSegE;
    const uint32_t* dnSegP;
    int mergeMC;          // segmented tables with equal class lists: one product per class
    // coefficient classes, interleaved (re, im), scale 2^-Fc
    int64_t coefUP[2 * kMaxCls];
    int64_t coefDN[2 * kMaxCls];
};

// Two-pass (striped) matvec for sectors whose down rows exceed shared memory
// (ed_matvec_striped.cu); the down index is in the op's permuted order.
struct StripedArgs {
    const int64_t* xq;        // FX input, permuted order
    int64_t* sdn;             // int64 down sums (pass D out, pass U in / FP64 out)
    int64_t dimUP, dimDN;
    const uint16_t* sched16;  // [cpad / 32][s8][32][8] offset in the chunk's window | sign << 15; idle: a zero slot
    const uint8_t* steps32;   // steps the warp of 32-column block k runs
    const uint8_t* negcnt;    // negative entries of each (permuted) column
    int64_t cpad;
    int s8;                   // groups of eight schedule steps
    int64_t bw;               // bandwidth of the permuted down index
    int chunk;                // columns per pass-D item
    int zbase;                // first of the 16 zero slots after the window
    const int64_t* dDNq;      // folded down diagonal, permuted
    const uint64_t* stDN;     // down bitstrings, permuted
    int* err;
};

}  // namespace ed

struct ed_op {
    int device = 0;
    int n_sites = 0, n_up = 0, n_dn = 0;
    bool cplx = false;
    int64_t dimUP = 0, dimDN = 0, D = 0;
    double U = 0.0;
    uint64_t mask = 0;
    ed::SpinBasis bup, bdn;
    ed::SpinTable tup, tdn;
    ed::MvArgs mv;  // static part of the matvec arguments
    // device tables
    uint32_t *d_upEnt = nullptr, *d_dnEnt = nullptr;
    uint8_t *d_upLen = nullptr, *d_dnLen = nullptr;
    uint8_t *d_upNpos = nullptr, *d_dnNpos = nullptr;
    uint32_t *d_upPtr = nullptr, *d_upEntC = nullptr, *d_dnPtr = nullptr, *d_dnEntC = nullptr;
    uint16_t* d_dnSched = nullptr;
    uint8_t* d_dnSteps = nullptr;
    uint32_t *d_rowStart = nullptr, *d_rowList = nullptr, *d_rowQueue = nullptr, *d_unitQueue = nullptr;
    uint32_t *d_upSegE = nullptr, *d_upSegP = nullptr, *d_dnSegE = nullptr, *d_dnSegP = nullptr;
    int* d_err = nullptr;
    int64_t *d_dUPq = nullptr, *d_dDNq = nullptr;
    uint64_t *d_stUP = nullptr, *d_stDN = nullptr;
    // perform-path workspace (grow-only)
    int64_t* d_xq = nullptr;
    int* d_emax = nullptr;
    int* d_flag = nullptr;
    double* h_stage = nullptr;  // pinned staging for host-pointer perform
    size_t h_stage_bytes = 0;
    double* d_io = nullptr;     // device x|y for host-pointer perform
    size_t d_io_bytes = 0;
    int stage_smem = 0;         // bytes of dynamic smem for the staged row (0 = no staging)
    int grid = 0;               // matvec grid
    int mv_threads = 256;       // matvec CTA size
    bool mv_fast = false;       // at most one coefficient class per spin
    int tma_smem = 0;           // >0: the shared-memory/TMA matvec is used
    int tma_grid = 0;
    // two-pass matvec (striped): down index permuted by perm (new -> old)
    bool striped = false;
    int st_grid = 0, st_win = 0, st_chunk = 0, st_zbase = 0;
    int st_s8 = 0;              // groups of eight steps of pass D's schedule (lane-packed layout)
    // tuning (ed_op_autotune): Lanczos kernels 0 by the default rule, 1 per
    // step, 2 persistent; weight of the persistent kernel's row queue
    int lz_mode = 0;
    int lz_grid = 0;            // persistent kernel's CTAs (0: tma_grid, two per SM)
    double row_cost = -1.0;
    int64_t st_bw = 0, st_cpad = 0;
    uint32_t* d_permDN = nullptr;
    uint16_t* d_sched16 = nullptr;
    uint8_t* d_steps32 = nullptr;
    uint8_t* d_negDN = nullptr;   // negative entries per permuted down column
    int64_t* d_dDNqP = nullptr;
    uint64_t* d_stDNp = nullptr;
    int64_t* d_sdn = nullptr;   // D down sums, allocated on first use
    std::string last_error;
};

namespace ed {

// Launch-level API used by the C ABI and the Lanczos driver.
cudaError_t launch_emax(const double* x, int64_t n, int* d_emax, int* d_flag, cudaStream_t s);
cudaError_t launch_to_fx(const double* x, int64_t n, const int* d_emax, int64_t* xq, cudaStream_t s);
// y = H x from the FX copy xq (exponent from d_emax), FP64 output.
cudaError_t launch_matvec_f64(const ed_op* op, const int64_t* xq, const int* d_emax, double* y,
                              cudaStream_t s);
// u = H x in FX with the Lanczos-step epilogue (dot and max partials).
// d_mx: device pointer to max|xq| (the Krylov slot's m entry).
cudaError_t launch_matvec_lz(const ed_op* op, const int64_t* xq, int64_t* uq, void* lz,
                             const uint64_t* d_mx, int step, cudaStream_t s);
int matvec_grid(const ed_op* op);
int matvec_threads(int64_t dimDN);
int tma_plan(const ed_op* op, MvArgs* a);
int tma_grid(const ed_op* op);
// Rows of each of the G CTAs: longest-processing-time-first under the cost
// model 1 + w * len_up(u) / mean len_up (w from ED_ROW_COST_UP, default kRowCostUp).
// queue: all rows in decreasing order of that cost.
// w < 0: ED_ROW_COST_UP or kRowCostUp.
void row_plan(const SpinTable& up, int G, std::vector<uint32_t>* start, std::vector<uint32_t>* list,
              std::vector<uint32_t>* queue, double w = -1.0);
cudaError_t launch_matvec_tma(const ed_op* op, const MvArgs& a, int out, cudaStream_t s);
cudaError_t launch_striped_down(const ed_op* op, const StripedArgs& g, cudaStream_t s);
cudaError_t launch_striped_up(const ed_op* op, const MvArgs& a, const StripedArgs& g, int out, cudaStream_t s);
cudaError_t launch_permute_f64(const ed_op* op, const double* in, double* out, int forward, cudaStream_t s);
cudaError_t launch_permute_i64(const ed_op* op, const int64_t* in, int64_t* out, int forward, cudaStream_t s);
cudaError_t launch_to_fx_perm(const ed_op* op, const double* x, const int* d_emax, int64_t* xq, cudaStream_t s);
// the striped path's scratch (D int64) and its arguments for input xq
cudaError_t striped_args(ed_op* op, const int64_t* xq, StripedArgs* g);

// Lanczos recurrence (ed_lanczos.cu); stop_beta >= 0 ends it at the first
// beta_k < stop_beta * beta_0 (Krylov time evolution).
ed_status lanczos_run(ed_op* op, void** ws_slot, const ed_lanczos_cfg* cfg, const double* start, int start_mem,
                      double* evec, int evec_mem, double* alpha_h, double* beta_h, ed_lanczos_result* res,
                      cudaStream_t s, double stop_beta = -1.0);
// The op's Lanczos workspace slot, and the stored basis of its last run:
// slot k at basis + k * stride holds q_k with w_k = q_k 2^e[k] (e on the device).
void** lanczos_ws_slot(ed_op* op);
// B fixed-step runs of operators sharing their hopping tables in one
// persistent launch (ed_lanczos.cu).
ed_status lanczos_batch_run(ed_op* const* ops, int B, const ed_lanczos_cfg* cfg, const double* starts, int start_mem,
                            double* evecs, int evec_mem, double* alpha_h, double* beta_h, ed_lanczos_result* res,
                            cudaStream_t s);
// Entanglement blocks (column-major m x n, m >= n, at blocks + off[k]) whose
// singular values the cluster bidiagonalisation computes: handled[k] = 1 and
// the values, descending, at (*sv_host)[svo[k] ..).  ED_EE_METHOD=gesvd
// leaves every block to cuSOLVER.
ed_status ee_bidiag_blocks(int device, cudaStream_t s, const double* blocks, const std::vector<int64_t>& off,
                           const std::vector<int>& mm, const std::vector<int>& nn, const std::vector<int64_t>& svo,
                           std::vector<double>* sv_host, std::vector<char>* handled);
void lanczos_basis(void* ws_slot, const int64_t** basis, int64_t* stride, const int** e_dev);
// The vectors of the last non-stored run on a workspace, regenerated one by
// one for visit(k, q_k) (ed_lanczos.cu).
ed_status lanczos_replay(ed_op* op, void* ws_slot, int n,
                         const std::function<cudaError_t(int, const int64_t*)>& visit, cudaStream_t s);

}  // namespace ed
