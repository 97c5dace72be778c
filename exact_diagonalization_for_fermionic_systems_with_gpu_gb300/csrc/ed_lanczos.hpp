// ed_lanczos.hpp — device-resident state of one Lanczos run.
//
// The Lanczos vectors are kept unnormalised (w_j, |w_j| = beta_j) in FX
// format, one exponent per vector; v_j = w_j / beta_j is never formed.  All
// scalar bookkeeping (alpha_j, beta_j, exponents, the integer coefficients
// of the next axpy) happens on the device: in the last block of each
// reduction of the per-step kernels (two launches per step), or in every
// CTA of the persistent kernel after its grid barriers (one launch per run).
#pragma once

#include <cstdint>

namespace ed {

constexpr int kLzMaxPartials = 152 * 16;  // entries of each partial-sum array
constexpr int kLzStamps = 9;              // timestamps per step of the persistent kernel
constexpr int kFxBits = 54;               // every FX Lanczos vector has |q| < 2^kFxBits

struct LzState {
    // per Krylov slot j (device arrays of length max_steps + 2)
    int* e;          // exponent: w_j[i] = q_j[i] * 2^e[j]
    uint64_t* m;     // max |q_j[i]|
    double* beta;    // beta[j] = |w_j|; beta[0] = |start vector|
    double* alpha;   // alpha[j] = <v_j, H v_j>
    // grid-reduction partials, one entry per block
    uint64_t* part_lo;
    uint64_t* part_hi;
    uint64_t* part_max;
    unsigned int* counter;  // [4] last-block counters (matvec, axpy, start, misc)
    // current step scalars
    int s_u;         // right shift applied to the exact matvec accumulator
    int e_u;         // exponent of u = H w_j
    uint64_t m_u;    // max |u_q|
    int Fa;          // fractional bits of the axpy coefficients
    int e_w;         // exponent of w_{j+1}
    int64_t at[3];   // integer axpy coefficients (u, w_j, w_{j-1})
    int sh[3];       // extra right shift of each product to the common Fa
    int status;      // 0 ok, 7 breakdown, 6 non-finite
    int min_bits;    // fewest significant bits of any w_j
    int steps_done;
};

// Grid-reduction accumulator of the persistent kernel: an exact 128-bit sum
// as three 42-bit limb sums (l2 holds the signed top limb) and a max.
struct LzRedSet {
    unsigned long long l0, l1, l2, mx;
};

// Arguments of the persistent Lanczos kernel (steps j0 .. j1-1 in one launch).
// Limits of the persistent kernels' grid-barrier waits: a CTA gives up after
// `spin` polls or `ns` nanoseconds of %globaltimer, whichever comes first.
// `extra` > 0 makes every barrier wait for that many arrivals more than the
// grid has, so that the wait runs out (the error path's test).
struct GridWait {
    long long spin;
    unsigned long long ns;
    unsigned int extra;
};

// Defaults (2^26 polls, 4 s), or ED_GRID_WAIT="<ns>[,<extra arrivals>]".
GridWait grid_wait_limits();

// Host-mapped mirror of the Lanczos scalars for the host-side stop test.
struct HostMirror {
    int done;     // alpha[0 .. done-1] and beta[0 .. done] are written
    int stop;     // host: nonzero n ends the run once n steps are done
    int pad_[2];
    double* alpha;  // device addresses of mapped arrays (max_steps + 2 each)
    double* beta;
};

struct LzFusedArgs {
    int64_t* basis;
    int64_t stride;      // slot stride in elements
    int stored;          // slot(j) = basis + (stored ? j : j % 3) * stride
    int j0, j1;
    int64_t* u;
    int64_t n;           // stored values (D * W)
    LzState* lz;
    unsigned int* gbar;  // grid-barrier arrivals, zero at launch
    LzRedSet* red;       // four accumulator sets, zero at launch
    unsigned int* taken; // two row-queue counters (step parity), zero at launch
    unsigned long long* stamps;  // optional: %globaltimer of block 0 at kLzStamps
                                 // points of every step (see ed_lanczos_fused.cu)
    unsigned long long* cta_stamps;  // optional: every CTA's rows-done and axpy-done
                                     // times, [step][2][gridDim.x]
    GridWait wait;
    // Stop test on the host while the launch runs (reference mode): block 0
    // mirrors alpha and beta into host-mapped memory and counts the slots
    // done; a nonzero host stop word s ends the launch at the first step end
    // with j + 1 >= s (the decision passed to every CTA through stop_word,
    // read after the step's last grid barrier).  All null when unused.
    HostMirror* mirror;  // device address of the mapped mirror
    int* stop_word;      // device word, zero at launch
};

// One instance of a batched run (k_lz_batch): instances share the hopping
// tables of the first operator (same sector and lattice terms) and differ in
// their folded diagonals and scalars.
constexpr int kLzBatchMax = 8;

struct LzInst {
    int64_t* basis;        // stored Krylov basis (slot stride LzBatchArgs::stride)
    int64_t* u;            // matvec output
    LzState* lz;
    const int64_t* dUPq;   // folded diagonals at the instance's scale 2^-Fc
    const int64_t* dDNq;
    int64_t Uq;            // U 2^Fc
    int64_t coefUP;        // the single hopping class of each table, 2^Fc units
    int64_t coefDN;
    int Fc;
    int unitUP, unitDN, mergeUD;
    int nclsUP, nclsDN;
    int bq_bits;
    int pad_;
};

struct LzBatchArgs {
    const LzInst* inst;    // B instances (device)
    int B;
    int j0, j1;
    int64_t stride;        // slot stride in elements
    int64_t n;             // stored values per vector
    unsigned int* gbar;    // grid-barrier arrivals, zero at launch
    LzRedSet* red;         // 4 * B accumulator sets (set r % 4 of instance b at (r % 4) * B + b), zero at launch
    unsigned int* taken;   // two item-queue counters (step parity), zero at launch
    GridWait wait;
};

struct MvArgs;

// Heterogeneous batch (k_lz_multi): instances of any sectors, real or
// complex, each with its own operator arguments; instances with equal
// `group` share the shared-memory tables (same sector and hopping terms).
constexpr int kLzMultiMax = 16;

// Row-engine variant of an operator (the k_lz_fused instantiation it takes).
enum LzKind : int {
    kKindRealSched = 0,  // real, one class per table, gather schedule
    kKindRealFast = 1,   // real, one class per table, CSR down table
    kKindRealSeg = 2,    // real, class-segmented tables
    kKindReal = 3,       // real, any classes
    kKindCplxFast = 4,   // complex, one class per table
    kKindCplxSeg = 5,    // complex, class-segmented tables
    kKindCplx = 6,       // complex, any classes
};

struct LzMultiInst {
    int64_t* basis;   // stored Krylov basis, slot stride `stride`
    int64_t* u;       // matvec output
    LzState* lz;
    int64_t n;        // stored values (rows, or 2 rows complex)
    int64_t stride;
    int kind;         // LzKind
    int group;        // instances with equal group share staged tables
    int dimUP;
    int pad_;
};

struct LzMultiArgs {
    const MvArgs* args;         // B operator arguments (device; err of the first)
    const LzMultiInst* inst;    // B instances (device)
    int B;
    int j0, j1;
    int smem;                   // dynamic shared memory of the launch
    unsigned int* gbar;         // grid-barrier arrivals, zero at launch
    LzRedSet* red;              // 4 * B accumulator sets, zero at launch
    unsigned int* taken;        // 2 * B row-queue counters (step parity, instance), zero at launch
    GridWait wait;
};

}  // namespace ed
