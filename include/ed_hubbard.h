/*
 * ed_hubbard.h — C ABI of the GB300-native Hubbard exact-diagonalisation
 * hot path: the Siro-Harju spin-split matvec
 *     y = (H_up (x) 1 + 1 (x) H_dn + U * sum_i n_i,up n_i,dn) x
 * over the fixed-(N_up, N_dn) product basis, and the Lanczos solver it drives.
 *
 * Conventions
 *  - Every function returns an ed_status (0 = ED_OK) unless it returns a size;
 *    nothing throws across this boundary.
 *  - Vectors are FP64, length ed_op_rows(op) (complex operators: interleaved
 *    re,im pairs, 2*rows doubles), indexed up-index-major exactly like the
 *    reference: element (a_up, a_dn) sits at a_up * dim_dn + a_dn, where a_s
 *    is the rank of the spin-s bitstring among N-bit words with Q_s bits set
 *    in ascending-integer order (= the combinatorial-number-system rank).
 *  - "stream" is a cudaStream_t passed as void* (NULL = legacy default stream).
 *  - Indices and sizes are 64-bit throughout.
 *
 * Reference interfaces replaced (paths inside the reference project
 * jeechul/Exact_Diagonalization_for_Fermionic_systems_with_GPU):
 *  - H_TBq (basis + per-spin tables)           MBL_test/include/fermi_operator.h:42-242
 *  - Hubbard ctor / Hubbard_mv                 MBL_test/include/HubMatrix_GPU.cuh:30-182
 *  - cuSpectra::Hubbard rows/cols/perform_op   TotalSpin/include/HubMatrix_TotalSpin.cuh:181-322
 *  - Lanczos::random_vector / eigen            MBL_test/include/HubMatrix_GPU.cuh:477-613
 *  - LAPACKf77::dsted (tridiagonal eigensolve)  MBL_test/include/MAGMA_LAPACK.h:296-326
 */
#ifndef ED_HUBBARD_H
#define ED_HUBBARD_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int ed_status;

enum {
    ED_OK = 0,
    ED_ERR_ARG = 1,          /* invalid argument (null pointer, bad size, bad site) */
    ED_ERR_CUDA = 2,         /* a CUDA runtime call failed */
    ED_ERR_ALLOC = 3,        /* device or host allocation failed */
    ED_ERR_TABLE = 4,        /* a table row needs more slots than the layout has */
    ED_ERR_RANGE = 5,        /* size beyond what the layout supports */
    ED_ERR_NONFINITE = 6,    /* NaN or Inf in an input vector */
    ED_ERR_BREAKDOWN = 7,    /* Lanczos residual vanished (invariant subspace) */
    ED_ERR_NOT_CONVERGED = 8,/* convergence test not met within max_steps */
    ED_ERR_TIMEOUT = 9,      /* a bounded device wait gave up */
    ED_ERR_NOT_BUILT = 10    /* requested feature not available in this build */
};

/* Human-readable name of a status code (static storage). */
const char* ed_status_string(ed_status s);
/* ABI version: major*10000 + minor*100 + patch. */
int ed_version(void);

/* ------------------------------------------------------------------ basis --
 * Combinatorial-number-system rank/unrank of N-bit words with Q bits set, in
 * ascending-integer order.  Bit-identical to H_TBq::state / H_TBq::address
 * (fermi_operator.h:44-53, 76-88).  Host functions. */
int64_t ed_binom(int n, int k);
/* words[i] = the ranks[i]-th word (0-based). */
ed_status ed_basis_unrank(int n_sites, int n_part, const int64_t* ranks, int64_t count, uint64_t* words);
/* ranks[i] = rank of words[i]; ED_ERR_ARG if a word has the wrong popcount. */
ed_status ed_basis_rank(int n_sites, int n_part, const uint64_t* words, int64_t count, int64_t* ranks);
/* Same two maps on the device (device pointers, asynchronous on stream). */
ed_status ed_basis_unrank_device(int n_sites, int n_part, const int64_t* ranks, int64_t count, uint64_t* words, void* stream);
ed_status ed_basis_rank_device(int n_sites, int n_part, const uint64_t* words, int64_t count, int64_t* ranks, void* stream);

/* ------------------------------------------------------------- one-body terms
 * A per-spin operator is an ordered list of terms, each one reference call:
 *   ED_TERM_HOP      H_TBq::Make_H(i, j, t)   fermi_operator.h:100-115
 *                    t (c+_i c_j + c+_j c_i), Jordan-Wigner sign
 *                    (-1)^(particles strictly between i and j)
 *   ED_TERM_CURRENT  H_TBq::Make_J(i, j, t)   fermi_operator.h:117-138
 *                    row state empty at i, full at j -> +t; reverse -> -t
 *   ED_TERM_DENSITY  H_TBq::Make_N(i, v)      fermi_operator.h:140-149
 *                    v n_i (j ignored)
 *   ED_TERM_PEIERLS  complex hop: t e^{+i phi} for the particle moving
 *                    i -> j and t e^{-i phi} for j -> i (same sign rule);
 *                    phi = 0 gives ED_TERM_HOP.  Requires ED_OP_COMPLEX.
 * value = t (or v), phase = phi (PEIERLS only). */
enum { ED_TERM_HOP = 0, ED_TERM_CURRENT = 1, ED_TERM_DENSITY = 2, ED_TERM_PEIERLS = 3 };

typedef struct {
    int32_t kind;
    int32_t i, j;
    int32_t pad_;
    double value;
    double phase;
} ed_term;

/* Reference ELL export: the exact tables H_TBq builds for the given term
 * list, slot-major with z*Q+1 = 10*Q+1 slots (Ax[s*count + a], Aj[s*count + a],
 * 0.0 marks an empty slot, first-empty-slot stacking, fermi_operator.h:64-73).
 * Real terms only.  ax, aj: count*(10*Q+1) entries; state: count entries (any
 * of the three may be NULL).  ED_ERR_TABLE if a row overflows its slots. */
ed_status ed_tables_ell(int n_sites, int n_part, const ed_term* terms, int n_terms,
                        double* ax, int64_t* aj, uint64_t* state);

/* --------------------------------------------------------------- operator -- */
typedef struct ed_op ed_op;

enum { ED_OP_REAL = 0, ED_OP_COMPLEX = 1 };
enum { ED_MEM_HOST = 0, ED_MEM_DEVICE = 1 };

typedef struct {
    int32_t n_sites;            /* N (<= 62) */
    int32_t n_up, n_dn;         /* Q_up, Q_dn */
    int32_t flags;              /* ED_OP_REAL | ED_OP_COMPLEX */
    const ed_term* up_terms;    /* spin-up term list (H_TBq of the up spin) */
    int32_t n_up_terms;
    int32_t pad0_;
    const ed_term* dn_terms;    /* spin-down term list */
    int32_t n_dn_terms;
    int32_t pad1_;
    double U;                   /* on-site interaction */
    uint64_t interaction_mask;  /* sites where U acts; 0 = all N sites
                                   (the reference "dilution" word,
                                   HubMatrix_GPU.cuh:72-95, 152-156) */
} ed_model_desc;

/* Build the operator on the given CUDA device: basis, per-spin tables and
 * the folded diagonal are built on the host and uploaded once (the reference
 * Hubbard ctor, HubMatrix_GPU.cuh:46-95). */
ed_status ed_op_create(ed_op** op, const ed_model_desc* desc, int device);
ed_status ed_op_destroy(ed_op* op);

/* Hilbert-space dimension dim_up * dim_dn (64-bit: the reference's int
 * rows() overflows at 2^31, HubMatrix_TotalSpin.cuh:279-280). */
int64_t ed_op_rows(const ed_op* op);
int64_t ed_op_cols(const ed_op* op);
int64_t ed_op_dim_up(const ed_op* op);
int64_t ed_op_dim_dn(const ed_op* op);
int ed_op_is_complex(const ed_op* op);

/* The matvec kernel of the operator's Lanczos steps: ED_MV_GENERIC (one
 * thread per element), ED_MV_ROWS (rows staged in shared memory by bulk
 * copies) or ED_MV_TWO_PASS (down sums over a bandwidth-reduced down index,
 * then the up term over L2-resident column stripes); -1 for a null op.
 * Chosen at ed_op_create from the sector's shape (ED_MATVEC overrides). */
enum { ED_MV_GENERIC = 0, ED_MV_ROWS = 1, ED_MV_TWO_PASS = 2 };
int ed_op_matvec_kind(const ed_op* op);

/* y = H x.  mem = ED_MEM_HOST: x, y are host pointers and the call is
 * synchronous — the cuSpectra::Hubbard::perform_op semantics
 * (HubMatrix_TotalSpin.cuh:282-311).  mem = ED_MEM_DEVICE: device pointers,
 * asynchronous on stream — the Hubbard::Hubbard_mv semantics
 * (HubMatrix_GPU.cuh:163-182) without its device-wide sync.  y is
 * overwritten; x and y must not overlap. */
ed_status ed_op_perform(ed_op* op, const double* x, double* y, int mem, void* stream);

/* y = H x on device vectors without any device allocation.  This entry has no
 * counterpart in the reference.  It is for callers that cannot let a library
 * allocate GPU memory: code whose device memory belongs to another allocator
 * (for example a framework's caching pool that has reserved the GPU) and loops
 * that cannot afford the implicit device synchronisation a cudaMalloc or
 * cudaFree may cause.  Same result and argument meaning as ed_op_perform with
 * ED_MEM_DEVICE (x, y device pointers, asynchronous on stream, y
 * overwritten), but the int64 copy of x lives in a fixed static device array
 * of 2^21 values (16 MiB, held on a GPU from the first call there until the
 * process exits): operators with more than 2^21 stored values (rows, or
 * 2*rows for complex operators) return ED_ERR_RANGE.  The first call on a
 * device resolves the array's device address (cudaGetSymbolAddress), which
 * under CUDA's lazy module loading also loads the module holding the array
 * and so reserves its 16 MiB: make that first call before any stream capture
 * and before another allocator reserves the device (ED_ERR_ALLOC if the
 * reservation fails).  All calls share the one array and it keeps the last
 * call's contents: calls that overlap on the GPU (other streams, other
 * threads, other operators on the same device) race.  NaN or Inf in x is not
 * detected by this entry (ED_OK is returned and y is undefined); use
 * ed_op_perform where that check is wanted. */
ed_status ed_op_perform_noalloc(ed_op* op, const double* x, double* y, void* stream);

/* ---------------------------------------------------------------- Lanczos -- */
enum { ED_LANCZOS_REFERENCE = 0,  /* stop test every 10 steps as in
                                       HubMatrix_GPU.cuh:585-597 */
       ED_LANCZOS_FIXED = 1 };    /* exactly max_steps steps */
enum { ED_RITZ_NONE = 0, ED_RITZ_STORED = 1, /* from the stored Krylov basis */
       ED_RITZ_RECOMPUTE = 2 };   /* second pass, as HubMatrix_GPU.cuh:600-612 */
enum { ED_START_RANDOM = 0, ED_START_USER = 1 };

typedef struct {
    int32_t max_steps;     /* Lanczos steps (reference maxN = 1000) */
    int32_t mode;          /* ED_LANCZOS_REFERENCE | ED_LANCZOS_FIXED */
    int32_t reorth;        /* 1 = full reorthogonalisation (needs ED_RITZ_STORED
                              storage; the basis is kept either way) */
    int32_t ritz;          /* ED_RITZ_* */
    int32_t start;         /* ED_START_RANDOM (counter-based, seed below) |
                              ED_START_USER (start vector given) */
    int32_t profile;       /* 1 = per-step kernels, every matvec / axpy launch
                              timed with CUDA events on the launching stream
                              (result fields matvec_ms, axpy_ms);
                              2 = persistent kernel with device timestamps
                              of its phases (matvec_ms, axpy_ms, reduce_ms) */
    uint64_t seed;         /* seed of the uniform(-1,1) start vector */
} ed_lanczos_cfg;

typedef struct {
    double e0;             /* lowest Ritz value */
    int32_t steps;         /* Lanczos steps taken (size of T) */
    int32_t converged;     /* reference stop test met */
    int32_t status;        /* ED_OK | ED_ERR_BREAKDOWN | ... */
    int32_t min_bits;      /* fewest significant bits any Lanczos vector kept */
    double residual;       /* |beta_{n} z_{n-1}| of the lowest Ritz pair */
    int64_t launches;      /* kernels this call launched */
    double matvec_ms;      /* profile: summed device time of the matvecs */
    double axpy_ms;        /* profile: summed device time of the axpys */
    int32_t n_matvec;      /* matvecs (Lanczos steps run) */
    int32_t pad_;
    double reduce_ms;      /* profile 2: time between the phases (block sums,
                              grid barriers, scalar updates) ... */
    double barrier_ms;     /* ... of which waiting at the grid barriers */
    double scalar_ms;      /* ... of which reading the grid totals and updating
                              the Lanczos scalars */
    double fused_ms;       /* profile 2: CUDA-event time of the persistent
                              kernel launches */
    double rows_spread_ms; /* profile 2: summed over steps, last minus first
                              CTA to finish its matvec rows */
    double axpy_spread_ms; /* profile 2: the same for the axpy slices */
} ed_lanczos_result;

/* Run Lanczos on op.  start: ED_START_USER start vector (rows doubles, mem
 * as start_mem), else ignored.  evec: output Ritz vector (normalised; rows
 * doubles at evec_mem) when cfg->ritz != ED_RITZ_NONE, may be NULL
 * otherwise.  alpha (max_steps) and beta (max_steps+1, beta[0] = |f|) are
 * optional HOST outputs of the tridiagonal T.  Synchronous. */
ed_status ed_lanczos_run(ed_op* op, const ed_lanczos_cfg* cfg,
                         const double* start, int start_mem,
                         double* evec, int evec_mem,
                         double* alpha, double* beta,
                         ed_lanczos_result* res, void* stream);

/* The operator as a dense rows x rows matrix, row-major (Hubbard::Write,
 * MBL_test/include/HubMatrix_GPU.cuh:184-240, for the dense-ED drivers
 * TotalSpinFull_* and tED): FP64 entries from the coefficients (interleaved
 * re, im pairs for complex operators), overwritten (the reference adds into a
 * zeroed matrix).  rows <= 65536.  H at mem; synchronous. */
ed_status ed_op_write_dense(ed_op* op, double* H, int mem, void* stream);

/* n_ops (1..16) fixed-step Lanczos runs in one persistent launch: the
 * batched form of the sweeps that call Lanczos::eigen once per disorder
 * realisation, sector or twist (MBL_test/src/Hubbard_EE_test.cu:62-72,
 * TotalSpinExcited_Lieb_randomHop.cu:110-136,
 * drude_v2_cal_Kagome_randomHop.cu:129-158).  The operators may belong to
 * different (N_up, N_dn) sectors of uneven dimension and be real or complex;
 * each needs a shared-memory plan (not the two-pass matvec of the largest
 * sectors; else ED_ERR_NOT_BUILT).  Up to 8 real one-class operators that
 * share their hopping tables run in a kernel specialised for that case,
 * anything else in the general one.  cfg: mode ED_LANCZOS_FIXED, no
 * reorthogonalisation, ritz ED_RITZ_STORED or ED_RITZ_NONE; start
 * ED_START_RANDOM (run b seeded cfg->seed + b) or ED_START_USER.  starts and
 * evecs (at start_mem / evec_mem) hold the runs one after another, rows_b
 * values each (2*rows_b for complex operators: n_ops x rows when all are
 * equal); alpha (n_ops x max_steps), beta (n_ops x (max_steps+1)) and res
 * (n_ops) are optional host outputs; each run's coefficients, E0 and Ritz
 * vector equal those of its own ed_lanczos_run bit for bit.  Synchronous. */
ed_status ed_lanczos_batch(ed_op* const* ops, int n_ops, const ed_lanczos_cfg* cfg, const double* starts,
                           int start_mem, double* evecs, int evec_mem, double* alpha, double* beta,
                           ed_lanczos_result* res, void* stream);

/* Autotuning of the Lanczos step for one operator, over the knobs that set
 * its speed per sector size: the per-step kernels against the persistent
 * kernel; for the persistent kernel, the row-cost weight of its work queue
 * (the cost of a row taken as 1 + w len_up(u) / mean len_up, w = 0.4, 0.8,
 * 1.2) and the rows each CTA takes (two 512-thread CTAs per SM, or one per SM
 * taking twice the rows); for sectors on the two-pass matvec (rows beyond
 * shared memory), the columns of a pass-D window (the chunk, largest that
 * fits and half of it).  Each candidate runs `steps` fixed Lanczos steps (one
 * warm-up run, best of two timed runs); with apply, the fastest becomes the
 * operator's choice for ed_lanczos_run and its users (ED_LZ_FUSED still
 * overrides).  Every candidate computes the same coefficients bit for bit;
 * only the time differs.  Synchronous. */
typedef struct {
    int32_t steps;           /* Lanczos steps per timed run (e.g. 30) */
    int32_t apply;           /* 1: keep the fastest on the operator */
} ed_tune_cfg;

typedef struct {
    int32_t persistent;      /* the choice: 1 persistent kernel, 0 per-step kernels */
    int32_t candidates;      /* configurations timed */
    double row_cost;         /* the choice's row-cost weight (persistent) */
    double us_per_step;      /* the choice's time per step, host clock */
    double per_step_us;      /* per-step kernels */
    double persistent_us[3]; /* persistent kernel, w = 0.4, 0.8, 1.2 (0: no shared-memory plan) */
    int32_t ctas_per_sm;     /* the choice's persistent CTAs per SM (2 or 1; 0 per-step) */
    int32_t chunk;           /* the choice's pass-D window columns (two-pass sectors; else 0) */
    double one_cta_us;       /* persistent kernel, one CTA per SM, the best weight (0: not timed) */
    double chunk_us[2];      /* two-pass: per-step time at the largest chunk and at half of it */
} ed_tune_result;

ed_status ed_op_autotune(ed_op* op, const ed_tune_cfg* cfg, ed_tune_result* res, void* stream);

/* Apply an ed_op_autotune result to another operator of the same shape
 * (e.g. the next twist or disorder sample of a sweep). */
ed_status ed_op_set_tuning(ed_op* op, const ed_tune_result* tuned);

/* Same generator on the device: out (device, n doubles), async on stream. */
ed_status ed_random_vector_device(int64_t n, uint64_t seed, double* out_device, void* stream);

/* The start vector ED_START_RANDOM uses: uniform(-1,1) from a counter-based
 * generator keyed by seed (Philox4x64-10, element k from counter k/4, word k%4), NOT
 * normalised.  Host output. */
ed_status ed_random_vector(int64_t n, uint64_t seed, double* out_host);

/* y = S_xy x, S_xy = (S+S- + S-S+)/2, the transverse part of the total spin
 * on the operator's (N, N_up, N_dn) product basis (TotalSpin::Hubbard::
 * Hubbard_mv, TotalSpin/include/HubMatrix_TotalSpin.cuh:20-66,120-175).
 * x, y: rows values (2*rows, interleaved re,im, for complex operators) at
 * mem; synchronous for host memory, asynchronous on stream otherwise. */
ed_status ed_s2_apply(ed_op* op, const double* x, double* y, int mem, void* stream);

/* For a normalised psi: out[0] = <psi|S_xy|psi>, out[1] = S^2 =
 * (N_up - N_dn)^2 / 4 + <S_xy> (ConservedTotalSpin_Kagome_randomHop.cu:
 * 113-116).  Synchronous. */
ed_status ed_s2_expect(ed_op* op, const double* psi, int mem, double* out, void* stream);

/* Lowest eigenpair of the symmetric tridiagonal (alpha[0..n-1], off-diagonal
 * beta[0..n-2]): eigenvalue e0 (Sturm bisection to adjacent doubles) and unit
 * eigenvector z (n doubles, inverse iteration, largest component positive;
 * may be NULL).  Host in/out, computed on the host (T is a few hundred rows);
 * replaces LAPACKf77::dsted for the Lanczos T. */
ed_status ed_tridiag_lowest(int n, const double* alpha, const double* offdiag,
                            double* e0, double* z);

/* All eigenpairs of the same tridiagonal (LAPACKf77::dsted with compz = 'I',
 * MBL_test/include/MAGMA_LAPACK.h:296-326, as Krylov::Make_tridiagonal_eigen
 * calls it, HubMatrix_GPU.cuh:672-680): evals ascending (n doubles), z the unit
 * eigenvectors as columns (n x n, column j = eigenvector of evals[j]; may be
 * NULL).  Implicit QR with Wilkinson shifts on the host.  ED_ERR_BREAKDOWN if
 * the iteration does not converge. */
ed_status ed_tridiag_eigen(int n, const double* alpha, const double* offdiag,
                           double* evals, double* z);

/* Singular values (descending) of the upper bidiagonal with diagonal d
 * (n) and superdiagonal e (n-1): Golub-Kahan SVD steps on the host, the
 * second half of the entanglement entropy's block SVD (LAPACK's dbdsqr as
 * cusolverDnDgesvd uses it).  ED_ERR_NOT_CONVERGED after 60 n sweeps. */
ed_status ed_bidiag_singular_values(int n, const double* d, const double* e, double* s);

/* out[t] = exp(-i T times[t]) e_0 (n complex values, interleaved re, im;
 * n_times x 2n doubles): the Krylov propagator coefficients of
 * Krylov::Krylov_time_evol (HubMatrix_GPU.cuh:684-690).  Host in/out. */
ed_status ed_tridiag_expm(int n, const double* alpha, const double* offdiag,
                          int n_times, const double* times, double* out);

/* ------------------------------------------------------------ observables --
 * What the reference drivers compute from a ground state.  psi is the Ritz
 * vector (rows doubles, or 2*rows for complex operators) at `mem`. */

/* <x, y> of n doubles (Thrust_Lin::thrust_Dotprod, HubMatrix_GPU.cuh:451-455),
 * deterministic reduction order. */
ed_status ed_vec_dot(int64_t n, const double* x, const double* y, int mem, double* out, void* stream);
/* sum_k conj(x_k) y_k over n complex numbers (interleaved); out[0] = re,
 * out[1] = im (HubMatrix_GPU.cuh:457-463). */
ed_status ed_vec_zdot(int64_t n, const double* x, const double* y, int mem, double* out, void* stream);
/* <psi|O|psi> (out[0] = re, out[1] = im), the Hubbard_mv + thrust_Dotprod
 * pair the drivers use for K_x and S^2 (drude_v2_cal_Kagome_randomHop.cu:213-214). */
ed_status ed_op_expect(ed_op* op, const double* psi, int mem, double* out, void* stream);
/* Per-site <n_i,up>, <n_i,dn> and <n_i,up n_i,dn> of psi (N entries each,
 * any pointer may be NULL): the Hellmann-Feynman derivatives dE0/d eps_i and
 * dE0/dU_i.  Accumulated exactly in 2^-60 fixed point. */
ed_status ed_site_densities(ed_op* op, const double* psi, int mem, double* n_up, double* n_dn, double* docc,
                            void* stream);
/* g(w) = norm2 / (w + E - a_0 - b_1^2/(w + E - a_1 - ...)) for nw complex
 * frequencies (re, im pairs), beta[0] unused
 * (correlator_continued_fraction, HubMatrix_GPU.cuh:820-835).  Host in/out. */
ed_status ed_continued_fraction(int n, const double* alpha, const double* beta, double norm2, double energy, int nw,
                                const double* omega, double* g);

typedef struct {
    int32_t lanczos_steps;   /* Lanczos::tridiagonal length (reference 200) */
    int32_t n_omega;         /* NOMEGA (reference 8000) */
    double omega_step;       /* OMEGA_STEP (0.004) */
    double delta;            /* DELTA, imaginary part of w (0.01) */
    double omega_cutoff;     /* OMEGA_CUTOFF (0.01) */
    double volume;           /* VOL */
} ed_kubo_cfg;

typedef struct {
    double drude;            /* (-<K> - 2 Vertex) / VOL */
    double kinetic;          /* <psi|K|psi> */
    double vertex;           /* sum_{w > cutoff} sigma(w) dw */
} ed_kubo_result;

/* drude_weight_Jx (drude_v2_cal_Kagome_randomHop.cu:183-220): sigma(w) =
 * -Im Lambda(w)/(pi w) with Lambda the continued fraction of the
 * lanczos_steps-step tridiagonalisation of H from J|psi>.  Real operators,
 * psi on the device; sigma_out (n_omega doubles, host) may be NULL. */
ed_status ed_drude_kubo(ed_op* H, ed_op* J, ed_op* K, const double* psi, double e0, const ed_kubo_cfg* cfg,
                        ed_kubo_result* res, double* sigma_out, void* stream);
/* First- and second-order energy response to a parameter theta with
 * dH = dH/dtheta and d2H = d2H/dtheta2 (psi normalised ground state, device):
 *   first  = <psi|dH|psi>                                  (Hellmann-Feynman)
 *   second = <psi|d2H|psi> - 2 <b|(H - E0)^-1|b>,  b = (1 - |psi><psi|) dH psi,
 * the resolvent from a `steps`-step Lanczos on H started at b.  For the flux
 * theta = Phi this is d2E0/dPhi2, the Drude weight without broadening. */
ed_status ed_response(ed_op* H, ed_op* dH, ed_op* d2H, const double* psi, double e0, int steps, double* first,
                      double* second, void* stream);

/* ed_response for n (1..16) operators at once, e.g. the twists of a flux
 * sweep: psis holds the n normalised ground states one after another (rows
 * values each, 2*rows for complex), device memory; e0, first, second are
 * host arrays of n.  The n linear-response Lanczos runs share one persistent
 * launch (the batched form of ed_lanczos_batch; one run each when the
 * operators have no persistent plan).  d2H and second may be NULL together.
 * Synchronous.  No counterpart in the reference (its drivers loop over
 * drude_weight_Jx, drude_v2_cal_Kagome_randomHop.cu:129-158). */
ed_status ed_response_batch(ed_op* const* H, ed_op* const* dH, ed_op* const* d2H, int n, const double* psis,
                            const double* e0, int steps, double* first, double* second, void* stream);

/* The same response for a degenerate ground level (a multiplet the reference
 * drivers do not treat: they differentiate whichever ground state Lanczos
 * returns, e.g. at the zero twist of drude_v2_cal_Kagome_randomHop.cu:
 * 129-158, where Kagome12 6+6 is two-fold degenerate).  psis: g (1..4)
 * linearly independent ground states, one after another (rows values each,
 * 2*rows for complex operators), device memory; the call orthonormalises a
 * copy of them in order (S below; ED_ERR_ARG when they are dependent).
 * Outputs, g x g complex row-major
 * (interleaved re, im; host):
 *   d1  = S^H dH S                                  (first-order matrix)
 *   d2m = S^H d2H S - 2 B^H (Q (H - E0) Q)^-1 B,     B = Q dH S, Q = 1 - S S^H
 * with each resolvent form from a `steps`-step Lanczos run (off-diagonal
 * elements by polarisation).  The branch derivatives of E0(theta) are the
 * eigenvalues of d1 and, where d1 vanishes, of d2m.  Synchronous. */
ed_status ed_response_subspace(ed_op* H, ed_op* dH, ed_op* d2H, const double* psis, int g, double e0, int steps,
                               double* d1, double* d2m, void* stream);
/* Entanglement entropy of psi for the sites in a_mask: the matrix
 * psi[(a_up a_dn), (b_up b_dn)] (entangle_entropy.h:177-197) is block-diagonal
 * in the particle numbers of A; singular values s of every block from a
 * Householder bidiagonalisation on a thread-block cluster and Golub-Kahan
 * SVD steps on the host (blocks too large for a cluster's shared memory:
 * cusolverDnDgesvd, as entangle_entropy.h:231-291; ED_EE_METHOD=gesvd for
 * every block).  s_vn = -sum s^2 ln s^2 (von Neumann entropy of the
 * reduced density matrix), s_ref = -sum s ln s (the sum the reference
 * drivers print, Hubbard_EE_test.cu:80-83).  Real operators. */
ed_status ed_entanglement_entropy(ed_op* op, const double* psi, int mem, uint64_t a_mask, double* s_vn,
                                  double* s_ref, void* stream);

/* The same for n_states states of op's sector (psis: n_states x rows at
 * mem, row-major; s_vn, s_ref: n_states values each), e.g. the ground
 * states of the disorder realisations of one ed_lanczos_batch call (any
 * operator of the sector serves as op).  All blocks of all states share
 * the bidiagonalisation launches and the host SVD threads; each state's
 * entropies equal those of its own ed_entanglement_entropy call bit for
 * bit.  Synchronous. */
ed_status ed_entanglement_entropy_batch(ed_op* op, int n_states, const double* psis, int mem, uint64_t a_mask,
                                        double* s_vn, double* s_ref, void* stream);

/* ---------------------------------------------------- several eigenpairs --
 * The nev lowest eigenpairs of a real operator (what TotalSpinExcited_*.cu
 * get from Spectra::SymEigsSolver<cuSpectra::Hubbard<double>> with
 * SortRule::SmallestAlge, TotalSpinExcited_Lieb_randomHop.cu:133-143; the
 * GPU copy of its restart logic is TotalSpin/include/SymEigsSolver.cuh):
 * thick-restart Lanczos (equivalent to implicit restarting with the unwanted
 * Ritz values as exact shifts) with full reorthogonalisation, every vector
 * in device memory.  Converged when |last component of z_i| * |f| <
 * tol * max(eps^(2/3), |theta_i|) for the nev wanted pairs (Spectra's test);
 * the restart keeps nev + min(nconv, (ncv - nev) / 2) Ritz vectors (ARPACK's
 * dsaup2 rule, as Spectra).  evals (host, nev, ascending), evecs (nev x rows
 * at evec_mem, vector i at evecs + i*rows; may be NULL), resid (host, nev;
 * may be NULL).  ED_ERR_NOT_CONVERGED when max_restarts ran out (the pairs
 * are still written).  Real operators.  Synchronous. */
typedef struct {
    int32_t nev;           /* eigenpairs wanted (lowest algebraic) */
    int32_t ncv;           /* Krylov subspace size, nev < ncv (the reference: 4 (nev + 1)) */
    int32_t max_restarts;  /* Spectra's maxit (the reference: 1000) */
    int32_t start;         /* ED_START_RANDOM | ED_START_USER */
    double tol;            /* Spectra's tol (the reference: 1e-10) */
    uint64_t seed;         /* seed of the uniform(-1,1) start vector */
} ed_eigs_cfg;

typedef struct {
    int32_t nconv;         /* converged pairs among the nev */
    int32_t restarts;      /* restarts done */
    int64_t n_matvec;      /* operator applications */
    int64_t launches;      /* kernels this call launched */
    double max_resid;      /* largest residual estimate of the nev pairs */
} ed_eigs_result;

ed_status ed_eigs_lowest(ed_op* op, const ed_eigs_cfg* cfg, const double* start, int start_mem, double* evals,
                         double* evecs, int evec_mem, double* resid, ed_eigs_result* res, void* stream);

/* Eigenpairs of a small dense symmetric matrix a (n x n, column-major; the
 * symmetric part is used): w ascending, z (n x n, column j = unit eigenvector
 * of w[j]; may be NULL).  Cyclic Jacobi on the host; the Rayleigh-Ritz solve
 * of ed_eigs_lowest.  ED_ERR_NOT_CONVERGED after 100 sweeps. */
ed_status ed_dense_sym_eigen(int n, const double* a, double* w, double* z);

/* ------------------------------------------------------- time evolution --
 * psi(t) = exp(-i H t) psi0 in the Krylov space of psi0
 * (Krylov::Make_tridiagonal_eigen + Krylov::Krylov_time_evol,
 * MBL_test/include/HubMatrix_GPU.cuh:619-728): the Lanczos recurrence from
 * psi0 (the same persistent Lanczos step as ed_lanczos_run, the basis kept in
 * device memory) stops at the first beta_k < tol * |psi0| (the reference:
 * 1e-10 for a normalised psi0) or after max_steps; then, for every time,
 * c = exp(-i T t) e_0 (ed_tridiag_expm) and psi(t) = |psi0| sum_k c_k v_k on
 * the device.  A real operator applied to a complex psi0 runs one recurrence
 * for each nonzero part (exp(-iHt) is linear).  psi0: 2*rows doubles
 * (complex, interleaved re, im) at psi0_mem; psi_out: n_times x 2*rows
 * doubles at out_mem, time-major, overwritten (added to with accumulate);
 * times: host.  Operators that need the two-pass matvec (sectors whose down
 * rows exceed shared memory) keep three vectors and regenerate the basis in
 * a second recurrence (as ED_RITZ_RECOMPUTE and the reference's
 * Krylov_time_evol do), adding each vector's share as it appears.
 * Synchronous. */
typedef struct {
    int32_t max_steps;   /* Krylov dimension cap (the reference's loop: 1000) */
    int32_t reorth;      /* 1: full reorthogonalisation of the basis */
    double tol;          /* stop at beta_k < tol * |psi0| */
    int32_t accumulate;  /* 1: psi_out += psi(t) (Krylov_time_evol adds into phi) */
    int32_t pad_;
} ed_krylov_cfg;

typedef struct {
    int32_t steps;       /* Krylov dimension used (largest of the recurrences) */
    int32_t runs;        /* recurrences run (0, 1 or 2) */
    double norm;         /* |psi0| */
    double err_est;      /* max over times and runs of beta_m |c_{m-1}(t)| |psi0_part|,
                            the a-posteriori error estimate of the truncation */
    int64_t launches;    /* kernels this call launched */
} ed_krylov_result;

ed_status ed_krylov_evolve(ed_op* op, const ed_krylov_cfg* cfg, const double* psi0, int psi0_mem, int n_times,
                           const double* times, double* psi_out, int out_mem, ed_krylov_result* res,
                           void* stream);

#ifdef __cplusplus
}
#endif
#endif /* ED_HUBBARD_H */
