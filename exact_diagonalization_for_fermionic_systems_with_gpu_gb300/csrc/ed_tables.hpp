// ed_tables.hpp — host-side basis and per-spin operator tables.
//
// The basis of one spin species is the list of N-bit words with Q bits set,
// in ascending-integer order (H_TBq::Labeling, fermi_operator.h:44-53); the
// rank of a word in that list is its combinatorial-number-system rank
// sum_k C(p_k, k+1) over its set-bit positions p_0 < p_1 < ...
//
// A per-spin operator is built from an ordered list of reference-style terms
// (Make_H / Make_J / Make_N, fermi_operator.h:100-149) into two layouts:
//  * SpinEll  — the reference's own ELL layout (10*Q+1 slots, slot-major,
//               first-empty-slot stacking) for bit-exact export and KATs;
//  * SpinTable — this build's device layout: the diagonal folded into one
//               FP64 value per state, and the off-diagonal entries of each
//               row packed into 32-bit words (column | coefficient class |
//               sign) sorted by class, stored slot-major with a per-row count.
//               A "class" is one distinct coefficient value up to sign, so a
//               row's contribution is  sum_c coef[c] * (sum of +-x over the
//               row's class-c entries)  — the inner sums are exact integer
//               adds on the device.
#pragma once

#include <complex>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/ed_hubbard.h"

namespace ed {

int64_t binom(int n, int k);
int popcount64(uint64_t v);
// Set bits strictly between sites i and j (fermi_operator.h:26-40).
int count_between(uint64_t word, int i, int j);

struct SpinBasis {
    int n_sites = 0, n_part = 0;
    int64_t count = 0;
    std::vector<uint64_t> state;   // state[rank] = word
    // binom_tab[p][k] = C(p, k) for p <= n_sites, k <= n_part+1
    std::vector<int64_t> binom_tab;
    void build(int n, int q);
    int64_t rank(uint64_t word) const;   // -1 if the popcount is wrong
    uint64_t unrank(int64_t r) const;
};

// Packed entry: bits 0..23 column, bits 24..29 class, bit 31 sign (1 = negative).
constexpr int kColBits = 24;
constexpr uint32_t kColMask = (1u << kColBits) - 1u;
constexpr int kClassShift = 24;
constexpr uint32_t kClassMask = 0x3Fu;
constexpr int kMaxClasses = 64;
constexpr uint32_t kSignBit = 0x80000000u;

struct SpinTable {
    int64_t count = 0;
    int max_len = 0;                      // slots per row in the slot-major layout
    std::vector<uint32_t> ent;            // ent[s * count + a], s < max_len
    std::vector<uint8_t> len;             // entries in row a
    std::vector<uint8_t> npos;            // single-class tables: the first npos[a]
                                          // entries of row a are +, the rest -
    std::vector<double> diag_re, diag_im; // folded diagonal (Make_N terms)
    std::vector<std::complex<double>> coef; // class -> coefficient (sign stripped)
    bool complex_coef = false;            // any class with a nonzero imaginary part
    int64_t nnz = 0;                      // off-diagonal entries
    double max_row_abs = 0.0;             // max_a sum_k |coef of row a| (off-diagonal)
    double max_diag_abs = 0.0;
};

struct SpinEll {
    int64_t count = 0;
    int nslots = 0;
    std::vector<double> ax;
    std::vector<int64_t> aj;
    bool overflow = false;
};

// Bank-conflict-free gather schedule for a real single-class table (the
// down-spin term of the shared-memory matvec).  The kernel keeps a row of x
// in shared memory as [x (neg_base words) | -x (neg_base words) | 16 zeros];
// a schedule entry is an index into that buffer (+x, -x or a zero), so the
// inner loop is load-index, load-value, add.  Column d is handled by lane
// d % 32 of a warp; the 16 lanes of a half warp load 8-byte words, and the
// word at index i sits in bank pair i % 16 (neg_base is a multiple of 16).
// Step s gives every column at most one of its entries, chosen so that the
// 16 columns of a half warp touch 16 different bank pairs: a proper edge
// colouring of the bipartite multigraph (columns x bank pairs, one edge per
// entry), which needs exactly as many colours as its largest degree
// (Koenig's theorem) and is found with alternating-path recolouring.  Lanes
// without an entry in a step read the zero of a bank pair no other lane of
// the half warp uses in that step.
constexpr int kSchedMaxCount = 32752;  // 2 * neg_base + 16 indices fit 16 bits

struct GatherSchedule {
    int steps = 0;                 // schedule length (max over the 32-column blocks)
    int64_t count_pad = 0;         // count rounded up to 32 (row stride of ent)
    int64_t neg_base = 0;          // count rounded up to 16: index of -x[0]
    std::vector<uint16_t> ent;     // ent[s * count_pad + d]: buffer index
    std::vector<uint8_t> steps32;  // steps the warp of 32-column block k runs
};

// False (with *err) when the table is not eligible: complex or several
// classes, more than kSchedMaxCount states, or more than 255 steps.
// bank_cap as in build_gather_schedule32.
bool build_gather_schedule(const SpinTable& t, GatherSchedule* g, std::string* err, int bank_cap = 1);

// Reverse Cuthill-McKee order of a table's hop graph (breadth-first from a
// pseudo-peripheral state, neighbours by increasing degree, reversed; every
// connected component in turn): perm[new] = old, inv[old] = new, and the
// bandwidth max |inv[a] - inv[b]| over the table's entries.  With this order
// the hops of a state stay within +-bandwidth of it.
void rcm_order(const SpinTable& t, std::vector<uint32_t>* perm, std::vector<uint32_t>* inv, int64_t* bandwidth);

// Reorders each aligned block of `block` consecutive entries of perm by
// decreasing row length (stable), so that the lanes of a warp have similar
// entry counts; updates inv and the bandwidth (which grows by < block).
void sort_blocks_by_degree(const SpinTable& t, int block, std::vector<uint32_t>* perm, std::vector<uint32_t>* inv,
                           int64_t* bandwidth);

// Conflict-free gather schedule over permuted columns for the two-pass
// matvec: column c' = inv[d] of the permuted table reads its entries
// (targets inv[col]) one per step, 32-bit words col' | sign << 31, idle
// lanes kSched32None; bank pair of a target = col' % 16 (the kernel's
// windows start at multiples of 16).
constexpr uint32_t kSched32None = 0xFFFFFFFFu;

struct GatherSchedule32 {
    int steps = 0;
    int64_t count_pad = 0;         // count rounded up to 32 (row stride of ent)
    std::vector<uint32_t> ent;     // ent[s * count_pad + c']
    std::vector<uint8_t> steps32;  // steps the warp of 32-column block k runs
};

// sign_filter: -1 every entry, 0 only the + entries, 1 only the - entries.
// bank_cap: 1 conflict-free steps; 2 at most two targets per bank pair in a
// step (a two-way conflict), which lets a step carry more lanes.
bool build_gather_schedule32(const SpinTable& t, const std::vector<uint32_t>& perm, const std::vector<uint32_t>& inv,
                             GatherSchedule32* g, std::string* err, int sign_filter = -1, int bank_cap = 1);

// The persistent Lanczos kernel's unit queue from a row queue rq for G CTAs:
// the rows past the last full wave (rq.size() mod G of them, the cheapest)
// each split into up to four column ranges.  An entry is a row, or
// row | part << 24 | log2(P) << 28 for part `part` of P: columns
// [part ch, min(dimDN, (part + 1) ch)) with ch = ceil(ceil(dimDN / P) / 32) 32,
// every part non-empty (P = 1, no split, when dimDN is too narrow).  At most
// rq.size() + 3 (G - 1) entries; rows below 2^24.
std::vector<uint32_t> unit_queue(const std::vector<uint32_t>& rq, int64_t dimDN, int G);

// Negative entries of each column of a schedule (count_pad values, idle
// lanes not counted).  Pass D adds v ^ m per step (m = -1 for a negative
// entry: v ^ -1 = -v - 1) and this count once per column.
std::vector<uint8_t> schedule_negcount(const GatherSchedule32& g);

// Pass D's schedule (two-pass matvec): the permuted schedule g as 16-bit
// words, step-major ([step][count_pad]), each the offset of the target in the
// window of its column's chunk, x[w0 .. w1) with w0 = (k chunk - bw) rounded
// down to 16 (at least 0) and w1 = min(count, (k+1) chunk + bw) rounded up to
// even, | sign << 15.  A window starts on a multiple of 16 columns, so an
// offset keeps its target's residue mod 16; the idle lanes of a half-warp
// step all read one zero slot zbase + z (a broadcast) at a residue z that no
// busy lane of that step uses, from 16 zero slots [zbase, zbase + 16) past
// every window.  False when a target lies outside its chunk's window, the
// chunk is not a multiple of 1024 columns, or the window needs 15 bits or more.
bool window_schedule16(const GatherSchedule32& g, int64_t count, int64_t chunk, int64_t bw, std::vector<uint16_t>* out,
                       int64_t* zbase);

// The [steps][cpad] window schedule rearranged lane-packed, [cpad / 32]
// [ceil(steps / 8)][32][8]: eight successive steps of a column in one
// 16-byte word, so that one load serves eight steps and a warp's load is
// one contiguous 512-byte segment.  Steps past the last are padded with the
// zero slot zbase (offset zbase, + sign).
std::vector<uint16_t> lane_packed16(const std::vector<uint16_t>& s16, int64_t cpad, int64_t steps, int64_t zbase);

// Build both layouts for one spin from a term list.  Returns ED_OK or an
// error (bad site, table overflow, complex term in a real operator when
// allow_complex is false).
ed_status build_spin(const SpinBasis& basis, const ed_term* terms, int n_terms,
                     bool allow_complex, SpinTable* table, SpinEll* ell,
                     std::string* err);

}  // namespace ed
