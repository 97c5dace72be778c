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

// Build both layouts for one spin from a term list.  Returns ED_OK or an
// error (bad site, table overflow, complex term in a real operator when
// allow_complex is false).
ed_status build_spin(const SpinBasis& basis, const ed_term* terms, int n_terms,
                     bool allow_complex, SpinTable* table, SpinEll* ell,
                     std::string* err);

}  // namespace ed
