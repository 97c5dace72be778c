// ed_tables.cpp — host-side basis (CNS rank/unrank) and per-spin tables.
#include "ed_tables.hpp"

#include <algorithm>
#include <cmath>
#include <map>

namespace ed {

int64_t binom(int n, int k) {
    if (k < 0 || n < 0 || k > n) return 0;
    if (k > n - k) k = n - k;
    unsigned __int128 r = 1;  // r * (n-k+i) can exceed 2^63 before the exact division
    for (int i = 1; i <= k; ++i) r = r * (unsigned)(n - k + i) / (unsigned)i;
    return (int64_t)r;
}

int popcount64(uint64_t v) { return __builtin_popcountll(v); }

int count_between(uint64_t word, int i, int j) {
    int lo = i < j ? i : j, hi = i < j ? j : i;
    if (hi - lo <= 1) return 0;
    uint64_t mask = ((1ULL << (hi - lo - 1)) - 1ULL) << (lo + 1);
    return popcount64(word & mask);
}

void SpinBasis::build(int n, int q) {
    n_sites = n;
    n_part = q;
    count = binom(n, q);
    const int kdim = q + 2;
    binom_tab.assign((size_t)(n + 1) * kdim, 0);
    for (int p = 0; p <= n; ++p)
        for (int k = 0; k < kdim; ++k) binom_tab[(size_t)p * kdim + k] = binom(p, k);
    state.resize(count);
    // Ascending-integer enumeration of popcount-q words: Gosper's next
    // combination step visits them in increasing order.
    if (q == 0) {
        if (count) state[0] = 0;
        return;
    }
    uint64_t w = (q >= 64) ? ~0ULL : ((1ULL << q) - 1ULL);
    for (int64_t r = 0; r < count; ++r) {
        state[r] = w;
        uint64_t c = w & (~w + 1ULL);
        uint64_t t = w + c;
        w = (((t ^ w) >> 2) / c) | t;
    }
}

// rank = sum over the set bits (p_0 < p_1 < ...) of C(p_k, k+1)
int64_t SpinBasis::rank(uint64_t word) const {
    if (popcount64(word) != n_part) return -1;
    if (n_sites < 64 && (word >> n_sites)) return -1;
    const int kdim = n_part + 2;
    int64_t r = 0;
    int k = 0;
    while (word) {
        int p = __builtin_ctzll(word);
        r += binom_tab[(size_t)p * kdim + (k + 1)];
        ++k;
        word &= word - 1;
    }
    return r;
}

uint64_t SpinBasis::unrank(int64_t r) const {
    const int kdim = n_part + 2;
    uint64_t w = 0;
    int p = n_sites - 1;
    for (int k = n_part; k >= 1; --k) {
        // largest p with C(p, k) <= r
        while (p >= 0 && binom_tab[(size_t)p * kdim + k] > r) --p;
        w |= 1ULL << p;
        r -= binom_tab[(size_t)p * kdim + k];
        --p;
    }
    return w;
}

namespace {

struct RowEntry {
    int64_t col;
    std::complex<double> value;
};

// Canonical class key of a coefficient up to sign.
std::complex<double> class_rep(std::complex<double> v, bool* negative) {
    bool neg = (v.real() < 0.0) || (v.real() == 0.0 && v.imag() < 0.0);
    *negative = neg;
    return neg ? -v : v;
}

struct CplxLess {
    bool operator()(const std::complex<double>& a, const std::complex<double>& b) const {
        if (a.real() != b.real()) return a.real() < b.real();
        return a.imag() < b.imag();
    }
};

}  // namespace

ed_status build_spin(const SpinBasis& basis, const ed_term* terms, int n_terms,
                     bool allow_complex, SpinTable* table, SpinEll* ell, std::string* err) {
    const int N = basis.n_sites;
    const int64_t count = basis.count;
    if (count > (int64_t)kColMask + 1) {
        if (err) *err = "spin basis larger than 2^24 states";
        return ED_ERR_RANGE;
    }
    for (int t = 0; t < n_terms; ++t) {
        const ed_term& tm = terms[t];
        bool two_site = tm.kind != ED_TERM_DENSITY;
        if (tm.kind < 0 || tm.kind > ED_TERM_PEIERLS || tm.i < 0 || tm.i >= N ||
            (two_site && (tm.j < 0 || tm.j >= N || tm.j == tm.i))) {
            if (err) *err = "bad term " + std::to_string(t);
            return ED_ERR_ARG;
        }
        if (tm.kind == ED_TERM_PEIERLS && !allow_complex) {
            if (err) *err = "Peierls term in a real operator";
            return ED_ERR_ARG;
        }
    }

    // Per-row entry lists in stacking order (the order H_TBq fills slots):
    // terms in call order, within a term rows ascending, one entry per row.
    std::vector<std::vector<RowEntry>> rows(count);
    for (int t = 0; t < n_terms; ++t) {
        const ed_term& tm = terms[t];
        for (int64_t a = 0; a < count; ++a) {
            uint64_t n = basis.state[a];
            if (tm.kind == ED_TERM_DENSITY) {
                if ((n >> tm.i) & 1ULL) rows[a].push_back({a, std::complex<double>(tm.value, 0.0)});
                continue;
            }
            int oi = (int)((n >> tm.i) & 1ULL), oj = (int)((n >> tm.j) & 1ULL);
            if (oi == oj) continue;
            uint64_t l = n ^ ((1ULL << tm.i) | (1ULL << tm.j));
            int64_t b = basis.rank(l);
            double sign = (count_between(n, tm.i, tm.j) & 1) ? -1.0 : 1.0;
            std::complex<double> v;
            if (tm.kind == ED_TERM_HOP) {
                v = sign * tm.value;
            } else if (tm.kind == ED_TERM_CURRENT) {
                v = (oi == 0 && oj == 1) ? sign * tm.value : sign * (-tm.value);
            } else {  // PEIERLS: row state n is reached from column state l.
                // Row has the particle at j (oj == 1): it moved i -> j, phase +phi.
                double ph = (oj == 1) ? tm.phase : -tm.phase;
                v = sign * tm.value * std::complex<double>(std::cos(ph), std::sin(ph));
            }
            rows[a].push_back({b, v});
        }
    }

    // ---- reference ELL layout (real values only) --------------------------
    if (ell) {
        ell->count = count;
        ell->nslots = 10 * basis.n_part + 1;
        ell->ax.assign((size_t)ell->nslots * count, 0.0);
        ell->aj.assign((size_t)ell->nslots * count, 0);
        ell->overflow = false;
        for (int64_t a = 0; a < count; ++a) {
            for (const RowEntry& e : rows[a]) {
                bool placed = false;
                for (int s = 0; s < ell->nslots; ++s) {
                    size_t idx = (size_t)s * count + a;
                    if (ell->ax[idx] == 0.0) {
                        ell->ax[idx] += e.value.real();
                        ell->aj[idx] = e.col;
                        placed = true;
                        break;
                    }
                }
                if (!placed) ell->overflow = true;
            }
        }
    }

    if (!table) return (ell && ell->overflow) ? ED_ERR_TABLE : ED_OK;

    // ---- device layout -------------------------------------------------------
    std::map<std::complex<double>, int, CplxLess> cls;
    table->count = count;
    table->diag_re.assign(count, 0.0);
    table->diag_im.assign(count, 0.0);
    table->coef.clear();
    table->nnz = 0;
    table->max_row_abs = 0.0;
    table->max_diag_abs = 0.0;
    table->complex_coef = false;
    std::vector<std::vector<uint32_t>> packed(count);
    int max_len = 0;
    for (int64_t a = 0; a < count; ++a) {
        double row_abs = 0.0;
        std::vector<std::pair<int, uint32_t>> tmp;
        for (const RowEntry& e : rows[a]) {
            if (e.col == a) {  // diagonal (Make_N): fold
                table->diag_re[a] += e.value.real();
                table->diag_im[a] += e.value.imag();
                continue;
            }
            if (e.value == std::complex<double>(0.0, 0.0)) continue;
            bool neg = false;
            std::complex<double> rep = class_rep(e.value, &neg);
            auto it = cls.find(rep);
            int c;
            if (it == cls.end()) {
                c = (int)cls.size();
                if (c >= kMaxClasses) {
                    if (err) *err = "more than 64 distinct hopping magnitudes in one spin table";
                    return ED_ERR_RANGE;
                }
                cls.emplace(rep, c);
                table->coef.push_back(rep);
                if (rep.imag() != 0.0) table->complex_coef = true;
            } else {
                c = it->second;
            }
            uint32_t w = (uint32_t)e.col | ((uint32_t)c << kClassShift) | (neg ? kSignBit : 0u);
            tmp.push_back({c, w});
            row_abs += std::abs(e.value);
        }
        // order within a row: by class, positive entries before negative
        // ones (the sums are exact integers, so the order is free)
        std::stable_sort(tmp.begin(), tmp.end(),
                         [](const std::pair<int, uint32_t>& x, const std::pair<int, uint32_t>& y) {
                             if (x.first != y.first) return x.first < y.first;
                             return (x.second & kSignBit) < (y.second & kSignBit);
                         });
        for (auto& p : tmp) packed[a].push_back(p.second);
        max_len = std::max(max_len, (int)packed[a].size());
        table->nnz += (int64_t)packed[a].size();
        table->max_row_abs = std::max(table->max_row_abs, row_abs);
        table->max_diag_abs = std::max(table->max_diag_abs, std::abs(std::complex<double>(table->diag_re[a], table->diag_im[a])));
    }
    if (max_len > 255) {
        if (err) *err = "row with more than 255 off-diagonal entries";
        return ED_ERR_RANGE;
    }
    table->max_len = max_len;
    table->ent.assign((size_t)std::max(max_len, 1) * count, 0u);
    table->len.assign(count, 0);
    table->npos.assign(count, 0);
    for (int64_t a = 0; a < count; ++a) {
        table->len[a] = (uint8_t)packed[a].size();
        int np = 0;
        for (size_t s = 0; s < packed[a].size(); ++s) {
            table->ent[s * count + a] = packed[a][s];
            if (!(packed[a][s] & kSignBit)) ++np;
        }
        table->npos[a] = (uint8_t)np;
    }
    if (ell && ell->overflow) return ED_ERR_TABLE;
    return ED_OK;
}

}  // namespace ed
