// ed_tables.cpp — host-side basis (CNS rank/unrank) and per-spin tables.
#include "ed_tables.hpp"

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdlib>
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

namespace {

struct GroupEdge {
    int lane, bank;
    uint32_t word;
};

// Proper edge colouring of one 16-column group (lanes x nbanks banks,
// nbanks <= 32) with as many colours as the largest degree;
// pick[c * 16 + l] = edge of lane l in colour c or -1, *free_banks[c] = the
// banks no edge of colour c uses (bit mask).
bool colour_group(const std::vector<GroupEdge>& edges, int* Dout, std::vector<int>* pick,
                  std::vector<int>* free_banks, std::string* err, int nbanks = 16) {
    constexpr int kL = 16;
    const int kB = nbanks;
    int degL[kL] = {0}, degB[32] = {0};
    for (const GroupEdge& e : edges) {
        ++degL[e.lane];
        ++degB[e.bank];
    }
    int D = 0;
    for (int i = 0; i < kL; ++i) D = std::max(D, degL[i]);
    for (int i = 0; i < kB; ++i) D = std::max(D, degB[i]);
    std::vector<int> cL((size_t)kL * D, -1), cB((size_t)kB * D, -1), color(edges.size(), -1);
    auto setc = [&](int e, int c) {
        color[e] = c;
        cL[(size_t)edges[e].lane * D + c] = e;
        cB[(size_t)edges[e].bank * D + c] = e;
    };
    for (int e = 0; e < (int)edges.size(); ++e) {
        const int l = edges[e].lane, b = edges[e].bank;
        int a = 0, bb = 0;
        while (cL[(size_t)l * D + a] != -1) ++a;   // free at the lane
        while (cB[(size_t)b * D + bb] != -1) ++bb; // free at the bank
        if (cB[(size_t)b * D + a] != -1) {
            // swap colours a and bb along the alternating path that leaves
            // bank b on colour a; it cannot reach lane l (no a-edge there)
            std::vector<int> path;
            bool at_bank = true;
            int node = b, c = a;
            for (;;) {
                const int pe = at_bank ? cB[(size_t)node * D + c] : cL[(size_t)node * D + c];
                if (pe == -1) break;
                path.push_back(pe);
                node = at_bank ? edges[pe].lane : edges[pe].bank;
                at_bank = !at_bank;
                c = (c == a) ? bb : a;
            }
            for (int pe : path) {
                cL[(size_t)edges[pe].lane * D + color[pe]] = -1;
                cB[(size_t)edges[pe].bank * D + color[pe]] = -1;
            }
            for (int pe : path) setc(pe, color[pe] == a ? bb : a);
        }
        setc(e, a);
    }
    // verify: one entry per lane and per bank pair in every colour
    pick->assign((size_t)D * kL, -1);
    free_banks->assign(D, 0);
    for (int c = 0; c < D; ++c) {
        uint32_t seen = 0;
        for (int l = 0; l < kL; ++l) {
            const int e = cL[(size_t)l * D + c];
            if (e < 0) continue;
            const uint32_t bit = 1u << edges[e].bank;
            if (seen & bit || color[e] != c) {
                if (err) *err = "gather schedule: colouring check failed";
                return false;
            }
            seen |= bit;
            (*pick)[(size_t)c * kL + l] = e;
        }
        (*free_banks)[c] = (int)(~seen & (kB == 32 ? 0xFFFFFFFFu : ((1u << kB) - 1u)));
    }
    for (int e = 0; e < (int)edges.size(); ++e)
        if (color[e] < 0) {
            if (err) *err = "gather schedule: uncoloured entry";
            return false;
        }
    *Dout = D;
    return true;
}

}  // namespace

bool build_gather_schedule(const SpinTable& t, GatherSchedule* g, std::string* err, int bank_cap) {
    if (t.complex_coef || t.coef.size() > 1) {
        if (err) *err = "gather schedule: needs a real single-class table";
        return false;
    }
    if (t.count > kSchedMaxCount) {
        if (err) *err = "gather schedule: too many states";
        return false;
    }
    const int64_t count = t.count;
    const int64_t cpad = (count + 31) / 32 * 32;
    const int64_t neg_base = (count + 15) / 16 * 16;
    const int64_t zero_base = 2 * neg_base;
    const int64_t ngroups = cpad / 16;
    constexpr int kL = 16;
    std::vector<std::vector<uint16_t>> group_steps(ngroups);  // [group] -> words by (step*16 + lane)
    std::vector<int> group_deg(ngroups, 0);
    int smax = 0;
    for (int64_t gi = 0; gi < ngroups; ++gi) {
        std::vector<GroupEdge> edges;
        int seen_res[16] = {0};
        for (int l = 0; l < kL; ++l) {
            const int64_t d = gi * 16 + l;
            if (d >= count) continue;
            for (int k = 0; k < t.len[d]; ++k) {
                const uint32_t e = t.ent[(size_t)k * count + d];
                const uint32_t col = e & kColMask;
                // bank_cap 2: a residue's targets alternate between two
                // virtual banks, so a step holds at most two of them
                const int r = (int)(col % 16);
                const int bank = bank_cap == 2 ? 2 * r + (seen_res[r]++ & 1) : r;
                edges.push_back({l, bank, (uint32_t)(col + ((e & kSignBit) ? neg_base : 0))});
            }
        }
        int D = 0;
        std::vector<int> pick, freeb;
        if (!colour_group(edges, &D, &pick, &freeb, err, bank_cap == 2 ? 32 : 16)) return false;
        // idle lanes take the zeros of the bank pairs left free (a step with
        // k idle lanes has at most 16 - k busy lanes, so k residues are free)
        std::vector<uint16_t> words((size_t)D * kL, 0);
        for (int c = 0; c < D; ++c) {
            int fb = freeb[c];
            if (bank_cap == 2) {
                int fr = 0;
                for (int r = 0; r < 16; ++r)
                    if (((freeb[c] >> (2 * r)) & 3) == 3) fr |= 1 << r;
                fb = fr;
            }
            for (int l = 0; l < kL; ++l) {
                const int e = pick[(size_t)c * kL + l];
                if (e >= 0) {
                    words[(size_t)c * kL + l] = (uint16_t)edges[e].word;
                } else {
                    const int b = __builtin_ctz(fb);
                    fb &= fb - 1;
                    words[(size_t)c * kL + l] = (uint16_t)(zero_base + b);
                }
            }
        }
        group_steps[gi] = std::move(words);
        group_deg[gi] = D;
        smax = std::max(smax, D);
    }
    if (smax > 255) {
        if (err) *err = "gather schedule: more than 255 steps";
        return false;
    }
    g->steps = smax;
    g->count_pad = cpad;
    g->neg_base = neg_base;
    // steps a group does not use read the zero of the lane's own bank pair
    g->ent.assign((size_t)std::max(smax, 1) * cpad, 0);
    for (int s2 = 0; s2 < std::max(smax, 1); ++s2)
        for (int64_t d = 0; d < cpad; ++d) g->ent[(size_t)s2 * cpad + d] = (uint16_t)(zero_base + d % 16);
    g->steps32.assign(cpad / 32, 0);
    for (int64_t gi = 0; gi < ngroups; ++gi) {
        const int D = group_deg[gi];
        for (int c = 0; c < D; ++c)
            for (int l = 0; l < kL; ++l) g->ent[(size_t)c * cpad + gi * 16 + l] = group_steps[gi][(size_t)c * kL + l];
        uint8_t& st = g->steps32[gi / 2];
        st = (uint8_t)std::max<int>(st, D);
    }
    return true;
}

bool window_schedule16(const GatherSchedule32& g, int64_t count, int64_t chunk, int64_t bw, std::vector<uint16_t>* out,
                       int64_t* zbase_out) {
    if (chunk <= 0 || chunk % 1024 != 0) return false;  // whole 32-column blocks per chunk
    const int64_t zbase = (chunk + 2 * bw + 16 + 15) / 16 * 16;
    if (zbase + 16 > 32768) return false;
    const int64_t cpad = g.count_pad, nsteps = std::max(g.steps, 1);
    out->assign((size_t)nsteps * cpad, 0);
    for (int64_t cg = 0; cg < cpad; cg += 16) {
        const int64_t k = cg / chunk;  // a chunk is a multiple of 1024 columns: one chunk per group
        const int64_t w0 = std::max<int64_t>(0, k * chunk - bw) & ~(int64_t)15;
        int64_t w1 = std::min<int64_t>(count, (k + 1) * chunk + bw);
        w1 = (w1 + 1) & ~(int64_t)1;
        for (int64_t st = 0; st < nsteps; ++st) {
            auto word = [&](int l) { return st < g.steps ? g.ent[(size_t)st * cpad + cg + l] : kSched32None; };
            uint32_t used = 0;
            for (int l = 0; l < 16; ++l) {
                const uint32_t e = word(l);
                if (e == kSched32None) continue;
                const int64_t off = (int64_t)(e & 0x7FFFFFFFu) - w0;
                if (off < 0 || off >= w1 - w0) return false;  // not within the chunk's window
                used |= 1u << (off & 15);
                (*out)[(size_t)st * cpad + cg + l] = (uint16_t)(off | ((e & 0x80000000u) ? 0x8000 : 0));
            }
            int z = 0;
            while (z < 16 && ((used >> z) & 1u)) ++z;  // a step with an idle lane leaves a residue free
            for (int l = 0; l < 16; ++l)
                if (word(l) == kSched32None) (*out)[(size_t)st * cpad + cg + l] = (uint16_t)(zbase + (z & 15));
        }
    }
    *zbase_out = zbase;
    return true;
}

void rcm_order(const SpinTable& t, std::vector<uint32_t>* perm, std::vector<uint32_t>* inv, int64_t* bandwidth) {
    const int64_t n = t.count;
    std::vector<std::vector<uint32_t>> adj(n);
    for (int64_t a = 0; a < n; ++a)
        for (int k = 0; k < t.len[a]; ++k) {
            const uint32_t col = t.ent[(size_t)k * n + a] & kColMask;
            if ((int64_t)col != a) adj[a].push_back(col);
        }
    std::vector<int> deg(n);
    for (int64_t a = 0; a < n; ++a) {
        std::sort(adj[a].begin(), adj[a].end());
        adj[a].erase(std::unique(adj[a].begin(), adj[a].end()), adj[a].end());
        deg[a] = (int)adj[a].size();
    }
    std::vector<char> seen(n, 0);
    std::vector<uint32_t> order;
    order.reserve(n);
    // breadth-first levels from s; returns the last level's minimum-degree state
    auto bfs_far = [&](uint32_t s0) {
        std::vector<int> lvl(n, -1);
        std::vector<uint32_t> q{s0};
        lvl[s0] = 0;
        size_t h = 0;
        while (h < q.size()) {
            const uint32_t v = q[h++];
            for (uint32_t w : adj[v])
                if (lvl[w] < 0) {
                    lvl[w] = lvl[v] + 1;
                    q.push_back(w);
                }
        }
        const int last = lvl[q.back()];
        uint32_t best = q.back();
        for (uint32_t v : q)
            if (lvl[v] == last && deg[v] < deg[best]) best = v;
        return best;
    };
    for (int64_t s = 0; s < n; ++s) {
        if (seen[s]) continue;
        // the component's minimum-degree state, then two sweeps towards the periphery
        uint32_t start = (uint32_t)s;
        {
            std::vector<uint32_t> comp{(uint32_t)s};
            size_t h = 0;
            std::vector<char>& vis = seen;  // temporarily mark the component
            vis[s] = 2;
            while (h < comp.size()) {
                const uint32_t v = comp[h++];
                if (deg[v] < deg[start]) start = v;
                for (uint32_t w : adj[v])
                    if (!vis[w]) {
                        vis[w] = 2;
                        comp.push_back(w);
                    }
            }
            for (uint32_t v : comp) vis[v] = 0;
        }
        start = bfs_far(bfs_far(start));
        std::vector<uint32_t> q{start};
        seen[start] = 1;
        size_t h = 0;
        while (h < q.size()) {
            const uint32_t v = q[h++];
            std::vector<uint32_t> nb;
            for (uint32_t w : adj[v])
                if (!seen[w]) {
                    seen[w] = 1;
                    nb.push_back(w);
                }
            std::stable_sort(nb.begin(), nb.end(), [&](uint32_t x, uint32_t y) { return deg[x] < deg[y]; });
            q.insert(q.end(), nb.begin(), nb.end());
        }
        order.insert(order.end(), q.begin(), q.end());
    }
    std::reverse(order.begin(), order.end());
    perm->assign(order.begin(), order.end());
    inv->assign(n, 0);
    for (int64_t i = 0; i < n; ++i) (*inv)[(*perm)[i]] = (uint32_t)i;
    int64_t bw = 0;
    for (int64_t a = 0; a < n; ++a)
        for (uint32_t b : adj[a]) bw = std::max<int64_t>(bw, std::llabs((int64_t)(*inv)[a] - (int64_t)(*inv)[b]));
    *bandwidth = bw;
}

void sort_blocks_by_degree(const SpinTable& t, int block, std::vector<uint32_t>* perm, std::vector<uint32_t>* inv,
                           int64_t* bandwidth) {
    for (size_t s = 0; s < perm->size(); s += (size_t)block) {
        const size_t e = std::min(perm->size(), s + (size_t)block);
        std::stable_sort(perm->begin() + s, perm->begin() + e,
                         [&](uint32_t a, uint32_t b) { return t.len[a] > t.len[b]; });
    }
    for (size_t k = 0; k < perm->size(); ++k) (*inv)[(*perm)[k]] = (uint32_t)k;
    int64_t bw = 0;
    for (int64_t a = 0; a < t.count; ++a)
        for (int k = 0; k < t.len[a]; ++k)
            bw = std::max<int64_t>(bw, std::llabs((int64_t)(*inv)[a] - (int64_t)(*inv)[t.ent[(size_t)k * t.count + a] & kColMask]));
    *bandwidth = bw;
}

bool build_gather_schedule32(const SpinTable& t, const std::vector<uint32_t>& perm, const std::vector<uint32_t>& inv,
                             GatherSchedule32* g, std::string* err, int sign_filter, int bank_cap) {
    if (t.complex_coef || t.coef.size() > 1) {
        if (err) *err = "gather schedule: needs a real single-class table";
        return false;
    }
    const int64_t count = t.count;
    const int64_t cpad = (count + 31) / 32 * 32;
    const int64_t ngroups = cpad / 16;
    constexpr int kL = 16;
    std::vector<std::vector<uint32_t>> group_steps(ngroups);
    std::vector<int> group_deg(ngroups, 0);
    int smax = 0;
    for (int64_t gi = 0; gi < ngroups; ++gi) {
        std::vector<GroupEdge> edges;
        int seen_res[16] = {0};
        for (int l = 0; l < kL; ++l) {
            const int64_t c = gi * 16 + l;  // permuted column
            if (c >= count) continue;
            const int64_t d = perm[c];      // its state in table order
            for (int k = 0; k < t.len[d]; ++k) {
                const uint32_t e = t.ent[(size_t)k * count + d];
                if (sign_filter >= 0 && ((e & kSignBit) != 0) != (sign_filter == 1)) continue;
                const uint32_t tc = inv[e & kColMask];
                // bank_cap 2: the targets of a residue alternate between two
                // virtual banks, so a step holds at most two of them
                const int r = (int)(tc % 16);
                const int bank = bank_cap == 2 ? 2 * r + (seen_res[r]++ & 1) : r;
                edges.push_back({l, bank, tc | (e & kSignBit)});
            }
        }
        int D = 0;
        std::vector<int> pick, freeb;
        if (!colour_group(edges, &D, &pick, &freeb, err, bank_cap == 2 ? 32 : 16)) return false;
        std::vector<uint32_t> words((size_t)D * kL, kSched32None);
        for (int c = 0; c < D; ++c)
            for (int l = 0; l < kL; ++l) {
                const int e = pick[(size_t)c * kL + l];
                if (e >= 0) words[(size_t)c * kL + l] = edges[e].word;
            }
        group_steps[gi] = std::move(words);
        group_deg[gi] = D;
        smax = std::max(smax, D);
    }
    if (smax > 255) {
        if (err) *err = "gather schedule: more than 255 steps";
        return false;
    }
    g->steps = smax;
    g->count_pad = cpad;
    g->ent.assign((size_t)std::max(smax, 1) * cpad, kSched32None);
    g->steps32.assign(cpad / 32, 0);
    for (int64_t gi = 0; gi < ngroups; ++gi) {
        const int D = group_deg[gi];
        for (int c = 0; c < D; ++c)
            for (int l = 0; l < kL; ++l) g->ent[(size_t)c * cpad + gi * 16 + l] = group_steps[gi][(size_t)c * kL + l];
        uint8_t& st = g->steps32[gi / 2];
        st = (uint8_t)std::max<int>(st, D);
    }
    return true;
}

std::vector<uint32_t> unit_queue(const std::vector<uint32_t>& rq, int64_t dimDN, int G) {
    const size_t k = G > 0 ? rq.size() % (size_t)G : 0;
    // parts of a multiple of 32 columns, every one of them non-empty
    int lg = 2;
    while (lg > 0) {
        const int64_t P = (int64_t)1 << lg, ch = ((dimDN + P - 1) / P + 31) / 32 * 32;
        if ((P - 1) * ch < dimDN) break;
        --lg;
    }
    if (k == 0 || lg == 0) return rq;
    std::vector<uint32_t> q(rq.begin(), rq.end() - (std::ptrdiff_t)k);
    for (size_t i = rq.size() - k; i < rq.size(); ++i)
        for (uint32_t part = 0; part < (1u << lg); ++part) q.push_back(rq[i] | part << 24 | (uint32_t)lg << 28);
    return q;
}

std::vector<uint8_t> schedule_negcount(const GatherSchedule32& g) {
    std::vector<uint8_t> neg((size_t)g.count_pad, 0);
    for (int st = 0; st < g.steps; ++st)
        for (int64_t c = 0; c < g.count_pad; ++c) {
            const uint32_t w = g.ent[(size_t)st * g.count_pad + c];
            if (w != kSched32None && (w & kSignBit)) ++neg[(size_t)c];
        }
    return neg;
}

std::vector<uint16_t> lane_packed16(const std::vector<uint16_t>& s16, int64_t cpad, int64_t steps, int64_t zbase) {
    const int64_t groups = (steps + 7) / 8;
    std::vector<uint16_t> out((size_t)((cpad / 32) * groups * 256), (uint16_t)zbase);
    for (int64_t c = 0; c < cpad; ++c)
        for (int64_t st = 0; st < steps; ++st)
            out[(size_t)((((c / 32) * groups + st / 8) * 32 + c % 32) * 8 + st % 8)] = s16[(size_t)(st * cpad + c)];
    return out;
}

}  // namespace ed
