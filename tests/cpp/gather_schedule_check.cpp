// Host-only check of the down-term gather schedule (build_gather_schedule):
// for spin tables of several lattices, every entry of every row appears in
// the schedule exactly once (as an index of +x or -x, the rest of the steps
// reading zeros), no step of a 16-column group touches a bank pair twice, and
// the per-block step counts cover the entries; the same for the permuted
// two-pass schedules, the hop-count ordering of columns and the variants with
// two targets per bank pair and split signs.  Prints one line
// per case: "<name> count <n> max_len <L> steps <S> ok".
#include <cstdio>
#include <algorithm>
#include <cstdlib>
#include <map>
#include <string>
#include <vector>

#include "ed_tables.hpp"

using namespace ed;

// A permuted 32-bit schedule against its table: every entry (of the sign the
// filter keeps) exactly once, nothing past a block's step count, at most
// `cap` targets per bank pair in a step of a 16-column group.
static int check32(const char* name, const SpinTable& t, const std::vector<uint32_t>& perm,
                   const std::vector<uint32_t>& inv, const GatherSchedule32& g32, int cap, int sign_filter) {
    const int64_t cnt = t.count;
    for (int64_t c = 0; c < g32.count_pad; ++c) {
        std::map<int64_t, int> want, got;
        if (c < cnt) {
            const int64_t d = perm[c];
            for (int k = 0; k < t.len[d]; ++k) {
                const uint32_t e = t.ent[(size_t)k * cnt + d];
                if (sign_filter >= 0 && ((e & kSignBit) != 0) != (sign_filter == 1)) continue;
                const int64_t tc = (int64_t)inv[e & kColMask] + 1;
                ++want[(e & kSignBit) ? -tc : tc];
            }
        }
        for (int s = 0; s < g32.steps; ++s) {
            const uint32_t w = g32.ent[(size_t)s * g32.count_pad + c];
            if (w == kSched32None) continue;
            if (s >= g32.steps32[c / 32]) {
                std::printf("%s cap%d/%d entry beyond the block's steps\n", name, cap, sign_filter);
                return 1;
            }
            const int64_t tc = (int64_t)(w & 0x7FFFFFFFu) + 1;
            ++got[(w & 0x80000000u) ? -tc : tc];
        }
        if (want != got) {
            std::printf("%s cap%d/%d column %lld differs from the table\n", name, cap, sign_filter, (long long)c);
            return 1;
        }
    }
    for (int64_t g0 = 0; g0 < g32.count_pad; g0 += 16)
        for (int s = 0; s < g32.steps; ++s) {
            int use[16] = {0};
            for (int l = 0; l < 16; ++l) {
                const uint32_t w = g32.ent[(size_t)s * g32.count_pad + g0 + l];
                if (w == kSched32None) continue;
                if (++use[(w & 0x7FFFFFFFu) % 16] > cap) {
                    std::printf("%s cap%d/%d: bank pair used more than %d times in a step\n", name, cap, sign_filter,
                                cap);
                    return 1;
                }
            }
        }
    return 0;
}

static int check(const char* name, int n, int q, const std::vector<ed_term>& terms) {
    SpinBasis b;
    b.build(n, q);
    SpinTable t;
    std::string err;
    if (build_spin(b, terms.data(), (int)terms.size(), false, &t, nullptr, &err) != ED_OK) {
        std::printf("%s build_spin failed: %s\n", name, err.c_str());
        return 1;
    }
    GatherSchedule g;
    if (!build_gather_schedule(t, &g, &err)) {
        std::printf("%s schedule failed: %s\n", name, err.c_str());
        return 1;
    }
    const int64_t cnt = t.count, cp = g.count_pad, nb = g.neg_base, zb = 2 * g.neg_base;
    if (cp % 32 != 0 || cp < cnt || nb % 16 != 0 || nb < cnt || (int64_t)g.steps32.size() != cp / 32) {
        std::printf("%s bad padding\n", name);
        return 1;
    }
    for (int64_t d = 0; d < cp; ++d) {
        std::map<int64_t, int> want, got;  // +-(col + 1)
        if (d < cnt)
            for (int k = 0; k < t.len[d]; ++k) {
                const uint32_t e = t.ent[(size_t)k * cnt + d];
                const int64_t c = (int64_t)(e & kColMask) + 1;
                ++want[(e & kSignBit) ? -c : c];
            }
        const int nst = g.steps32[d / 32];
        for (int s = 0; s < nst; ++s) {
            const int64_t w = g.ent[(size_t)s * cp + d];
            if (w >= zb + 16 || (w >= cnt && w < nb) || (w >= nb + cnt && w < zb)) {
                std::printf("%s index out of the buffer (d %lld s %d)\n", name, (long long)d, s);
                return 1;
            }
            if (w >= zb) continue;
            ++got[w < nb ? w + 1 : -(w - nb + 1)];
        }
        if (want != got) {
            std::printf("%s row %lld: schedule entries differ from the table\n", name, (long long)d);
            return 1;
        }
    }
    for (int64_t g0 = 0; g0 < cp; g0 += 16) {
        const int nst = g.steps32[g0 / 32];
        for (int s = 0; s < nst; ++s) {
            int seen = 0;
            for (int l = 0; l < 16; ++l) {
                const int bit = 1 << (g.ent[(size_t)s * cp + g0 + l] % 16);
                if (seen & bit) {
                    std::printf("%s bank conflict at group %lld step %d\n", name, (long long)g0, s);
                    return 1;
                }
                seen |= bit;
            }
        }
    }
    // the reverse Cuthill-McKee order and the permuted 32-bit schedule
    std::vector<uint32_t> perm, inv;
    int64_t bw = 0;
    rcm_order(t, &perm, &inv, &bw);
    std::vector<char> hit(cnt, 0);
    for (int64_t c = 0; c < cnt; ++c) {
        if (perm[c] >= cnt || hit[perm[c]] || inv[perm[c]] != c) {
            std::printf("%s rcm order is not a permutation\n", name);
            return 1;
        }
        hit[perm[c]] = 1;
    }
    GatherSchedule32 g32;
    if (!build_gather_schedule32(t, perm, inv, &g32, &err)) {
        std::printf("%s schedule32 failed: %s\n", name, err.c_str());
        return 1;
    }
    int64_t bw_seen = 0;
    for (int64_t c = 0; c < g32.count_pad; ++c) {
        std::map<int64_t, int> want, got;
        if (c < cnt) {
            const int64_t d = perm[c];
            for (int k = 0; k < t.len[d]; ++k) {
                const uint32_t e = t.ent[(size_t)k * cnt + d];
                const int64_t tc = (int64_t)inv[e & kColMask] + 1;
                ++want[(e & kSignBit) ? -tc : tc];
                bw_seen = std::max<int64_t>(bw_seen, std::llabs((int64_t)inv[e & kColMask] - c));
            }
        }
        for (int s = 0; s < g32.steps; ++s) {
            const uint32_t w = g32.ent[(size_t)s * g32.count_pad + c];
            if (w == kSched32None) continue;
            if (s >= g32.steps32[c / 32]) {
                std::printf("%s schedule32 entry beyond the block's steps\n", name);
                return 1;
            }
            const int64_t tc = (int64_t)(w & 0x7FFFFFFFu) + 1;
            ++got[(w & 0x80000000u) ? -tc : tc];
        }
        if (want != got) {
            std::printf("%s schedule32 column %lld differs from the table\n", name, (long long)c);
            return 1;
        }
    }
    for (int64_t g0 = 0; g0 < g32.count_pad; g0 += 16)
        for (int s = 0; s < g32.steps; ++s) {
            int seen = 0;
            for (int l = 0; l < 16; ++l) {
                const uint32_t w = g32.ent[(size_t)s * g32.count_pad + g0 + l];
                if (w == kSched32None) continue;
                const int bit = 1 << ((w & 0x7FFFFFFFu) % 16);
                if (seen & bit) {
                    std::printf("%s schedule32 bank conflict\n", name);
                    return 1;
                }
                seen |= bit;
            }
        }
    if (bw_seen > bw) {
        std::printf("%s rcm bandwidth %lld below an entry's distance %lld\n", name, (long long)bw, (long long)bw_seen);
        return 1;
    }
    // columns ordered by hop count within 256-column blocks: still a
    // permutation, lengths non-increasing inside a block, bandwidth updated
    std::vector<uint32_t> perm2 = perm, inv2 = inv;
    int64_t bw2 = 0;
    sort_blocks_by_degree(t, 256, &perm2, &inv2, &bw2);
    std::vector<char> hit2(cnt, 0);
    int64_t bw2_seen = 0;
    for (int64_t c = 0; c < cnt; ++c) {
        if (perm2[c] >= cnt || hit2[perm2[c]] || inv2[perm2[c]] != c ||
            (c % 256 != 0 && t.len[perm2[c]] > t.len[perm2[c - 1]])) {
            std::printf("%s degree-sorted order broken at %lld\n", name, (long long)c);
            return 1;
        }
        hit2[perm2[c]] = 1;
        for (int k = 0; k < t.len[perm2[c]]; ++k)
            bw2_seen = std::max<int64_t>(bw2_seen,
                                         std::llabs((int64_t)inv2[t.ent[(size_t)k * cnt + perm2[c]] & kColMask] - c));
    }
    if (bw2_seen != bw2) {
        std::printf("%s sorted bandwidth %lld, entries reach %lld\n", name, (long long)bw2, (long long)bw2_seen);
        return 1;
    }
    // two targets per bank pair (pass D's schedule), and the sign-split
    // schedules, over the sorted order
    for (int sf = -1; sf <= 1; ++sf) {
        GatherSchedule32 gc;
        if (!build_gather_schedule32(t, perm2, inv2, &gc, &err, sf, 2)) {
            std::printf("%s cap2 schedule failed: %s\n", name, err.c_str());
            return 1;
        }
        if (check32(name, t, perm2, inv2, gc, 2, sf)) return 1;
    }
    // pass D's 16-bit window schedule (what k_mv_down reads): every entry of
    // every column once as window offset + window start, offsets inside the
    // window or on the zero slots, at most two targets per bank pair in a
    // half-warp step, idle lanes on one zero slot of a residue no busy lane
    // of the step uses
    {
        GatherSchedule32 gc;
        build_gather_schedule32(t, perm2, inv2, &gc, &err, -1, 2);
        // the per-column count of negative entries that k_mv_down adds once
        const std::vector<uint8_t> neg = schedule_negcount(gc);
        if ((int64_t)neg.size() != gc.count_pad) {
            std::printf("%s negative counts: size\n", name);
            return 1;
        }
        for (int64_t c = 0; c < gc.count_pad; ++c) {
            int want = 0;
            if (c < cnt)
                for (int k = 0; k < t.len[perm2[c]]; ++k)
                    want += (t.ent[(size_t)k * cnt + perm2[c]] & kSignBit) ? 1 : 0;
            if (neg[(size_t)c] != want) {
                std::printf("%s negative count of column %lld\n", name, (long long)c);
                return 1;
            }
        }
        for (int64_t chunk : {(int64_t)1024, (int64_t)2048}) {
            std::vector<uint16_t> s16;
            int64_t zb16 = 0;
            if (!window_schedule16(gc, cnt, chunk, bw2, &s16, &zb16)) {
                std::printf("%s window schedule (chunk %lld) refused\n", name, (long long)chunk);
                return 1;
            }
            const int64_t cpd = gc.count_pad, nst = std::max(gc.steps, 1);
            if ((int64_t)s16.size() != nst * cpd || zb16 % 16 != 0) {
                std::printf("%s window schedule shape\n", name);
                return 1;
            }
            // the lane-packed copy k_mv_down reads: word (c, st) at
            // (((c / 32) g8 + st / 8) 32 + c % 32) 8 + st % 8, the steps past
            // the last on the zero slot zb16
            const int64_t g8 = (nst + 7) / 8;
            const std::vector<uint16_t> bm = lane_packed16(s16, cpd, nst, zb16);
            if ((int64_t)bm.size() != (cpd / 32) * g8 * 256) {
                std::printf("%s lane-packed schedule size\n", name);
                return 1;
            }
            for (int64_t c = 0; c < cpd; ++c)
                for (int64_t st = 0; st < g8 * 8; ++st) {
                    const uint16_t want = st < nst ? s16[(size_t)(st * cpd + c)] : (uint16_t)zb16;
                    if (bm[(size_t)((((c / 32) * g8 + st / 8) * 32 + c % 32) * 8 + st % 8)] != want) {
                        std::printf("%s lane-packed schedule\n", name);
                        return 1;
                    }
                }
            for (int64_t c = 0; c < cpd; ++c) {
                const int64_t k = c / chunk;
                const int64_t w0 = std::max<int64_t>(0, k * chunk - bw2) & ~(int64_t)15;
                int64_t w1 = std::min<int64_t>(cnt, (k + 1) * chunk + bw2);
                w1 = (w1 + 1) & ~(int64_t)1;
                std::map<int64_t, int> want, got;
                if (c < cnt)
                    for (int kk = 0; kk < t.len[perm2[c]]; ++kk) {
                        const uint32_t e = t.ent[(size_t)kk * cnt + perm2[c]];
                        const int64_t tc = (int64_t)inv2[e & kColMask] + 1;
                        ++want[(e & kSignBit) ? -tc : tc];
                    }
                for (int st = 0; st < gc.steps32[c / 32]; ++st) {
                    const uint32_t w = s16[(size_t)st * cpd + c];
                    const int64_t off = w & 0x7FFF;
                    if (off >= zb16 + 16 || (off >= zb16 && (w & 0x8000))) {
                        std::printf("%s window offset out of the buffer\n", name);
                        return 1;
                    }
                    if (off >= zb16) continue;
                    if (off >= w1 - w0) {
                        std::printf("%s window offset past the copied window\n", name);
                        return 1;
                    }
                    const int64_t tc = off + w0 + 1;
                    ++got[(w & 0x8000) ? -tc : tc];
                }
                if (want != got) {
                    std::printf("%s window schedule column %lld differs from the table\n", name, (long long)c);
                    return 1;
                }
            }
            for (int64_t g0 = 0; g0 < cpd; g0 += 16)
                for (int st = 0; st < gc.steps32[g0 / 32]; ++st) {
                    int use[16] = {0};
                    int zres = -1;
                    for (int l = 0; l < 16; ++l) {
                        const int64_t off = s16[(size_t)st * cpd + g0 + l] & 0x7FFF;
                        if (off >= zb16) {
                            if (zres >= 0 && zres != (int)(off - zb16)) {
                                std::printf("%s idle lanes on different zero slots\n", name);
                                return 1;
                            }
                            zres = (int)(off - zb16);
                        } else if (++use[off % 16] > 2) {
                            std::printf("%s window schedule: more than two targets on a bank pair\n", name);
                            return 1;
                        }
                    }
                    if (zres >= 0 && use[zres]) {
                        std::printf("%s zero slot shares a bank pair with a target\n", name);
                        return 1;
                    }
                }
        }
    }
    // the row engine's schedule with two targets per bank pair
    GatherSchedule g2;
    if (!build_gather_schedule(t, &g2, &err, 2)) {
        std::printf("%s row-engine cap2 schedule failed: %s\n", name, err.c_str());
        return 1;
    }
    for (int64_t d = 0; d < cp; ++d) {
        std::map<int64_t, int> want, got;
        if (d < cnt)
            for (int k = 0; k < t.len[d]; ++k) {
                const uint32_t e = t.ent[(size_t)k * cnt + d];
                const int64_t c = (int64_t)(e & kColMask) + 1;
                ++want[(e & kSignBit) ? -c : c];
            }
        for (int s = 0; s < g2.steps32[d / 32]; ++s) {
            const int64_t w = g2.ent[(size_t)s * cp + d];
            if (w >= zb + 16) {
                std::printf("%s row-engine cap2 index out of the buffer\n", name);
                return 1;
            }
            if (w >= zb) continue;
            ++got[w < nb ? w + 1 : -(w - nb + 1)];
        }
        if (want != got) {
            std::printf("%s row-engine cap2 row %lld differs from the table\n", name, (long long)d);
            return 1;
        }
    }
    for (int64_t g0 = 0; g0 < cp; g0 += 16)
        for (int s = 0; s < g2.steps32[g0 / 32]; ++s) {
            std::map<int64_t, int> addr_of_res[16];
            for (int l = 0; l < 16; ++l) {
                const int64_t w = g2.ent[(size_t)s * cp + g0 + l];
                ++addr_of_res[w % 16][w];
            }
            for (int r = 0; r < 16; ++r)
                if (addr_of_res[r].size() > 2) {
                    std::printf("%s row-engine cap2: more than two addresses on a bank pair\n", name);
                    return 1;
                }
        }
    std::printf("%s count %lld max_len %d steps %d rcm_bandwidth %lld steps32 %d ok\n", name, (long long)cnt, t.max_len,
                g.steps, (long long)bw, g32.steps);
    return 0;
}

// The persistent kernel's unit queue: every (row, column) exactly once,
// ranges of a multiple of 32 columns and non-empty, at most 3 (G - 1) more
// entries than rows, whole rows first in the row queue's order.
static int check_units() {
    for (int64_t dimUP : {1, 5, 300, 924, 1000})
        for (int64_t dimDN : {1, 20, 31, 32, 33, 64, 70, 100, 495, 924, 1000})
            for (int G : {1, 7, 152, 304}) {
                std::vector<uint32_t> rq((size_t)dimUP);
                for (int64_t u = 0; u < dimUP; ++u) rq[(size_t)u] = (uint32_t)((u * 7919) % dimUP);
                const std::vector<uint32_t> uq = unit_queue(rq, dimDN, G);
                if (uq.size() > rq.size() + 3 * (size_t)(G - 1)) {
                    std::printf("units %lld x %lld G %d: %zu entries\n", (long long)dimUP, (long long)dimDN, G, uq.size());
                    return 1;
                }
                std::vector<int> hit((size_t)(dimUP * dimDN), 0);
                size_t whole = 0;
                for (size_t q = 0; q < uq.size(); ++q) {
                    const uint32_t e = uq[q], u = e & 0xFFFFFFu;
                    int64_t lo = 0, hi = dimDN;
                    if (e >> 24) {
                        const int64_t P = (int64_t)1 << (e >> 28), ch = ((dimDN + P - 1) / P + 31) / 32 * 32;
                        lo = (int64_t)((e >> 24) & 0xFu) * ch;
                        hi = std::min<int64_t>(dimDN, lo + ch);
                        if (lo % 32 != 0 || lo >= hi || ((e >> 24) & 0xFu) >= (uint32_t)P) {
                            std::printf("units %lld x %lld G %d: bad range\n", (long long)dimUP, (long long)dimDN, G);
                            return 1;
                        }
                    } else {
                        if (q != whole || rq[q] != u) {
                            std::printf("units %lld x %lld G %d: whole rows out of order\n", (long long)dimUP,
                                        (long long)dimDN, G);
                            return 1;
                        }
                        ++whole;
                    }
                    for (int64_t d = lo; d < hi; ++d) ++hit[(size_t)(u * dimDN + d)];
                }
                for (int h : hit)
                    if (h != 1) {
                        std::printf("units %lld x %lld G %d: coverage\n", (long long)dimUP, (long long)dimDN, G);
                        return 1;
                    }
            }
    std::printf("unit queue ok\n");
    return 0;
}

static std::vector<ed_term> bonds(const std::vector<std::pair<int, int>>& bs, double t) {
    std::vector<ed_term> v;
    for (auto& p : bs) v.push_back({ED_TERM_HOP, p.first, p.second, 0, t, 0.0});
    return v;
}

int main() {
    int fails = 0;
    {
        std::vector<std::pair<int, int>> bs;
        for (int i = 0; i < 14; ++i) bs.push_back({i, (i + 1) % 14});
        fails += check("chain14_q7", 14, 7, bonds(bs, -1.0));
    }
    {
        // 12 sites, every site on four bonds (ring plus second neighbours)
        std::vector<std::pair<int, int>> bs;
        for (int i = 0; i < 12; ++i) {
            bs.push_back({i, (i + 1) % 12});
            bs.push_back({i, (i + 2) % 12});
        }
        fails += check("ring12_nnn_q6", 12, 6, bonds(bs, -1.0));
        fails += check("ring12_nnn_q5", 12, 5, bonds(bs, 1.0));
    }
    {
        // 16 sites, random bonds (fixed LCG), 6 particles
        std::vector<std::pair<int, int>> bs;
        uint64_t x = 12345;
        for (int k = 0; k < 40; ++k) {
            x = x * 6364136223846793005ULL + 1442695040888963407ULL;
            const int i = (int)((x >> 33) % 16);
            x = x * 6364136223846793005ULL + 1442695040888963407ULL;
            const int j = (int)((x >> 33) % 16);
            if (i != j) bs.push_back({i, j});
        }
        fails += check("random16_q6", 16, 6, bonds(bs, 0.5));
    }
    {
        std::vector<std::pair<int, int>> bs = {{0, 1}};
        fails += check("dimer_q1", 2, 1, bonds(bs, -1.0));
    }
    fails += check_units();
    return fails ? 1 : 0;
}
