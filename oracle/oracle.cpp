/*
 * oracle.cpp -- CPU restatement of immunodbscan's DBSCAN clone-collapsing
 * path (rules S1-S7), C++17 + OpenMP.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  PARITY UNPINNED: the reference has
 * no tests or fixtures and its CUDA path cannot run here; known-answer tests
 * under tests/ pin this restatement instead.
 *
 * The structure deliberately follows the reference, not the GPU design of this
 * project: every pair of uniques of a repertoire is visited (the reference's
 * all-pairs grids, cuda/PSDBSCAN.hcu:1115-1178 and :1200-1257), Levenshtein is
 * the full O(m*n) DP with no band and no early exit (cuda/PSDBSCAN.hcu:246-290),
 * and a Hamming test precedes it for equal lengths (cuda/PSDBSCAN.hcu:801-811).
 * That makes it both the parity checker and an honest CPU baseline.
 */
#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <map>
#include <numeric>
#include <string>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct StrCol {
    const char *data;
    const int64_t *off;
    const char *fallback;   // used when data == nullptr
    const char *ptr(uint32_t i) const { return data ? data + off[i] : fallback; }
    uint32_t len(uint32_t i) const {
        return data ? (uint32_t)(off[i + 1] - off[i]) : (uint32_t)std::strlen(fallback);
    }
};

// S1 -- bit g is set iff gene name g occurs as a byte-exact substring of the
// call string (cuda/BitsetVector.inl:118-176: sliding comparison, bit set by
// atomicOr at :112-115).  An empty name launches a zero-thread block in the
// reference and never sets a bit; a name longer than the call never matches
// (loop guard at :151).
bool occurs(const char *hay, uint32_t hl, const char *needle, uint32_t nl) {
    if (nl == 0 || nl > hl) return false;
    for (uint32_t p = 0; p + nl <= hl; ++p)
        if (std::memcmp(hay + p, needle, nl) == 0) return true;
    return false;
}

void build_bitsets(uint32_t n, const StrCol &calls, const StrCol &genes, uint32_t n_genes,
                   std::vector<uint32_t> &words, uint32_t &width) {
    // int32 words, width = ceil(n_genes/32) (cuda/BitsetVector.inl:34)
    width = (n_genes + 31) / 32;
    words.assign((size_t)n * width, 0u);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        const char *c = calls.ptr((uint32_t)i);
        uint32_t cl = calls.len((uint32_t)i);
        for (uint32_t g = 0; g < n_genes; ++g)
            if (occurs(c, cl, genes.ptr(g), genes.len(g)))
                words[(size_t)i * width + g / 32] |= 1u << (g % 32);
    }
}

}  // namespace

extern "C" int32_t ora_eps(uint32_t lx, uint32_t ly, float threshold, int32_t abs_eps) {
    // S2 -- (int)truncf((float)max(Lx,Ly) * threshold) in single precision
    // (cuda/SpecialFunctors.hcu:257-261, instantiated with <false> at
    // cuda/PSDBSCAN.hcu:1119,1204 for both distance modes).  The absolute eps
    // is this project's added key; when both are set the smaller one wins.
    bool rel = !std::isnan(threshold);
    bool ab = abs_eps >= 0;
    if (!rel && !ab) return INT32_MIN;
    int32_t e = INT32_MAX;
    if (rel) {
        volatile float m = (float)std::max(lx, ly);   // keep the product in float
        volatile float prod = m * threshold;
        float t = truncf(prod);
        e = (int32_t)t;
    }
    if (ab) e = std::min(e, abs_eps);
    return e;
}

extern "C" int32_t ora_levenshtein(const char *a, uint32_t la, const char *b, uint32_t lb) {
    // Unit-cost edit distance on bytes, full DP, no band, no early exit
    // (cuda/PSDBSCAN.hcu:246-290 evaluates every anti-diagonal).
    std::vector<int32_t> prev(lb + 1), cur(lb + 1);
    for (uint32_t j = 0; j <= lb; ++j) prev[j] = (int32_t)j;
    for (uint32_t i = 1; i <= la; ++i) {
        cur[0] = (int32_t)i;
        for (uint32_t j = 1; j <= lb; ++j) {
            int32_t sub = prev[j - 1] + (a[i - 1] != b[j - 1]);
            int32_t del = prev[j] + 1, ins = cur[j - 1] + 1;
            cur[j] = std::min(sub, std::min(del, ins));
        }
        std::swap(prev, cur);
    }
    return prev[lb];
}

extern "C" int32_t ora_levenshtein_within(const char *a, uint32_t la, const char *b, uint32_t lb,
                                          int32_t e) {
    // Ukkonen's cutoff: a cell (i, j) with |i - j| > e holds more than e, so
    // only the band |i - j| <= e is computed (cells outside read as e + 1), and
    // once every cell of a row exceeds e the distance does.
    if (e < 0) return 0;
    if ((int64_t)la - (int64_t)lb > e || (int64_t)lb - (int64_t)la > e) return 0;
    const int32_t big = e + 1;
    thread_local std::vector<int32_t> prev, cur;
    prev.assign(lb + 2, big);
    cur.assign(lb + 2, big);
    for (uint32_t j = 0; j <= lb && (int32_t)j <= e; ++j) prev[j] = (int32_t)j;
    for (uint32_t i = 1; i <= la; ++i) {
        const int64_t lo = std::max<int64_t>(1, (int64_t)i - e);
        const int64_t hi = std::min<int64_t>(lb, (int64_t)i + e);
        cur[lo - 1] = (lo == 1 && (int32_t)i <= e) ? (int32_t)i : big;
        int32_t rowmin = cur[lo - 1];
        for (int64_t j = lo; j <= hi; ++j) {
            int32_t v = prev[j - 1] + (a[i - 1] != b[j - 1]);
            v = std::min(v, prev[j] + 1);
            v = std::min(v, cur[j - 1] + 1);
            cur[j] = std::min(v, big);
            rowmin = std::min(rowmin, cur[j]);
        }
        if (hi + 1 <= (int64_t)lb) cur[hi + 1] = big;
        if (rowmin > e) return 0;
        std::swap(prev, cur);
    }
    return prev[lb] <= e;
}

extern "C" int32_t ora_hamming(const char *a, const char *b, uint32_t len) {
    // Count of differing positions (cuda/PSDBSCAN.hcu:410-428).
    int32_t d = 0;
    for (uint32_t k = 0; k < len; ++k) d += a[k] != b[k];
    return d;
}

extern "C" int ora_gene_bitsets(uint32_t n_rows, const char *c_data, const int64_t *c_off,
                                const char *g_data, const int64_t *g_off, uint32_t n_genes,
                                uint32_t *words_out) {
    StrCol calls{c_data, c_off, "V"}, genes{g_data, g_off, "V"};
    std::vector<uint32_t> w;
    uint32_t width;
    build_bitsets(n_rows, calls, genes, n_genes, w, width);
    std::memcpy(words_out, w.data(), w.size() * sizeof(uint32_t));
    return 0;
}

namespace {

struct Rows {
    uint32_t n;
    StrCol seq;
    std::vector<uint32_t> vb, jb;   // int32 words as the reference stores them
    uint32_t vw, jw;
    float threshold;
    int32_t abs_eps;

    uint32_t len(uint32_t i) const { return seq.len(i); }
    const char *s(uint32_t i) const { return seq.ptr(i); }
    // compare_bitset_values: OR over words of (a & b), required non-zero for V
    // AND for J (cuda/BitsetVector.inl:214-237, :298-314).
    bool overlap(uint32_t x, uint32_t y) const {
        uint32_t v = 0, j = 0;
        for (uint32_t k = 0; k < vw; ++k) v |= vb[(size_t)x * vw + k] & vb[(size_t)y * vw + k];
        for (uint32_t k = 0; k < jw; ++k) j |= jb[(size_t)x * jw + k] & jb[(size_t)y * jw + k];
        return v != 0 && j != 0;
    }
    // singlet_bitset_values_equal: every word equal (cuda/BitsetVector.inl:340-357).
    bool bits_equal(uint32_t x, uint32_t y) const {
        for (uint32_t k = 0; k < vw; ++k)
            if (vb[(size_t)x * vw + k] != vb[(size_t)y * vw + k]) return false;
        for (uint32_t k = 0; k < jw; ++k)
            if (jb[(size_t)x * jw + k] != jb[(size_t)y * jw + k]) return false;
        return true;
    }
    // eps per length pair, tabulated up to the longest sequence
    uint32_t max_len = 0;
    std::vector<int32_t> eps_tab;
    void tabulate_eps() {
        for (uint32_t i = 0; i < n; ++i) max_len = std::max(max_len, len(i));
        eps_tab.resize((size_t)(max_len + 1) * (max_len + 1));
        for (uint32_t a = 0; a <= max_len; ++a)
            for (uint32_t b = 0; b <= max_len; ++b)
                eps_tab[(size_t)a * (max_len + 1) + b] = ora_eps(a, b, threshold, abs_eps);
    }
    int32_t eps(uint32_t a, uint32_t b) const { return eps_tab[(size_t)a * (max_len + 1) + b]; }
};

// S4 -- neighbour predicate on two uniques (x != y).
//  Levenshtein mode (cuda/PSDBSCAN.hcu:776-812): V and J overlap, |Lx-Ly| <= eps,
//  then Hamming <= eps if the lengths agree, else (or if that fails) the full
//  Levenshtein DP <= eps.
//  Hamming mode (cuda/PSDBSCAN.hcu:608-651): equal lengths, V and J overlap, and
//  a Hamming count that stops once it exceeds eps.
bool neighbours(const Rows &R, uint32_t x, uint32_t y, bool hamming_mode, bool indexed,
                bool &admissible) {
    uint32_t lx = R.len(x), ly = R.len(y);
    int32_t e = R.eps(lx, ly);
    admissible = false;
    if (hamming_mode) {
        if (lx != ly) return false;
        if (!R.overlap(x, y)) return false;
        if (e < 0) return false;
        admissible = true;
        const char *a = R.s(x), *b = R.s(y);
        int32_t d = 0;
        for (uint32_t k = 0; k < lx; ++k)
            if (a[k] != b[k] && ++d > e) return false;
        return true;
    }
    int32_t gap = lx > ly ? (int32_t)(lx - ly) : (int32_t)(ly - lx);
    if (!R.overlap(x, y) || gap > e) return false;
    admissible = true;
    if (lx == ly && ora_hamming(R.s(x), R.s(y), lx) <= e) return true;
    if (indexed) return ora_levenshtein_within(R.s(x), lx, R.s(y), ly, e) != 0;
    return ora_levenshtein(R.s(x), lx, R.s(y), ly) <= e;
}

struct DSU {   // union-find with link-to-min: the root of a set is its minimum index
    std::vector<uint32_t> p;
    explicit DSU(size_t n) : p(n) { std::iota(p.begin(), p.end(), 0u); }
    uint32_t find(uint32_t x) {
        while (p[x] != x) { p[x] = p[p[x]]; x = p[x]; }
        return x;
    }
    void unite(uint32_t a, uint32_t b) {
        a = find(a); b = find(b);
        if (a == b) return;
        if (a < b) p[b] = a; else p[a] = b;
    }
};

}  // namespace

extern "C" int ora_cluster(uint32_t n_rows,
                           const char *v_data, const int64_t *v_off,
                           const char *j_data, const int64_t *j_off,
                           const char *s_data, const int64_t *s_off,
                           const char *vg_data, const int64_t *vg_off, uint32_t n_vg,
                           const char *jg_data, const int64_t *jg_off, uint32_t n_jg,
                           uint32_t n_rep, const uint32_t *rep_off,
                           const ora_params *prm, ora_result *out) {
    if (!prm || !out) return 1;
#ifdef _OPENMP
    if (prm->n_threads > 0) omp_set_num_threads(prm->n_threads);
#endif
    // Missing gene columns: every row "V" against ["V"] (cpp/TableHolder.hpp:293-296,
    // :311-314); missing sequence column: every row "Gene" (:326-328).
    Rows R;
    R.n = n_rows;
    R.seq = StrCol{s_data, s_off, "Gene"};
    R.threshold = prm->threshold;
    R.abs_eps = prm->abs_eps;
    {
        StrCol vc{v_data, v_off, "V"}, vg{v_data ? vg_data : nullptr, vg_off, "V"};
        build_bitsets(n_rows, vc, vg, v_data ? n_vg : 1u, R.vb, R.vw);
        StrCol jc{j_data, j_off, "V"}, jg{j_data ? jg_data : nullptr, jg_off, "V"};
        build_bitsets(n_rows, jc, jg, j_data ? n_jg : 1u, R.jb, R.jw);
    }
    R.tabulate_eps();
    const bool indexed = prm->indexed != 0;
    int32_t max_gap = 0;   // the largest eps of any length pair bounds an admissible gap
    for (int32_t v : R.eps_tab) max_gap = std::max(max_gap, v);
    std::vector<uint32_t> roff;
    if (rep_off && n_rep > 0) roff.assign(rep_off, rep_off + n_rep + 1);
    else roff = {0u, n_rows};
    const uint32_t nrep = (uint32_t)roff.size() - 1;
    const bool ham = prm->use_hamming != 0;
    const int K = std::max(prm->max_candidates, 0);

    // S3 -- exact duplicates: equal length, equal V and J bitsets and equal
    // bytes (the 32-bit std::hash at cuda/StringOperations.hcu:94-96 is only a
    // prefilter and cannot change the result).  union_a_and_b links the larger
    // index to the smaller one (cuda/PSDBSCAN.hcu:76-107), so the representative
    // is the minimum row index of the class; copies[rep] = class size and
    // copies[dup] = 0 (cuda/PSDBSCAN.hcu:1074-1085).
    std::vector<uint32_t> rep(n_rows), copies(n_rows, 0u);
    for (uint32_t r = 0; r < nrep; ++r) {
        std::unordered_map<std::string, uint32_t> first;
        first.reserve((size_t)(roff[r + 1] - roff[r]) * 2 + 1);
        for (uint32_t i = roff[r]; i < roff[r + 1]; ++i) {
            std::string key;
            uint32_t L = R.len(i);
            key.append(reinterpret_cast<const char *>(&L), 4);
            key.append(reinterpret_cast<const char *>(&R.vb[(size_t)i * R.vw]), R.vw * 4);
            key.append(reinterpret_cast<const char *>(&R.jb[(size_t)i * R.jw]), R.jw * 4);
            key.append(R.s(i), L);
            auto it = first.emplace(key, i).first;
            rep[i] = it->second;   // rows are visited in ascending order
            copies[rep[i]] += 1;
        }
    }
    // uniques = ascending indices with copies != 0 (cuda/PSDBSCAN.hcu:1102-1111)
    std::vector<std::vector<uint32_t>> uniq(nrep);
    uint32_t n_uniques = 0;
    for (uint32_t r = 0; r < nrep; ++r)
        for (uint32_t i = roff[r]; i < roff[r + 1]; ++i)
            if (copies[i]) { uniq[r].push_back(i); ++n_uniques; }

    // S4 + S5 -- all pairs of uniques; count[x] starts at copies[x]
    // (cuda/PSDBSCAN.hcu:1099) and each neighbour pair adds the other side's
    // copies to both sides (:824-826, :648-650).
    std::vector<std::atomic<uint64_t>> count(n_rows);
    for (uint32_t i = 0; i < n_rows; ++i) count[i].store(copies[i], std::memory_order_relaxed);
    std::vector<std::vector<std::pair<uint32_t, uint32_t>>> nbr_lists;
    uint64_t adm_total = 0, nbr_total = 0, all_total = 0;
    for (uint32_t r = 0; r < nrep; ++r) {
        const std::vector<uint32_t> &U = uniq[r];
        const int64_t nu = (int64_t)U.size();
        all_total += (uint64_t)nu * (uint64_t)(nu > 0 ? nu - 1 : 0) / 2;
        int nthr = 1;
#ifdef _OPENMP
        nthr = omp_get_max_threads();
#endif
        std::vector<std::vector<std::pair<uint32_t, uint32_t>>> local(nthr);
        uint64_t adm = 0;
        // indexed mode: uniques in (length, row) order, and each one is paired
        // with the later ones up to the largest admissible length gap (equal
        // lengths only in Hamming mode); the full mode pairs every two uniques
        std::vector<uint32_t> V(U);
        if (indexed)
            std::stable_sort(V.begin(), V.end(),
                             [&](uint32_t p, uint32_t q) { return R.len(p) < R.len(q); });
        const uint32_t gap = ham ? 0u : (uint32_t)max_gap;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : adm)
        for (int64_t a = 0; a < nu; ++a) {
            int t = 0;
#ifdef _OPENMP
            t = omp_get_thread_num();
#endif
            uint32_t x = V[a];
            const uint32_t lx = R.len(x);
            for (int64_t b = a + 1; b < nu; ++b) {
                uint32_t y = V[b];
                if (indexed && R.len(y) > lx + gap) break;
                bool is_adm;
                if (neighbours(R, x, y, ham, indexed, is_adm)) {
                    local[t].emplace_back(x, y);
                    count[x].fetch_add(copies[y], std::memory_order_relaxed);
                    count[y].fetch_add(copies[x], std::memory_order_relaxed);
                }
                adm += is_adm;
            }
        }
        adm_total += adm;
        for (auto &l : local) { nbr_total += l.size(); nbr_lists.push_back(std::move(l)); }
    }

    // core = count >= minPts (cuda/PSDBSCAN.hcu:1180).  Duplicates keep count 0
    // and are core only when minPts == 0.
    std::vector<uint8_t> core(n_rows);
    uint32_t n_cores = 0;
    for (uint32_t i = 0; i < n_rows; ++i) {
        core[i] = count[i].load() >= (uint64_t)prm->min_pts;
        if (core[i] && copies[i]) ++n_cores;
    }

    // S6 -- core-core neighbour pairs are merged (union_a_and_b, link to min);
    // a non-core unique is claimed by a core neighbour (first-wins atomicCAS at
    // cuda/PSDBSCAN.hcu:113-122, racy).  Deterministic rule used here: the
    // minimum-index core neighbour.  All core neighbours' clusters are recorded
    // as the admissible set for the reference's race.
    DSU dsu(n_rows);
    std::vector<uint32_t> border_min(n_rows, UINT32_MAX);
    std::vector<std::vector<uint32_t>> core_nbrs(K > 0 ? n_rows : 0);
    for (auto &l : nbr_lists)
        for (auto &e : l) {
            uint32_t x = e.first, y = e.second;
            bool cx = core[x] && copies[x], cy = core[y] && copies[y];
            if (cx && cy) dsu.unite(x, y);
            if (cx && !cy) { border_min[y] = std::min(border_min[y], x); if (K) core_nbrs[y].push_back(x); }
            if (cy && !cx) { border_min[x] = std::min(border_min[x], y); if (K) core_nbrs[x].push_back(y); }
        }

    // S7 -- root of every core component is its minimum core index; labels are
    // 1 + rank of the root among the repertoire's core roots in ascending order,
    // noise = 0 (cuda/PSDBSCAN.hcu:1263-1294).
    std::vector<uint32_t> label_of_root(n_rows, 0u);
    uint32_t n_clusters = 0;
    for (uint32_t r = 0; r < nrep; ++r) {
        uint32_t next = 1;
        for (uint32_t i : uniq[r])
            if (core[i] && dsu.find(i) == i) label_of_root[i] = next++;
        n_clusters += next - 1;
    }
    auto unique_label = [&](uint32_t u) -> uint32_t {
        if (core[u]) return label_of_root[dsu.find(u)];
        if (border_min[u] != UINT32_MAX) return label_of_root[dsu.find(border_min[u])];
        return 0u;
    };
    for (uint32_t i = 0; i < n_rows; ++i) {
        uint32_t u = rep[i];
        out->clone_id[i] = unique_label(u);
        out->core[i] = core[i] ? 1 : 0;
        out->copies[i] = copies[i];
        if (out->n_cand) {
            uint32_t nc = 0;
            if (!core[u] && K > 0) {
                std::vector<uint32_t> labs;
                for (uint32_t x : core_nbrs[u]) labs.push_back(label_of_root[dsu.find(x)]);
                std::sort(labs.begin(), labs.end());
                labs.erase(std::unique(labs.begin(), labs.end()), labs.end());
                nc = (uint32_t)labs.size();
                if (out->cand)
                    for (uint32_t k = 0; k < nc && k < (uint32_t)K; ++k)
                        out->cand[(size_t)i * K + k] = labs[k];
            }
            out->n_cand[i] = nc;
        }
    }
    out->n_uniques = n_uniques;
    out->n_cores = n_cores;
    out->n_clusters = n_clusters;
    out->admissible_pairs = adm_total;
    out->neighbour_pairs = nbr_total;
    out->all_pairs = all_total;
    return 0;
}
