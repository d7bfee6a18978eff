// k_buckets.cu -- bucketing of the uniques and the work list of the distance
// kernel.
//
// The reference compares every pair of uniques (an n_u x n_u block grid,
// cuda/PSDBSCAN.hcu:1115-1178, and n_cores x n_u at :1200-1257) and tests V/J
// compatibility and the length gap inside each pair (:785-788).  Here the
// uniques are first placed in bins keyed by (repertoire, V gene, J gene,
// length); a unique with ambiguous calls sits in |V|*|J| bins.  Two uniques are
// V- and J-compatible (both bitset intersections non-empty,
// cuda/BitsetVector.inl:214-237) iff they share a bin, so only pairs inside a
// bin, or between the bins of one (repertoire, V, J) whose lengths are within
// the threshold, are ever evaluated.  Bins are laid out densely with the length
// fastest, so the partner bin of length L+g is the bin index + g.
//
// Each bin is further split into kKeyClasses sub-buckets: class 0 holds the
// uniques of small call groups, classes 1.. hold the uniques of large groups
// of identical (V set, J set) -- the members of a big clonal family.  Every
// sub-bucket keeps the AND of its entries' signatures (the genes each entry
// has below the bin's V gene and below its J gene).  A pair of sub-buckets whose
// signature ANDs intersect shares a lower gene in every pair, so none of its
// pairs is canonical here and the pair of sub-buckets is not scheduled: a
// family's internal pairs are evaluated once, in its lowest (V, J) bin, and not
// again in each of the |V|*|J| bins it occupies.
//
// Hamming with eps <= 2 at every length takes its candidates from a segment
// join instead (the k_join_* kernels below): groups of uniques that share one
// whole segment of eps+1, which every neighbour pair does (pigeonhole).
#include "idb_internal.cuh"

namespace idb {

namespace {

constexpr int kThreads = 256;

inline int grid_for(uint64_t n, int threads = kThreads) {
    uint64_t g = (n + threads - 1) / threads;
    uint64_t cap = (uint64_t)sm_count() * 8;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

struct BinGeom {
    uint32_t Gv, Gj, NL, Lmin, VW, JW, K;
    __device__ __forceinline__ bool in_range(uint32_t L) const { return L >= Lmin && L - Lmin < NL; }
    // sub-bucket index: ((((r*Gv + v)*Gj + j)*NL + L-Lmin)*K + class
    __device__ __forceinline__ uint32_t bin(uint32_t r, uint32_t v, uint32_t j, uint32_t L,
                                            uint32_t c) const {
        return (((r * Gv + v) * Gj + j) * NL + (L - Lmin)) * K + c;
    }
};

// genes of `bits` (first word) below gene index g
__device__ __forceinline__ uint64_t below(uint64_t word0, uint32_t g) {
    return g >= 64 ? word0 : (word0 & ((1ull << g) - 1ull));
}

// ---------------------------------------------------------------------------
// Call groups: uniques with identical (repertoire, length, V bits, J bits).
// Open addressing on the (reset) duplicate table; a group of >= kBigGroup
// members gets class 1 + (slot % (K-1)), all others class 0.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool same_group(const uint64_t *vbits, const uint64_t *jbits,
                                           uint32_t VW, uint32_t JW, uint32_t ra, uint32_t rb) {
    for (uint32_t w = 0; w < VW; ++w)
        if (vbits[(size_t)ra * VW + w] != vbits[(size_t)rb * VW + w]) return false;
    for (uint32_t w = 0; w < JW; ++w)
        if (jbits[(size_t)ra * JW + w] != jbits[(size_t)rb * JW + w]) return false;
    return true;
}

__global__ void k_group_insert(BinGeom g, Counters *ctr, const uint32_t *__restrict__ urow,
                               const uint32_t *__restrict__ ulen, const uint32_t *__restrict__ urep,
                               const uint64_t *__restrict__ vbits, const uint64_t *__restrict__ jbits,
                               uint32_t *table, uint32_t *tcount, uint32_t *uslot, uint64_t mask) {
    const uint32_t nu = ctr->n_uniques;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < nu; u += stride) {
        const uint32_t row = urow[u], L = ulen[u], r = urep[u];
        uint64_t h = mix64(0xA0761D6478BD642Full + r, L);
        for (uint32_t w = 0; w < g.VW; ++w) h = mix64(h, vbits[(size_t)row * g.VW + w]);
        for (uint32_t w = 0; w < g.JW; ++w) h = mix64(h, jbits[(size_t)row * g.JW + w]);
        uint64_t sl = h & mask;
        uint32_t it = 0;
        for (;; ++it) {
            if (it > mask || it >= kSpinCap) {
                atomicOr(&ctr->error, kErrHashStall);
                sl = kNone;
                break;
            }
            uint32_t cur = *((volatile uint32_t *)&table[sl]);
            if (cur == kNone) {
                const uint32_t prev = atomicCAS(&table[sl], kNone, u);
                if (prev == kNone) break;
                cur = prev;
            }
            if (urep[cur] == r && ulen[cur] == L &&
                same_group(vbits, jbits, g.VW, g.JW, urow[cur], row))
                break;
            sl = (sl + 1) & mask;
        }
        uslot[u] = (uint32_t)sl;
        const uint32_t grp = __match_any_sync(__activemask(), (uint32_t)sl);
        if ((threadIdx.x & 31) == (uint32_t)__ffs(grp) - 1 && sl != kNone)
            atomicAdd(&tcount[sl], (uint32_t)__popc(grp));
    }
}

__global__ void k_group_class(const Counters *__restrict__ ctr, const uint32_t *__restrict__ uslot,
                              const uint32_t *__restrict__ tcount, uint32_t K, uint32_t big,
                              uint32_t *__restrict__ uclass) {
    const uint32_t nu = ctr->n_uniques;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < nu; u += stride) {
        const uint32_t sl = uslot[u];
        uint32_t c = 0;
        if (K > 1 && sl != kNone && tcount[sl] >= big) c = 1 + (uint32_t)(mix64(sl, 7) % (K - 1));
        uclass[u] = c;
    }
}

// Entries per unique: |V bits| * |J bits|, one histogram increment per entry.
__global__ void k_bin_hist(BinGeom g, const Counters *__restrict__ ctr,
                           const uint32_t *__restrict__ urow, const uint32_t *__restrict__ ulen,
                           const uint32_t *__restrict__ urep, const uint32_t *__restrict__ uclass,
                           const uint64_t *__restrict__ vbits,
                           const uint64_t *__restrict__ jbits, uint32_t *__restrict__ hist) {
    const uint32_t nu = ctr->n_uniques;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < nu; u += stride) {
        const uint32_t row = urow[u], L = ulen[u], r = urep[u];
        if (!g.in_range(L)) continue;   // only after a replay on changed data (flagged)
        for (uint32_t vw = 0; vw < g.VW; ++vw) {
            uint64_t vb = vbits[(size_t)row * g.VW + vw];
            while (vb) {
                const uint32_t v = vw * 64 + lowest_bit64(vb);
                vb &= vb - 1;
                if (v >= g.Gv) break;
                for (uint32_t jw = 0; jw < g.JW; ++jw) {
                    uint64_t jb = jbits[(size_t)row * g.JW + jw];
                    while (jb) {
                        const uint32_t j = jw * 64 + lowest_bit64(jb);
                        jb &= jb - 1;
                        if (j >= g.Gj) break;
                        // one increment per bin among the lanes here together
                        const uint32_t b = g.bin(r, v, j, L, uclass[u]);
                        const uint32_t grp = __match_any_sync(__activemask(), b);
                        if ((threadIdx.x & 31) == (uint32_t)__ffs(grp) - 1)
                            atomicAdd(&hist[b], (uint32_t)__popc(grp));
                    }
                }
            }
        }
    }
}

// Record of one unique.
//  planes (Hamming, fast path): Bp bit planes x W words; bit i of word
//    p*W + i/32 is bit p of the code of residue i.  Hamming distance of two
//    records = sum over words of popc(OR_p (x_p ^ y_p)).
//  codes (Levenshtein and generic path): one code byte per residue.
// Codes are a bijection of the byte values present, so equality of codes is
// equality of bytes.
// The record of one unique (fast paths: at most NR 16-byte words): bit planes
// (Hamming) or code bytes (Levenshtein), residues read 4 at a time.
// Bit planes of one sequence (L <= 128): bit i of wd[p][w] is bit p of the
// code of residue 32w + i; positions past L keep code 0.  Residues are read 4
// at a time.
__device__ __forceinline__ void build_planes(const uint8_t *s, uint32_t L, const uint8_t *cm,
                                             uint32_t (&wd)[5][4]) {
#pragma unroll
    for (int p = 0; p < 5; ++p)
#pragma unroll
        for (int w = 0; w < 4; ++w) wd[p][w] = 0;
#pragma unroll
    for (int w = 0; w < 4; ++w) {
        if (32u * w >= L) break;
        uint32_t cw[8];
        load_chunk32(s, L, (uint32_t)w, cw);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const uint32_t i0 = 32u * w + 4u * k;
            const uint32_t v = cw[k];
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const uint32_t c = i0 + b < L ? (uint32_t)cm[(v >> (8 * b)) & 0xFFu] : 0u;
#pragma unroll
                for (int p = 0; p < 5; ++p) wd[p][w] |= ((c >> p) & 1u) << (4 * k + b);
            }
        }
    }
}

template <int NR>
__device__ __forceinline__ void build_small_record(const uint8_t *s, uint32_t L,
                                                   const uint8_t *cm, int planes, uint32_t W,
                                                   uint4 (&rec)[NR]) {
    if (planes > 0) {
        uint32_t wd[5][4];
        build_planes(s, L, cm, wd);
        // layout: word p*W + w
        uint32_t flat[4 * NR];
#pragma unroll
        for (int k = 0; k < 4 * NR; ++k) flat[k] = 0;
#pragma unroll
        for (int p = 0; p < 5; ++p)
#pragma unroll
            for (int w = 0; w < 4; ++w)
                if (p < planes && (uint32_t)w < W) {
                    const uint32_t k = (uint32_t)p * W + w;
#pragma unroll
                    for (int kk = 0; kk < 4 * NR; ++kk)
                        if ((uint32_t)kk == k) flat[kk] = wd[p][w];
                }
#pragma unroll
        for (int q = 0; q < NR; ++q) rec[q] = make_uint4(flat[4 * q], flat[4 * q + 1], flat[4 * q + 2], flat[4 * q + 3]);
    } else {
        GlobalReader rd(s, L);
#pragma unroll
        for (int q = 0; q < NR; ++q) {
            uint32_t wv[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const uint32_t i0 = q * 16 + e * 4;
                const uint32_t v = i0 < L ? rd.next() : 0u;
                uint32_t acc = 0;
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    const uint32_t c = i0 + t < L ? (uint32_t)cm[(v >> (8 * t)) & 0xFFu] : 0u;
                    acc |= c << (8 * t);
                }
                wv[e] = acc;
            }
            rec[q] = make_uint4(wv[0], wv[1], wv[2], wv[3]);
        }
    }
}

// RSC: record size in 16-byte words when it is a compile-time 1..8 (the fast
// paths: the record is built once, in RSC uint4 registers), 0 for the long
// records of the generic path (code bytes packed per entry).
template <int RSC>
__global__ void __launch_bounds__(256)
k_bin_fill(BinGeom g, const Counters *__restrict__ ctr,
                           const uint32_t *__restrict__ urow, const uint32_t *__restrict__ ulen,
                           const uint32_t *__restrict__ urep, const uint32_t *__restrict__ uclass,
                           unsigned long long *__restrict__ sig_and,
                           const uint64_t *__restrict__ vbits,
                           const uint64_t *__restrict__ jbits, const uint8_t *__restrict__ seq,
                           const int64_t *__restrict__ seq_off, const uint8_t *__restrict__ codemap,
                           const uint32_t *__restrict__ bin_start, uint32_t *__restrict__ cursor,
                           uint32_t *__restrict__ ent_uid, uint4 *__restrict__ ent_rec,
                           uint4 *__restrict__ ent_meta,
                           uint32_t rs16, int planes, uint32_t W, uint64_t cap_entries,
                           uint32_t *err) {
    __shared__ uint8_t cm[256];
    for (int k = threadIdx.x; k < 256; k += blockDim.x) cm[k] = codemap[k];
    __syncthreads();
    const uint32_t nu = ctr->n_uniques;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < nu; u += stride) {
        const uint32_t row = urow[u], L = ulen[u], r = urep[u];
        if (!g.in_range(L)) continue;
        const uint8_t *s = seq + seq_off[row];
        // the record depends on the unique only: build it once (registers when it
        // is at most 128 bytes, the fast paths), store it in every bin
        constexpr int NR = RSC > 0 ? RSC : 1;
        uint4 rec[NR];
        constexpr bool small = RSC > 0;
        if (small) build_small_record<NR>(s, L, cm, planes, W, rec);
        for (uint32_t vw = 0; vw < g.VW; ++vw) {
            uint64_t vb = vbits[(size_t)row * g.VW + vw];
            while (vb) {
                const uint32_t v = vw * 64 + lowest_bit64(vb);
                vb &= vb - 1;
                if (v >= g.Gv) break;
                for (uint32_t jw = 0; jw < g.JW; ++jw) {
                    uint64_t jb = jbits[(size_t)row * g.JW + jw];
                    while (jb) {
                        const uint32_t j = jw * 64 + lowest_bit64(jb);
                        jb &= jb - 1;
                        if (j >= g.Gj) break;
                        const uint32_t b = g.bin(r, v, j, L, uclass[u]);
                        const uint64_t sv = below(vbits[(size_t)row * g.VW], v);
                        const uint64_t sj = below(jbits[(size_t)row * g.JW], j);
                        // the ANDs only clear bits: no atomic when nothing would change
                        // (a stale read can only cost an unneeded atomic)
                        const unsigned long long cv = sig_and[2 * (size_t)b];
                        if ((cv & sv) != cv) atomicAnd(&sig_and[2 * (size_t)b], sv);
                        const unsigned long long cj = sig_and[2 * (size_t)b + 1];
                        if ((cj & sj) != cj) atomicAnd(&sig_and[2 * (size_t)b + 1], sj);
                        // one cursor increment per bin among the lanes here together
                        const uint32_t am = __activemask();
                        const uint32_t grp = __match_any_sync(am, b);
                        const uint32_t lane = threadIdx.x & 31, ld = (uint32_t)__ffs(grp) - 1;
                        uint32_t base = 0;
                        if (lane == ld) base = atomicAdd(&cursor[b], (uint32_t)__popc(grp));
                        base = __shfl_sync(grp, base, ld);
                        const uint64_t pos = (uint64_t)bin_start[b] + base +
                                             __popc(grp & ((1u << lane) - 1u));
                        if (pos >= cap_entries) { atomicOr(err, kErrEntryOverflow); continue; }
                        ent_uid[pos] = u;
                        // side record: signature below (v, j) and the unique id
                        ent_meta[pos] = make_uint4((uint32_t)sv, (uint32_t)(sv >> 32), (uint32_t)sj, u);
                        uint4 *dst = ent_rec + pos * rs16;
                        if (small) {
#pragma unroll
                            for (int q = 0; q < NR; ++q) dst[q] = rec[q];
                            continue;
                        }
                        // long records (generic path): code bytes, 16 at a time
                        for (uint32_t q = 0; q < rs16; ++q) {
                            uint32_t wv[4];
#pragma unroll
                            for (int e = 0; e < 4; ++e) {
                                uint32_t acc = 0;
#pragma unroll
                                for (int t = 0; t < 4; ++t) {
                                    const uint32_t i = q * 16 + e * 4 + t;
                                    const uint32_t c = i < L ? cm[s[i]] : 0u;
                                    acc |= c << (8 * t);
                                }
                                wv[e] = acc;
                            }
                            dst[q] = make_uint4(wv[0], wv[1], wv[2], wv[3]);
                        }
                    }
                }
            }
        }
    }
}

// Bin pairs: sub-bucket pairs (b,c) x (b+g,c') for every admissible length gap
// g (eps(L,L+g) >= g; Hamming compares equal lengths only,
// cuda/PSDBSCAN.hcu:615); for g = 0 only c <= c'.  Pairs whose signature ANDs
// intersect hold no canonical pair and are left out.
struct PairGeom {
    uint32_t NL, Lmin, Gv, Gj, K;
    int dLmax;
    bool hamming;
    uint32_t TX, TY, q;
};

__device__ __forceinline__ bool pair_ok(const PairGeom &pg, const int16_t *eps_tab, uint32_t li,
                                        int gap) {
    if (li + gap >= pg.NL) return false;
    if (pg.hamming && gap != 0) return false;
    const int e = eps_tab[(size_t)li * pg.NL + li + gap];
    return e >= gap;
}

__device__ __forceinline__ bool sig_disjoint(const unsigned long long *sig, uint32_t a, uint32_t b) {
    return ((sig[2 * (size_t)a] & sig[2 * (size_t)b]) | (sig[2 * (size_t)a + 1] & sig[2 * (size_t)b + 1])) == 0;
}

template <bool FILL>
__device__ __forceinline__ uint32_t visit_pairs(uint32_t sb, const PairGeom &pg,
                                                const int16_t *eps_tab, const uint32_t *bin_start,
                                                const unsigned long long *sig, BinPair *out,
                                                uint32_t k, uint64_t cap_bp, uint32_t *err) {
    const uint32_t a0 = bin_start[sb], nA = bin_start[sb + 1] - a0;
    if (nA == 0) return 0;
    const uint32_t b = sb / pg.K, c = sb % pg.K;
    const uint32_t li = b % pg.NL;
    uint32_t n = 0;
    for (int g = 0; g <= pg.dLmax; ++g) {
        if (!pair_ok(pg, eps_tab, li, g)) continue;
        for (uint32_t c2 = (g == 0 ? c : 0); c2 < pg.K; ++c2) {
            const uint32_t sb2 = (b + g) * pg.K + c2;
            const uint32_t b0 = bin_start[sb2], nB = bin_start[sb2 + 1] - b0;
            if (nB == 0) continue;
            const bool same = g == 0 && c2 == c;
            if (same && nA < 2) continue;
            if (!sig_disjoint(sig, sb, sb2)) continue;
            if (FILL) {
                const uint32_t kk = k + n;
                if (kk >= cap_bp) { atomicOr(err, kErrBinPairOverflow); ++n; continue; }
                const uint32_t rest = b / pg.NL;
                BinPair P;
                P.a_start = a0; P.a_n = nA; P.b_start = b0; P.b_n = nB;
                P.unit_base = 0;
                P.ncx = (nA + pg.TX - 1) / pg.TX;
                P.la = (uint16_t)(pg.Lmin + li); P.lb = (uint16_t)(pg.Lmin + li + g);
                P.v = (uint16_t)((rest / pg.Gj) % pg.Gv); P.j = (uint16_t)(rest % pg.Gj);
                P.eps = eps_tab[(size_t)li * pg.NL + li + g];
                P.same = same;
                const uint64_t cost = same ? (uint64_t)nA * (nA - 1) / 2 : (uint64_t)nA * nB;
                P.cls = (uint8_t)(cost ? 63 - __clzll((long long)cost) : 0);
                P.cost_lo = (uint32_t)min(cost, (uint64_t)0xFFFFFFFFu);
                out[kk] = P;
            }
            ++n;
        }
    }
    return n;
}

__global__ void k_binpairs_count(uint32_t nsub, PairGeom pg, const int16_t *__restrict__ eps_tab,
                                 const uint32_t *__restrict__ bin_start,
                                 const unsigned long long *__restrict__ sig,
                                 uint32_t *__restrict__ cnt) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t sb = blockIdx.x * blockDim.x + threadIdx.x; sb < nsub; sb += stride)
        cnt[sb] = visit_pairs<false>(sb, pg, eps_tab, bin_start, sig, nullptr, 0, 0, nullptr);
}

__global__ void k_binpairs_fill(uint32_t nsub, PairGeom pg, const int16_t *__restrict__ eps_tab,
                                const uint32_t *__restrict__ bin_start,
                                const unsigned long long *__restrict__ sig,
                                const uint32_t *__restrict__ bp_off, uint64_t cap_bp,
                                BinPair *__restrict__ out, uint32_t *err) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t sb = blockIdx.x * blockDim.x + threadIdx.x; sb < nsub; sb += stride)
        visit_pairs<true>(sb, pg, eps_tab, bin_start, sig, out, bp_off[sb], cap_bp, err);
}

// Schedule: heavy bin pairs first (counting sort on log2 of the cost, cost =
// pairs for the static schedule or the predicted cost for the learned one).
__global__ void k_cls_hist(const Counters *__restrict__ ctr, const BinPair *__restrict__ bp,
                           const float *__restrict__ pred, uint32_t *__restrict__ hist) {
    __shared__ uint32_t h[64];
    if (threadIdx.x < 64) h[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t n = ctr->n_binpairs;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        uint32_t cls = bp[i].cls;
        if (pred) {
            const float c = fmaxf(pred[i], 1.0f);
            cls = min(63u, (uint32_t)(log2f(c) * 2.0f));
        }
        atomicAdd(&h[63 - cls], 1u);
    }
    __syncthreads();
    if (threadIdx.x < 64 && h[threadIdx.x]) atomicAdd(&hist[threadIdx.x], h[threadIdx.x]);
}

__global__ void k_cls_scatter(const Counters *__restrict__ ctr, const BinPair *__restrict__ bp,
                              const float *__restrict__ pred, const uint32_t *__restrict__ start,
                              uint32_t *__restrict__ cursor, BinPair *__restrict__ out,
                              uint32_t *__restrict__ units, uint32_t TX, uint32_t TY, uint32_t q,
                              int small_mode, uint32_t *__restrict__ small_list,
                              uint32_t *__restrict__ n_small, uint32_t *__restrict__ n_tiny,
                              uint32_t small_cap) {
    const uint32_t n = ctr->n_binpairs;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        BinPair P = bp[i];
        uint32_t cls = P.cls;
        if (pred) {
            const float c = fmaxf(pred[i], 1.0f);
            cls = min(63u, (uint32_t)(log2f(c) * 2.0f));
        }
        // one cursor increment per class among the warp's active lanes
        const uint32_t act = __activemask();
        const uint32_t grp = __match_any_sync(act, cls);
        const uint32_t lane = threadIdx.x & 31, leader = (uint32_t)__ffs(grp) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(&cursor[63 - cls], (uint32_t)__popc(grp));
        base = __shfl_sync(act, base, leader);
        const uint32_t pos = start[63 - cls] + base + __popc(grp & ((1u << lane) - 1u));
        P.cls = (uint8_t)cls;
        out[pos] = P;
        uint64_t nu;
        if (small_mode && P.a_n <= kSmallSide && (P.same || P.b_n <= kSmallSide)) {
            nu = 0;                               // pair-parallel path, no tiled units
            // small bin pairs from the front of the list, tiny ones from its end
            const bool tiny = P.same && P.a_n <= kTinySide;
            const uint32_t am = __activemask();
            const uint32_t tm = __ballot_sync(am, tiny), sm = am & ~tm;
            const uint32_t ld = (uint32_t)__ffs(am) - 1;
            uint32_t b0 = 0, t0 = 0;
            if (lane == ld) {
                if (sm) b0 = atomicAdd(n_small, (uint32_t)__popc(sm));
                if (tm) t0 = atomicAdd(n_tiny, (uint32_t)__popc(tm));
            }
            b0 = __shfl_sync(am, b0, ld);
            t0 = __shfl_sync(am, t0, ld);
            const uint32_t below = (1u << lane) - 1u;
            if (tiny) small_list[small_cap - 1u - (t0 + __popc(tm & below))] = pos;
            else small_list[b0 + __popc(sm & below)] = pos;
        } else if (P.same) {
            const uint32_t ncy = (P.a_n + TY - 1) / TY;
            nu = tri_units(P.ncx, ncy, q);
        } else {
            const uint32_t ncy = (P.b_n + TY - 1) / TY;
            nu = (uint64_t)P.ncx * ncy;
        }
        units[pos] = (uint32_t)nu;
    }
}

__global__ void k_set_unit_base(const Counters *__restrict__ ctr, BinPair *__restrict__ bp,
                                const uint32_t *__restrict__ base) {
    const uint32_t n = ctr->n_binpairs;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        bp[i].unit_base = base[i];
}


// ---------------------------------------------------------------------------
// Segment join (Hamming, eps(L,L) <= kJoinMaxEps for every length).  Split a
// sequence of length L into S = eps+1 segments [k*L/S, (k+1)*L/S): two
// sequences of length L within Hamming distance eps differ in at most eps
// positions, so at least one segment is identical (pigeonhole).  Every unique
// is entered once per segment under the key (repertoire, L, k, segment bytes);
// the uniques that share a key form a group, and only pairs inside a group are
// evaluated.  A pair is emitted from its lowest identical segment only, and
// only if its V sets and J sets intersect, so each neighbour pair appears once
// and the pairs are exactly those of the bucket path.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t seg_count(const int16_t *eps_tab, uint32_t NL, uint32_t li) {
    const int e = eps_tab[(size_t)li * NL + li];
    return e < 0 ? 1u : (uint32_t)e + 1u;
}

// Key of segment k of a unique: repertoire (24 bits), length (8), segment (2)
// and 30 bits of a hash of the segment's residue codes.  Codes are a bijection
// of the bytes, so identical segments always share a key; two different
// segments that share one only make a group larger (the distance kernel
// checks that segment k is identical before it emits a pair).
__device__ __forceinline__ unsigned long long seg_key(const uint32_t (&wd)[5][4], uint32_t r,
                                                      uint32_t L, uint32_t k, uint32_t lo,
                                                      uint32_t hi) {
    unsigned long long h = mix64(0x5E6A1F00ull, ((unsigned long long)r << 16) | (L << 2) | k);
#pragma unroll
    for (int w = 0; w < 4; ++w) {
        const uint32_t a0 = max(lo, 32u * w), a1 = min(hi, 32u * w + 32u);
        if (a0 < a1) {
            const uint32_t n = a1 - a0;
            const uint32_t m = (n >= 32 ? 0xFFFFFFFFu : ((1u << n) - 1u)) << (a0 - 32u * w);
            unsigned long long acc = 0;
#pragma unroll
            for (int p = 0; p < 5; ++p) acc = acc * 0x9E3779B97F4A7C15ull + (wd[p][w] & m);
            h = mix64(h, acc);
        }
    }
    return ((unsigned long long)r << 40) | ((unsigned long long)L << 32) |
           ((unsigned long long)k << 30) | (h >> 34);
}

// Slots of the join table in use: about 1.5 slots per possible key (join_smax
// per unique), a power of two, at most the allocation.  The allocation is sized
// for every row being unique; the uniques are counted on the device, so the
// table a call probes (and clears) is the smaller one they need.
__device__ __forceinline__ uint32_t join_mask(uint32_t nu, uint32_t smax, uint64_t cap_mask) {
    const uint64_t want = max((3ull * smax * nu + 1) / 2, 1024ull);
    uint64_t c = 1024;
    while (c < want) c <<= 1;
    return (uint32_t)min(c - 1, cap_mask);
}

// The probed prefix is sized by the unique count, or by `rows` (an upper
// bound) when the inserts run by row chunk, before the count is known.
__global__ void k_join_clear(Counters *ctr, uint32_t smax, uint64_t cap_mask,
                             unsigned long long *__restrict__ key, uint32_t *__restrict__ cnt,
                             uint32_t rows) {
    const uint32_t n = join_mask(rows ? rows : ctr->n_uniques, smax, cap_mask) + 1u;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ctr->n_jslots = n;
        ctr->n_jslots1 = n + 1;
    }
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        key[i] = ~0ull;
        cnt[i] = 0u;
    }
}

__global__ void __launch_bounds__(256)
k_join_insert(BinGeom g, Counters *ctr, const uint32_t *__restrict__ urow,
              const uint32_t *__restrict__ ulen, const uint32_t *__restrict__ urep,
              const uint8_t *__restrict__ seq, const int64_t *__restrict__ seq_off,
              const uint8_t *__restrict__ codemap, const int16_t *__restrict__ eps_tab,
              unsigned long long *tkey, uint32_t *tcnt, uint32_t *__restrict__ islot,
              uint32_t *__restrict__ irank, uint32_t smax,
              int chunk) {
    __shared__ uint8_t cm[256];
    for (int k = threadIdx.x; k < 256; k += blockDim.x) cm[k] = codemap[k];
    __syncthreads();
    // every unique, or (chunk >= 0) the uniques of one row chunk
    uint32_t u0 = 0, u1 = ctr->n_uniques;
    if (chunk >= 0) {
        u0 = 0;
        for (int m = 0; m < chunk; ++m) u0 += ctr->chunk_uniques[m];
        u1 = u0 + ctr->chunk_uniques[chunk];
    }
    const uint32_t mask = ctr->n_jslots - 1u;   // the prefix k_join_clear prepared
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t u = u0 + blockIdx.x * blockDim.x + threadIdx.x; u < u1; u += stride) {
        const uint32_t row = urow[u], L = ulen[u], r = urep[u];
        const uint32_t S = g.in_range(L) ? seg_count(eps_tab, g.NL, L - g.Lmin) : 0u;
        uint32_t wd[5][4];
        build_planes(seq + seq_off[row], S ? L : 0u, cm, wd);
        for (uint32_t k = 0; k < 4; ++k) {
            uint32_t sl = kNone;
            if (k < S) {
                const unsigned long long key = seg_key(wd, r, L, k, k * L / S, (k + 1) * L / S);
                sl = (uint32_t)(mix64(key, 0x51ull) & mask);
                for (uint32_t it = 0;; ++it) {
                    if (it > mask || it >= kSpinCap) {
                        atomicOr(&ctr->error, kErrHashStall);
                        sl = kNone;
                        break;
                    }
                    unsigned long long cur = *((volatile unsigned long long *)&tkey[sl]);
                    if (cur == ~0ull) {
                        cur = atomicCAS(&tkey[sl], ~0ull, key);
                        if (cur == ~0ull) break;   // this entry created the key
                    }
                    if (cur == key) break;
                    sl = (sl + 1) & (uint32_t)mask;
                }
            }
            islot[(size_t)u * 4 + k] = sl;
            // one count increment per key among the lanes here together; the
            // count before it ranks the entry within its key's group (its
            // place in the group's entries, k_join_fill)
            const uint32_t am = __activemask();
            const uint32_t grp = __match_any_sync(am, sl);
            const int leader = __ffs(grp) - 1;
            uint32_t base = 0;
            if (lane == (uint32_t)leader && sl != kNone) base = atomicAdd(&tcnt[sl], (uint32_t)__popc(grp));
            base = __shfl_sync(am, base, leader);
            if (k < S) irank[(size_t)u * smax + k] = base + (uint32_t)__popc(grp & ((1u << lane) - 1u));
        }
    }
}

// Size of every key's group, per table slot (0 for an empty slot and for a
// key held by one unique), and the bin-pair index of the slots that hold
// groups.  A sequential pass over the probed prefix of the table, four slots
// per thread (16-byte loads and stores), with one counter atomic per block and
// pass of 4 x 256 slots (the counter's atomics bounded the pass at one slot per
// thread).
__global__ void __launch_bounds__(256)
k_join_sizes(Counters *ctr, const uint32_t *__restrict__ tcnt, uint32_t *__restrict__ sizes,
             uint32_t *__restrict__ bpidx) {
    __shared__ uint32_t s_w[8];
    __shared__ uint32_t s_base;
    const uint32_t ns = ctr->n_jslots;
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t stride = 4 * gridDim.x * blockDim.x;
    if (blockIdx.x == 0 && threadIdx.x == 0) sizes[ns] = 0u;   // the scan's end: the total
    for (uint32_t h0 = 4 * blockIdx.x * blockDim.x; h0 < ns; h0 += stride) {
        const uint32_t h = h0 + 4 * threadIdx.x;
        uint32_t c[4] = {0u, 0u, 0u, 0u};
        if (h + 4 <= ns) {   // the probed prefix is a power of two >= 1024: whole quads
            const uint4 v = *reinterpret_cast<const uint4 *>(tcnt + h);
            c[0] = v.x; c[1] = v.y; c[2] = v.z; c[3] = v.w;
        }
        uint32_t mine = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (c[k] < 2) c[k] = 0;
            mine += c[k] != 0;
        }
        if (h + 4 <= ns) *reinterpret_cast<uint4 *>(sizes + h) = make_uint4(c[0], c[1], c[2], c[3]);
        // rank of this thread's groups in the block: warp scan, then warp sums
        uint32_t incl = mine;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if (lane >= (uint32_t)d) incl += t;
        }
        if (lane == 31) s_w[wid] = incl;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t t = 0;
            for (uint32_t w = 0; w < blockDim.x / 32; ++w) { const uint32_t x = s_w[w]; s_w[w] = t; t += x; }
            s_base = t ? atomicAdd(&ctr->n_groups, t) : 0u;
        }
        __syncthreads();
        uint32_t idx = s_base + s_w[wid] + incl - mine;
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (c[k]) bpidx[h + k] = idx++;
        __syncthreads();
    }
}

// Entries: each unique once per segment whose key forms a group, at the
// group's start plus the entry's rank from the insert; the side record carries
// the segment index and the unique id.
template <int RSC>
__global__ void __launch_bounds__(256)
k_join_fill(BinGeom g, const Counters *__restrict__ ctr, const uint32_t *__restrict__ urow,
            const uint32_t *__restrict__ ulen, const uint8_t *__restrict__ seq,
            const int64_t *__restrict__ seq_off, const uint8_t *__restrict__ codemap,
            const int16_t *__restrict__ eps_tab, const uint32_t *__restrict__ islot,
            const uint64_t *__restrict__ vbits, const uint64_t *__restrict__ jbits,
            const uint32_t *__restrict__ start,
            const uint32_t *__restrict__ irank, uint32_t smax, uint4 *__restrict__ ent_rec,
            uint4 *__restrict__ ent_meta, int planes, uint32_t W, uint64_t cap_entries,
            uint32_t *err) {
    __shared__ uint8_t cm[256];
    for (int k = threadIdx.x; k < 256; k += blockDim.x) cm[k] = codemap[k];
    __syncthreads();
    const uint32_t nu = ctr->n_uniques;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < nu; u += stride) {
        const uint32_t row = urow[u], L = ulen[u];
        if (!g.in_range(L)) continue;
        const uint32_t S = seg_count(eps_tab, g.NL, L - g.Lmin);
        uint4 rec[RSC];
        build_small_record<RSC>(seq + seq_off[row], L, cm, planes, W, rec);
        for (uint32_t k = 0; k < S; ++k) {
            const uint32_t sl = islot[(size_t)u * 4 + k];
            if (sl == kNone) continue;
            const uint32_t s0 = start[sl];
            if (start[sl + 1] - s0 < 2) continue;              // a key of one unique: no group
            const uint64_t pos = (uint64_t)s0 + irank[(size_t)u * smax + k];
            if (pos >= cap_entries) { atomicOr(err, kErrEntryOverflow); continue; }
            // side record (its unique id is the entry's: the join's distance
            // kernel reads no separate id array): V bits, J bits with the segment index in the top two bits
            const uint64_t vb = vbits[(size_t)row * g.VW];
            const uint32_t jb = (uint32_t)jbits[(size_t)row * g.JW];
            ent_meta[pos] = make_uint4((uint32_t)vb, (uint32_t)(vb >> 32), jb | (k << 30), u);
            uint4 *dst = ent_rec + pos * RSC;
#pragma unroll
            for (int q = 0; q < RSC; ++q) dst[q] = rec[q];
        }
        (void)lane;
    }
}

__global__ void k_join_nbp(Counters *ctr) {
    if (threadIdx.x == 0 && blockIdx.x == 0) ctr->n_binpairs = ctr->n_groups;
}

// One bin pair (a group against itself) per key held by two or more uniques:
// a sequential pass over the probed prefix of the table.
__global__ void k_join_bp_fill(BinGeom g, const Counters *__restrict__ ctr,
                               const unsigned long long *__restrict__ tkey, const uint32_t *__restrict__ start,
                               const uint32_t *__restrict__ bpidx, const int16_t *__restrict__ eps_tab,
                               uint32_t TX, uint64_t cap_bp, BinPair *__restrict__ out, uint32_t *err) {
    const uint32_t ns = ctr->n_jslots;   // a power of two >= 1024: whole quads of slots
    const uint32_t stride = 4 * gridDim.x * blockDim.x;
    for (uint32_t h0 = 4 * (blockIdx.x * blockDim.x + threadIdx.x); h0 < ns; h0 += stride) {
        // four slots a thread: their starts in one 16-byte load, and the next
        // quad's first start (start has ns + 1 entries)
        const uint4 v = *reinterpret_cast<const uint4 *>(start + h0);
        const uint32_t sv[5] = {v.x, v.y, v.z, v.w, start[h0 + 4]};
#pragma unroll
        for (uint32_t q = 0; q < 4; ++q) {
            const uint32_t h = h0 + q, s0 = sv[q], c = sv[q + 1] - s0;
            if (c < 2) continue;
            const uint32_t k = bpidx[h];
            if (k >= cap_bp) { atomicOr(err, kErrBinPairOverflow); continue; }
            const unsigned long long key = tkey[h];
            const uint32_t L = (uint32_t)(key >> 32) & 0xFFu;
            const uint32_t li = L - g.Lmin;
            BinPair P;
            P.a_start = s0; P.a_n = c; P.b_start = s0; P.b_n = c;
            P.unit_base = 0;
            P.ncx = (c + TX - 1) / TX;
            P.la = (uint16_t)L; P.lb = (uint16_t)L;
            P.v = (uint16_t)((key >> 30) & 3u);                   // segment of the group
            P.j = (uint16_t)seg_count(eps_tab, g.NL, li);         // segments of length L
            P.eps = eps_tab[(size_t)li * g.NL + li];
            P.same = 1;
            const uint64_t cost = (uint64_t)c * (c - 1) / 2;
            P.cls = (uint8_t)(cost ? 63 - __clzll((long long)cost) : 0);
            P.cost_lo = (uint32_t)min(cost, (uint64_t)0xFFFFFFFFu);
            out[k] = P;
        }
    }
}
}  // namespace

void launch_join_init(const Plan &P, const Buffers &B, cudaStream_t s) {
    cudaMemsetAsync(&B.ctr->n_jslots, 0, 2 * sizeof(uint32_t), s);   // n_jslots, n_groups
    k_join_clear<<<grid_wave(k_join_clear, B.jn_mask + 1, kThreads), kThreads, 0, s>>>(
        B.ctr, P.join_smax, B.jn_mask, B.jn_key, B.jn_cnt, P.front_join ? P.N : 0u);
}

void launch_join_insert(const Plan &P, const Buffers &B, int chunk, cudaStream_t s) {
    BinGeom g{P.Gv, P.Gj, P.NL, P.Lmin, P.VW, P.JW, P.K};
    const uint32_t rows = chunk < 0 ? P.N : P.chunk_row[chunk + 1] - P.chunk_row[chunk];
    if (rows == 0) return;
    k_join_insert<<<grid_wave(k_join_insert, rows, kThreads), kThreads, 0, s>>>(
        g, B.ctr, B.urow, B.ulen, B.urep, B.seq, B.seq_off, B.codemap, B.eps_tab, B.jn_key, B.jn_cnt,
        B.jn_islot, B.jn_cur, P.join_smax, chunk);
}

void launch_buckets(const Plan &P, const Buffers &B, cudaStream_t s) {
    BinGeom g{P.Gv, P.Gj, P.NL, P.Lmin, P.VW, P.JW, P.K};
    if (P.join) {
        const uint64_t slots = B.jn_mask + 1;   // the allocation; the probed prefix is on the device
        if (!P.front_join) {                    // else the row chunks did these
            launch_join_init(P, B, s);
            launch_join_insert(P, B, -1, s);
        }
        k_join_sizes<<<grid_wave(k_join_sizes, slots, kThreads), kThreads, 0, s>>>(
            B.ctr, B.jn_cnt, B.jn_start, B.jn_bpidx);
        scan_u32(B.jn_start, B.jn_start, (uint32_t)slots + 1, &B.ctr->n_jslots1, &B.ctr->n_entries,
                 B.scan_part, B.scan_part_cap, s);
        return;
    }
    const uint32_t nb = (uint32_t)P.nbins;
    // call groups (the duplicate table is free again once the uniques exist)
    cudaMemsetAsync(B.table, 0xFF, sizeof(uint32_t) * (B.table_mask + 1), s);
    cudaMemsetAsync(B.tcount, 0, sizeof(uint32_t) * (B.table_mask + 1), s);
    k_group_insert<<<grid_wave(k_group_insert, P.N, kThreads), kThreads, 0, s>>>(g, B.ctr, B.urow, B.ulen, B.urep, B.vbits,
                                                       B.jbits, B.table, B.tcount, B.slot,
                                                       B.table_mask);
    k_group_class<<<grid_wave(k_group_class, P.N, kThreads), kThreads, 0, s>>>(B.ctr, B.slot, B.tcount, P.K, P.big_group,
                                                      B.uclass);
    cudaMemsetAsync(B.bin_hist, 0, sizeof(uint32_t) * (P.nbins + 1), s);
    k_bin_hist<<<grid_wave(k_bin_hist, P.N, kThreads), kThreads, 0, s>>>(g, B.ctr, B.urow, B.ulen, B.urep, B.uclass,
                                                    B.vbits, B.jbits, B.bin_hist);
    scan_u32(B.bin_hist, B.bin_hist, nb + 1, nullptr, &B.ctr->n_entries, B.scan_part,
             B.scan_part_cap, s);
}

void launch_fill(const Plan &P, const Buffers &B, cudaStream_t s) {
    if (P.join) {
        BinGeom g{P.Gv, P.Gj, P.NL, P.Lmin, P.VW, P.JW, P.K};
        const int planes = (int)P.B;
        auto go = [&](auto kern) {
            kern<<<grid_wave(kern, P.N, kThreads), kThreads, 0, s>>>(g, B.ctr, B.urow, B.ulen, B.seq, B.seq_off,
                                                     B.codemap, B.eps_tab, B.jn_islot, B.vbits,
                                                     B.jbits, B.jn_start, B.jn_cur, P.join_smax,
                                                     B.ent_rec, B.ent_meta, planes, P.W,
                                                     P.cap_entries, &B.ctr->error);
        };
        switch (P.RS / 16) {   // Hamming fast path: 1..8 words of bit planes
            case 1: go(k_join_fill<1>); break;
            case 2: go(k_join_fill<2>); break;
            case 3: go(k_join_fill<3>); break;
            case 4: go(k_join_fill<4>); break;
            case 5: go(k_join_fill<5>); break;
            case 6: go(k_join_fill<6>); break;
            case 7: go(k_join_fill<7>); break;
            default: go(k_join_fill<8>); break;
        }
        return;
    }
    BinGeom g{P.Gv, P.Gj, P.NL, P.Lmin, P.VW, P.JW, P.K};
    cudaMemsetAsync(B.bin_cursor, 0, sizeof(uint32_t) * P.nbins, s);
    cudaMemsetAsync(B.sig_and, 0xFF, sizeof(unsigned long long) * 2 * P.nbins, s);
    const int planes = (P.fast && P.hamming) ? (int)P.B : 0;
    const uint32_t rs16 = P.RS / 16;
    auto go = [&](auto kern) {
        kern<<<grid_wave(kern, P.N, kThreads), kThreads, 0, s>>>(
            g, B.ctr, B.urow, B.ulen, B.urep, B.uclass, B.sig_and, B.vbits, B.jbits, B.seq, B.seq_off,
            B.codemap, B.bin_hist, B.bin_cursor, B.ent_uid, B.ent_rec, B.ent_meta, rs16, planes, P.W,
            P.cap_entries, &B.ctr->error);
    };
    switch (rs16) {
        case 1: go(k_bin_fill<1>); break;
        case 2: go(k_bin_fill<2>); break;
        case 3: go(k_bin_fill<3>); break;
        case 4: go(k_bin_fill<4>); break;
        case 5: go(k_bin_fill<5>); break;
        case 6: go(k_bin_fill<6>); break;
        case 7: go(k_bin_fill<7>); break;
        case 8: go(k_bin_fill<8>); break;
        default: go(k_bin_fill<0>); break;
    }
}

void launch_binpairs(const Plan &P, const Buffers &B, cudaStream_t s) {
    if (P.join) {
        k_join_nbp<<<1, 32, 0, s>>>(B.ctr);
        return;
    }
    PairGeom pg{P.NL, P.Lmin, P.Gv, P.Gj, P.K, P.dLmax, P.hamming, P.TX, P.TY, P.TY / P.TX};
    const uint32_t nb = (uint32_t)P.nbins;
    k_binpairs_count<<<grid_for(nb), kThreads, 0, s>>>(nb, pg, B.eps_tab, B.bin_hist, B.sig_and,
                                                        B.bp_count);
    scan_u32(B.bp_count, B.bp_count, nb, nullptr, &B.ctr->n_binpairs, B.scan_part,
             B.scan_part_cap, s);
}

void launch_binpairs_fill(const Plan &P, const Buffers &B, cudaStream_t s) {
    if (P.join) {
        BinGeom g{P.Gv, P.Gj, P.NL, P.Lmin, P.VW, P.JW, P.K};
        k_join_bp_fill<<<grid_wave(k_join_bp_fill, B.jn_mask + 1, kThreads), kThreads, 0, s>>>(
            g, B.ctr, B.jn_key, B.jn_start, B.jn_bpidx, B.eps_tab, P.TX, P.cap_binpairs, B.bp,
            &B.ctr->error);
        return;
    }
    PairGeom pg{P.NL, P.Lmin, P.Gv, P.Gj, P.K, P.dLmax, P.hamming, P.TX, P.TY, P.TY / P.TX};
    const uint32_t nb = (uint32_t)P.nbins;
    k_binpairs_fill<<<grid_for(nb), kThreads, 0, s>>>(nb, pg, B.eps_tab, B.bin_hist, B.sig_and,
                                                       B.bp_count, P.cap_binpairs, B.bp,
                                                       &B.ctr->error);
}

void launch_schedule(const Plan &P, const Buffers &B, cudaStream_t s) {
    const uint32_t q = P.TY / P.TX;
    const float *pred = P.schedule == 1 ? B.pred : nullptr;
    cudaMemsetAsync(B.cls_hist, 0, sizeof(uint32_t) * 130, s);
    k_cls_hist<<<grid_for(P.cap_binpairs), kThreads, 0, s>>>(B.ctr, B.bp, pred, B.cls_hist);
    scan_u32(B.cls_hist, B.cls_hist, 64, nullptr, nullptr, B.scan_part, B.scan_part_cap, s);
    cudaMemsetAsync(&B.ctr->n_small, 0, 2 * sizeof(uint32_t), s);   // n_small, small_cursor
    cudaMemsetAsync(&B.ctr->n_tiny, 0, 2 * sizeof(uint32_t), s);    // n_tiny, tiny_cursor
    k_cls_scatter<<<grid_for(P.cap_binpairs), kThreads, 0, s>>>(
        B.ctr, B.bp, pred, B.cls_hist, B.cls_hist + 64, B.bp_sorted, B.bp_units, P.TX, P.TY, q,
        (P.fast && P.hamming) ? 1 : 0, B.bp_small, &B.ctr->n_small, &B.ctr->n_tiny,
        (uint32_t)P.cap_binpairs + 1u);
    scan_u32(B.bp_units, B.bp_units, (uint32_t)P.cap_binpairs, &B.ctr->n_binpairs,
             &B.ctr->n_units, B.scan_part, B.scan_part_cap, s);
    k_set_unit_base<<<grid_for(P.cap_binpairs), kThreads, 0, s>>>(B.ctr, B.bp_sorted, B.bp_units);
}

}  // namespace idb
