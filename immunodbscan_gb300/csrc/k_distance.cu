// k_distance.cu -- the neighbour search (rule S4), one persistent launch.
//
// Reference: half_core_points / half_hamming_core_points
// (cuda/PSDBSCAN.hcu:585-657, 751-833) and their second sweep fuse_clusters /
// fuse_hamming_clusters (:664-742, 840-931).  The reference runs one block per
// pair with an anti-diagonal DP and a __syncthreads per diagonal, twice.  Here
// the distance work is done once: every neighbour pair becomes an edge of the
// neighbour graph, and core marking and cluster growth run on that graph.
//
// Work decomposition
//  * A work unit is an x-chunk of TX = 32*RX entries of bin A against a y-chunk
//    of TY entries of bin B (B = A for a same-bin pair; then only pairs with
//    y after x in the bin are kept).  Units are numbered in schedule order (heavy
//    bin pairs first) and handed out by an atomic queue; each warp owns a unit.
//  * Lane l holds x-entries l, l+32, ... of the chunk in registers.  The
//    y-records are staged into the warp's shared memory with coalesced 128-bit
//    loads and read back as broadcasts, so a y-record costs two shared loads
//    per RX pairs.
//  * Hamming (fast path): residues are bit-sliced (Bp planes of W 32-bit
//    words); a pair costs Bp*W XOR/OR plus a population test.
//  * Levenshtein (fast path): Myers/Hyyro bit-parallel recurrence with the
//    x-pattern's match masks (Peq) in shared memory and the y-text broadcast;
//    the value on the diagonal through (m, n) is checked every 4 columns and a
//    warp leaves a y early once all its pairs exceed eps (the diagonal value
//    never decreases, so the early exit is exact).
//  * A neighbour pair is kept only in the bin of its lowest common V gene and
//    lowest common J gene, so a pair that shares several bins counts once.
//  * Segment join (Hamming, eps <= 2): the "bins" are groups of uniques that
//    share one whole segment; a pair is kept only in the group of its lowest
//    identical segment, and only if its V and J sets intersect.
//  * Bin pairs of at most 32 entries a side are scored pair-parallel (records
//    by shuffles), and a bin with itself of at most 8 entries by one lane.
//  * Hits are queued per lane and written as one warp-compacted bulk append.
#include "idb_internal.cuh"

namespace idb {

namespace {

constexpr int kWarps = 4;            // warps per block
constexpr int kYB = 64;              // y-records staged per batch

struct DistArgs {
    const BinPair *bp;
    const uint32_t *unit_base;
    const uint4 *rec;
    const uint32_t *ent_uid;
    const uint32_t *urow;
    const uint64_t *vbits, *jbits;
    uint32_t VW, JW;
    uint32_t rs16;                   // record size in 16-byte words
    uint32_t TX, TY, q;
    uint32_t A;                      // number of codes (Levenshtein)
    uint2 *edges;
    uint64_t cap_edges;
    Counters *ctr;
    unsigned long long *bp_cycles;   // optional per bin-pair cycle log
    uint32_t *bp_hits;
    const uint4 *meta;               // per entry {sigV lo, sigV hi, sigJ, uid}
    int sig_exact;                   // signatures decide canonicity exactly
    const uint32_t *small_list;      // schedule positions of the small bin pairs (from the
                                     // front) and of the tiny ones (from small_cap - 1 down)
    uint32_t small_cap;
    // segment join: a hit is a neighbour pair if the V and J sets intersect and
    // no lower segment is identical (that segment's group emits it)
    int join;
    // where neighbour pairs go: kSinkEdges = the edge list; kSinkCount /
    // kSinkGrow = the two sweeps of the streamed mode (no edge list kept)
    uint32_t sink;
    uint32_t *cnt;                   // copies-weighted neighbour counts (count sweep)
    const uint32_t *ucopies;
    const uint32_t *ucore;           // core flags (grow sweep)
    uint32_t *parent;                // union-find forest (grow sweep)
    uint32_t *bmin;                  // minimum core neighbour of a non-core unique
};

// Streamed mode, for neighbour graphs larger than the edge memory allowed: the
// distance work runs twice and no pair is stored.  The count sweep adds each
// side's copies to the other's count (rule S5); after the core flags, the grow
// sweep merges core-core pairs into the union-find forest (link to the smaller
// root, as the reference's union_a_and_b does, cuda/PSDBSCAN.hcu:76-107) and
// keeps for every non-core unique its minimum core neighbour (atomicMin: the
// same border rule as the edge-list path).  Both are order-independent.
__device__ __forceinline__ uint32_t sweep_find(uint32_t *p, uint32_t x) {
    volatile uint32_t *vp = p;
    while (true) {   // parent[y] <= y: x strictly decreases
        const uint32_t px = vp[x];
        if (px == x) return x;
        const uint32_t ppx = vp[px];
        if (ppx == px) return px;
        vp[x] = ppx;   // path halving
        x = ppx;
    }
}

__device__ __noinline__ void sink_streamed(const DistArgs &a, uint32_t lo, uint32_t hi) {
    if (a.sink == kSinkCount) {
        atomicAdd(&a.cnt[lo], __ldg(&a.ucopies[hi]));
        atomicAdd(&a.cnt[hi], __ldg(&a.ucopies[lo]));
        return;
    }
    const uint32_t clo = a.ucore[lo], chi = a.ucore[hi];
    if (clo != chi) {
        atomicMin(&a.bmin[clo ? hi : lo], clo ? lo : hi);
        return;
    }
    if (!clo) return;
    uint32_t x = lo, y = hi, it = 0;
    for (; it < kSpinCap; ++it) {
        uint32_t rx = sweep_find(a.parent, x), ry = sweep_find(a.parent, y);
        if (rx == ry) break;
        if (rx < ry) { const uint32_t t = rx; rx = ry; ry = t; }
        if (atomicCAS(&a.parent[rx], rx, ry) == rx) break;   // hook the larger root
        x = rx;
        y = ry;
    }
    if (it == kSpinCap) atomicOr(&a.ctr->error, kErrUnionStall);
}

// One neighbour pair (lo < hi, unique ids) at edge slot `slot`.
__device__ __forceinline__ void put_edge(const DistArgs &a, uint64_t slot, uint32_t lo, uint32_t hi) {
    if (a.sink == kSinkEdges) {
        if (slot < a.cap_edges) a.edges[slot] = make_uint2(lo, hi);
    } else {
        sink_streamed(a, lo, hi);
    }
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Edge writer: each warp reserves kEdgeChunk slots at a time; slots a warp
// does not fill are set to the sentinel (x = kNone) before it moves on.
struct EdgeWriter {
    uint64_t base;     // kNone64 = no chunk held
    uint32_t fill;
    uint32_t written;
    static constexpr uint64_t kNoChunk = ~0ull;

    __device__ void init() { base = kNoChunk; fill = 0; written = 0; }

    __device__ void pad(const DistArgs &a, int lane) {
        if (base == kNoChunk || a.sink != kSinkEdges) return;
        for (uint32_t t = fill + lane; t < kEdgeChunk; t += 32) {
            const uint64_t slot = base + t;
            if (slot < a.cap_edges) a.edges[slot] = make_uint2(kNone, kNone);
        }
    }

    // warp-uniform call; lanes with ok=true append (lo, hi)
    __device__ void append(const DistArgs &a, int lane, bool ok, uint32_t lo, uint32_t hi) {
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, ok);
        if (!m) return;
        const uint32_t n = __popc(m);
        if (base == kNoChunk || fill + n > kEdgeChunk) {
            pad(a, lane);
            uint32_t b = 0;
            if (lane == 0) b = atomicAdd(&a.ctr->edge_reserved, kEdgeChunk);
            b = __shfl_sync(0xFFFFFFFFu, b, 0);
            base = b;
            fill = 0;
            if ((uint64_t)b + kEdgeChunk > a.cap_edges && lane == 0)
                atomicOr(&a.ctr->error, kErrEdgeOverflow);
        }
        if (ok) put_edge(a, base + fill + __popc(m & lanemask_lt()), lo, hi);
        fill += n;
        written += n;
    }

    // Bulk append, warp-uniform: the warp appends T edges at logical positions
    // 0..T-1 (each lane knows its own); the room left in the held chunk is
    // used first, then as many new chunks as needed, reserved with one atomic.
    struct Bulk { uint64_t b0; uint32_t f0; uint64_t nb; };
    __device__ Bulk reserve(const DistArgs &a, int lane, uint32_t T) {
        Bulk k;
        k.f0 = base == kNoChunk ? kEdgeChunk : fill;
        k.b0 = base;
        k.nb = kNoChunk;
        const uint32_t room = kEdgeChunk - k.f0;
        if (T > room) {
            const uint32_t nch = (T - room + kEdgeChunk - 1) / kEdgeChunk;
            uint32_t nb = 0;
            if (lane == 0) nb = atomicAdd(&a.ctr->edge_reserved, nch * kEdgeChunk);
            nb = __shfl_sync(0xFFFFFFFFu, nb, 0);
            if ((uint64_t)nb + (uint64_t)nch * kEdgeChunk > a.cap_edges && lane == 0)
                atomicOr(&a.ctr->error, kErrEdgeOverflow);
            k.nb = nb;
            base = (uint64_t)nb + (uint64_t)(nch - 1) * kEdgeChunk;
            fill = (T - room) - (nch - 1) * kEdgeChunk;
        } else {
            fill = k.f0 + T;
        }
        written += T;
        return k;
    }
    __device__ __forceinline__ uint64_t slot_of(const Bulk &k, uint32_t i) const {
        const uint32_t room = kEdgeChunk - k.f0;
        return i < room ? k.b0 + k.f0 + i : k.nb + (i - room);
    }
};

// lowest common gene of two uniques in one column, -1 if none
__device__ __forceinline__ int lowest_common(const uint64_t *bits, uint32_t W, uint32_t rx,
                                             uint32_t ry) {
    for (uint32_t w = 0; w < W; ++w) {
        const uint64_t c = bits[(size_t)rx * W + w] & bits[(size_t)ry * W + w];
        if (c) return (int)(w * 64) + lowest_bit64(c);
    }
    return -1;
}

__device__ __forceinline__ bool canonical(const DistArgs &a, const BinPair &P, uint32_t ux,
                                          uint32_t uy) {
    const uint32_t rx = a.urow[ux], ry = a.urow[uy];
    return lowest_common(a.vbits, a.VW, rx, ry) == (int)P.v &&
           lowest_common(a.jbits, a.JW, rx, ry) == (int)P.j;
}

// Warp-cooperative lookup of the bin pair that owns unit u (largest i with
// unit_base[i] <= u); 32-ary search.
__device__ __forceinline__ uint32_t find_binpair(const uint32_t *base, uint32_t n, uint32_t u,
                                                 int lane) {
    uint32_t lo = 0, hi = n;
    while (hi - lo > 32) {
        const uint32_t step = (hi - lo + 31) / 32;
        const uint32_t idx = lo + (uint32_t)lane * step;
        const bool ok = idx < hi && __ldg(base + idx) <= u;
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, ok);
        const uint32_t t = 31 - __clz(m);
        lo = lo + t * step;
        hi = min(hi, lo + step);
    }
    const uint32_t idx = lo + lane;
    const bool ok = idx < hi && __ldg(base + idx) <= u;
    const uint32_t m = __ballot_sync(0xFFFFFFFFu, ok);
    return lo + (31 - __clz(m));
}

struct Unit {
    BinPair P;
    uint32_t xbase, nx, ybase, ny;
    uint32_t bpi;             // index of the bin pair in schedule order
    long long t0;             // clock64 at the start (profiling only)
};

__device__ __forceinline__ bool next_unit(const DistArgs &a, uint32_t n_units, uint32_t n_bp,
                                          int lane, Unit &U) {
    uint32_t u = 0;
    if (lane == 0) u = atomicAdd(&a.ctr->unit_cursor, 1u);
    u = __shfl_sync(0xFFFFFFFFu, u, 0);
    if (u >= n_units) return false;
    const uint32_t i = find_binpair(a.unit_base, n_bp, u, lane);
    U.bpi = i;
    if (a.bp_cycles) U.t0 = clock64();
    U.P = a.bp[i];
    const uint64_t k = u - a.unit_base[i];
    uint32_t cx, cy;
    if (U.P.same) {
        tri_decode(k, U.P.ncx, a.q, cx, cy);
    } else {
        cy = (uint32_t)(k / U.P.ncx);
        cx = (uint32_t)(k % U.P.ncx);
    }
    U.xbase = cx * a.TX;
    U.nx = min(a.TX, U.P.a_n - U.xbase);
    U.ybase = cy * a.TY;
    const uint32_t bn = U.P.same ? U.P.a_n : U.P.b_n;
    U.ny = min(a.TY, bn - U.ybase);
    return true;
}

// profiling: device cycles spent on each bin pair (learned-schedule training data)
__device__ __forceinline__ void log_unit(const DistArgs &a, const Unit &U, int lane) {
    if (a.bp_cycles && lane == 0)
        atomicAdd(&a.bp_cycles[U.bpi], (unsigned long long)(clock64() - U.t0));
}

// pairs of the unit that the method evaluates (y after x for a same-bin pair)
__device__ __forceinline__ uint64_t unit_pairs(const Unit &U, uint32_t xpos) {
    if (!U.P.same) return U.ny;
    const uint32_t lo = max(U.ybase, xpos + 1), hi = U.ybase + U.ny;
    return hi > lo ? hi - lo : 0;
}

__device__ __forceinline__ void finish(const DistArgs &a, EdgeWriter &ew, uint64_t pairs,
                                       int lane) {
    ew.pad(a, lane);
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) pairs += __shfl_xor_sync(0xFFFFFFFFu, pairs, d);
    if (lane == 0) {
        if (pairs) atomicAdd(&a.ctr->pairs_evaluated, (unsigned long long)pairs);
        if (ew.written) atomicAdd(&a.ctr->n_edges, ew.written);
    }
}

// Segment join with the gene bits in the side records: V and J sets intersect,
// segment k (the group's) is identical and no lower segment is, read from the
// difference words d[w] (bit i of word w: residue 32w+i differs) of the
// length-L pair split into S segments.  Groups are keyed by a hash of the
// segment, so the test on segment k itself keeps a shared key of two different
// segments from emitting a pair twice.
template <int W>
__device__ __forceinline__ bool join_meta_ok(const uint4 &mx, const uint4 &my, const uint32_t (&d)[W],
                                             uint32_t L, uint32_t S, uint32_t k) {
    if (((mx.x & my.x) | (mx.y & my.y)) == 0) return false;
    if ((mx.z & my.z & 0x3FFFFFFFu) == 0) return false;
    for (uint32_t kk = 0; kk <= k; ++kk) {
        const uint32_t lo = kk * L / S, hi = (kk + 1) * L / S;
        uint32_t any = 0;
#pragma unroll
        for (int w = 0; w < W; ++w) {
            const uint32_t a0 = max(lo, 32u * w), a1 = min(hi, 32u * w + 32u);
            if (a0 < a1) {
                const uint32_t n = a1 - a0;
                const uint32_t m = (n >= 32 ? 0xFFFFFFFFu : ((1u << n) - 1u)) << (a0 - 32u * w);
                any |= d[w] & m;
            }
        }
        if (kk < k && any == 0) return false;   // identical (or empty) lower segment: emitted there
        if (kk == k && any != 0) return false;  // segment k differs: a shared key only
    }
    return true;
}

// ---------------------------------------------------------------------------
// Neighbour hits of one y against the calling lane's x-entries (bit r of `hit`
// = x-entry xbase + 32*r + lane).  Kept out of line: hits are rare, and the
// hot loops stay small enough for the instruction cache.
// ---------------------------------------------------------------------------
__device__ __noinline__ void emit_hits(const DistArgs &a, EdgeWriter &ew, uint32_t hit,
                                       uint32_t a_start, uint32_t xbase, uint32_t y_entry,
                                       uint32_t ypos, uint32_t same, uint32_t v, uint32_t j,
                                       int lane) {
    uint32_t any = __reduce_or_sync(0xFFFFFFFFu, hit);
    const uint32_t uy = a.ent_uid[y_entry];
    while (any) {
        const int r = __ffs(any) - 1;
        any &= any - 1;
        const uint32_t xpos = xbase + 32u * r + lane;
        bool ok = (hit >> r) & 1u;
        if (ok && same && ypos <= xpos) ok = false;
        uint32_t ux = 0;
        if (ok) {
            ux = a.ent_uid[a_start + xpos];
            const uint32_t rx = a.urow[ux], ry = a.urow[uy];
            ok = lowest_common(a.vbits, a.VW, rx, ry) == (int)v &&
                 lowest_common(a.jbits, a.JW, rx, ry) == (int)j;
        }
        ew.append(a, lane, ok, min(ux, uy), max(ux, uy));
    }
}

// Pair p of a small bin pair -> (i, j).  One bin: i < j < n, ordered by j
// (pairs of j start at j(j-1)/2).  Two bins: i = p mod n, j = p div n.
__device__ __forceinline__ void small_pair(uint32_t p, bool same, uint32_t n, uint32_t &i,
                                           uint32_t &j) {
    if (same) {
        uint32_t jj = (uint32_t)((1.0f + sqrtf(8.0f * (float)p + 1.0f)) * 0.5f);
        while (jj > 1 && jj * (jj - 1) / 2 > p) --jj;
        while (jj * (jj + 1) / 2 <= p) ++jj;
        j = jj;
        i = p - jj * (jj - 1) / 2;
    } else {
        j = p / n;
        i = p - j * n;
    }
}

// Bulk append of a lane's edges given as bits: bit b stands for pair index
// p0 + stride*b of a small or tiny bin pair (i, j from the pair index; the
// unique ids from the side records).  Warp-uniform.
__device__ __forceinline__ void emit_pair_bits(const DistArgs &a, EdgeWriter &ew, int lane,
                                               uint32_t bits, uint32_t p0, uint32_t stride,
                                               bool same, uint32_t n, uint32_t xstart,
                                               uint32_t ystart) {
    const uint32_t c = (uint32_t)__popc(bits);
    uint32_t incl = c;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, d);
        if (lane >= d) incl += t;
    }
    const uint32_t T = __shfl_sync(0xFFFFFFFFu, incl, 31);
    if (T == 0) return;
    const EdgeWriter::Bulk bk = ew.reserve(a, lane, T);
    uint32_t k = incl - c;
    for (uint32_t b = bits; b; b &= b - 1) {
        const uint32_t p = p0 + stride * ((uint32_t)__ffs(b) - 1u);
        uint32_t i, j;
        small_pair(p, same, n, i, j);
        const uint32_t ux = __ldg(&a.meta[xstart + i].w), uy = __ldg(&a.meta[ystart + j].w);
        put_edge(a, ew.slot_of(bk, k++), min(ux, uy), max(ux, uy));
    }
}

// A small bin pair (at most kSmallSide entries a side), pair-parallel: lane l
// holds entry l of each side; each round the lanes take 32 pairs and fetch
// the two records by shuffles.  Canonicity of a hit is decided from the side
// records (global loads: hits are rare).
template <int BP, int W, int EM, bool JN>
__device__ __forceinline__ void hamming_small(const DistArgs &a, EdgeWriter &ew, const BinPair &P,
                                              uint32_t idx, int lane, uint64_t &pairs) {
    constexpr int NW = BP * W;
    constexpr int R16 = (NW + 3) / 4;
    const long long t0 = a.bp_cycles ? clock64() : 0;
    const bool same = P.same != 0;
    const uint32_t n = P.a_n, m = same ? P.a_n : P.b_n;
    const uint32_t ystart = same ? P.a_start : P.b_start;
    uint32_t xr[NW], yr[NW];
    {
        const uint4 *src = a.rec + (size_t)(P.a_start + ((uint32_t)lane < n ? lane : 0)) * R16;
        const uint4 *srcy = a.rec + (size_t)(ystart + ((uint32_t)lane < m ? lane : 0)) * R16;
#pragma unroll
        for (int q = 0; q < R16; ++q) {
            const uint4 v = __ldg(src + q);
            const uint4 u = same ? v : __ldg(srcy + q);
            const uint32_t w4[4] = {v.x, v.y, v.z, v.w};
            const uint32_t u4[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
            for (int e = 0; e < 4; ++e)
                if (4 * q + e < NW) { xr[4 * q + e] = w4[e]; yr[4 * q + e] = u4[e]; }
        }
    }
    const uint32_t npairs = same ? n * (n - 1) / 2 : n * m;
    if (lane == 0) pairs += npairs;
    const uint32_t thr = EM == 0 ? (uint32_t)max(P.eps, 0) : 0u;
    const bool neg = EM == 0 && P.eps < 0;
    static_assert(kSmallSide * kSmallSide <= 32 * 32, "small round mask");
    uint32_t rmask = 0;           // bit k: the lane's pair of round k is an edge
    for (uint32_t p0 = 0; p0 < npairs && !neg; p0 += 32) {
        const uint32_t p = p0 + lane;
        const bool act = p < npairs;
        uint32_t i = 0, j = 0;
        if (act) small_pair(p, same, n, i, j);
        uint32_t sc;
        uint32_t dw[W];
        if (W == 1) {
            uint32_t d = __shfl_sync(0xFFFFFFFFu, xr[0], i) ^ __shfl_sync(0xFFFFFFFFu, yr[0], j);
#pragma unroll
            for (int q = 1; q < BP; ++q)
                d |= __shfl_sync(0xFFFFFFFFu, xr[q], i) ^ __shfl_sync(0xFFFFFFFFu, yr[q], j);
            dw[0] = d;
            sc = EM == 2 ? d : (EM == 1 ? (d & (d - 1u)) : (uint32_t)__popc(d));
        } else {
            uint32_t dist = 0;
#pragma unroll
            for (int w = 0; w < W; ++w) {
                uint32_t d = __shfl_sync(0xFFFFFFFFu, xr[w], i) ^ __shfl_sync(0xFFFFFFFFu, yr[w], j);
#pragma unroll
                for (int q = 1; q < BP; ++q)
                    d |= __shfl_sync(0xFFFFFFFFu, xr[q * W + w], i) ^
                         __shfl_sync(0xFFFFFFFFu, yr[q * W + w], j);
                dw[w] = d;
                dist += __popc(d);
            }
            sc = dist;
        }
        if (act && sc <= thr) {
            const uint4 mx = __ldg(a.meta + P.a_start + i), my = __ldg(a.meta + ystart + j);
            bool ok;
            if (JN) {
                ok = join_meta_ok<W>(mx, my, dw, P.la, P.j, P.v);
            } else if (a.sig_exact) {
                ok = ((mx.x & my.x) | (mx.y & my.y) | (mx.z & my.z)) == 0;
            } else {
                const uint32_t rx = a.urow[mx.w], ry = a.urow[my.w];
                ok = lowest_common(a.vbits, a.VW, rx, ry) == (int)P.v &&
                     lowest_common(a.jbits, a.JW, rx, ry) == (int)P.j;
            }
            rmask |= (uint32_t)ok << (p0 >> 5);
        }
    }
    // every round's edges of the lane, one bulk append for the warp
    emit_pair_bits(a, ew, lane, rmask, (uint32_t)lane, 32u, same, n, P.a_start, ystart);
    if (a.bp_cycles && lane == 0)
        atomicAdd(&a.bp_cycles[idx], (unsigned long long)(clock64() - t0));
}

// Small bin pairs of a warp: the warp claims kSmallBatch schedule positions
// with one atomic, each lane loads one of their bin pairs, and while one bin
// pair is scored the next one's records are prefetched into L1 (a small bin
// pair is otherwise a chain of dependent loads: position, bin pair, records).
constexpr uint32_t kSmallBatch = 16;

__device__ __forceinline__ BinPair shfl_binpair(const BinPair &p, int src) {
    static_assert(sizeof(BinPair) % 4 == 0, "BinPair words");
    constexpr int NWD = (int)(sizeof(BinPair) / 4);
    uint32_t w[NWD];
    memcpy(w, &p, sizeof(BinPair));
#pragma unroll
    for (int k = 0; k < NWD; ++k) w[k] = __shfl_sync(0xFFFFFFFFu, w[k], src);
    BinPair q;
    memcpy(&q, w, sizeof(BinPair));
    return q;
}

__device__ __forceinline__ void prefetch_l1(const void *p) {
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

template <int BP, int W, int EM, bool JN>
__device__ __forceinline__ void hamming_small_all(const DistArgs &a, EdgeWriter &ew, int lane,
                                                  uint64_t &pairs) {
    constexpr int R16 = (BP * W + 3) / 4;
    const uint32_t n_small = a.ctr->n_small;
    for (;;) {
        uint32_t s0 = 0;
        if (lane == 0) s0 = atomicAdd(&a.ctr->small_cursor, kSmallBatch);
        s0 = __shfl_sync(0xFFFFFFFFu, s0, 0);
        if (s0 >= n_small) break;
        const uint32_t cnt = min(kSmallBatch, n_small - s0);
        uint32_t myidx = 0;
        BinPair myP;
        memset(&myP, 0, sizeof(BinPair));
        if ((uint32_t)lane < cnt) {
            myidx = a.small_list[s0 + lane];
            myP = a.bp[myidx];
        }
        for (uint32_t g = 0; g < cnt; ++g) {
            if (g + 1 < cnt) {
                const uint32_t na = __shfl_sync(0xFFFFFFFFu, myP.a_start, g + 1);
                const uint32_t nn = __shfl_sync(0xFFFFFFFFu, myP.a_n, g + 1);
                const uint32_t nb = __shfl_sync(0xFFFFFFFFu, myP.b_start, g + 1);
                const uint32_t nm = __shfl_sync(0xFFFFFFFFu, myP.b_n, g + 1);
                const uint32_t ns = __shfl_sync(0xFFFFFFFFu, (uint32_t)myP.same, g + 1);
                if ((uint32_t)lane < nn) prefetch_l1(a.rec + (size_t)(na + lane) * R16);
                if (!ns && (uint32_t)lane < nm) prefetch_l1(a.rec + (size_t)(nb + lane) * R16);
            }
            const BinPair P = shfl_binpair(myP, (int)g);
            hamming_small<BP, W, EM, JN>(a, ew, P, __shfl_sync(0xFFFFFFFFu, myidx, g), lane, pairs);
        }
    }
}

// Tiny bin pairs (a bin with itself, at most kTinySide entries): lane l takes
// every pair of the l-th bin pair of a batch of 32, so the latency of loading
// a bin pair and its records is paid once per 32 bin pairs.  Records are read
// per pair from L1 (a tiny bin's records share one or two cache lines).
template <int BP, int W, int EM, bool JN>
__device__ __forceinline__ void hamming_tiny_all(const DistArgs &a, EdgeWriter &ew, int lane,
                                                 uint64_t &pairs) {
    constexpr int NW = BP * W;
    constexpr int R16 = (NW + 3) / 4;
    const uint32_t n_tiny = a.ctr->n_tiny;
    for (;;) {
        uint32_t s0 = 0;
        if (lane == 0) s0 = atomicAdd(&a.ctr->tiny_cursor, 32u);
        s0 = __shfl_sync(0xFFFFFFFFu, s0, 0);
        if (s0 >= n_tiny) break;
        const long long t0 = a.bp_cycles ? clock64() : 0;
        const bool act = s0 + (uint32_t)lane < n_tiny;
        uint32_t idx = 0;
        BinPair P;
        memset(&P, 0, sizeof(BinPair));
        if (act) {
            idx = a.small_list[a.small_cap - 1u - (s0 + (uint32_t)lane)];
            P = a.bp[idx];
        }
        const uint32_t n = P.a_n;
        const uint32_t np = (EM == 0 && P.eps < 0) ? 0u : n * (n - 1) / 2;
        pairs += n * (n - 1) / 2;
        const uint32_t thr = EM == 0 ? (uint32_t)max((int)P.eps, 0) : 0u;
        const uint4 *rec = a.rec + (size_t)P.a_start * R16;
        // pass 1: each lane scores its bin pair's pairs and keeps the edges
        // as bits of pair indices (at most 28 pairs)
        static_assert(kTinySide * (kTinySide - 1) / 2 <= 32, "tiny pair mask");
        uint32_t emask = 0;
        for (uint32_t p = 0; p < np; ++p) {
            uint32_t i, j;
            small_pair(p, true, n, i, j);
            uint32_t xw[4 * R16], yw[4 * R16];
#pragma unroll
            for (int q = 0; q < R16; ++q) {
                const uint4 u = __ldg(rec + (size_t)i * R16 + q), v = __ldg(rec + (size_t)j * R16 + q);
                xw[4 * q] = u.x; xw[4 * q + 1] = u.y; xw[4 * q + 2] = u.z; xw[4 * q + 3] = u.w;
                yw[4 * q] = v.x; yw[4 * q + 1] = v.y; yw[4 * q + 2] = v.z; yw[4 * q + 3] = v.w;
            }
            uint32_t dw[W], dist = 0;
#pragma unroll
            for (int w = 0; w < W; ++w) {
                uint32_t d = xw[w] ^ yw[w];
#pragma unroll
                for (int q = 1; q < BP; ++q) d |= xw[q * W + w] ^ yw[q * W + w];
                dw[w] = d;
                dist += __popc(d);
            }
            const uint32_t sc = EM == 2 ? dw[0] : (EM == 1 ? (dw[0] & (dw[0] - 1u)) : dist);
            if (sc > thr) continue;
            const uint4 mx = __ldg(a.meta + P.a_start + i), my = __ldg(a.meta + P.a_start + j);
            bool ok;
            if (JN) {
                ok = join_meta_ok<W>(mx, my, dw, P.la, P.j, P.v);
            } else if (a.sig_exact) {
                ok = ((mx.x & my.x) | (mx.y & my.y) | (mx.z & my.z)) == 0;
            } else {
                const uint32_t rx = a.urow[mx.w], ry = a.urow[my.w];
                ok = lowest_common(a.vbits, a.VW, rx, ry) == (int)P.v &&
                     lowest_common(a.jbits, a.JW, rx, ry) == (int)P.j;
            }
            emask |= (uint32_t)ok << p;
        }
        // pass 2: one bulk append for the warp
        emit_pair_bits(a, ew, lane, emask, 0u, 1u, true, n, P.a_start, P.a_start);
        if (a.bp_cycles) {
            // the batch's cycles, shared out by pairs (every lane takes part in
            // the reduction; lanes past the list's end hold n = 0)
            const uint32_t mine = n * (n - 1) / 2;
            const uint32_t tot = __reduce_add_sync(0xFFFFFFFFu, mine);
            const unsigned long long dt = (unsigned long long)(clock64() - t0);
            if (act) atomicAdd(&a.bp_cycles[idx], dt * mine / (tot ? tot : 1u));
        }
    }
}

// Deferred hits: the Hamming loop only records, per lane, (y index in the staged
// chunk, hit bits) in a small shared-memory queue; the queue is drained here when
// a lane's queue is full or the chunk ends, with every lane taking part.
constexpr int kHitQ = 8;   // queued (y, hits) records per lane
constexpr uint32_t kLevQ = 256;          // queued candidate pairs per warp (Levenshtein)
constexpr uint32_t kOff = 0x40000000u;   // score of a masked x-entry (never a hit)

// The queue holds (y index in the chunk, hit bits) per lane.  Hits are
// compacted over the whole warp before they are written: each lane first keeps
// the bits of its own queue that are edges (pair order and canonical bin),
// then one warp scan gives every lane its place in one bulk append.
template <bool JN>
__device__ __forceinline__ void drain_hits(const DistArgs &a, EdgeWriter &ew, uint32_t *q,
                                        uint32_t qn, const uint4 *xm, const uint4 *ym,
                                        uint32_t xbase, uint32_t ypos0, uint32_t same,
                                        uint32_t v, uint32_t j, int lane) {
    uint32_t c = 0;
    for (uint32_t k = 0; k < qn; ++k) {
        const uint32_t e = q[k * 32 + lane];
        const uint32_t t = e >> 8, ypos = ypos0 + t;
        const uint4 my = ym[t];
        uint32_t keep = 0;
        for (uint32_t b = e & 0xFFu; b; b &= b - 1) {
            const uint32_t r = (uint32_t)__ffs(b) - 1u;
            const uint32_t xpos = xbase + 32u * r + (uint32_t)lane;
            bool ok = !(same && ypos <= xpos);
            if (ok && !JN) {
                const uint4 m = xm[32 * r + lane];
                if (a.sig_exact) {
                    ok = ((m.x & my.x) | (m.y & my.y) | (m.z & my.z)) == 0;
                } else {
                    const uint32_t rx = a.urow[m.w], ry = a.urow[my.w];
                    ok = lowest_common(a.vbits, a.VW, rx, ry) == (int)v &&
                         lowest_common(a.jbits, a.JW, rx, ry) == (int)j;
                }
            }
            keep |= (uint32_t)ok << r;   // the join was checked when the hit was queued
        }
        q[k * 32 + lane] = (t << 8) | keep;
        c += (uint32_t)__popc(keep);
    }
    uint32_t incl = c;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t n = __shfl_up_sync(0xFFFFFFFFu, incl, d);
        if (lane >= d) incl += n;
    }
    const uint32_t T = __shfl_sync(0xFFFFFFFFu, incl, 31);
    if (T == 0) return;
    const EdgeWriter::Bulk bk = ew.reserve(a, lane, T);
    uint32_t i = incl - c;
    for (uint32_t k = 0; k < qn; ++k) {
        const uint32_t e = q[k * 32 + lane];
        const uint32_t uy = ym[e >> 8].w;
        for (uint32_t b = e & 0xFFu; b; b &= b - 1) {
            const uint32_t r = (uint32_t)__ffs(b) - 1u;
            const uint32_t ux = xm[32 * r + lane].w;
            put_edge(a, ew.slot_of(bk, i++), min(ux, uy), max(ux, uy));
        }
    }
}

// The y loop of one Hamming unit.  FULL: every r-block of the lane's x-entries
// is inside the unit, so all RX chains run without branches; otherwise the
// chains of r-blocks past the unit's end are skipped.
template <int BP, int W, int RX, int EM, bool FULL, bool JN>
__device__ __forceinline__ void hamming_unit_y(const DistArgs &a, EdgeWriter &ew, const Unit &U,
                                               const uint32_t (&x)[RX][BP * W],
                                               const uint32_t (&vmask)[RX], uint32_t valid,
                                               uint4 *sy, uint4 *sym, uint4 *sxm, uint32_t *shq,
                                               const uint32_t *sseg, int lane) {
    constexpr int NW = BP * W;
    constexpr int R16 = (NW + 3) / 4;
    const uint32_t rb = (U.nx + 31) >> 5;   // r-blocks holding entries
    const uint32_t jk = U.P.v;              // segment join: the group's segment
    // a pair is a hit iff its score <= thr (score: d&(d-1) for eps 1, d for
    // eps 0, the popcount otherwise); masked entries score >= kOff
    const uint32_t thr = EM == 0 ? (uint32_t)max(U.P.eps, 0) : 0u;
    const bool neg = EM == 0 && U.P.eps < 0;       // no pair can be a neighbour
    const uint32_t same = U.P.same;
    const uint32_t yrow0 = (same ? U.P.a_start : U.P.b_start) + U.ybase;
    // same bin: y-entries at or before the first x-entry pair with nothing
    const uint32_t y0 = (same && U.xbase >= U.ybase) ? min(U.ny, U.xbase - U.ybase + 1) : 0u;
    for (uint32_t yb = y0; yb < U.ny && !neg; yb += kYB) {
        const uint32_t nb = min((uint32_t)kYB, U.ny - yb);
        const uint4 *src = a.rec + (size_t)(yrow0 + yb) * R16;
        for (uint32_t t = lane; t < nb * R16; t += 32) sy[t] = __ldg(src + t);
        for (uint32_t t = lane; t < nb; t += 32) sym[t] = __ldg(a.meta + yrow0 + yb + t);
        __syncwarp();
        uint32_t qn = 0;
        // y-entries inside the unit's own x range (same bin) need the mask of the
        // x-entries before them; they come first in the chunk (y ascending, all
        // after xbase), the rest pair with every x-entry of the unit
        uint32_t tdiag = 0;
        if (same && U.ybase + yb < U.xbase + U.nx)
            tdiag = min(nb, U.xbase + U.nx - (U.ybase + yb));
        auto score = [&](uint32_t t, uint32_t (&sc)[RX]) {
            uint32_t y[NW];
#pragma unroll
            for (int q = 0; q < R16; ++q) {
                const uint4 v = sy[t * R16 + q];
                const uint32_t w4[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (4 * q + e < NW) y[4 * q + e] = w4[e];
            }
            // FULL: all RX chains without branches (independent, interleaved);
            // otherwise only the r-blocks that hold entries (warp-uniform test)
#pragma unroll
            for (int r = 0; r < RX; ++r) {
                if (!FULL && r >= rb) { sc[r] = kOff; continue; }
                if (W == 1) {
                    uint32_t d = x[r][0] ^ y[0];
#pragma unroll
                    for (int p = 1; p < BP; ++p) d |= x[r][p] ^ y[p];
                    sc[r] = (EM == 2 ? d : (EM == 1 ? (d & (d - 1u)) : (uint32_t)__popc(d))) | vmask[r];
                } else {
                    uint32_t dist = 0;
#pragma unroll
                    for (int w = 0; w < W; ++w) {
                        uint32_t d = x[r][w] ^ y[w];
#pragma unroll
                        for (int p = 1; p < BP; ++p) d |= x[r][p * W + w] ^ y[p * W + w];
                        dist += __popc(d);
                    }
                    sc[r] = dist | vmask[r];
                }
            }
        };
        auto record = [&](uint32_t t, const uint32_t (&sc)[RX]) {
            // with exact signatures a hit outside its canonical bin is dropped
            // here: sig_x & sig_y must be empty
            const uint4 ym = sym[t];
            uint32_t hit = 0;
#pragma unroll
            for (int r = 0; r < RX; ++r)
                if (sc[r] <= thr) {
                    bool ok = true;
                    if (JN) {
                        // segment join: V and J sets intersect, the group's
                        // segment is identical and no lower one is (masks of
                        // segment kk, word w at sseg[4 kk + w])
                        const uint4 m = sxm[32 * r + lane];
                        ok = ((m.x & ym.x) | (m.y & ym.y)) != 0 && (m.z & ym.z & 0x3FFFFFFFu) != 0;
                        if (ok) {
                            const uint32_t *yw = reinterpret_cast<const uint32_t *>(sy + t * R16);
                            uint32_t dk = 0, l0 = 0, l1 = 0, l2 = 0;
#pragma unroll
                            for (int w = 0; w < W; ++w) {
                                uint32_t d = x[r][w] ^ yw[w];
#pragma unroll
                                for (int p = 1; p < BP; ++p) d |= x[r][p * W + w] ^ yw[p * W + w];
                                dk |= d & sseg[4 * jk + w];
                                l0 |= d & sseg[w];
                                l1 |= d & sseg[4 + w];
                                l2 |= d & sseg[8 + w];
                            }
                            ok = dk == 0 && (jk < 1 || l0 != 0) && (jk < 2 || l1 != 0) &&
                                 (jk < 3 || l2 != 0);
                        }
                    } else if (a.sig_exact) {
                        const uint4 m = sxm[32 * r + lane];
                        ok = ((m.x & ym.x) | (m.y & ym.y) | (m.z & ym.z)) == 0;
                    }
                    hit |= (uint32_t)ok << r;
                }
            hit &= valid;
            if (hit) shq[qn++ * 32 + lane] = (t << 8) | hit;
        };
        auto drain_if_full = [&](uint32_t room) {
            if (__any_sync(0xFFFFFFFFu, qn + room > (uint32_t)kHitQ)) {
                __syncwarp();
                drain_hits<JN>(a, ew, shq, qn, sxm, sym, U.xbase, U.ybase + yb, same, U.P.v, U.P.j, lane);
                qn = 0;
                __syncwarp();
            }
        };
        for (uint32_t t = 0; t < tdiag; ++t) {
            uint32_t sc[RX];
            score(t, sc);
            const uint32_t nact = U.ybase + yb + t - U.xbase;   // x-entries before y
#pragma unroll
            for (int r = 0; r < RX; ++r)
                if ((uint32_t)r * 32 + lane >= nact) sc[r] |= kOff;
            uint32_t z = sc[0];
#pragma unroll
            for (int r = 1; r < RX; ++r) z = min(z, sc[r]);
            if (z <= thr) record(t, sc);
            drain_if_full(1);
        }
        uint32_t t = tdiag;
        for (; t + 1 < nb; t += 2) {      // two y-entries per step: twice the chains
            uint32_t sa[RX], sb[RX];
            score(t, sa);
            score(t + 1, sb);
            uint32_t za = sa[0], zb = sb[0];
#pragma unroll
            for (int r = 1; r < RX; ++r) { za = min(za, sa[r]); zb = min(zb, sb[r]); }
            if (za <= thr) record(t, sa);
            if (zb <= thr) record(t + 1, sb);
            drain_if_full(2);
        }
        if (t < nb) {
            uint32_t sc[RX];
            score(t, sc);
            uint32_t z = sc[0];
#pragma unroll
            for (int r = 1; r < RX; ++r) z = min(z, sc[r]);
            if (z <= thr) record(t, sc);
        }
        if (__any_sync(0xFFFFFFFFu, qn)) {
            __syncwarp();
            drain_hits<JN>(a, ew, shq, qn, sxm, sym, U.xbase, U.ybase + yb, same, U.P.v, U.P.j, lane);
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Hamming, fast path.  BP planes x W words per record; RX x-entries per lane.
// EM: 0 = popcount test, 1 = eps == 1 (d & (d-1)) == 0, 2 = eps == 0.
// ---------------------------------------------------------------------------
template <int BP, int W, int RX, int EM, bool JN>
__global__ void __launch_bounds__(kWarps * 32, (W == 1 && RX <= 2 ? 6 : (W == 1 && RX <= 4 ? 5 : 4)))
k_hamming(DistArgs a) {
    constexpr int NW = BP * W;                 // words per record used
    constexpr int R16 = (NW + 3) / 4;          // 16-byte words per record
    __shared__ uint4 sy[kWarps][kYB * R16];
    __shared__ uint4 sym[kWarps][kYB];            // y side records
    __shared__ uint4 sxm[kWarps][32 * RX];        // x side records
    __shared__ uint32_t shq[kWarps][kHitQ * 32];  // deferred hits
    __shared__ uint32_t sseg[kWarps][16];         // segment join: masks of segment kk, word w
    static_assert(RX <= 8 && kYB < (1 << 24), "hit record layout");
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t n_units = a.ctr->n_units, n_bp = a.ctr->n_binpairs;
    EdgeWriter ew;
    ew.init();
    uint64_t pairs = 0;
    Unit U;
    while (next_unit(a, n_units, n_bp, lane, U)) {
        uint32_t x[RX][NW];
        uint32_t vmask[RX];          // kOff for x-entries outside the unit
        uint32_t valid = 0;
#pragma unroll
        for (int r = 0; r < RX; ++r) {
            const uint32_t xi = (uint32_t)r * 32 + lane;
            const bool ok = xi < U.nx;
            valid |= (uint32_t)ok << r;
            vmask[r] = ok ? 0u : kOff;
            const uint4 *src = a.rec + (size_t)(U.P.a_start + U.xbase + (ok ? xi : 0)) * R16;
#pragma unroll
            for (int q = 0; q < R16; ++q) {
                const uint4 v = __ldg(src + q);
                const uint32_t w4[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (4 * q + e < NW) x[r][4 * q + e] = w4[e];
            }
            if (ok) pairs += unit_pairs(U, U.xbase + xi);
            sxm[wid][xi] = __ldg(a.meta + U.P.a_start + U.xbase + (ok ? xi : 0));
        }
        if (JN && lane < 16) {
            // segment kk = lane / 4 of length la split into j segments, word w = lane % 4
            const uint32_t kk = (uint32_t)lane >> 2, w = (uint32_t)lane & 3u;
            const uint32_t L = U.P.la, S = U.P.j;
            const uint32_t lo = kk < S ? kk * L / S : 0u, hi = kk < S ? (kk + 1) * L / S : 0u;
            const uint32_t a0 = max(lo, 32u * w), a1 = min(hi, 32u * w + 32u);
            uint32_t m = 0;
            if (a0 < a1) {
                const uint32_t n = a1 - a0;
                m = (n >= 32 ? 0xFFFFFFFFu : ((1u << n) - 1u)) << (a0 - 32u * w);
            }
            sseg[wid][lane] = m;
        }
        __syncwarp();
        if (U.nx == (uint32_t)(32 * RX))
            hamming_unit_y<BP, W, RX, EM, true, JN>(a, ew, U, x, vmask, valid, sy[wid], sym[wid], sxm[wid],
                                                shq[wid], sseg[wid], lane);
        else
            hamming_unit_y<BP, W, RX, EM, false, JN>(a, ew, U, x, vmask, valid, sy[wid], sym[wid],
                                                 sxm[wid], shq[wid], sseg[wid], lane);
        log_unit(a, U, lane);
    }
    // then the small bin pairs (they also fill the tail of the tiled work)
    hamming_small_all<BP, W, EM, JN>(a, ew, lane, pairs);
    hamming_tiny_all<BP, W, EM, JN>(a, ew, lane, pairs);
    finish(a, ew, pairs, lane);
}

// ---------------------------------------------------------------------------
// Levenshtein, fast path.  Codes records (one byte per residue, RS bytes);
// pattern <= 32*W residues; RX patterns per lane.
// ---------------------------------------------------------------------------
template <int W, int RX>
__global__ void __launch_bounds__(kWarps * 32, 4)
k_levenshtein(DistArgs a) {
    extern __shared__ uint32_t smem[];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t A = a.A;
    const uint32_t peq_words = RX * A * W * 32;          // per warp
    const uint32_t ybuf_words = kYB * a.rs16 * 4;        // per warp
    const uint32_t meta_words = (kYB + 32 * RX) * 4;     // per warp
    constexpr uint32_t kCW = 8;                          // count words: 4 codes each, A <= 32
    uint32_t *peq = smem + wid * (peq_words + ybuf_words + meta_words + kYB +
                                  kCW * (kYB + 32 * RX) + kLevQ);
    uint4 *sy = reinterpret_cast<uint4 *>(peq + peq_words);
    uint4 *sym = sy + kYB * a.rs16;                      // y side records
    uint4 *sxm = sym + kYB;                              // x side records
    uint32_t *spres = reinterpret_cast<uint32_t *>(sxm + 32 * RX);   // y residue sets
    uint32_t *sycnt = spres + kYB;                       // y residue counts [kYB][kCW]
    uint32_t *sxcnt = sycnt + kCW * kYB;                 // x residue counts [RX][kCW][32]
    uint32_t *lq = sxcnt + kCW * 32 * RX;                // queued candidate pairs [kLevQ]
    const uint32_t cw = (A + 3) / 4;                     // count words in use
    const uint32_t n_units = a.ctr->n_units, n_bp = a.ctr->n_binpairs;
    EdgeWriter ew;
    ew.init();
    uint64_t pairs = 0, cols = 0;
    Unit U;
    while (next_unit(a, n_units, n_bp, lane, U)) {
        const int m = U.P.la, n = U.P.lb, eps = U.P.eps;
        const int dg = n - m;
        uint32_t xpos[RX];
        bool xval[RX];
        uint32_t xpres[RX];        // set of residue codes of each x-entry (A <= 32)
        // Peq[r][c][w][lane]
        for (uint32_t k = 0; k < (uint32_t)RX * A * W; ++k) peq[k * 32 + lane] = 0u;
        for (uint32_t k = 0; k < (uint32_t)RX * kCW; ++k) sxcnt[k * 32 + lane] = 0u;
        __syncwarp();
#pragma unroll
        for (int r = 0; r < RX; ++r) {
            xpos[r] = U.xbase + r * 32 + lane;
            xval[r] = xpos[r] < U.xbase + U.nx;
            xpres[r] = 0;
            sxm[r * 32 + lane] = __ldg(a.meta + U.P.a_start + (xval[r] ? xpos[r] : U.xbase));
            if (xval[r]) {
                pairs += unit_pairs(U, xpos[r]);
                const uint8_t *codes =
                    reinterpret_cast<const uint8_t *>(a.rec + (size_t)(U.P.a_start + xpos[r]) * a.rs16);
                for (int i = 0; i < m; ++i) {
                    const uint32_t c = __ldg(codes + i);
                    peq[((r * A + c) * W + (i >> 5)) * 32 + lane] |= 1u << (i & 31);
                    xpres[r] |= 1u << c;
                    sxcnt[(r * kCW + (c >> 2)) * 32 + lane] += 1u << (8 * (c & 3));
                }
            }
        }
        uint32_t xcnt[RX][kCW];    // residue counts, one byte per code (lengths < 256)
#pragma unroll
        for (int r = 0; r < RX; ++r)
#pragma unroll
            for (uint32_t k = 0; k < kCW; ++k) xcnt[r][k] = sxcnt[(r * kCW + k) * 32 + lane];
        // An edit changes the set of residues present by at most two (a
        // substitution drops one and adds one, an indel one), so a pair whose
        // sets differ in more than 2*eps residues is not within eps.  Likewise
        // an edit changes the residue counts by at most 2 in total (sum of
        // absolute differences), so a pair with that sum above 2*eps is not.
        const int pres_max = 2 * eps;
        __syncwarp();
        const uint32_t yrow0 = (U.P.same ? U.P.a_start : U.P.b_start) + U.ybase;
        for (uint32_t yb = 0; yb < U.ny; yb += kYB) {
            const uint32_t nb = min((uint32_t)kYB, U.ny - yb);
            const uint4 *src = a.rec + (size_t)(yrow0 + yb) * a.rs16;
            for (uint32_t t = lane; t < nb * a.rs16; t += 32) sy[t] = __ldg(src + t);
            for (uint32_t t = lane; t < nb; t += 32) sym[t] = __ldg(a.meta + yrow0 + yb + t);
            __syncwarp();
            for (uint32_t t = lane; t < nb; t += 32) {
                const uint8_t *yc = reinterpret_cast<const uint8_t *>(sy + t * a.rs16);
                uint32_t *yk = sycnt + t * kCW;
#pragma unroll
                for (uint32_t k = 0; k < kCW; ++k) yk[k] = 0u;
                uint32_t pr = 0;
                for (int j = 0; j < n; ++j) {
                    const uint32_t c = yc[j];
                    pr |= 1u << c;
                    yk[c >> 2] += 1u << (8 * (c & 3));
                }
                spres[t] = pr;
            }
            __syncwarp();
            // 1. filters: the pairs that survive go to a warp queue as
            //    (owner lane, r, t), so the DP below runs with every lane busy
            uint32_t qn = 0;
            for (uint32_t t = 0; t < nb; ++t) {
                const uint32_t ypos = U.ybase + yb + t;
                const uint32_t ypres = spres[t];
                uint32_t ycnt[kCW];
#pragma unroll
                for (uint32_t k = 0; k < kCW; ++k) ycnt[k] = k < cw ? sycnt[t * kCW + k] : 0u;
#pragma unroll
                for (int r = 0; r < RX; ++r) {
                    bool alive = xval[r] && !(U.P.same && ypos <= xpos[r]) &&
                                 __popc(xpres[r] ^ ypres) <= pres_max;
                    if (alive) {
                        uint32_t sad = 0;
#pragma unroll
                        for (uint32_t k = 0; k < kCW; ++k) sad = __vsadu4(xcnt[r][k], ycnt[k]) + sad;
                        alive = (int)sad <= pres_max;
                    }
                    const uint32_t mk = __ballot_sync(0xFFFFFFFFu, alive);
                    if (alive) lq[qn + __popc(mk & lanemask_lt())] = (uint32_t)lane | ((uint32_t)r << 5) | (t << 8);
                    qn += __popc(mk);
                }
                if (qn > kLevQ - 32 * RX || t + 1 == nb) {
                    __syncwarp();
                    // 2. bit-parallel DP of the queued pairs, 32 at a time
                    for (uint32_t k0 = 0; k0 < qn; k0 += 32) {
                        const bool has = k0 + lane < qn;
                        const uint32_t it = has ? lq[k0 + lane] : 0u;
                        const uint32_t owner = it & 31u, r = (it >> 5) & 7u, tt = it >> 8;
                        const uint8_t *yc = reinterpret_cast<const uint8_t *>(sy + tt * a.rs16);
                        uint32_t Pv[W], Mv[W];
#pragma unroll
                        for (int w = 0; w < W; ++w) { Pv[w] = 0xFFFFFFFFu; Mv[w] = 0u; }
                        bool live = has;
                        for (int j = 0; j < n; ++j) {
                            const uint32_t c = yc[j];
                            const uint32_t *pe = peq + ((r * A + c) * W) * 32 + owner;
                            if (W == 1) {
                                myers_step1(Pv[0], Mv[0], pe[0]);
                            } else {
                                int h = 1;
#pragma unroll
                                for (int w = 0; w < W; ++w) h = myers_block(Pv[w], Mv[w], pe[w * 32], h);
                            }
                            if ((j & 3) == 3) {
                                const int col = j + 1;
                                const int i = col - dg;
                                if (i >= 0 && i <= m) {
                                    if (live && myers_value<W>(Pv, Mv, i, col) > eps) {
                                        live = false;
                                        cols += (uint32_t)col;
                                    }
                                    if (!__any_sync(0xFFFFFFFFu, live)) break;
                                }
                            }
                        }
                        bool hit = false;
                        if (live) {
                            cols += (uint32_t)n;
                            hit = myers_value<W>(Pv, Mv, m, n) <= eps;
                        }
                        if (__any_sync(0xFFFFFFFFu, hit)) {
                            bool ok = hit;
                            const uint4 mx = sxm[r * 32 + owner], my = sym[tt];
                            if (ok) {
                                if (a.sig_exact) {
                                    ok = ((mx.x & my.x) | (mx.y & my.y) | (mx.z & my.z)) == 0;
                                } else {
                                    const uint32_t rx = a.urow[mx.w], ry = a.urow[my.w];
                                    ok = lowest_common(a.vbits, a.VW, rx, ry) == (int)U.P.v &&
                                         lowest_common(a.jbits, a.JW, rx, ry) == (int)U.P.j;
                                }
                            }
                            ew.append(a, lane, ok, min(mx.w, my.w), max(mx.w, my.w));
                        }
                    }
                    qn = 0;
                    __syncwarp();
                }
            }
            __syncwarp();
        }
        log_unit(a, U, lane);
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) cols += __shfl_xor_sync(0xFFFFFFFFu, cols, d);
    if (lane == 0 && cols) atomicAdd(&a.ctr->lev_columns, (unsigned long long)cols);
    finish(a, ew, pairs, lane);
}

// ---------------------------------------------------------------------------
// Generic path (more than 32 distinct residues, or longer than 128): one pair
// per lane, code bytes read from global memory.  Hamming stops once the count
// exceeds eps (cuda/PSDBSCAN.hcu:628-636); Levenshtein is a DP restricted to
// the diagonals |j - i| <= eps with a cut-off once a row exceeds eps.
// ---------------------------------------------------------------------------
__device__ bool generic_lev_leq(const uint8_t *x, int m, const uint8_t *y, int n, int eps) {
    if (eps < 0) return false;
    if (m - n > eps || n - m > eps) return false;
    // D restricted to the band; values above eps are clamped to eps+1
    short row[2][kGenericMaxLen + 1];
    const int big = eps + 1;
    for (int j = 0; j <= n; ++j) row[0][j] = (short)min(j, big);
    int cur = 0;
    for (int i = 1; i <= m; ++i) {
        const int nx = cur ^ 1;
        const int jlo = max(1, i - eps), jhi = min(n, i + eps);
        row[nx][0] = (short)min(i, big);
        if (jlo > 1) row[nx][jlo - 1] = (short)big;
        int rmin = row[nx][0];
        for (int j = jlo; j <= jhi; ++j) {
            int v = row[cur][j - 1] + (x[i - 1] != y[j - 1]);
            const int up = (j <= i - 1 + eps) ? row[cur][j] + 1 : big;
            const int left = row[nx][j - 1] + 1;
            v = min(v, min(up, left));
            v = min(v, big);
            row[nx][j] = (short)v;
            rmin = min(rmin, v);
        }
        if (jhi < n) row[nx][jhi + 1] = (short)big;
        cur = nx;
        if (rmin > eps) return false;
    }
    return row[cur][n] <= eps;
}

template <bool HAM>
__global__ void __launch_bounds__(kWarps * 32)
k_generic(DistArgs a) {
    const int lane = threadIdx.x & 31;
    const uint32_t n_units = a.ctr->n_units, n_bp = a.ctr->n_binpairs;
    EdgeWriter ew;
    ew.init();
    uint64_t pairs = 0;
    Unit U;
    while (next_unit(a, n_units, n_bp, lane, U)) {
        const int m = U.P.la, n = U.P.lb, eps = U.P.eps;
        const uint32_t yrow0 = (U.P.same ? U.P.a_start : U.P.b_start) + U.ybase;
        const uint32_t total = U.nx * U.ny;
        for (uint32_t p0 = 0; p0 < total; p0 += 32) {
            const uint32_t p = p0 + lane;
            bool ok = false;
            uint32_t ux = 0, uy = 0;
            if (p < total) {
                const uint32_t xi = p / U.ny, yi = p % U.ny;
                const uint32_t xpos = U.xbase + xi, ypos = U.ybase + yi;
                if (!(U.P.same && ypos <= xpos)) {
                    ++pairs;
                    const uint8_t *xc =
                        reinterpret_cast<const uint8_t *>(a.rec + (size_t)(U.P.a_start + xpos) * a.rs16);
                    const uint8_t *yc =
                        reinterpret_cast<const uint8_t *>(a.rec + (size_t)(yrow0 + yi) * a.rs16);
                    if (HAM) {
                        int d = 0;
                        ok = eps >= 0;
                        for (int k = 0; k < m && ok; ++k)
                            if (xc[k] != yc[k] && ++d > eps) ok = false;
                    } else {
                        ok = generic_lev_leq(xc, m, yc, n, eps);
                    }
                    if (ok) {
                        ux = a.ent_uid[U.P.a_start + xpos];
                        uy = a.ent_uid[yrow0 + yi];
                        ok = canonical(a, U.P, ux, uy);
                    }
                }
            }
            ew.append(a, lane, ok, min(ux, uy), max(ux, uy));
        }
        log_unit(a, U, lane);
    }
    finish(a, ew, pairs, lane);
}

// ---------------------------------------------------------------------------
// Admissible-pair count (the throughput metric's numerator): unique pairs that
// share a bin (V and J overlap) with an admissible length gap, each counted in
// its canonical bin only.  One pair per lane; run once per workload.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kWarps * 32)
k_count_admissible(DistArgs a) {
    const int lane = threadIdx.x & 31;
    const uint32_t n_units = a.ctr->n_units, n_bp = a.ctr->n_binpairs;
    unsigned long long cnt = 0;
    Unit U;
    while (next_unit(a, n_units, n_bp, lane, U)) {
        const uint32_t yrow0 = (U.P.same ? U.P.a_start : U.P.b_start) + U.ybase;
        const uint32_t total = U.nx * U.ny;
        for (uint32_t p = lane; p < total; p += 32) {
            const uint32_t xi = p / U.ny, yi = p % U.ny;
            const uint32_t xpos = U.xbase + xi, ypos = U.ybase + yi;
            if (U.P.same && ypos <= xpos) continue;
            if (U.P.eps < 0) continue;
            const uint32_t ux = a.ent_uid[U.P.a_start + xpos], uy = a.ent_uid[yrow0 + yi];
            cnt += canonical(a, U.P, ux, uy);
        }
    }
    const uint32_t n_small = a.ctr->n_small, n_tiny = a.ctr->n_tiny;
    for (;;) {
        uint32_t s = 0;
        if (lane == 0) s = atomicAdd(&a.ctr->small_cursor, 1u);
        s = __shfl_sync(0xFFFFFFFFu, s, 0);
        if (s >= n_small + n_tiny) break;
        const uint32_t sidx = s < n_small ? a.small_list[s] : a.small_list[a.small_cap - 1u - (s - n_small)];
        const BinPair P = a.bp[sidx];
        if (P.eps < 0) continue;
        const bool same = P.same != 0;
        const uint32_t ystart = same ? P.a_start : P.b_start;
        const uint32_t npairs = same ? P.a_n * (P.a_n - 1) / 2 : P.a_n * P.b_n;
        for (uint32_t p = lane; p < npairs; p += 32) {
            uint32_t i, j;
            small_pair(p, same, P.a_n, i, j);
            cnt += canonical(a, P, a.ent_uid[P.a_start + i], a.ent_uid[ystart + j]);
        }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) cnt += __shfl_xor_sync(0xFFFFFFFFu, cnt, d);
    if (lane == 0 && cnt) atomicAdd(&a.ctr->admissible_pairs, cnt);
}

template <typename K>
int occupancy_grid(K kernel, size_t smem) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kWarps * 32, smem);
    if (per_sm < 1) per_sm = 1;
    return per_sm * sm_count();
}

template <typename K>
void run(K kernel, const DistArgs &a, size_t smem, int grid, cudaStream_t s) {
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (grid <= 0) grid = occupancy_grid(kernel, smem);
    kernel<<<grid, kWarps * 32, smem, s>>>(a);
}

// The segment join and the buckets are separate instantiations, so the
// bucket path's hot loop carries none of the join's per-hit tests (and the
// instruction cache holds one of them, not both).
template <int BP, int W, int RX, bool JN>
void run_hamming_jn(const Plan &P, const DistArgs &a, int grid, cudaStream_t s) {
    if (P.hamming_eps_mode == 2) run(k_hamming<BP, W, RX, 2, JN>, a, 0, grid, s);
    else if (P.hamming_eps_mode == 1 && W == 1) run(k_hamming<BP, W, RX, 1, JN>, a, 0, grid, s);
    else run(k_hamming<BP, W, RX, 0, JN>, a, 0, grid, s);
}

template <int BP, int W, int RX>
void run_hamming(const Plan &P, const DistArgs &a, int grid, cudaStream_t s) {
    if (P.join) run_hamming_jn<BP, W, RX, true>(P, a, grid, s);
    else run_hamming_jn<BP, W, RX, false>(P, a, grid, s);
}

}  // namespace

static DistArgs make_args(const Plan &P, const Buffers &B) {
    DistArgs a;
    a.bp = B.bp_sorted;
    a.unit_base = B.bp_units;
    a.rec = B.ent_rec;
    a.ent_uid = B.ent_uid;
    a.urow = B.urow;
    a.vbits = B.vbits; a.jbits = B.jbits;
    a.VW = P.VW; a.JW = P.JW;
    a.rs16 = P.RS / 16;
    a.TX = P.TX; a.TY = P.TY; a.q = P.TY / P.TX;
    a.A = P.A;
    a.edges = B.edges;
    a.cap_edges = P.cap_edges;
    a.ctr = B.ctr;
    a.bp_cycles = B.bp_cycles;   // set only while profiling
    a.bp_hits = B.bp_hits;
    a.meta = B.ent_meta;
    a.sig_exact = (P.sig_exact && !P.join) ? 1 : 0;
    a.small_list = B.bp_small;
    a.small_cap = (uint32_t)P.cap_binpairs + 1u;
    a.join = P.join ? 1 : 0;
    a.sink = kSinkEdges;
    a.cnt = B.cnt;
    a.ucopies = B.ucopies;
    a.ucore = B.ucore;
    a.parent = B.parent;
    a.bmin = B.bmin;
    return a;
}

void launch_count_admissible(const Plan &P, const Buffers &B, cudaStream_t s) {
    DistArgs a = make_args(P, B);
    cudaMemsetAsync(&B.ctr->unit_cursor, 0, sizeof(uint32_t), s);
    cudaMemsetAsync(&B.ctr->small_cursor, 0, sizeof(uint32_t), s);
    cudaMemsetAsync(&B.ctr->tiny_cursor, 0, sizeof(uint32_t), s);
    run(k_count_admissible, a, 0, 0, s);
}

const char *distance_variant_name(const Plan &P) {
    if (!P.fast) return P.hamming ? "k_generic<hamming>" : "k_generic<levenshtein>";
    return P.hamming ? "k_hamming" : "k_levenshtein";
}

void launch_distance(const Plan &P, const Buffers &B, int grid, cudaStream_t s, uint32_t sink) {
    DistArgs a = make_args(P, B);
    a.sink = sink;
    if (sink != kSinkEdges) {   // no list: nothing to overflow
        a.edges = nullptr;
        a.cap_edges = ~0ull;
    }
    cudaMemsetAsync(&B.ctr->unit_cursor, 0, sizeof(uint32_t), s);
    cudaMemsetAsync(&B.ctr->small_cursor, 0, sizeof(uint32_t), s);
    cudaMemsetAsync(&B.ctr->tiny_cursor, 0, sizeof(uint32_t), s);
    if (!P.fast) {
        if (P.hamming) run(k_generic<true>, a, 0, grid, s);
        else run(k_generic<false>, a, 0, grid, s);
        return;
    }
    if (P.hamming) {
        const int RX = (int)P.RX;
        if (P.B <= 2) {
            switch (P.W) {
                case 1:
                    if (RX == 2 && P.join) run_hamming_jn<2, 1, 2, true>(P, a, grid, s);
                    else if (RX == 8) run_hamming<2, 1, 8>(P, a, grid, s);
                    else run_hamming<2, 1, 4>(P, a, grid, s);
                    break;
                case 2: run_hamming<2, 2, 4>(P, a, grid, s); break;
                case 3: run_hamming<2, 3, 4>(P, a, grid, s); break;
                default: run_hamming<2, 4, 4>(P, a, grid, s); break;
            }
        } else {
            switch (P.W) {
                case 1:
                    if (RX == 2 && P.join) run_hamming_jn<5, 1, 2, true>(P, a, grid, s);
                    else if (RX == 8) run_hamming<5, 1, 8>(P, a, grid, s);
                    else run_hamming<5, 1, 4>(P, a, grid, s);
                    break;
                case 2: run_hamming<5, 2, 4>(P, a, grid, s); break;
                case 3: run_hamming<5, 3, 4>(P, a, grid, s); break;
                default: run_hamming<5, 4, 4>(P, a, grid, s); break;
            }
        }
        return;
    }
    const size_t smem = (size_t)kWarps * ((size_t)P.RX * P.A * P.W * 32 * 4 + (size_t)kYB * P.RS +
                                          16 * ((size_t)kYB + 32 * P.RX) + 4 * (size_t)kYB +
                                          4 * 8 * ((size_t)kYB + 32 * P.RX) + 4 * (size_t)kLevQ);
    switch (P.W) {
        case 1: if (P.RX == 2) run(k_levenshtein<1, 2>, a, smem, grid, s); else run(k_levenshtein<1, 1>, a, smem, grid, s); break;
        case 2: run(k_levenshtein<2, 1>, a, smem, grid, s); break;
        case 3: run(k_levenshtein<3, 1>, a, smem, grid, s); break;
        default: run(k_levenshtein<4, 1>, a, smem, grid, s); break;
    }
}

}  // namespace idb
