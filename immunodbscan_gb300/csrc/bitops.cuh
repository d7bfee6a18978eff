// bitops.cuh -- integer helpers shared by the device kernels and the host-side
// unit tests (compiled by nvcc for sm_103a and by g++ for the CPU tests).
//
// Contents
//  * popcount / find-first-set wrappers
//  * Myers/Hyyro bit-parallel global edit distance on 32-bit blocks
//    (G. Myers, "A fast bit-vector algorithm for approximate string matching
//    based on dynamic programming", J. ACM 46(3), 1999; H. Hyyro, "A bit-vector
//    algorithm for computing Levenshtein and Damerau edit distances", Nordic J.
//    Computing 10, 2003 -- block-based form with a horizontal delta carried
//    between 32-row blocks).  The reference computes the same quantity with a
//    full anti-diagonal DP (cuda/PSDBSCAN.hcu:246-290).
//  * closed-form decode of triangular work-unit grids
//  * a 64-bit mixing hash for the duplicate table
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define IDB_HD __host__ __device__ __forceinline__
#else
#define IDB_HD inline
#endif

namespace idb {

IDB_HD int popc32(uint32_t x) {
#if defined(__CUDA_ARCH__)
    return __popc(x);
#else
    return __builtin_popcount(x);
#endif
}

IDB_HD int popc64(uint64_t x) {
#if defined(__CUDA_ARCH__)
    return __popcll(x);
#else
    return __builtin_popcountll(x);
#endif
}

// index of the lowest set bit, -1 if none
IDB_HD int lowest_bit64(uint64_t x) {
#if defined(__CUDA_ARCH__)
    return __ffsll((long long)x) - 1;
#else
    return x ? __builtin_ctzll(x) : -1;
#endif
}

IDB_HD uint32_t low_mask32(int i) {   // bits [0, i) set, 0 <= i <= 32
    return i >= 32 ? 0xFFFFFFFFu : ((1u << i) - 1u);
}

// ---------------------------------------------------------------------------
// One column of the bit-parallel edit-distance recurrence for one 32-row block.
// Pv/Mv hold the vertical deltas D[i][j-1]-D[i-1][j-1] = +1 / -1 of the block's
// rows; eq has bit i set iff pattern row i matches the text character.
// h_in is the horizontal delta D[r0][j]-D[r0][j-1] entering from the row above
// the block (+1 for the first block: D[0][j] = j).  Returns the delta leaving
// the block's top bit (row r0+32).
// ---------------------------------------------------------------------------
IDB_HD int myers_block(uint32_t &Pv, uint32_t &Mv, uint32_t eq, int h_in) {
    const uint32_t in_neg = (uint32_t)(h_in < 0);
    const uint32_t in_pos = (uint32_t)(h_in > 0);
    const uint32_t Xv = eq | Mv;
    eq |= in_neg;                            // a -1 entering from above acts like a match
    const uint32_t Xh = (((eq & Pv) + Pv) ^ Pv) | eq;
    uint32_t Ph = Mv | ~(Xh | Pv);
    uint32_t Mh = Pv & Xh;
    const int h_out = (int)(Ph >> 31) - (int)(Mh >> 31);
    Ph = (Ph << 1) | in_pos;
    Mh = (Mh << 1) | in_neg;
    Pv = Mh | ~(Xv | Ph);
    Mv = Ph & Xv;
    return h_out;
}

// Single-block specialisation (pattern <= 32, h_in = +1 always).
IDB_HD void myers_step1(uint32_t &Pv, uint32_t &Mv, uint32_t eq) {
    const uint32_t Xv = eq | Mv;
    const uint32_t Xh = (((eq & Pv) + Pv) ^ Pv) | eq;
    uint32_t Ph = Mv | ~(Xh | Pv);
    uint32_t Mh = Pv & Xh;
    Ph = (Ph << 1) | 1u;
    Mh = Mh << 1;
    Pv = Mh | ~(Xv | Ph);
    Mv = Ph & Xv;
}

// D[i][j] recovered from the vertical deltas of column j (D[0][j] = j).
template <int W>
IDB_HD int myers_value(const uint32_t (&Pv)[W], const uint32_t (&Mv)[W], int i, int j) {
    int d = j;
#pragma unroll
    for (int w = 0; w < W; ++w) {
        int lo = w * 32;
        int take = i - lo;
        if (take <= 0) break;
        uint32_t m = low_mask32(take);
        d += popc32(Pv[w] & m) - popc32(Mv[w] & m);
    }
    return d;
}

// Reference edit distance of two code strings via the block recurrence
// (used by the host unit tests; the kernels inline the same steps).
template <int W>
IDB_HD int myers_distance(const uint8_t *p, int m, const uint8_t *t, int n) {
    uint32_t Pv[W], Mv[W];
#pragma unroll
    for (int w = 0; w < W; ++w) { Pv[w] = 0xFFFFFFFFu; Mv[w] = 0u; }
    for (int j = 0; j < n; ++j) {
        int h = 1;
#pragma unroll
        for (int w = 0; w < W; ++w) {
            uint32_t eq = 0;
            for (int b = 0; b < 32; ++b) {
                int i = w * 32 + b;
                if (i < m && p[i] == t[j]) eq |= 1u << b;
            }
            h = myers_block(Pv[w], Mv[w], eq, h);
        }
    }
    return myers_value<W>(Pv, Mv, m, n);
}

// ---------------------------------------------------------------------------
// Work units of a same-bucket (triangular) bucket pair.  The bucket holds n
// entries; x-chunks have TX entries, y-chunks TY = q*TX.  Unit (cx, cy) exists
// iff some y of chunk cy lies above some x of chunk cx, i.e. cx < (cy+1)*q.
// Units are numbered row by row (cy major).
// ---------------------------------------------------------------------------
IDB_HD uint64_t tri_units(uint32_t ncx, uint32_t ncy, uint32_t q) {
    uint64_t s = ncx / q;                  // rows cy < s are unsaturated
    if (s > ncy) s = ncy;
    return (uint64_t)q * s * (s + 1) / 2 + (uint64_t)(ncy - s) * ncx;
}

IDB_HD void tri_decode(uint64_t k, uint32_t ncx, uint32_t q, uint32_t &cx, uint32_t &cy) {
    uint64_t s = ncx / q;
    uint64_t head = (uint64_t)q * s * (s + 1) / 2;
    if (k < head) {
        // largest c with q*c*(c+1)/2 <= k
        double kk = (double)k / (double)q;
#if defined(__CUDA_ARCH__)
        uint64_t c = (uint64_t)((sqrt(8.0 * kk + 1.0) - 1.0) * 0.5);
#else
        uint64_t c = (uint64_t)((__builtin_sqrt(8.0 * kk + 1.0) - 1.0) * 0.5);
#endif
        while (c > 0 && (uint64_t)q * c * (c + 1) / 2 > k) --c;
        while ((uint64_t)q * (c + 1) * (c + 2) / 2 <= k) ++c;
        cy = (uint32_t)c;
        cx = (uint32_t)(k - (uint64_t)q * c * (c + 1) / 2);
    } else {
        uint64_t r = k - head;
        cy = (uint32_t)(s + r / ncx);
        cx = (uint32_t)(r % ncx);
    }
}

// ---------------------------------------------------------------------------
// 64-bit mixing hash (splitmix64 finaliser applied per absorbed word).
// ---------------------------------------------------------------------------
IDB_HD uint64_t mix64(uint64_t h, uint64_t v) {
    h ^= v + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
    h ^= h >> 30;
    h *= 0xBF58476D1CE4E5B9ull;
    h ^= h >> 27;
    h *= 0x94D049BB133111EBull;
    h ^= h >> 31;
    return h;
}

}  // namespace idb
