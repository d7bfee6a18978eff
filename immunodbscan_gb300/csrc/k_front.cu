// k_front.cu -- front of the clustering path: input survey, V/J gene bitsets,
// exact-duplicate collapse, unique numbering, and the device-wide scan used by
// every compaction of the pipeline.
//
// Reference counterparts:
//  survey/lengths      cuda/StringOperations.hcu:77-116 (lengths, max_strlen)
//  gene bitsets (S1)   cuda/BitsetVector.inl:28-45, 118-209 (110 serial launches,
//                      one block per row); here one launch, one warp per row
//  duplicates (S3)     cuda/PSDBSCAN.hcu:525-573 (an N^2 thread grid) + 1074-1085
//                      (sort / reduce_by_key / scatter); here one hash-table pass
//  uniques             cuda/PSDBSCAN.hcu:1102-1111 (remove_if over copies != 0)
#include <algorithm>

#include "idb_internal.cuh"

namespace idb {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ uint32_t rep_of_row(const uint32_t *rep_off, uint32_t R, uint32_t i) {
    // largest r with rep_off[r] <= i
    uint32_t lo = 0, hi = R;   // invariant: rep_off[lo] <= i < rep_off[hi]
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (rep_off[mid] <= i) lo = mid; else hi = mid;
    }
    return lo;
}

// ---------------------------------------------------------------------------
// Survey: sequence length range and the set of byte values present.
// ---------------------------------------------------------------------------
__global__ void k_survey(const uint8_t *__restrict__ seq, const int64_t *__restrict__ off,
                         uint32_t N, Counters *ctr) {
    __shared__ uint32_t used[8];
    __shared__ uint32_t smax, smin;
    if (threadIdx.x < 8) used[threadIdx.x] = 0;
    if (threadIdx.x == 0) { smax = 0; smin = 0xFFFFFFFFu; }
    __syncthreads();
    uint32_t lmax = 0, lmin = 0xFFFFFFFFu;
    const uint32_t stride = gridDim.x * blockDim.x;
    // four rows (and below four 16-byte words) per step: their loads in flight together
    for (uint32_t i0 = blockIdx.x * blockDim.x + threadIdx.x; i0 < N; i0 += 4 * stride) {
        int64_t a[4], b[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint64_t i = (uint64_t)i0 + (uint64_t)u * stride;
            a[u] = i < N ? off[i] : 0;
            b[u] = i < N ? off[i + 1] : 0;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if ((uint64_t)i0 + (uint64_t)u * stride < N) {
                const uint32_t L = (uint32_t)(b[u] - a[u]);
                lmax = max(lmax, L);
                lmin = min(lmin, L);
            }
    }
    // byte values present: 16 bytes per thread and step (aligned 16-byte loads,
    // the ragged ends byte by byte); values 64..127 (the letters) go to a
    // per-thread 64-bit mask, the rest straight to shared memory
    const int64_t b0 = N ? off[0] : 0, b1 = N ? off[N] : 0;
    unsigned long long m64 = 0;
    auto note = [&](uint32_t b) {
        if ((b & 0xC0u) == 0x40u) {
            m64 |= 1ull << (b & 63u);
        } else {
            const uint32_t bit = 1u << (b & 31);
            if (!(used[b >> 5] & bit)) atomicOr(&used[b >> 5], bit);
        }
    };
    const int64_t a0 = (int64_t)((reinterpret_cast<uintptr_t>(seq + b0) + 15) & ~(uintptr_t)15) -
                       (int64_t)reinterpret_cast<uintptr_t>(seq);   // first aligned byte
    const int64_t head_end = a0 < b1 ? a0 : b1;
    const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x;
    for (int64_t p = b0 + gtid; p < head_end; p += stride) note(seq[p]);
    const int64_t nvec = b1 > head_end ? (b1 - head_end) >> 4 : 0;
    const uint4 *vec = reinterpret_cast<const uint4 *>(seq + head_end);
    for (int64_t k0 = gtid; k0 < nvec; k0 += 4 * (int64_t)stride) {
        uint4 v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int64_t k = k0 + (int64_t)u * stride;
            v[u] = k < nvec ? __ldg(vec + k) : make_uint4(0x41414141u, 0x41414141u, 0x41414141u, 0x41414141u);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (k0 + (int64_t)u * stride >= nvec) break;
            const uint32_t w4[4] = {v[u].x, v[u].y, v[u].z, v[u].w};
#pragma unroll
            for (int e = 0; e < 4; ++e)
#pragma unroll
                for (int q = 0; q < 4; ++q) note((w4[e] >> (8 * q)) & 0xFFu);
        }
    }
    for (int64_t p = head_end + 16 * nvec + gtid; p < b1; p += stride) note(seq[p]);
    {
        const uint32_t lo = __reduce_or_sync(0xFFFFFFFFu, (uint32_t)m64);
        const uint32_t hi = __reduce_or_sync(0xFFFFFFFFu, (uint32_t)(m64 >> 32));
        if ((threadIdx.x & 31) == 0) {
            if (lo) atomicOr(&used[2], lo);
            if (hi) atomicOr(&used[3], hi);
        }
    }
    atomicMax(&smax, lmax);
    atomicMin(&smin, lmin);
    __syncthreads();
    if (threadIdx.x < 8 && used[threadIdx.x]) atomicOr(&ctr->used[threadIdx.x], used[threadIdx.x]);
    if (threadIdx.x == 0) {
        atomicMax(&ctr->lmax, smax);
        atomicMin(&ctr->lmin, smin);
    }
}

// Every row carries the literal "Gene" (no sequence column configured).
__global__ void k_const_strings(uint8_t *blob, int64_t *off, uint32_t N) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i <= N; i += stride) {
        off[i] = 4 * (int64_t)i;
        if (i < N) {
            blob[4 * (size_t)i + 0] = 'G';
            blob[4 * (size_t)i + 1] = 'e';
            blob[4 * (size_t)i + 2] = 'n';
            blob[4 * (size_t)i + 3] = 'e';
        }
    }
}

// ---------------------------------------------------------------------------
// S1 -- gene bitsets.  Bit g of a row is set iff reference gene name g is a
// byte-exact substring of the row's call (cuda/BitsetVector.inl:149-175, one
// launch and one block per row per gene there).  Empty names never match (the
// reference launches a zero-thread block for them).
//
// Calls repeat heavily (a repertoire has a few hundred distinct V calls over
// millions of rows), so a column is collapsed by string first:
//   k_call_slots  hashes every row's call and inserts (hash, row) into a bounded
//                 open-addressing table; the first row of every distinct string,
//                 and any row that finds no slot within kCallProbe probes, is
//                 queued;
//   k_gene_bits   computes the bitsets of the queued rows;
//   k_call_copy   copies each representative's bitset to the rows that share
//                 its string.
// A bitset is a function of the string alone, so the result does not depend
// on which row wins a slot.  The three kernels run per row chunk (host columns
// arrive chunk by chunk): a chunk's rows find the slots of earlier chunks'
// strings, and each chunk lists the rows that compute their own bitset in its
// own part of the todo array.
//
// k_gene_bits: a warp takes up to 32 queued rows, gathers their call bytes into
// its shared-memory slice, collects the bytes that start some gene name into a
// candidate queue with ballots, and verifies one candidate per lane: a rolling
// hash over the following bytes is looked up in the gene table at every length
// some name has, and every hit is checked byte by byte.  A row longer than the
// slice, or a table with a name longer than 255 bytes, takes one warp per row
// and one lane per gene instead.
// ---------------------------------------------------------------------------
constexpr int kGbWarps = 8;                 // warps per block
constexpr int kGbRows = 32;                 // rows per warp window
constexpr int kGbBytes = 2048;              // staged call bytes per warp
constexpr int kGbNameBytes = 16384;         // gene names kept in shared memory
constexpr uint32_t kCallProbe = 64;         // probes before a row computes its own bitset
constexpr unsigned long long kCallEmpty = ~0ull;

__device__ __forceinline__ bool name_at(const uint8_t *c, uint32_t cl, const uint8_t *name,
                                        uint32_t nl) {
    if (nl == 0 || nl > cl) return false;
    const uint8_t first = name[0];
    for (uint32_t p = 0; p + nl <= cl; ++p) {
        if (c[p] != first) continue;
        uint32_t k = 1;
        while (k < nl && c[p + k] == name[k]) ++k;
        if (k == nl) return true;
    }
    return false;
}

// one warp, one row: lane l tests genes l, l+32, ...
__device__ void gene_bits_row_naive(const uint8_t *c, uint32_t cl, const uint8_t *genes,
                                    const int32_t *goff, uint32_t G, uint32_t GW, int lane,
                                    uint64_t *out) {
    uint64_t acc[kMaxGeneWords];
#pragma unroll
    for (int w = 0; w < kMaxGeneWords; ++w) acc[w] = 0;
    for (uint32_t gb = 0; gb * 32 < G; ++gb) {
        const uint32_t g = gb * 32 + lane;
        bool found = false;
        if (g < G) {
            const int32_t n0 = goff[g];
            found = name_at(c, cl, genes + n0, (uint32_t)(goff[g + 1] - n0));
        }
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, found);
#pragma unroll
        for (int w = 0; w < kMaxGeneWords; ++w)
            if ((int)(gb >> 1) == w) acc[w] |= (uint64_t)m << (32 * (gb & 1));
    }
#pragma unroll
    for (int w = 0; w < kMaxGeneWords; ++w)
        if (lane == w && (uint32_t)w < GW) out[w] = acc[w];
}

// A warp's shared-memory slice: bitsets, row offsets, candidate queue, bytes.
struct GbSlice {
    uint64_t *bits;     // [kGbRows * GW]
    uint32_t *roff;     // [kGbRows + 1] byte offset of each staged row
    uint16_t *cand;     // [kGbBytes]
    uint32_t *words;    // [kGbBytes / 4 + 1]
    __device__ const uint8_t *bytes() const { return reinterpret_cast<const uint8_t *>(words); }
};

__host__ __device__ constexpr size_t gb_slice_bytes(uint32_t GW) {
    return (size_t)kGbBytes + 4 + 2 * kGbBytes + 4 * (kGbRows + 1) + 8 * (size_t)kGbRows * GW + 16;
}

// The call-collapse kernel stages bytes only: row offsets and words.
__host__ __device__ constexpr size_t cs_slice_bytes() {
    return 4 * (kGbRows + 1) + (size_t)kGbBytes + 4 + 16;
}

__device__ GbSlice cs_slice(uint8_t *base, int wid) {
    uint8_t *w = base + (cs_slice_bytes() + 15) / 16 * 16 * wid;
    GbSlice g;
    g.bits = nullptr;
    g.cand = nullptr;
    g.roff = reinterpret_cast<uint32_t *>(w);
    g.words = g.roff + kGbRows + 1;
    return g;
}

__device__ GbSlice gb_slice(uint8_t *base, uint32_t GW, int wid) {
    const size_t slice = (gb_slice_bytes(GW) + 15) / 16 * 16;
    uint8_t *w = base + slice * wid;
    GbSlice g;
    g.bits = reinterpret_cast<uint64_t *>(w);
    g.roff = reinterpret_cast<uint32_t *>(g.bits + kGbRows * GW);
    g.cand = reinterpret_cast<uint16_t *>(g.roff + kGbRows + 1);
    g.words = reinterpret_cast<uint32_t *>(
        (reinterpret_cast<uintptr_t>(g.cand + kGbBytes) + 3) & ~(uintptr_t)3);
    return g;
}

// Stages the longest prefix of rows [r, end) of the window (row k is rows[k], or
// k itself when rows is null) whose call bytes fit the slice.  Returns the
// number of rows staged, 0 if row r alone does not fit.  *my_row receives the
// row of lane l (entry r + l).  With rows == null the rows are contiguous and are
// copied with aligned 4-byte loads; otherwise row by row.
__device__ uint32_t gb_stage(const uint8_t *__restrict__ calls, const int64_t *__restrict__ off,
                             const uint32_t *__restrict__ rows, uint32_t r, uint32_t end, int lane,
                             const GbSlice &w, uint32_t *my_row) {
    const uint32_t k = r + lane;
    uint32_t row = 0, len = 0;
    int64_t st = 0;
    if (k < end) {
        row = rows ? rows[k] : k;
        st = off[row];
        len = (uint32_t)(off[row + 1] - st);
    }
    *my_row = row;
    // shift: alignment slack of the contiguous copy (0 for the gather)
    const int64_t base = __shfl_sync(0xFFFFFFFFu, st, 0);
    const uint32_t shift = rows ? 0u : (uint32_t)(reinterpret_cast<uintptr_t>(calls + base) & 3u);
    uint32_t incl = len;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, d);
        if (lane >= d) incl += t;
    }
    const bool fit = k < end && incl + shift + 4 <= (uint32_t)kGbBytes;
    const uint32_t nr = __popc(__ballot_sync(0xFFFFFFFFu, fit));
    if (nr == 0) return 0;
    const uint32_t excl = incl - len;
    if ((uint32_t)lane < nr) w.roff[lane] = excl + shift;
    const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, nr - 1);
    if (lane == 0) w.roff[nr] = total + shift;
    if (!rows) {
        // aligned words covering [calls + base, + total); the edge words are read
        // byte by byte where they reach outside that range
        const uint32_t *src = reinterpret_cast<const uint32_t *>(
            reinterpret_cast<uintptr_t>(calls + base) - shift);
        const uint32_t qend = shift + total, nwords = (qend + 3) >> 2;
        for (uint32_t t = lane; t < nwords; t += 32) {
            if (4 * t >= shift && 4 * t + 4 <= qend) {
                w.words[t] = src[t];
            } else {
                uint32_t v = 0;
                for (uint32_t b = 0; b < 4; ++b) {
                    const uint32_t q = 4 * t + b;
                    if (q >= shift && q < qend) v |= (uint32_t)calls[base + (q - shift)] << (8 * b);
                }
                w.words[t] = v;
            }
        }
    } else {
        // gather: every lane copies its own row with aligned 4-byte loads (a
        // word that holds a row byte never leaves that byte's page), so the
        // loads of all the window's rows are in flight together
        if ((uint32_t)lane < nr && len) {
            uint8_t *dst = reinterpret_cast<uint8_t *>(w.words) + excl;
            const uintptr_t a = reinterpret_cast<uintptr_t>(calls + st);
            const uint32_t sh = (uint32_t)(a & 3u);
            const uint32_t *gw = reinterpret_cast<const uint32_t *>(a - sh);
            const uint32_t nw = (sh + len + 3) >> 2;
#pragma unroll 4
            for (uint32_t t = 0; t < nw; ++t) {
                const uint32_t v = __ldg(gw + t);
#pragma unroll
                for (uint32_t b = 0; b < 4; ++b) {
                    const int q = (int)(4 * t + b) - (int)sh;
                    if (q >= 0 && (uint32_t)q < len) dst[q] = (uint8_t)(v >> (8 * b));
                }
            }
        }
    }
    __syncwarp();
    return nr;
}

__global__ void __launch_bounds__(kGbWarps * 32)
k_gene_bits(const uint8_t *__restrict__ calls, const int64_t *__restrict__ off,
            const uint32_t *__restrict__ rows, const uint32_t *__restrict__ n_dev, uint32_t n_host,
            const uint8_t *__restrict__ genes, const int32_t *__restrict__ goff, uint32_t G,
            uint32_t GW, const GeneEntry *__restrict__ tab, GeneMatcher gm,
            uint64_t *__restrict__ bits) {
    extern __shared__ __align__(16) uint8_t sm[];
    // rows per warp window: up to kGbRows, fewer when the rows are few (the
    // distinct calls of a column), so that every warp of the grid gets some;
    // blocks past the last window leave before loading the tables
    const uint32_t n = n_dev ? *n_dev : n_host;
    const uint32_t nwarps = gridDim.x * kGbWarps;
    const uint32_t rpc = max(1u, min((uint32_t)kGbRows, (n + nwarps - 1) / nwarps));
    const uint32_t nchunks = (n + rpc - 1) / rpc;
    if (blockIdx.x * kGbWarps >= nchunks) return;
    // block-wide tables
    GeneEntry *s_tab = reinterpret_cast<GeneEntry *>(sm);
    int32_t *s_goff = reinterpret_cast<int32_t *>(s_tab + gm.ts);
    const uint32_t name_bytes = (uint32_t)goff[G] <= (uint32_t)kGbNameBytes ? (uint32_t)goff[G] : 0u;
    uint8_t *s_names = reinterpret_cast<uint8_t *>(s_goff + G + 1);
    uint8_t *wbase = reinterpret_cast<uint8_t *>(
        (reinterpret_cast<uintptr_t>(s_names + name_bytes) + 15) & ~(uintptr_t)15);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const GbSlice w = gb_slice(wbase, GW, wid);
    const uint8_t *wb = w.bytes();
    __shared__ uint32_t s_first[8], s_len[8];
    for (uint32_t k = threadIdx.x; k < gm.ts; k += blockDim.x) s_tab[k] = tab[k];
    for (uint32_t k = threadIdx.x; k <= G; k += blockDim.x) s_goff[k] = goff[k];
    for (uint32_t k = threadIdx.x; k < name_bytes; k += blockDim.x) s_names[k] = genes[k];
#pragma unroll
    for (int k = 0; k < 8; ++k)      // constant indices keep the parameter out of local memory
        if (threadIdx.x == k) {
            s_first[k] = gm.firstmask[k];
            s_len[k] = gm.lenmask[k];
        }
    __syncthreads();
    const uint8_t *names = name_bytes ? s_names : genes;
    const uint32_t gwarp = blockIdx.x * kGbWarps + wid;
    for (uint32_t ch = gwarp; ch < nchunks; ch += nwarps) {
        const uint32_t end = min(ch * rpc + rpc, n);
        uint32_t r = ch * rpc;
        while (r < end) {
            uint32_t my_row = 0;
            const uint32_t nr = gm.long_names ? 0u : gb_stage(calls, off, rows, r, end, lane, w, &my_row);
            if (nr == 0) {   // one row (or every row: long names) the slow way
                const uint32_t row = rows ? rows[r] : r;
                const int64_t c0 = off[row];
                gene_bits_row_naive(calls + c0, (uint32_t)(off[row + 1] - c0), names, s_goff, G,
                                    GW, lane, bits + (size_t)row * GW);
                ++r;
                continue;
            }
            for (uint32_t k = lane; k < nr * GW; k += 32) w.bits[k] = 0;
            // candidates: positions whose byte starts some gene name
            uint32_t ncand = 0;
            const uint32_t qbeg = w.roff[0], qend = w.roff[nr];
            for (uint32_t q0 = qbeg; q0 < qend; q0 += 32) {
                const uint32_t q = q0 + lane;
                bool cand = false;
                if (q < qend) {
                    const uint32_t c = wb[q];
                    cand = (s_first[c >> 5] >> (c & 31)) & 1u;
                }
                const uint32_t m = __ballot_sync(0xFFFFFFFFu, cand);
                if (cand) w.cand[ncand + __popc(m & ((1u << lane) - 1u))] = (uint16_t)q;
                ncand += __popc(m);
            }
            __syncwarp();
            for (uint32_t k = lane; k < ncand; k += 32) {
                const uint32_t q = w.cand[k];
                uint32_t lo = 0, hi = nr;   // row: largest i with roff[i] <= q
                while (hi - lo > 1) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if (w.roff[mid] <= q) lo = mid; else hi = mid;
                }
                const uint32_t ri = lo, rend = w.roff[ri + 1];
                uint32_t h = 0;
                for (uint32_t t = 0; t < gm.maxlen && q + t < rend; ++t) {
                    h = h * kGeneHashMul + wb[q + t];
                    const uint32_t L = t + 1;
                    if (!((s_len[L >> 5] >> (L & 31)) & 1u)) continue;
                    uint32_t sl = h & (gm.ts - 1);
                    while (s_tab[sl].len != 0) {
                        const GeneEntry e = s_tab[sl];
                        if (e.h == h && e.len == L) {
                            const uint8_t *name = names + s_goff[e.gene];
                            uint32_t i = 0;
                            while (i < L && name[i] == wb[q + i]) ++i;
                            if (i == L)
                                atomicOr(reinterpret_cast<unsigned long long *>(&w.bits[ri * GW + (e.gene >> 6)]),
                                         1ull << (e.gene & 63));
                        }
                        sl = (sl + 1) & (gm.ts - 1);
                    }
                }
            }
            __syncwarp();
            if (rows) {
                for (uint32_t k = lane; k < nr * GW; k += 32)
                    bits[(size_t)rows[r + k / GW] * GW + k % GW] = w.bits[k];
            } else {
                for (uint32_t k = lane; k < nr * GW; k += 32) bits[(size_t)r * GW + k] = w.bits[k];
            }
            __syncwarp();
            r += nr;
        }
    }
}

size_t gene_bits_smem(uint32_t G, uint32_t GW, uint32_t ts, uint32_t name_bytes) {
    const size_t nb = name_bytes <= (uint32_t)kGbNameBytes ? name_bytes : 0;
    return sizeof(GeneEntry) * ts + sizeof(int32_t) * (G + 1) + nb + 16 +
           kGbWarps * ((gb_slice_bytes(GW) + 15) / 16 * 16);
}

// Sequential reader of a staged call: aligned 4-byte shared-memory loads
// joined by a funnel shift, 4 call bytes per step (bytes past the call are
// whatever the slice holds there: callers mask them).
struct StagedReader {
    const uint32_t *w;
    uint32_t idx, sh, prev;
    __device__ __forceinline__ StagedReader(const uint32_t *words, uint32_t q)
        : w(words), idx(q >> 2), sh(8 * (q & 3)), prev(words[q >> 2]) {}
    __device__ __forceinline__ uint32_t next() {
        const uint32_t cur = w[++idx];
        const uint32_t out = __funnelshift_r(prev, cur, sh);
        prev = cur;
        return out;
    }
};

// Mask of the first n (0..4) bytes of a word.
__device__ __forceinline__ uint32_t byte_mask(uint32_t n) {
    return n >= 4 ? 0xFFFFFFFFu : ((1u << (8 * n)) - 1u);
}

// Byte equality of a call in global memory with the staged bytes at offset q0.
// Reads only the aligned 4-byte words that hold the call's bytes (so no read
// leaves the call's pages), joined by a funnel shift; no early exit.  Whole
// words first, the ragged last word masked.
__device__ __forceinline__ bool bytes_equal_global(const uint8_t *g, const uint32_t *words,
                                                   uint32_t q0, uint32_t len) {
    if (len == 0) return true;
    const uintptr_t a = reinterpret_cast<uintptr_t>(g);
    const uint32_t sh = (uint32_t)(a & 3u);
    const uint32_t *gw = reinterpret_cast<const uint32_t *>(a - sh);
    const uint32_t last = (sh + len - 1) >> 2;       // last word holding a call byte
    StagedReader rd(words, q0);
    uint32_t gprev = __ldg(gw);
    uint32_t diff = 0;
    const uint32_t full = len >> 2;                  // words whose 4 bytes are all in the call
    uint32_t t = 0;
#pragma unroll 2
    for (; t < full; ++t) {
        const uint32_t gnext = t + 1 <= last ? __ldg(gw + t + 1) : 0u;
        diff |= __funnelshift_r(gprev, gnext, 8 * sh) ^ rd.next();
        gprev = gnext;
    }
    if (len & 3u) {
        const uint32_t gnext = t + 1 <= last ? __ldg(gw + t + 1) : 0u;
        diff |= (__funnelshift_r(gprev, gnext, 8 * sh) ^ rd.next()) & byte_mask(len & 3u);
    }
    return diff == 0;
}

// Equality of two staged calls of equal length.
__device__ __forceinline__ bool staged_equal(const uint32_t *words, uint32_t qa, uint32_t qb,
                                             uint32_t len) {
    StagedReader ra(words, qa), rb(words, qb);
    uint32_t diff = 0;
    const uint32_t full = len >> 2;
#pragma unroll 2
    for (uint32_t t = 0; t < full; ++t) diff |= ra.next() ^ rb.next();
    if (len & 3u) diff |= (ra.next() ^ rb.next()) & byte_mask(len & 3u);
    return diff == 0;
}

// String hash of a staged call: two 32-bit multiplicative lanes over 4-byte
// words, finished by mix64 (equality is then checked byte by byte).
__device__ __forceinline__ unsigned long long call_hash(const uint32_t *words, uint32_t q0,
                                                        uint32_t len) {
    StagedReader rd(words, q0);
    uint32_t h1 = 0x811C9DC5u ^ len, h2 = 0x2545F491u + len;
    const uint32_t full = len >> 2;
#pragma unroll 2
    for (uint32_t t = 0; t < full; ++t) {
        const uint32_t v = rd.next();
        h1 = (h1 ^ v) * 0x01000193u;
        h2 = (h2 + v) * 0x9E3779B1u;
    }
    if (len & 3u) {
        const uint32_t v = rd.next() & byte_mask(len & 3u);
        h1 = (h1 ^ v) * 0x01000193u;
        h2 = (h2 + v) * 0x9E3779B1u;
    }
    return mix64(((unsigned long long)h1 << 32) | h2, len);
}

// Collapse of a call column by string: ref[row] = slot of the row's string, or
// kNone when the row computes its own bitset (it won the slot, or found none);
// those rows are appended to todo.
__global__ void __launch_bounds__(kGbWarps * 32)
k_call_slots(const uint8_t *__restrict__ calls, const int64_t *__restrict__ off, uint32_t r0,
             uint32_t r1, unsigned long long *tab, uint32_t tmask, uint32_t *__restrict__ ref,
             uint32_t *__restrict__ todo, uint32_t *n_todo) {
    extern __shared__ __align__(16) uint8_t sm[];
    // rows that compute their own bitset, gathered per warp and appended to
    // todo a batch at a time (one atomic per batch, not per window)
    __shared__ uint32_t s_todo[kGbWarps][2 * kGbRows];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t tcnt = 0;
    auto flush_todo = [&]() {
        __syncwarp();
        uint32_t b0 = 0;
        if (lane == 0 && tcnt) b0 = atomicAdd(n_todo, tcnt);
        b0 = __shfl_sync(0xFFFFFFFFu, b0, 0);
        for (uint32_t k = (uint32_t)lane; k < tcnt; k += 32) todo[b0 + k] = s_todo[wid][k];
        __syncwarp();
        tcnt = 0;
    };
    const GbSlice w = cs_slice(sm, wid);
    const uint8_t *wb = w.bytes();
    const uint32_t nwin = (r1 - r0 + kGbRows - 1) / kGbRows;
    const uint32_t gwarp = blockIdx.x * kGbWarps + wid, nwarps = gridDim.x * kGbWarps;
    for (uint32_t ch = gwarp; ch < nwin; ch += nwarps) {
        const uint32_t end = min(r0 + ch * kGbRows + kGbRows, r1);
        uint32_t r = r0 + ch * kGbRows;
        while (r < end) {
            uint32_t my_row = 0;
            const uint32_t nr = gb_stage(calls, off, nullptr, r, end, lane, w, &my_row);
            bool own = false;
            uint32_t myref = kNone;
            if (nr == 0) {                      // too long to stage: computes its own bitset
                own = lane == 0;
            } else {
                const bool act = (uint32_t)lane < nr;
                uint32_t q0 = 0, len = 0;
                unsigned long long h = 0;
                if (act) {
                    q0 = w.roff[lane];
                    len = w.roff[lane + 1] - q0;
                    h = call_hash(w.words, q0, len);
                }
                // equal calls inside the window: the lowest lane of each hash group
                // looks the string up, the others check their bytes against it
                const uint32_t grp = __match_any_sync(0xFFFFFFFFu, act ? h : kCallEmpty);
                const int leader = __ffs(grp) - 1;
                const uint32_t lq0 = __shfl_sync(0xFFFFFFFFu, q0, leader);
                const uint32_t llen = __shfl_sync(0xFFFFFFFFu, len, leader);
                bool follow = false;
                if (act && leader != lane && llen == len) follow = staged_equal(w.words, q0, lq0, len);
                uint32_t slot = kNone;          // the string's slot, kNone if none was found
                if (act && !follow) {
                    const unsigned long long key = (h & 0xFFFFFFFF00000000ull) | my_row;
                    uint32_t sl = (uint32_t)h & tmask;
                    own = true;                 // unless an equal string is found below
                    for (uint32_t it = 0; it < kCallProbe; ++it) {
                        unsigned long long cur = *((volatile unsigned long long *)&tab[sl]);
                        if (cur == kCallEmpty) {
                            const unsigned long long prev = atomicCAS(&tab[sl], kCallEmpty, key);
                            if (prev == kCallEmpty) { slot = sl; break; }   // representative
                            cur = prev;
                        }
                        if ((cur >> 32) == (h >> 32)) {
                            const uint32_t other = (uint32_t)cur;
                            const int64_t o0 = off[other];
                            if ((uint32_t)(off[other + 1] - o0) == len &&
                                bytes_equal_global(calls + o0, w.words, q0, len)) {
                                own = false;
                                slot = sl;
                                break;
                            }
                        }
                        sl = (sl + 1) & tmask;
                    }
                }
                const uint32_t lslot = __shfl_sync(0xFFFFFFFFu, slot, leader);
                if (follow) {
                    own = lslot == kNone;       // the leader found no slot: own bitset too
                    slot = lslot;
                }
                myref = slot;
            }
            if (own) myref = kNone;
            const uint32_t m = __ballot_sync(0xFFFFFFFFu, own);
            if (m) {
                if (tcnt + 32u > 2u * kGbRows) flush_todo();
                if (own) s_todo[wid][tcnt + __popc(m & ((1u << lane) - 1u))] = nr == 0 ? r : my_row;
                tcnt += (uint32_t)__popc(m);
            }
            if (nr == 0) {
                if (lane == 0) ref[r] = kNone;
                ++r;
            } else {
                if ((uint32_t)lane < nr) ref[my_row] = myref;
                r += nr;
            }
            __syncwarp();
        }
    }
    flush_todo();
}

// Rows that share a representative's string take its bitset.
__global__ void k_call_copy(uint32_t r0, uint32_t r1, uint32_t N, const uint32_t *__restrict__ ref,
                            const unsigned long long *__restrict__ tab, uint32_t tmask, uint32_t GW,
                            uint64_t *__restrict__ bits) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = r0 + blockIdx.x * blockDim.x + threadIdx.x; i < r1; i += stride) {
        const uint32_t s = ref[i];
        if (s > tmask) continue;                 // kNone: the row has its own bitset
        const uint32_t src = (uint32_t)tab[s];
        if (src >= N) continue;
        for (uint32_t k = 0; k < GW; ++k) bits[(size_t)i * GW + k] = bits[(size_t)src * GW + k];
    }
}

// No gene column: every row carries bit 0 ("V" against ["V"]).
__global__ void k_gene_bits_const(uint32_t N, uint64_t *bits) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += stride) bits[i] = 1ull;
}

// ---------------------------------------------------------------------------
// S3 -- exact duplicates.  Key = (repertoire, length, V bits, J bits, bytes).
// Open addressing; a slot holds a row index, the class's minimum row wins via
// atomicMin (the reference links larger indices to smaller ones,
// cuda/PSDBSCAN.hcu:85-86, so its representative is the minimum index too).
// Equality is checked on the full key; the hash only spreads the probes.
// ---------------------------------------------------------------------------
struct DedupArgs {
    const uint8_t *seq; const int64_t *off;
    const uint64_t *vbits, *jbits; uint32_t VW, JW;
    const uint32_t *rep_off; uint32_t R;
    uint32_t r0, r1;      // the rows inserted by this launch
    uint2 *dtab;          // slot: {row of the class, ~(class size)}; all ones when empty
    uint32_t *slot;
    uint64_t mask;
    Counters *ctr;
};

// Row x (repertoire rx, bytes [ox, ox+lx)) equals row y: same repertoire,
// length, V and J bitsets and bytes.  Independent loads, no early exit.
__device__ bool rows_equal(const DedupArgs &a, uint32_t x, uint32_t y, uint32_t rx, int64_t ox,
                           uint32_t lx) {
    const int64_t oy = a.off[y], oy1 = a.off[y + 1];
    const uint32_t r0 = a.rep_off[rx], r1 = a.rep_off[rx + 1];
    if ((uint32_t)(oy1 - oy) != lx || y < r0 || y >= r1) return false;
    uint64_t d = 0;
    for (uint32_t w = 0; w < a.VW; ++w) d |= a.vbits[(size_t)x * a.VW + w] ^ a.vbits[(size_t)y * a.VW + w];
    for (uint32_t w = 0; w < a.JW; ++w) d |= a.jbits[(size_t)x * a.JW + w] ^ a.jbits[(size_t)y * a.JW + w];
    GlobalReader rx_(a.seq + ox, lx), ry_(a.seq + oy, lx);
    uint32_t db = 0;
    for (uint32_t k = 0; k < lx; k += 4) db |= rx_.next() ^ ry_.next();   // past the end: 0 ^ 0
    return d == 0 && db == 0;
}

constexpr uint32_t kRepSmem = 2048;   // repertoire offsets kept in shared memory

__global__ void __launch_bounds__(kThreads) k_dedupe_insert(DedupArgs a) {
    __shared__ uint32_t s_rep[kRepSmem + 1];
    const bool rep_smem = a.R + 1 <= kRepSmem + 1;
    if (rep_smem)
        for (uint32_t k = threadIdx.x; k <= a.R; k += blockDim.x) s_rep[k] = a.rep_off[k];
    __syncthreads();
    const uint32_t *rep_off = rep_smem ? s_rep : a.rep_off;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = a.r0 + blockIdx.x * blockDim.x + threadIdx.x; i < a.r1; i += stride) {
        const uint32_t r = rep_of_row(rep_off, a.R, i);
        const int64_t o = a.off[i];
        const uint32_t L = (uint32_t)(a.off[i + 1] - o);
        uint64_t h = mix64(0x1234567ull + r, L);
        for (uint32_t w = 0; w < a.VW; ++w) h = mix64(h, a.vbits[(size_t)i * a.VW + w]);
        for (uint32_t w = 0; w < a.JW; ++w) h = mix64(h, a.jbits[(size_t)i * a.JW + w]);
        GlobalReader rd(a.seq + o, L);
        for (uint32_t k = 0; k < L; k += 8) {
            const uint32_t lo = rd.next();
            const uint32_t hi = k + 4 < L ? rd.next() : 0u;
            h = mix64(h, ((uint64_t)hi << 32) | lo);
        }
        uint64_t s = h & a.mask;
        uint32_t it = 0;
        for (;; ++it) {
            if (it > a.mask || it >= kSpinCap) {   // table full: cannot happen at load <= 1/2
                atomicOr(&a.ctr->error, kErrHashStall);
                s = kNone;
                break;
            }
            uint32_t cur = *((volatile uint32_t *)&a.dtab[s].x);
            if (cur == kNone) {
                uint32_t prev = atomicCAS(&a.dtab[s].x, kNone, i);
                if (prev == kNone) break;
                cur = prev;
            }
            if (rows_equal(a, i, cur, r, o, L)) break;
            s = (s + 1) & a.mask;
        }
        a.slot[i] = (uint32_t)s;
        // one class-size increment and one minimum per class among the warp's
        // rows (lanes hold ascending rows, so the lowest lane has the smallest)
        const uint32_t grp = __match_any_sync(__activemask(), (uint32_t)s);
        if ((threadIdx.x & 31) == (uint32_t)(__ffs(grp) - 1) && s != kNone) {
            atomicSub(&a.dtab[s].y, (uint32_t)__popc(grp));   // the size is kept complemented
            atomicMin(&a.dtab[s].x, i);
        }
    }
}

// Representative and "is a representative" flag of rows [r0, r1).  Final as
// soon as every row up to r1 is in the table: later rows have larger indices,
// so they never lower a class's minimum row.
__global__ void k_dedupe_final(uint32_t r0, uint32_t r1, const uint32_t *__restrict__ slot,
                               const uint2 *__restrict__ dtab, uint32_t *__restrict__ rep_row,
                               uint32_t *__restrict__ flag) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = r0 + blockIdx.x * blockDim.x + threadIdx.x; i < r1; i += stride) {
        const uint32_t s = slot[i];
        const uint32_t r = s == kNone ? i : dtab[s].x;
        rep_row[i] = r;
        flag[i] = (r == i);
    }
}

// Unique numbering: uid = rank of the representative row among representatives
// (ascending row order, cuda/PSDBSCAN.hcu:1102-1111).  Also the per-unique
// columns and the row -> uid map.
__global__ void k_uniques(uint32_t N, const int64_t *__restrict__ off,
                          const uint32_t *__restrict__ rep_off, uint32_t R,
                          const uint32_t *__restrict__ slot, const uint2 *__restrict__ dtab,
                          const uint32_t *__restrict__ rep_row, const uint32_t *__restrict__ uid_of_row,
                          uint32_t *__restrict__ urow, uint32_t *__restrict__ ucopies,
                          uint32_t *__restrict__ ulen, uint32_t *__restrict__ urep,
                          uint32_t *__restrict__ row2uid) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += stride) {
        const uint32_t r = rep_row[i];
        if (r == i) {
            const uint32_t u = uid_of_row[i];
            urow[u] = i;
            ucopies[u] = slot[i] == kNone ? 1u : ~dtab[slot[i]].y;
            ulen[u] = (uint32_t)(off[i + 1] - off[i]);
            urep[u] = rep_of_row(rep_off, R, i);
        }
        row2uid[i] = uid_of_row[r];
    }
}

// First unique of every repertoire (its first row is a representative: a
// class never leaves its repertoire), and n_uniques at the end.
__global__ void k_uid_first(uint32_t N, uint32_t R, const uint32_t *__restrict__ rep_off,
                            const uint32_t *__restrict__ row2uid, const Counters *ctr,
                            uint32_t *__restrict__ uid_first) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r <= R) {
        const uint32_t row = rep_off[r];
        uid_first[r] = row < N ? row2uid[row] : ctr->n_uniques;
    }
}

// Row chunks: the chunk boundaries and the unique count of every chunk before
// k give chunk k's first unique id.
struct ChunkRows {
    uint32_t n;
    uint32_t row[kMaxRowChunks + 1];
};

__device__ __forceinline__ uint32_t chunk_uid_base(const Counters *ctr, uint32_t k) {
    uint32_t b = 0;
    for (uint32_t m = 0; m < k; ++m) b += ctr->chunk_uniques[m];
    return b;
}

// Unique numbering of row chunk k (rows [r0, r1)), once its representatives
// are final: uid = chunk k's first uid + the rank among the chunk's
// representatives (uid_of_row, scanned per chunk), so uids ascend with the row
// as in the one-pass numbering.  A duplicate takes its representative's uid,
// which may lie in an earlier chunk.  The copies come later (k_uniques_finish):
// a class may still grow in later chunks.
__global__ void k_uniques_rows(uint32_t k, ChunkRows cr, const int64_t *__restrict__ off,
                               const uint32_t *__restrict__ rep_off, uint32_t R,
                               const uint32_t *__restrict__ rep_row,
                               const uint32_t *__restrict__ uid_of_row, const Counters *ctr,
                               uint32_t *__restrict__ urow, uint32_t *__restrict__ ulen,
                               uint32_t *__restrict__ urep, uint32_t *__restrict__ row2uid) {
    const uint32_t r0 = cr.row[k], r1 = cr.row[k + 1];
    const uint32_t base = chunk_uid_base(ctr, k);
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = r0 + blockIdx.x * blockDim.x + threadIdx.x; i < r1; i += stride) {
        const uint32_t r = rep_row[i];
        uint32_t rb = base;
        if (r < r0) {                       // the representative is in an earlier chunk
            uint32_t j = 0;
            while (j + 1 < k && cr.row[j + 1] <= r) ++j;
            rb = chunk_uid_base(ctr, j);
        }
        const uint32_t u = rb + uid_of_row[r];
        row2uid[i] = u;
        if (r == i) {
            urow[u] = i;
            ulen[u] = (uint32_t)(off[i + 1] - off[i]);
            urep[u] = rep_of_row(rep_off, R, i);
        }
    }
}

// After the last chunk: the unique count and every unique's copies (its
// class size, final now).
__global__ void k_uniques_finish(uint32_t nchunks, Counters *ctr, const uint32_t *__restrict__ urow,
                                 const uint32_t *__restrict__ slot, const uint2 *__restrict__ dtab,
                                 uint32_t *__restrict__ ucopies) {
    const uint32_t nu = chunk_uid_base(ctr, nchunks);
    if (blockIdx.x == 0 && threadIdx.x == 0) ctr->n_uniques = nu;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < nu; u += stride) {
        const uint32_t sl = slot[urow[u]];
        ucopies[u] = sl == kNone ? 1u : ~dtab[sl].y;
    }
}

// ---------------------------------------------------------------------------
// Exclusive scan (reduce, scan of block sums, down-sweep).  4096 items per block.
// ---------------------------------------------------------------------------
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr uint32_t kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t t = __shfl_up_sync(0xFFFFFFFFu, v, d);
        if (lane >= d) v += t;
    }
    return v;
}

// exclusive block scan of one value per thread; returns prefix, *sum = total
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *sum) {
    __shared__ uint32_t wsum[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    uint32_t inc = warp_incl_scan(v);
    if (lane == 31) wsum[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        uint32_t w = lane < nw ? wsum[lane] : 0u;
        uint32_t wi = warp_incl_scan(w);
        if (lane < nw) wsum[lane] = wi - w;
        if (lane == nw - 1) wsum[31] = wi;
    }
    __syncthreads();
    uint32_t res = inc - v + wsum[wid];
    *sum = wsum[31];
    __syncthreads();
    return res;
}

__global__ void __launch_bounds__(kScanThreads)
k_scan_reduce(const uint32_t *__restrict__ in, uint32_t n_host, const uint32_t *n_dev,
              uint32_t *__restrict__ part) {
    const uint32_t n = n_dev ? min(*n_dev, n_host) : n_host;
    const uint64_t base = (uint64_t)blockIdx.x * kScanTile;
    uint32_t s = 0;
    for (int k = 0; k < kScanItems; ++k) {
        uint64_t i = base + (uint64_t)k * kScanThreads + threadIdx.x;
        if (i < n) s += in[i];
    }
    uint32_t total;
    block_excl_scan(s, &total);
    if (threadIdx.x == 0) part[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024)
k_scan_parts(uint32_t *__restrict__ part, uint32_t nb, uint32_t *total_out) {
    const uint32_t per = (nb + blockDim.x - 1) / blockDim.x;
    const uint32_t b0 = threadIdx.x * per;
    uint32_t s = 0;
    for (uint32_t k = 0; k < per; ++k)
        if (b0 + k < nb) s += part[b0 + k];
    uint32_t total;
    uint32_t pre = block_excl_scan(s, &total);
    for (uint32_t k = 0; k < per; ++k)
        if (b0 + k < nb) {
            uint32_t v = part[b0 + k];
            part[b0 + k] = pre;
            pre += v;
        }
    if (threadIdx.x == 0 && total_out) *total_out = total;
}

__global__ void __launch_bounds__(kScanThreads)
k_scan_down(const uint32_t *in, uint32_t *out, uint32_t n_host, const uint32_t *n_dev,
            const uint32_t *__restrict__ part, int vec) {
    const uint32_t n = n_dev ? min(*n_dev, n_host) : n_host;
    const uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
    // a thread's 16 items are 64 bytes, aligned when both arrays are: then a
    // thread whose items are all inside moves them as four 16-byte words
    static_assert(kScanItems % 4 == 0, "vector items");
    const bool whole = vec && base + kScanItems <= n;
    uint32_t v[kScanItems];
    uint32_t s = 0;
    if (whole) {
#pragma unroll
        for (int q = 0; q < kScanItems / 4; ++q) {
            const uint4 u = *reinterpret_cast<const uint4 *>(in + base + 4 * q);
            v[4 * q] = u.x; v[4 * q + 1] = u.y; v[4 * q + 2] = u.z; v[4 * q + 3] = u.w;
        }
    } else {
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            const uint64_t i = base + k;
            v[k] = i < n ? in[i] : 0u;
        }
    }
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) s += v[k];
    uint32_t total;
    uint32_t pre = block_excl_scan(s, &total) + part[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const uint32_t x = v[k];
        v[k] = pre;
        pre += x;
    }
    if (whole) {
#pragma unroll
        for (int q = 0; q < kScanItems / 4; ++q)
            *reinterpret_cast<uint4 *>(out + base + 4 * q) =
                make_uint4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
    } else {
#pragma unroll
        for (int k = 0; k < kScanItems; ++k)
            if (base + k < n) out[base + k] = v[k];
    }
}

// Phase time stamps: the device's global nanosecond timer, written by a
// one-thread kernel between phases (works inside a captured graph).
__global__ void k_stamp(unsigned long long *dst) {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    *dst = t;
}

// A replayed plan is only valid while lengths and byte values stay inside the
// ones it was built for.
struct PlanShape {
    uint32_t lmin, lmax;
    uint32_t used[8];
};

__global__ void k_check_plan(PlanShape ps, Counters *ctr) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    uint32_t err = 0;
    if (ctr->lmax > ps.lmax || ctr->lmin < ps.lmin) err |= kErrLength;
    for (int k = 0; k < 8; ++k)
        if (ctr->used[k] & ~ps.used[k]) err |= kErrAlphabet;
    if (err) atomicOr(&ctr->error, err);
}

inline int grid_for(uint64_t n, int threads = kThreads) {
    uint64_t g = (n + threads - 1) / threads;
    uint64_t cap = (uint64_t)sm_count() * 8;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

}  // namespace

// ---------------------------------------------------------------------------
uint32_t scan_part_needed(uint64_t n) { return (uint32_t)((n + kScanTile - 1) / kScanTile + 1); }

void scan_u32(const uint32_t *in, uint32_t *out, uint32_t n, const uint32_t *n_dev,
              uint32_t *total, uint32_t *part, uint32_t part_cap, cudaStream_t s) {
    const uint32_t nb = (uint32_t)((n + kScanTile - 1) / kScanTile);
    if (nb == 0) {
        if (total) cudaMemsetAsync(total, 0, sizeof(uint32_t), s);
        return;
    }
    (void)part_cap;
    const int vec = ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15u) == 0;
    k_scan_reduce<<<nb, kScanThreads, 0, s>>>(in, n, n_dev, part);
    k_scan_parts<<<1, 1024, 0, s>>>(part, nb, total);
    k_scan_down<<<nb, kScanThreads, 0, s>>>(in, out, n, n_dev, part, vec);
}

void launch_stamp(unsigned long long *dst, cudaStream_t s) { k_stamp<<<1, 1, 0, s>>>(dst); }

void launch_check_plan(const Plan &P, const Buffers &B, cudaStream_t s) {
    PlanShape ps;
    ps.lmin = P.Lmin;
    ps.lmax = P.Lmax;
    for (int k = 0; k < 8; ++k) ps.used[k] = 0;
    for (int b = 0; b < 256; ++b)
        if (P.codemap[b] != 0 || b == P.first_byte) ps.used[b >> 5] |= 1u << (b & 31);
    k_check_plan<<<1, 32, 0, s>>>(ps, B.ctr);
}

void launch_survey(const Plan &P, const Buffers &B, cudaStream_t s) {
    k_survey<<<grid_wave(k_survey, P.N, kThreads), kThreads, 0, s>>>(B.seq, B.seq_off, P.N, B.ctr);
}

void launch_const_strings(uint8_t *blob, int64_t *off, uint32_t N, cudaStream_t s) {
    k_const_strings<<<grid_for((uint64_t)N + 1), kThreads, 0, s>>>(blob, off, N);
}

void launch_call_init(const Plan &P, const Buffers &B, bool v_column, cudaStream_t s) {
    if (v_column ? P.no_v : P.no_j) {
        uint64_t *bits = v_column ? B.vbits : B.jbits;
        k_gene_bits_const<<<grid_for(P.N), kThreads, 0, s>>>(P.N, bits);
        return;
    }
    const CallScratch &cs = B.call[v_column ? 0 : 1];
    cudaMemsetAsync(cs.tab, 0xFF, sizeof(unsigned long long) * ((size_t)cs.mask + 1), s);
    cudaMemsetAsync(cs.ntodo, 0, sizeof(uint32_t) * kMaxRowChunks, s);
}

void launch_gene_bits(const Plan &P, const Buffers &B, bool v_column, uint32_t chunk, cudaStream_t s) {
    if (v_column ? P.no_v : P.no_j) return;   // constant bitsets, set by launch_call_init
    const uint32_t r0 = P.chunk_row[chunk], r1 = P.chunk_row[chunk + 1];
    if (r1 <= r0) return;
    const uint32_t nrows = r1 - r0;
    uint64_t *bits = v_column ? B.vbits : B.jbits;
    const CallScratch &cs = B.call[v_column ? 0 : 1];
    const uint32_t G = v_column ? P.Gv : P.Gj;
    const uint32_t GW = v_column ? P.VW : P.JW;
    const uint8_t *calls = v_column ? B.vcall : B.jcall;
    const int64_t *off = v_column ? B.v_off : B.j_off;
    const uint8_t *genes = v_column ? B.vgenes : B.jgenes;
    const int32_t *goff = v_column ? B.vg_off : B.jg_off;
    const GeneEntry *tab = v_column ? B.vtab : B.jtab;
    const GeneMatcher &gm = v_column ? P.vmatch : P.jmatch;
    const uint32_t name_bytes = v_column ? P.gene_bytes_v : P.gene_bytes_j;
    uint32_t *todo = cs.todo + r0, *ntodo = cs.ntodo + chunk;
    // 1. collapse the chunk's calls by string
    const size_t smem_slots = kGbWarps * ((cs_slice_bytes() + 15) / 16 * 16);
    static_assert(kGbWarps * ((cs_slice_bytes() + 15) / 16 * 16) <= 48 * 1024, "default smem limit");
    const int grid_rows = grid_wave(k_call_slots, ((uint64_t)nrows + kGbRows - 1) / kGbRows * 32,
                                    kGbWarps * 32, smem_slots);
    k_call_slots<<<grid_rows > 0 ? grid_rows : 1, kGbWarps * 32, smem_slots, s>>>(
        calls, off, r0, r1, cs.tab, cs.mask, cs.ref, todo, ntodo);
    // 2. bitsets of the representatives
    const size_t smem = gene_bits_smem(G, GW, gm.ts, name_bytes);
    static thread_local size_t attr_set = 0;
    if (smem > 48 * 1024 && smem > attr_set) {
        cudaFuncSetAttribute(k_gene_bits, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr_set = smem;
    }
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gene_bits, kGbWarps * 32, smem);
    const uint64_t want = ((uint64_t)nrows + kGbRows * kGbWarps - 1) / (kGbRows * kGbWarps);
    const int grid = (int)std::min<uint64_t>(want, (uint64_t)sm_count() * (per_sm > 0 ? per_sm : 1));
    k_gene_bits<<<grid > 0 ? grid : 1, kGbWarps * 32, smem, s>>>(
        calls, off, todo, ntodo, nrows, genes, goff, G, GW, tab, gm, bits);
    // 3. everybody else (a representative is a row of this chunk or of an earlier one)
    k_call_copy<<<grid_wave(k_call_copy, nrows, kThreads), kThreads, 0, s>>>(
        r0, r1, P.N, cs.ref, cs.tab, cs.mask, GW, bits);
}

void launch_dedupe_init(const Plan &P, const Buffers &B, cudaStream_t s) {
    cudaMemsetAsync(B.table, 0xFF, sizeof(uint2) * (B.table_mask + 1), s);
}

// Rows of one chunk into the duplicate table: their gene bitsets are complete,
// and so are those of every row already in the table (earlier chunks).
void launch_dedupe_rows(const Plan &P, const Buffers &B, uint32_t chunk, cudaStream_t s) {
    const uint32_t r0 = P.chunk_row[chunk], r1 = P.chunk_row[chunk + 1];
    if (r1 <= r0) return;
    DedupArgs a;
    a.seq = B.seq; a.off = B.seq_off;
    a.vbits = B.vbits; a.jbits = B.jbits; a.VW = P.VW; a.JW = P.JW;
    a.rep_off = B.rep_off; a.R = P.R; a.r0 = r0; a.r1 = r1;
    a.dtab = reinterpret_cast<uint2 *>(B.table); a.slot = B.slot;
    a.mask = B.table_mask; a.ctr = B.ctr;
    k_dedupe_insert<<<grid_wave(k_dedupe_insert, r1 - r0, kThreads), kThreads, 0, s>>>(a);
}

void launch_dedupe_final(const Plan &P, const Buffers &B, cudaStream_t s) {
    k_dedupe_final<<<grid_wave(k_dedupe_final, P.N, kThreads), kThreads, 0, s>>>(
        0, P.N, B.slot, reinterpret_cast<const uint2 *>(B.table), B.rep_row, B.flag);
}

void launch_uniques(const Plan &P, const Buffers &B, cudaStream_t s) {
    scan_u32(B.flag, B.uid_of_row, P.N, nullptr, &B.ctr->n_uniques, B.scan_part,
             B.scan_part_cap, s);
    k_uniques<<<grid_wave(k_uniques, P.N, kThreads), kThreads, 0, s>>>(P.N, B.seq_off, B.rep_off, P.R, B.slot,
                                                   reinterpret_cast<const uint2 *>(B.table),
                                                   B.rep_row, B.uid_of_row, B.urow, B.ucopies,
                                                   B.ulen, B.urep, B.row2uid);
    k_uid_first<<<(P.R + 1 + 255) / 256, 256, 0, s>>>(P.N, P.R, B.rep_off, B.row2uid, B.ctr,
                                                     B.uid_first);
}

void launch_uniques_rows(const Plan &P, const Buffers &B, uint32_t chunk, cudaStream_t s) {
    const uint32_t r0 = P.chunk_row[chunk], r1 = P.chunk_row[chunk + 1];
    if (r1 <= r0) return;   // its unique count stays 0
    k_dedupe_final<<<grid_wave(k_dedupe_final, r1 - r0, kThreads), kThreads, 0, s>>>(
        r0, r1, B.slot, reinterpret_cast<const uint2 *>(B.table), B.rep_row, B.flag);
    scan_u32(B.flag + r0, B.uid_of_row + r0, r1 - r0, nullptr, &B.ctr->chunk_uniques[chunk],
             B.scan_part, B.scan_part_cap, s);
    ChunkRows cr;
    cr.n = P.nchunks;
    for (uint32_t k = 0; k <= kMaxRowChunks; ++k) cr.row[k] = k <= P.nchunks ? P.chunk_row[k] : P.N;
    k_uniques_rows<<<grid_wave(k_uniques_rows, r1 - r0, kThreads), kThreads, 0, s>>>(
        chunk, cr, B.seq_off, B.rep_off, P.R, B.rep_row, B.uid_of_row, B.ctr, B.urow, B.ulen,
        B.urep, B.row2uid);
}

void launch_uniques_finish(const Plan &P, const Buffers &B, cudaStream_t s) {
    k_uniques_finish<<<grid_wave(k_uniques_finish, P.N, kThreads), kThreads, 0, s>>>(
        P.nchunks, B.ctr, B.urow, B.slot, reinterpret_cast<const uint2 *>(B.table), B.ucopies);
    k_uid_first<<<(P.R + 1 + 255) / 256, 256, 0, s>>>(P.N, P.R, B.rep_off, B.row2uid, B.ctr,
                                                     B.uid_first);
}

}  // namespace idb
