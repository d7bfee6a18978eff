// idb_internal.cuh -- device data layout, plan constants and kernel launchers
// shared by the translation units of libimmunodbscan_gb300.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "bitops.cuh"

namespace idb {

constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr int kMaxGeneWords = 8;        // 512 reference genes per gene column
constexpr int kFastMaxCodes = 32;       // alphabet of the fast (bit-plane) path
constexpr int kFastMaxWords = 4;        // 128 residues on the fast path
constexpr int kGenericMaxLen = 1024;    // Levenshtein on the generic path
constexpr int kDepthMax = 50;           // tree-depth histogram cap (cuda/PSDBSCAN.hcu:1029)
constexpr uint32_t kEdgeChunk = 256;    // edge slots reserved per warp at a time
constexpr uint32_t kSpinCap = 1u << 22; // bound of every device-side retry loop
constexpr int kMaxRowChunks = 8;        // host columns uploaded in at most this many row chunks
// Bin pairs with at most kSmallSide entries on each side (Hamming fast path) are
// evaluated pair-parallel: lanes take pairs, records travel by shuffles.
constexpr uint32_t kSmallSide = 32;
// A bin paired with itself with at most kTinySide entries is a tiny bin pair:
// one lane takes all of its pairs, 32 tiny bin pairs per warp at once.
constexpr uint32_t kTinySide = 8;
// Hamming with eps <= kJoinMaxEps for every length uses the segment join: two
// equal-length sequences within eps agree exactly on one of eps+1 segments.
// At eps 3 the quarter-length segments make groups large enough that the
// buckets evaluate their pairs faster (64 repertoires, 1M rows: 2.92 against
// 3.09 ms per call; eps 1: 1.25 against 0.99 ms for the join).
constexpr int kJoinMaxEps = 2;
constexpr int kMlpIn = 16;              // learned scheduler: features per bin pair
constexpr int kMlpHidden = 64;          // two hidden layers of 64
constexpr int kMlpParams = kMlpIn * kMlpHidden + kMlpHidden + kMlpHidden * kMlpHidden + kMlpHidden +
                           kMlpHidden + 1;

// where the distance kernel sends neighbour pairs
enum : uint32_t {
    kSinkEdges = 0u,   // the edge list (the graph phase reads it)
    kSinkCount = 1u,   // streamed mode, first sweep: copies-weighted counts
    kSinkGrow = 2u,    // streamed mode, second sweep: unions and border minima
};

// error bits raised by kernels (Counters::error)
enum : uint32_t {
    kErrHashStall = 1u,       // duplicate-table probe exceeded its bound
    kErrUnionStall = 2u,      // union-find retry exceeded its bound
    kErrEdgeOverflow = 4u,    // edge buffer too small (count still exact)
    kErrUnitOverflow = 8u,    // work-unit list exceeded its capacity
    kErrAlphabet = 16u,       // a byte outside the plan's code map
    kErrLength = 32u,         // a length outside the plan's range
    kErrBinPairOverflow = 64u,
    kErrEntryOverflow = 128u,
};

// Gene-name lookup table (built on the host per call): open addressing on the
// rolling hash h = h*kGeneHashMul + byte of a name; len 0 marks an empty slot.
constexpr uint32_t kGeneHashMul = 0x01000193u;
struct GeneEntry {
    uint32_t h;
    uint16_t len;
    uint16_t gene;
};
struct GeneMatcher {
    uint32_t ts = 0;             // table slots (power of two), 0 = no table
    uint32_t maxlen = 0;         // longest name
    uint32_t firstmask[8] = {};  // bytes that start some name
    uint32_t lenmask[8] = {};    // name lengths present (1..255)
    uint32_t long_names = 0;     // a name longer than 255 bytes exists
};

#ifdef __CUDACC__
// Sequential reader of a byte string in global memory, 4 bytes per step.  It
// loads only the aligned 4-byte words that hold bytes of the string (so no load
// leaves the string's pages) and joins neighbours with a funnel shift; bytes
// past the end of the string read as 0.
struct GlobalReader {
    const uint32_t *gw;
    uint32_t t, last, sh, prev, rem;
    __device__ __forceinline__ GlobalReader(const uint8_t *p, uint32_t len) {
        const uintptr_t a = reinterpret_cast<uintptr_t>(p);
        sh = (uint32_t)(a & 3u);
        gw = reinterpret_cast<const uint32_t *>(a - sh);
        last = len ? (sh + len - 1) >> 2 : 0u;
        t = 0;
        rem = len;
        prev = len ? __ldg(gw) : 0u;
    }
    __device__ __forceinline__ uint32_t next() {
        const uint32_t nx = t + 1 <= last ? __ldg(gw + t + 1) : 0u;
        uint32_t out = __funnelshift_r(prev, nx, 8 * sh);
        if (rem < 4) out &= (1u << (8 * rem)) - 1u;
        rem = rem < 4 ? 0u : rem - 4;
        prev = nx;
        ++t;
        return out;
    }
};
#endif

// Bytes [32c, 32c + 32) of a string p[0..L) as 8 little-endian words, bytes
// past L zero.  The aligned 4-byte words that hold those bytes are read with
// independent loads (all in flight at once), then shifted into place.
__device__ __forceinline__ void load_chunk32(const uint8_t *p, uint32_t L, uint32_t c,
                                             uint32_t (&w)[8]) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(p) + 32u * c;
    const uint32_t sh = (uint32_t)(a & 3u);
    const uint32_t *gw = reinterpret_cast<const uint32_t *>(a - sh);
    const uint32_t rem = L > 32u * c ? min(L - 32u * c, 32u) : 0u;
    const uint32_t nw = (sh + rem + 3u) >> 2;
    uint32_t v[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) v[k] = (uint32_t)k < nw ? __ldg(gw + k) : 0u;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        uint32_t o = __funnelshift_r(v[k], v[k + 1], 8u * sh);
        const uint32_t b = 4u * (uint32_t)k;
        if (b >= rem) o = 0u;
        else if (rem - b < 4u) o &= (1u << (8u * (rem - b))) - 1u;
        w[k] = o;
    }
}


// Device-resident counters of one clustering call (one struct, zeroed first).
struct Counters {
    uint32_t lmax, lmin;
    uint32_t used[8];            // 256-bit byte-presence map of the sequences
    uint32_t n_uniques;
    uint32_t n_entries;
    uint32_t n_binpairs;
    uint32_t n_units;
    uint32_t unit_cursor;        // persistent work queue head
    uint32_t edge_reserved;      // edge slots handed out (chunks)
    uint32_t n_edges;            // real edges written
    uint32_t n_cores;
    uint32_t n_clusters;
    uint32_t n_noise_rows;
    uint32_t error;
    uint32_t heavy_count;
    unsigned long long pairs_evaluated;
    unsigned long long admissible_pairs;
    unsigned long long stamp[8];  // %globaltimer at the phase boundaries (ns)
    unsigned long long lev_columns;  // text columns consumed by live Levenshtein pairs
    uint32_t n_small;            // small bin pairs handed to the pair-parallel path
    uint32_t small_cursor;       // their work queue head
    uint32_t n_heavy;            // bin pairs the learned predictor evaluates
    uint32_t n_core_edges;       // neighbour pairs with both ends core
    uint32_t n_jslots;           // segment join: table slots in use (the probed prefix)
    uint32_t n_jslots1;          // n_jslots + 1: the scan of group sizes ends with their total
    uint32_t chunk_uniques[kMaxRowChunks];   // uniques of each row chunk (numbered by chunk)
    uint32_t n_groups;           // segment join: keys held by two or more uniques
    uint32_t n_tiny;             // tiny bin pairs (one lane each), listed from the small list's end
    uint32_t tiny_cursor;        // their work queue head
};

// One bucket ("bin") holds the uniques of one (repertoire, V gene, J gene,
// length); a unique with V/J ambiguity sets sits in |V|*|J| bins.  Two uniques
// are V- and J-compatible iff they share a bin, and each compatible pair is
// evaluated in exactly one bin: its lowest common V gene and lowest common J
// gene (checked when a pair is a neighbour).
struct BinPair {
    uint32_t a_start, a_n;      // x entries [a_start, a_start+a_n)
    uint32_t b_start, b_n;      // y entries
    uint32_t unit_base;         // first work unit (exclusive scan, schedule order)
    uint32_t ncx;               // x chunks
    uint16_t la, lb;            // lengths of the two bins
    uint16_t v, j;              // the bins' V gene and J gene
    int16_t eps;                // neighbour threshold of the length pair
    uint8_t same;               // 1: a and b are the same bin (triangular units)
    uint8_t cls;                // schedule class
    uint32_t cost_lo;           // predicted cost (pairs or learned), low 32 bits
};
static_assert(sizeof(BinPair) == 40, "BinPair layout");

// Host-side plan of one call (everything the kernels need as constants).
struct Plan {
    uint32_t N = 0, R = 1;
    uint32_t Gv = 1, Gj = 1, VW = 1, JW = 1;     // genes and uint64 words per column
    uint32_t gene_bytes_v = 0, gene_bytes_j = 0; // bytes of the reference name lists
    GeneMatcher vmatch, jmatch;
    bool no_v = true, no_j = true, no_seq = false;
    bool hamming = false;
    uint32_t min_pts = 2;
    uint32_t Lmin = 0, Lmax = 0, NL = 1;
    uint32_t A = 1, B = 1, W = 1;                 // codes, bit planes, 32-bit words
    bool fast = true;
    uint32_t RS = 16;                             // record bytes per entry
    int dLmax = 0;                                // largest admissible length gap
    uint64_t nbins = 0;                           // sub-buckets (bins x K classes)
    uint32_t K = 4;                               // classes per bin
    uint32_t big_group = 64;                      // call-group size that gets its own class
    uint32_t TX = 256, TY = 256, RX = 8;          // unit shape (entries)
    int schedule = 0;
    int hamming_eps_mode = 0;                     // 0 popcount, 1 eps==1, 2 eps==0
    bool sig_exact = true;                        // V genes <= 64 and J genes <= 32
    bool join = false;                            // Hamming by segment join (eps <= kJoinMaxEps)
    uint32_t join_smax = 1;                       // most segments of any length
    bool streamed = false;                        // neighbour pairs not stored: the
                                                  // distance work runs twice
    uint64_t edge_budget = 0;                     // bytes for the edge list (0: no limit)
    // row chunks of the front end: host columns arrive chunk by chunk and the
    // gene-bitset and duplicate kernels of chunk k wait only for its rows
    uint32_t nchunks = 1;
    uint32_t chunk_row[kMaxRowChunks + 1] = {};   // [nchunks+1] row boundaries
    bool front_join = false;                      // segment-join inserts run by row chunk
    uint8_t codemap[256];
    int first_byte = -1;                          // byte value with code 0
    // capacities
    uint64_t cap_entries = 0, cap_binpairs = 0, cap_units = 0, cap_edges = 0;
};

// Scratch of the call-string collapse of one gene column.
struct CallScratch {
    unsigned long long *tab = nullptr;              // [mask+1] (hash hi 32 | row)
    uint32_t mask = 0;
    uint32_t *ref = nullptr;                        // [N] slot of the row's string or kNone
    uint32_t *todo = nullptr;                       // [N] rows that compute their own bitset;
                                                    // row chunk k lists its rows from chunk_row[k]
    uint32_t *ntodo = nullptr;                      // [kMaxRowChunks] list lengths per chunk
};

// Device buffers of one call (all carved from the context arena).
struct Buffers {
    // inputs (device)
    const uint8_t *seq = nullptr;  const int64_t *seq_off = nullptr;
    const uint8_t *vcall = nullptr; const int64_t *v_off = nullptr;
    const uint8_t *jcall = nullptr; const int64_t *j_off = nullptr;
    const uint8_t *vgenes = nullptr; const int32_t *vg_off = nullptr;
    const uint8_t *jgenes = nullptr; const int32_t *jg_off = nullptr;
    const GeneEntry *vtab = nullptr, *jtab = nullptr;
    const uint32_t *rep_off = nullptr;              // [R+1]
    const int16_t *eps_tab = nullptr;               // [NL*NL]
    const uint8_t *codemap = nullptr;               // [256]
    // row level [N]
    uint64_t *vbits = nullptr, *jbits = nullptr;    // [N*VW], [N*JW]
    uint64_t *rhash = nullptr;
    uint32_t *slot = nullptr, *rep_row = nullptr, *flag = nullptr, *uid_of_row = nullptr;
    uint32_t *row2uid = nullptr;
    // duplicate table
    uint32_t *table = nullptr, *tcount = nullptr;
    uint64_t table_mask = 0;
    // call-string collapse, one per gene column (V, J)
    CallScratch call[2];
    // uniques [N]
    uint32_t *urow = nullptr, *ucopies = nullptr, *ulen = nullptr, *urep = nullptr;
    // bins
    uint32_t *bin_hist = nullptr;                   // [nbins+1] -> bin_start
    uint32_t *bin_cursor = nullptr;                 // [nbins]
    uint32_t *uclass = nullptr;                     // [N] sub-bucket class per unique
    unsigned long long *sig_and = nullptr;          // [2*nbins] AND of V / J signatures
    uint32_t *ent_uid = nullptr;                    // [cap_entries]
    uint4 *ent_meta = nullptr;                      // [cap_entries] {sigV lo, sigV hi, sigJ, uid}
    uint4 *ent_rec = nullptr;                       // [cap_entries * RS/16]
    uint32_t *bp_count = nullptr;                   // [nbins+1]
    BinPair *bp = nullptr, *bp_sorted = nullptr;    // [cap_binpairs]
    uint32_t *bp_units = nullptr;                   // [cap_binpairs+1]
    uint32_t *bp_small = nullptr;                   // [cap_binpairs] schedule positions of small bin pairs
    // segment join: table of (unique, segment) keys and the groups they form
    // segment-join table: the keys (all ones = empty slot) and, apart, how
    // many (unique, segment) entries hold each key, so that the passes over
    // the slots read 4 bytes per slot
    unsigned long long *jn_key = nullptr;           // [jn_mask+1]
    uint32_t *jn_cnt = nullptr;                     // [jn_mask+1]
    uint64_t jn_mask = 0;
    uint32_t *jn_islot = nullptr;                   // [4*N] slot of (unique, segment)
    uint32_t *jn_start = nullptr;                   // [jn_mask+2] group size -> start, per table slot
    uint32_t *jn_bpidx = nullptr;                   // [jn_mask+2] bin pair of a slot's group
    uint32_t *jn_cur = nullptr;                     // [join_smax*N] rank of (unique, segment) in its group
    uint32_t *cls_hist = nullptr;                   // [65]
    float *pred = nullptr;                          // learned cost per bin pair
    // graph
    uint2 *edges = nullptr;                         // [cap_edges]
    uint32_t *cnt = nullptr;                        // [N] neighbour copies count
    uint32_t *ucore = nullptr;                      // [N]
    uint32_t *parent = nullptr;                     // [N]
    uint32_t *bmin = nullptr;                       // [N]
    uint32_t *rootflag = nullptr;                   // [N+1] -> rank
    uint32_t *uid_first = nullptr;                  // [R+1]
    uint32_t *depth_hist = nullptr;                 // [kDepthMax+1]
    // scan scratch
    uint32_t *scan_part = nullptr;                  // [scan_part_cap]
    uint32_t scan_part_cap = 0;
    // outputs (device)
    uint32_t *clone_id = nullptr;
    int32_t *core = nullptr;
    uint32_t *copies = nullptr;
    uint32_t *uniques = nullptr;
    Counters *ctr = nullptr;
    // per bin-pair timing log (optional)
    unsigned long long *bp_cycles = nullptr;
    uint32_t *bp_hits = nullptr;
};

// ---- launchers (each enqueues on `s`, never synchronises) ----
void launch_survey(const Plan &P, const Buffers &B, cudaStream_t s);
void launch_check_plan(const Plan &P, const Buffers &B, cudaStream_t s);
void launch_stamp(unsigned long long *dst, cudaStream_t s);
// The front end runs by row chunks [chunk_row[k], chunk_row[k+1]): the two
// init launchers once, then per chunk launch_gene_bits (V, then J) and
// launch_dedupe_rows, then launch_dedupe_final over all rows.
void launch_call_init(const Plan &P, const Buffers &B, bool v_column, cudaStream_t s);
void launch_gene_bits(const Plan &P, const Buffers &B, bool v_column, uint32_t chunk, cudaStream_t s);
void launch_dedupe_init(const Plan &P, const Buffers &B, cudaStream_t s);
void launch_dedupe_rows(const Plan &P, const Buffers &B, uint32_t chunk, cudaStream_t s);
void launch_dedupe_final(const Plan &P, const Buffers &B, cudaStream_t s);
// more than one row chunk: representatives and unique ids chunk by chunk
// (launch_uniques_rows after the chunk's launch_dedupe_rows), then the unique
// count and copies (launch_uniques_finish) in place of launch_dedupe_final +
// launch_uniques
void launch_uniques_rows(const Plan &P, const Buffers &B, uint32_t chunk, cudaStream_t s);
void launch_uniques_finish(const Plan &P, const Buffers &B, cudaStream_t s);
void launch_uniques(const Plan &P, const Buffers &B, cudaStream_t s);
void launch_buckets(const Plan &P, const Buffers &B, cudaStream_t s);
// segment join: clear the table (sized by the rows when front_join), then the
// inserts of every unique (chunk < 0) or of one row chunk's uniques
void launch_join_init(const Plan &P, const Buffers &B, cudaStream_t s);
void launch_join_insert(const Plan &P, const Buffers &B, int chunk, cudaStream_t s);
void launch_binpairs(const Plan &P, const Buffers &B, cudaStream_t s);
void launch_schedule(const Plan &P, const Buffers &B, cudaStream_t s);
void launch_distance(const Plan &P, const Buffers &B, int grid, cudaStream_t s,
                     uint32_t sink = kSinkEdges);
void launch_count_admissible(const Plan &P, const Buffers &B, cudaStream_t s);
// core_out: when set, the row core flags are written right after the core
// marking and the event is recorded there (an external record node in a
// captured graph), so their copy to the host can start before the labels.
void launch_graph(const Plan &P, const Buffers &B, bool trees, cudaStream_t s,
                  cudaEvent_t core_out = nullptr);
// streamed mode: both distance sweeps (counts, core flags, unions and border
// minima), then depths, compression and labels
void launch_streamed_sweeps(const Plan &P, const Buffers &B, cudaStream_t s);
void launch_streamed_labels(const Plan &P, const Buffers &B, bool trees, cudaStream_t s);
constexpr uint32_t kOutClone = 1, kOutCore = 2, kOutCopies = 4, kOutAll = 7;
void launch_outputs(const Plan &P, const Buffers &B, cudaStream_t s, uint32_t what = kOutAll);

// exclusive scan of n (host) or *n_dev (device, capacity n) uint32 values;
// out may alias in; *total (device) receives the sum when non-null.
void scan_u32(const uint32_t *in, uint32_t *out, uint32_t n, const uint32_t *n_dev,
              uint32_t *total, uint32_t *part, uint32_t part_cap, cudaStream_t s);
uint32_t scan_part_needed(uint64_t n);

void launch_features(const Buffers &B, uint32_t cap, float *feats, cudaStream_t s);
void launch_mlp_predict(const Buffers &B, uint32_t cap, const void *wq_bf16, cudaStream_t s);
void launch_mlp_grad(const float *X, const float *T, uint32_t n, const float *p, float scale,
                     float *grad, float *loss, cudaStream_t s);
void launch_adam(float *p, const float *grad, float *m, float *v, float lr, int step, cudaStream_t s);
void launch_to_bf16(const float *p, void *q, cudaStream_t s);
void launch_mlp_forward_rows(const float *X, uint32_t n, const void *wq_bf16, float *y,
                             cudaStream_t s);

int sm_count();
const char *distance_variant_name(const Plan &P);

// Blocks of a kernel resident on one SM at once (threads per block, dynamic
// shared memory), from the occupancy calculator; cached per kernel and device.
int resident_blocks(const void *kern, int threads, size_t smem);

// Grid of a grid-stride kernel over n items: one block per `threads` items, at
// most one full wave of resident blocks, so that no block starts in a second
// wave after the first has drained.
template <typename F>
inline int grid_wave(F *kern, uint64_t n, int threads, size_t smem = 0) {
    uint64_t g = (n + (uint64_t)threads - 1) / (uint64_t)threads;
    const uint64_t cap = (uint64_t)sm_count() *
                         (uint64_t)resident_blocks(reinterpret_cast<const void *>(kern), threads, smem);
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

}  // namespace idb
