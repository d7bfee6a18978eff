// idb_api.cu -- C ABI, contexts, workspace, plan and pipeline orchestration.
//
// The reference's boundary is InterlinkClass (cuda/Interlink.cu:34-95): build
// the V and J bitset containers, the string set, run DBSCAN::doScan
// (cuda/PSDBSCAN.hcu:1300-1356, nine phases each followed by
// cudaDeviceSynchronize) and copy clusters, cores, uniques and copies back.
// idb_cluster is that boundary with plain C types.  The pipeline here is
// device-driven: every kernel reads its work counts from device memory, so the
// same launch sequence runs eagerly (with a few size read-backs that grow the
// workspace) or replays from a captured CUDA graph (idb_batch_run).
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/immunodbscan_gb300.h"
#include "../../include/immunodbscan_gb300_diag.h"
#include "idb_internal.cuh"

namespace idb {
void launch_const_strings(uint8_t *blob, int64_t *off, uint32_t N, cudaStream_t s);
void launch_fill(const Plan &P, const Buffers &B, cudaStream_t s);
void launch_binpairs_fill(const Plan &P, const Buffers &B, cudaStream_t s);
}

namespace {

using namespace idb;

thread_local std::string g_err;

idb_status fail(idb_status st, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return st;
}

#define CU(call)                                                                        \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            if (e_ == cudaErrorMemoryAllocation)                                        \
                return fail(IDB_ERR_OUT_OF_MEMORY, "%s: %s", #call, cudaGetErrorString(e_)); \
            return fail(IDB_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_));         \
        }                                                                               \
    } while (0)

#define TRY(expr)                                 \
    do {                                          \
        idb_status st_ = (expr);                  \
        if (st_ != IDB_OK) return st_;            \
    } while (0)

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
};

enum BufId {
    bSeq, bSeqOff, bV, bVOff, bJ, bJOff, bVGenes, bVGOff, bJGenes, bJGOff, bRepOff, bEps, bCode,
    bVBits, bJBits, bSlot, bRepRow, bFlag, bUidOfRow, bRow2Uid, bTable, bTCount,
    bURow, bUCopies, bULen, bURep, bBinHist, bBinCursor, bEntUid, bEntRec, bBpCount, bBp,
    bBpSorted, bBpUnits, bClsHist, bPred, bEdges, bCnt, bUCore,
    bParent, bBMin, bRootFlag, bUidFirst, bDepth, bScanPart, bClone, bCore, bCopies, bUniques,
    bCtr, bVTab, bJTab, bSigAnd, bUClass, bEntMeta, bCallAux, bCallTab, bCallRef, bCallTodo, bBpSmall,
    bJnTab, bJnISlot, bJnStart, bJnCur, bJnBpIdx, bNumBufs
};

}  // namespace

struct idb_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t copy_stream = nullptr;   // host->device copies of the columns
    cudaStream_t side_stream = nullptr;   // the J column's call collapse, beside the V column's
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaEvent_t ev_seq = nullptr;         // sequence column copied
    cudaEvent_t ev_chunk[kMaxRowChunks] = {};   // call columns of row chunk k copied
    cudaEvent_t ev_out[2] = {};           // replays: row copies / core flags written
    DevBuf buf[bNumBufs];
    Counters *h_ctr = nullptr;        // pinned mirror of the counters
    cudaEvent_t ev[16] = {};
    // batch (graph) state
    bool planned = false;
    Plan plan;
    Buffers bufs;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    idb_output out_dev{};
    bool trees = false;
    uint32_t graph_kernels = 0;
    // learned schedule: MLP parameters (BF16 for inference)
    void *mlp_bf16 = nullptr;
    bool has_model = false;
    // bumped whenever a workspace buffer moves: a graph captured at another
    // generation would read freed memory and is not replayed
    uint64_t generation = 0;
    uint64_t batch_generation = 0;
    // bumped by every call that stages inputs: the staged gene tables,
    // repertoire offsets and columns a graph reads are those of that call
    uint64_t stage_epoch = 0;
    uint64_t batch_epoch = 0;
    // idb_cluster's plan cache (host inputs): the launch sequence of the last
    // input shape, captured after an eager call and replayed by later calls
    // with the same shape (see host_plan_*)
    struct HostPlan {
        bool valid = false;
        uint64_t generation = 0, epoch = 0;
        uint32_t N = 0, R = 0;
        std::vector<uint32_t> roff;
        idb_params prm{};
        bool no_v = false, no_j = false, no_seq = false, uniques = false, model = false;
        bool early_out = false;   // the graph records ev_out (row copies, row core flags)
        std::vector<char> vgenes, jgenes;
        std::vector<int64_t> vgoff, jgoff;
        Plan P;
        Buffers B;
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        uint32_t kernels = 0;
    } hp;
};

namespace {

idb_status ensure(idb_context *c, BufId id, size_t bytes, bool exact = false) {
    DevBuf &b = c->buf[id];
    if (bytes == 0) bytes = 16;
    if (b.cap >= bytes) return IDB_OK;
    if (b.p) CU(cudaFree(b.p));
    b.p = nullptr;
    b.cap = 0;
    ++c->generation;
    size_t want = exact ? bytes : bytes + bytes / 8 + 256;
    want = (want + 255) & ~(size_t)255;
    cudaError_t e = cudaMalloc(&b.p, want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(IDB_ERR_OUT_OF_MEMORY, "device allocation of %zu bytes failed", want);
    }
    b.cap = want;
    return IDB_OK;
}

template <typename T>
T *ptr(idb_context *c, BufId id) { return reinterpret_cast<T *>(c->buf[id].p); }

idb_status check_launch() {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(IDB_ERR_CUDA, "kernel launch: %s", cudaGetErrorString(e));
    return IDB_OK;
}

uint64_t next_pow2(uint64_t x) {
    uint64_t p = 1;
    while (p < x) p <<= 1;
    return p;
}

// eps(Lx,Ly) exactly as the reference computes it in single precision:
// (int)truncf((float)max(Lx,Ly) * threshold) (cuda/SpecialFunctors.hcu:257-261),
// capped by the absolute eps when that key is set.
int eps_value(uint32_t lx, uint32_t ly, float threshold, int32_t abs_eps) {
    int64_t e = INT32_MAX;
    if (!std::isnan(threshold)) {
        volatile float m = (float)(lx > ly ? lx : ly);
        volatile float prod = m * threshold;
        float t = truncf(prod);
        if (t >= 2147483647.0f) e = INT32_MAX;
        else if (t <= -2147483648.0f) e = INT32_MIN;
        else e = (int64_t)t;
    }
    if (abs_eps >= 0 && abs_eps < e) e = abs_eps;
    return (int)e;
}

// Bounds on the edit distance of two sequences joined through one or two
// intermediate neighbours (triangle inequality over the per-hop eps), as the
// reference's epsilonTwoFunctorClass / epsilonThreeFunctorClass define them
// (cuda/SpecialFunctors.hcu:276-344; unused by its clustering).  Single
// precision, in the reference's order of operations: an intermediate sequence
// within eps of a length-L sequence is at most L / (1 - t) long, so
//   two hops, Levenshtein: b = min(Lx/(1-t), Ly/(1-t));
//                          trunc((max(Lx, b) + max(b, Ly)) * t)
//   three hops:            b = min(Lx/(1-t), Ly/(1-t)/(1-t)),
//                          c = min(Ly/(1-t), Lx/(1-t)/(1-t));
//                          trunc((max(Lx, b) + max(c, b) + max(Ly, c)) * t)
//   Hamming (equal lengths): trunc(Lx * t * hops).
int eps_hops_value(uint32_t lx, uint32_t ly, float threshold, int hops, bool hamming) {
    volatile float t = threshold;
    volatile float fx = (float)lx, fy = (float)ly;
    if (hamming) {
        volatile float p = fx * t;
        volatile float q = p * (float)hops;
        return (int)truncf(q);
    }
    volatile float one_t = 1.0f - t;
    auto mx = [](float a, float b) { return a > b ? a : b; };
    auto mn = [](float a, float b) { return a < b ? a : b; };
    if (hops == 2) {
        volatile float bx = fx / one_t, by = fy / one_t;
        volatile float b = mn(bx, by);
        volatile float sum = mx(fx, b) + mx(b, fy);
        volatile float prod = sum * t;
        return (int)truncf(prod);
    }
    volatile float bx = fx / one_t, byy0 = fy / one_t;
    volatile float byy = byy0 / one_t;
    volatile float b = mn(bx, byy);
    volatile float cy = fy / one_t, cxx0 = fx / one_t;
    volatile float cxx = cxx0 / one_t;
    volatile float c = mn(cy, cxx);
    volatile float s1 = mx(fx, b) + mx(c, b);
    volatile float sum = s1 + mx(fy, c);
    volatile float prod = sum * t;
    return (int)truncf(prod);
}

idb_status get_ctx(idb_context **pc);

struct HostInputs {
    // staged or caller device pointers
    const uint8_t *seq; const int64_t *seq_off;
    const uint8_t *v; const int64_t *v_off;
    const uint8_t *j; const int64_t *j_off;
};

idb_status validate(const idb_input *in, const idb_params *prm, const idb_output *out) {
    if (!in || !prm || !out) return fail(IDB_ERR_INVALID_ARG, "NULL argument");
    if (in->n_rows > 0 && (!out->clone_id || !out->core || !out->copies))
        return fail(IDB_ERR_INVALID_ARG, "clone_id, core and copies outputs are required");
    if ((in->v_calls == nullptr) != (in->v_offsets == nullptr))
        return fail(IDB_ERR_INVALID_ARG, "v_calls and v_offsets must both be set or both NULL");
    if ((in->j_calls == nullptr) != (in->j_offsets == nullptr))
        return fail(IDB_ERR_INVALID_ARG, "j_calls and j_offsets must both be set or both NULL");
    if ((in->seqs == nullptr) != (in->seq_offsets == nullptr))
        return fail(IDB_ERR_INVALID_ARG, "seqs and seq_offsets must both be set or both NULL");
    if (in->v_calls && in->n_v_genes && (!in->v_genes || !in->v_gene_offsets))
        return fail(IDB_ERR_INVALID_ARG, "V reference gene list missing");
    if (in->j_calls && in->n_j_genes && (!in->j_genes || !in->j_gene_offsets))
        return fail(IDB_ERR_INVALID_ARG, "J reference gene list missing");
    if (in->v_calls && in->n_v_genes > 64u * kMaxGeneWords)
        return fail(IDB_ERR_UNSUPPORTED, "at most %d V reference genes", 64 * kMaxGeneWords);
    if (in->j_calls && in->n_j_genes > 64u * kMaxGeneWords)
        return fail(IDB_ERR_UNSUPPORTED, "at most %d J reference genes", 64 * kMaxGeneWords);
    if (std::isnan(prm->threshold) && prm->abs_eps < 0)
        return fail(IDB_ERR_INVALID_ARG, "neither threshold nor abs_eps is set");
    if (prm->candidates != 0 && prm->candidates != 1)
        return fail(IDB_ERR_INVALID_ARG, "candidates must be 0 (automatic) or 1 (buckets)");
    if (prm->row_chunks < 0 || prm->row_chunks > kMaxRowChunks)
        return fail(IDB_ERR_INVALID_ARG, "row_chunks must be 0 (automatic) to %d", kMaxRowChunks);
    if (in->n_repertoires > 0 && in->rep_offsets) {
        if (in->rep_offsets[0] != 0 || in->rep_offsets[in->n_repertoires] != in->n_rows)
            return fail(IDB_ERR_INVALID_ARG, "rep_offsets must start at 0 and end at n_rows");
        for (uint32_t r = 0; r < in->n_repertoires; ++r)
            if (in->rep_offsets[r] > in->rep_offsets[r + 1])
                return fail(IDB_ERR_INVALID_ARG, "rep_offsets must be non-decreasing");
    }
    if (in->n_rows >= 0x7FFFFFFFu) return fail(IDB_ERR_UNSUPPORTED, "at most 2^31-2 rows");
    return IDB_OK;
}

// Gene name lists -> device (host memory always), plus the hash table of the
// names used by the gene-bitset kernel.
idb_status upload_genes(idb_context *c, const char *names, const int64_t *off, uint32_t G,
                        BufId blob_id, BufId off_id, BufId tab_id, uint32_t *bytes_out,
                        GeneMatcher *gm) {
    ++c->stage_epoch;   // the gene tables a captured graph reads are replaced
    std::vector<int32_t> o(G + 1);
    const int64_t base = G ? off[0] : 0;
    for (uint32_t g = 0; g <= G; ++g) o[g] = (int32_t)(off[g] - base);
    const size_t nb = G ? (size_t)(off[G] - base) : 0;
    // table: slots >= 2*G, power of two
    *gm = GeneMatcher();
    uint32_t ts = 16;
    while (ts < 2 * G) ts <<= 1;
    std::vector<GeneEntry> tab(ts, GeneEntry{0, 0, 0});
    for (uint32_t g = 0; g < G; ++g) {
        const uint32_t L = (uint32_t)(o[g + 1] - o[g]);
        if (L == 0) continue;                         // an empty name never matches
        if (L > 255) { gm->long_names = 1; continue; }
        const uint8_t *nm = reinterpret_cast<const uint8_t *>(names + base + o[g]);
        uint32_t h = 0;
        for (uint32_t k = 0; k < L; ++k) h = h * kGeneHashMul + nm[k];
        uint32_t sl = h & (ts - 1);
        while (tab[sl].len != 0) sl = (sl + 1) & (ts - 1);
        tab[sl] = GeneEntry{h, (uint16_t)L, (uint16_t)g};
        gm->firstmask[nm[0] >> 5] |= 1u << (nm[0] & 31);
        gm->lenmask[L >> 5] |= 1u << (L & 31);
        gm->maxlen = std::max(gm->maxlen, L);
    }
    gm->ts = ts;
    TRY(ensure(c, blob_id, nb + 16));
    TRY(ensure(c, off_id, sizeof(int32_t) * (G + 1)));
    TRY(ensure(c, tab_id, sizeof(GeneEntry) * ts));
    if (nb) CU(cudaMemcpyAsync(c->buf[blob_id].p, names + base, nb, cudaMemcpyHostToDevice, c->stream));
    CU(cudaMemcpyAsync(c->buf[off_id].p, o.data(), sizeof(int32_t) * (G + 1), cudaMemcpyHostToDevice,
                       c->stream));
    CU(cudaMemcpyAsync(c->buf[tab_id].p, tab.data(), sizeof(GeneEntry) * ts, cudaMemcpyHostToDevice,
                       c->stream));
    CU(cudaStreamSynchronize(c->stream));   // o and tab are locals
    *bytes_out = (uint32_t)nb;
    return IDB_OK;
}

struct Pipeline {
    idb_context *c = nullptr;
    Plan P;
    Buffers B;
    bool trees = false;
    bool timing = false;
    std::vector<int16_t> eps_host;
    // host inputs arrive on the copy stream: the sequence column first (the
    // survey waits for it), then the call columns row chunk by row chunk (the
    // gene-bitset kernels of chunk k wait for its event).  In a graph capture
    // the waits become external event-wait nodes, so a replay waits for the
    // copies its own call issued.
    cudaEvent_t wait_seq = nullptr;
    cudaEvent_t wait_chunk[kMaxRowChunks] = {};
    bool external_waits = false;
    // a captured call writes the row copies after the uniques and the row core
    // flags after the core marking, each followed by an event record node, so
    // that a replay copies them to the host while the rest of the path runs
    bool early_out = false;
    bool copies_issued = false;
    bool allow_join = true;   // the segment join finds neighbours, not all admissible pairs
    // every return path (errors included) leaves no copy from the caller's host
    // buffers in flight
    ~Pipeline() {
        if (copies_issued && c) cudaStreamSynchronize(c->copy_stream);
    }
};

void record(Pipeline &pl, int k) {
    if (pl.timing) launch_stamp(&pl.B.ctr->stamp[k], pl.c->stream);
}

// phase durations from the device time stamps (ms)
void phase_times(const Counters &h, idb_stats *st) {
    for (int k = 0; k < 5; ++k)
        st->ms_phase[k] = h.stamp[k + 1] > h.stamp[k] ? 1e-6 * (double)(h.stamp[k + 1] - h.stamp[k]) : 0.0;
    st->ms_distance = st->ms_phase[2];
}

// Row chunks of the front end.  Host columns of 2^20 rows or more are copied
// and pre-processed in kMaxRowChunks chunks (or `want`, 1..kMaxRowChunks), so
// that the gene-bitset and duplicate kernels of a chunk run while the next
// chunks are being copied; device-resident columns are one chunk.  Chunk i of
// k holds (k - i) / (k (k + 1) / 2) of the rows: the first chunks are the
// largest and the last one, whose front end runs after the last copy, is the
// smallest.  (A chunk's front end takes less time than its copy, so every
// earlier chunk is done before the next one has arrived.)  Inner boundaries
// are multiples of 32 rows.
void set_row_chunks(Plan &P, bool host_inputs, int want) {
    uint32_t k = 1;
    if (host_inputs) {
        if (want > 0) k = (uint32_t)std::min(want, kMaxRowChunks);
        else if (P.N >= (1u << 20)) k = kMaxRowChunks;
    }
    P.nchunks = k;
    P.chunk_row[0] = 0;
    const uint64_t total = (uint64_t)k * (k + 1) / 2;
    uint64_t acc = 0;
    for (uint32_t i = 1; i < k; ++i) {
        acc += k - (i - 1);
        P.chunk_row[i] = (uint32_t)(((uint64_t)P.N * acc / total) & ~31ull);
    }
    P.chunk_row[k] = P.N;
}

// Host columns onto the copy stream in the order the device needs them: the
// sequences (for the survey), then the V and J calls of each row chunk, each
// followed by its event.  Copies of a column go into its staging buffer at the
// host offsets, so chunk k's bytes and offsets land where the kernels read them.
idb_status issue_host_copies(idb_context *c, const Plan &P, const idb_input *in) {
    cudaStream_t cs = c->copy_stream;
    const size_t N = P.N;
    if (!P.no_seq) {
        if (in->seq_offsets[N])
            CU(cudaMemcpyAsync(c->buf[bSeq].p, in->seqs, (size_t)in->seq_offsets[N],
                               cudaMemcpyHostToDevice, cs));
        CU(cudaMemcpyAsync(c->buf[bSeqOff].p, in->seq_offsets, 8 * (N + 1), cudaMemcpyHostToDevice, cs));
    }
    CU(cudaEventRecord(c->ev_seq, cs));
    // a chunk's bytes are copied from and to 16-byte boundaries (copies that
    // start and end unaligned ran about 10 % slower): the 16-byte block that
    // holds a chunk boundary is copied by both chunks, with the same bytes
    auto column = [&](const char *src, const int64_t *off, BufId bid, BufId oid, uint32_t r0,
                      uint32_t r1) -> idb_status {
        const int64_t b0 = off[r0] & ~(int64_t)15, b1 = std::min<int64_t>((off[r1] + 15) & ~(int64_t)15, off[N]);
        if (b1 > b0)
            CU(cudaMemcpyAsync(static_cast<char *>(c->buf[bid].p) + b0, src + b0, (size_t)(b1 - b0),
                               cudaMemcpyHostToDevice, cs));
        CU(cudaMemcpyAsync(static_cast<int64_t *>(c->buf[oid].p) + r0, off + r0,
                           8 * ((size_t)(r1 - r0) + 1), cudaMemcpyHostToDevice, cs));
        return IDB_OK;
    };
    for (uint32_t k = 0; k < P.nchunks; ++k) {
        const uint32_t r0 = P.chunk_row[k], r1 = P.chunk_row[k + 1];
        if (!P.no_v) TRY(column(in->v_calls, in->v_offsets, bV, bVOff, r0, r1));
        if (!P.no_j) TRY(column(in->j_calls, in->j_offsets, bJ, bJOff, r0, r1));
        CU(cudaEventRecord(c->ev_chunk[k], cs));
    }
    return IDB_OK;
}

// Stage 0: inputs in place, counters zeroed, survey run and read back.
idb_status stage_inputs_and_survey(Pipeline &pl, const idb_input *in, bool host_inputs,
                                   int row_chunks = 0) {
    idb_context *c = pl.c;
    Plan &P = pl.P;
    Buffers &B = pl.B;
    cudaStream_t s = c->stream;
    ++c->stage_epoch;
    P.N = in->n_rows;
    P.R = (in->n_repertoires > 0 && in->rep_offsets) ? in->n_repertoires : 1;
    P.no_v = in->v_calls == nullptr;
    P.no_j = in->j_calls == nullptr;
    P.no_seq = in->seqs == nullptr;
    set_row_chunks(P, host_inputs, row_chunks);
    TRY(ensure(c, bCtr, sizeof(Counters)));
    B.ctr = ptr<Counters>(c, bCtr);
    CU(cudaMemsetAsync(B.ctr, 0, sizeof(Counters), s));
    CU(cudaMemsetAsync(&B.ctr->lmin, 0xFF, sizeof(uint32_t), s));   // min starts at max
    // staging buffers of host columns (device columns are read in place)
    auto place = [&](const char *src, const int64_t *off, BufId bid, BufId oid,
                     const uint8_t **dst, const int64_t **doff) -> idb_status {
        if (!host_inputs) {
            *dst = reinterpret_cast<const uint8_t *>(src);
            *doff = off;
            return IDB_OK;
        }
        TRY(ensure(c, bid, (size_t)(P.N ? off[P.N] : 0) + 16));
        TRY(ensure(c, oid, sizeof(int64_t) * ((size_t)P.N + 1)));
        *dst = ptr<uint8_t>(c, bid);
        *doff = ptr<int64_t>(c, oid);
        return IDB_OK;
    };
    if (P.no_seq) {
        TRY(ensure(c, bSeq, 4 * (size_t)P.N + 16));
        TRY(ensure(c, bSeqOff, sizeof(int64_t) * ((size_t)P.N + 1)));
        launch_const_strings(ptr<uint8_t>(c, bSeq), ptr<int64_t>(c, bSeqOff), P.N, s);
        B.seq = ptr<uint8_t>(c, bSeq);
        B.seq_off = ptr<int64_t>(c, bSeqOff);
    } else {
        TRY(place(in->seqs, in->seq_offsets, bSeq, bSeqOff, &B.seq, &B.seq_off));
    }
    if (!P.no_v) TRY(place(in->v_calls, in->v_offsets, bV, bVOff, &B.vcall, &B.v_off));
    if (!P.no_j) TRY(place(in->j_calls, in->j_offsets, bJ, bJOff, &B.jcall, &B.j_off));
    if (host_inputs) {
        // every copy is issued now; the survey waits for the sequences only and
        // the host derives the plan while the call columns are still arriving
        pl.copies_issued = true;
        TRY(issue_host_copies(c, P, in));
        CU(cudaStreamWaitEvent(s, c->ev_seq, 0));
        for (uint32_t k = 0; k < P.nchunks; ++k) pl.wait_chunk[k] = c->ev_chunk[k];
    }
    // repertoire offsets
    std::vector<uint32_t> roff(P.R + 1);
    if (in->n_repertoires > 0 && in->rep_offsets) {
        for (uint32_t r = 0; r <= P.R; ++r) roff[r] = in->rep_offsets[r];
    } else {
        roff[0] = 0;
        roff[1] = P.N;
    }
    TRY(ensure(c, bRepOff, sizeof(uint32_t) * (P.R + 1)));
    CU(cudaMemcpyAsync(c->buf[bRepOff].p, roff.data(), sizeof(uint32_t) * (P.R + 1),
                       cudaMemcpyHostToDevice, s));
    B.rep_off = ptr<uint32_t>(c, bRepOff);
    // gene lists
    P.Gv = P.no_v ? 1 : in->n_v_genes;
    P.Gj = P.no_j ? 1 : in->n_j_genes;
    if (!P.no_v)
        TRY(upload_genes(c, in->v_genes, in->v_gene_offsets, P.Gv, bVGenes, bVGOff, bVTab,
                         &P.gene_bytes_v, &P.vmatch));
    if (!P.no_j)
        TRY(upload_genes(c, in->j_genes, in->j_gene_offsets, P.Gj, bJGenes, bJGOff, bJTab,
                         &P.gene_bytes_j, &P.jmatch));
    B.vgenes = ptr<uint8_t>(c, bVGenes); B.vg_off = ptr<int32_t>(c, bVGOff);
    B.jgenes = ptr<uint8_t>(c, bJGenes); B.jg_off = ptr<int32_t>(c, bJGOff);
    B.vtab = ptr<GeneEntry>(c, bVTab); B.jtab = ptr<GeneEntry>(c, bJTab);
    P.VW = P.Gv > 64 ? (P.Gv + 63) / 64 : 1;
    P.JW = P.Gj > 64 ? (P.Gj + 63) / 64 : 1;
    if (P.Gv == 0) P.Gv = 1;   // a V column with an empty reference list: all bitsets 0
    if (P.Gj == 0) P.Gj = 1;
    record(pl, 0);
    launch_survey(P, B, s);
    TRY(check_launch());
    CU(cudaMemcpyAsync(c->h_ctr, B.ctr, sizeof(Counters), cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    return IDB_OK;
}

// Work-unit shape: rx x-entries per lane (the kernels are compiled for
// Hamming 4 or 8 with one word, 4 otherwise, and 2 with one word for the
// segment join; Levenshtein 1, or 2 with one word) and ty y-entries, a multiple
// of 32*rx up to 4096.  Invalid values are ignored.
void apply_shape(Plan &P, int rx, int ty) {
    if (rx > 0) {
        if (P.hamming && (rx == 4 || ((rx == 8 || rx == 2) && P.W == 1))) P.RX = rx;
        if (!P.hamming && (rx == 1 || (rx == 2 && P.W == 1))) P.RX = rx;
        P.TX = 32 * P.RX;
    }
    if (P.TY % P.TX) P.TY = P.TX * ((P.TY + P.TX - 1) / P.TX);
    if (ty > 0 && ty >= (int)P.TX && ty % (int)P.TX == 0 && ty <= 4096) P.TY = ty;
}

// Plan constants from the survey.
idb_status derive_plan(Pipeline &pl, const idb_params *prm) {
    Plan &P = pl.P;
    const Counters &h = *pl.c->h_ctr;
    P.hamming = prm->use_hamming != 0;
    P.min_pts = prm->min_pts;
    P.schedule = prm->schedule;
    P.streamed = prm->edge_memory_mb < 0;
    P.edge_budget = prm->edge_memory_mb > 0 ? (uint64_t)prm->edge_memory_mb << 20 : 0;
    P.Lmin = P.N ? h.lmin : 0;
    P.Lmax = P.N ? h.lmax : 0;
    if (P.Lmin > P.Lmax) P.Lmin = P.Lmax;
    if (P.Lmax > 65535) return fail(IDB_ERR_UNSUPPORTED, "sequences longer than 65535 bytes");
    P.NL = P.Lmax - P.Lmin + 1;
    // alphabet: codes = ranks of the byte values present
    std::memset(P.codemap, 0, sizeof P.codemap);
    uint32_t A = 0;
    P.first_byte = -1;
    for (int b = 0; b < 256; ++b)
        if ((h.used[b >> 5] >> (b & 31)) & 1u) {
            if (A == 0) P.first_byte = b;
            P.codemap[b] = (uint8_t)A++;
        }
    P.A = A ? A : 1;
    P.W = P.Lmax > 32 ? (P.Lmax + 31) / 32 : 1;
    P.fast = P.A <= (uint32_t)kFastMaxCodes && P.Lmax <= 32u * kFastMaxWords;
    if (!P.hamming && !P.fast && P.Lmax > (uint32_t)kGenericMaxLen)
        return fail(IDB_ERR_UNSUPPORTED, "Levenshtein mode supports sequences up to %d bytes",
                    kGenericMaxLen);
    if (P.fast && P.hamming) {
        P.B = P.A <= 4 ? 2 : 5;
        P.RS = ((P.B * P.W * 4) + 15) & ~15u;
    } else {
        P.B = 8;
        P.RS = ((P.Lmax > 0 ? P.Lmax : 1) + 15) & ~15u;
    }
    // unit shape
    if (P.fast && P.hamming) {
        P.RX = P.W == 1 ? 8 : 4;
        P.TX = 32 * P.RX;
        P.TY = 256;
    } else if (P.fast) {
        P.RX = 1;
        P.TX = 32;
        P.TY = 256;
    } else {
        P.RX = 1;
        P.TX = 32;
        P.TY = 256;
    }
    if (P.fast) apply_shape(P, prm->tile_rx, prm->tile_ty);
    // eps table over the length range, and the largest admissible gap
    pl.eps_host.assign((size_t)P.NL * P.NL, 0);
    int dl = 0;
    int emin_same = INT32_MAX, emax_same = INT32_MIN;
    for (uint32_t a = 0; a < P.NL; ++a)
        for (uint32_t b = 0; b < P.NL; ++b) {
            int e = eps_value(P.Lmin + a, P.Lmin + b, prm->threshold, prm->abs_eps);
            if (e > 32767) e = 32767;
            if (e < -1) e = -1;
            pl.eps_host[(size_t)a * P.NL + b] = (int16_t)e;
            if (b >= a && e >= (int)(b - a) && (int)(b - a) > dl) dl = (int)(b - a);
            if (a == b) { emin_same = std::min(emin_same, e); emax_same = std::max(emax_same, e); }
        }
    P.dLmax = P.hamming ? 0 : dl;
    P.hamming_eps_mode = 0;
    if (P.hamming && emin_same == emax_same && emin_same == 1) P.hamming_eps_mode = 1;
    if (P.hamming && emin_same == emax_same && emin_same == 0) P.hamming_eps_mode = 2;
    P.K = 4;
    P.big_group = 64;
    P.sig_exact = P.Gv <= 64 && P.Gj <= 32;
    // Hamming with a small eps at every length: candidate pairs by segment join
    // (the side records then carry the V bits and the J bits with the segment;
    // a key holds the repertoire in 24 bits and the table at most 2^31 slots)
    P.join = pl.allow_join && prm->candidates == 0 && P.hamming && P.fast && emax_same <= kJoinMaxEps &&
             P.Gv <= 64 && P.Gj <= 30 && P.R < (1u << 24) - 1 &&
             2ull * (uint64_t)(emax_same + 1) * P.N <= (1ull << 30);
    P.join_smax = P.join ? (uint32_t)std::max(1, emax_same + 1) : 1u;
    // with row chunks the uniques are numbered and the join's inserts run chunk
    // by chunk, while later chunks are still being copied
    P.front_join = P.join && P.nchunks > 1;
    if (P.hamming && P.RX == 2 && !P.join) {   // 2 x-entries per lane: segment join only
        P.RX = 4;
        P.TX = 128;
        if (P.TY % P.TX) P.TY = P.TX * ((P.TY + P.TX - 1) / P.TX);
    }
    // segment join without a requested shape: 2 x-entries per lane, 512 y-entries
    // (its groups are mostly small: narrower x-chunks leave fewer lanes idle)
    if (P.join && P.W == 1 && prm->tile_rx <= 0) {
        P.RX = 2;
        P.TX = 64;
        if (prm->tile_ty <= 0) P.TY = 512;
        if (P.TY % P.TX) P.TY = P.TX * ((P.TY + P.TX - 1) / P.TX);
    }
    P.nbins = (uint64_t)P.R * P.Gv * P.Gj * P.NL * P.K;
    if (P.nbins >= (1ull << 31))
        return fail(IDB_ERR_UNSUPPORTED, "too many buckets (repertoires x V genes x J genes x lengths = %llu)",
                    (unsigned long long)P.nbins);
    return IDB_OK;
}

// Scratch of the call-string collapse of both gene columns: per column a
// table of min(N, 2^20) rounded up to a power of two 8-byte slots (at least
// 512), a slot per row and a list of the rows that compute their own bitset.
// Its own memory, so that a row chunk's duplicate kernel can run between the
// call collapses of the next chunk.
idb_status alloc_call_scratch(idb_context *c, Buffers &B, uint64_t N) {
    const uint64_t slots = std::min<uint64_t>(next_pow2(std::max<uint64_t>(N, 512)), 1u << 20);
    TRY(ensure(c, bCallTab, 2 * 8 * slots));
    TRY(ensure(c, bCallRef, 2 * 4 * N));
    TRY(ensure(c, bCallTodo, 2 * 4 * N));
    TRY(ensure(c, bCallAux, 2 * 4 * kMaxRowChunks));
    for (int k = 0; k < 2; ++k) {
        CallScratch &cs = B.call[k];
        cs.tab = ptr<unsigned long long>(c, bCallTab) + k * slots;
        cs.mask = (uint32_t)(slots - 1);
        cs.ref = ptr<uint32_t>(c, bCallRef) + k * N;
        cs.todo = ptr<uint32_t>(c, bCallTodo) + k * N;
        cs.ntodo = ptr<uint32_t>(c, bCallAux) + k * kMaxRowChunks;
    }
    return IDB_OK;
}

// Workspace for everything sized by N and the plan.

idb_status alloc_fixed(Pipeline &pl) {
    idb_context *c = pl.c;
    Plan &P = pl.P;
    Buffers &B = pl.B;
    const size_t N = P.N, N1 = N + 1;
    TRY(ensure(c, bEps, sizeof(int16_t) * pl.eps_host.size()));
    TRY(ensure(c, bCode, 256));
    CU(cudaMemcpyAsync(c->buf[bEps].p, pl.eps_host.data(), sizeof(int16_t) * pl.eps_host.size(),
                       cudaMemcpyHostToDevice, c->stream));
    CU(cudaMemcpyAsync(c->buf[bCode].p, P.codemap, 256, cudaMemcpyHostToDevice, c->stream));
    B.eps_tab = ptr<int16_t>(c, bEps);
    B.codemap = ptr<uint8_t>(c, bCode);
    TRY(ensure(c, bVBits, sizeof(uint64_t) * N * P.VW));
    TRY(ensure(c, bJBits, sizeof(uint64_t) * N * P.JW));
    TRY(ensure(c, bSlot, 4 * N));
    TRY(ensure(c, bRepRow, 4 * N));
    TRY(ensure(c, bFlag, 4 * N1));
    TRY(ensure(c, bUidOfRow, 4 * N1));
    TRY(ensure(c, bRow2Uid, 4 * N));
    const uint64_t tcap = next_pow2(std::max<uint64_t>(2 * N, 1024));
    TRY(ensure(c, bTable, 8 * tcap));     // duplicate table: {row, ~size} per slot
    TRY(ensure(c, bTCount, 4 * tcap));
    TRY(ensure(c, bURow, 4 * N1));
    TRY(ensure(c, bUCopies, 4 * N1));
    TRY(ensure(c, bULen, 4 * N1));
    TRY(ensure(c, bURep, 4 * N1));
    TRY(ensure(c, bBinHist, 4 * (P.nbins + 1)));
    TRY(ensure(c, bBinCursor, 4 * (P.nbins + 1)));
    TRY(ensure(c, bSigAnd, 16 * (P.nbins + 1)));
    TRY(ensure(c, bUClass, 4 * N1));
    TRY(ensure(c, bBpCount, 4 * (P.nbins + 1)));
    TRY(ensure(c, bClsHist, 4 * 130));
    TRY(ensure(c, bCnt, 4 * N1));
    TRY(ensure(c, bUCore, 4 * N1));
    TRY(ensure(c, bParent, 4 * N1));
    TRY(ensure(c, bBMin, 4 * N1));
    TRY(ensure(c, bRootFlag, 4 * N1));
    TRY(ensure(c, bUidFirst, 4 * (P.R + 1)));
    TRY(ensure(c, bDepth, 4 * (kDepthMax + 1)));
    uint64_t scan_n = std::max<uint64_t>(N1, P.nbins + 1);
    if (P.join) {
        // keys: at most join_smax per unique; the table at load <= 1/2
        const uint64_t heads = (uint64_t)P.join_smax * N;
        const uint64_t jcap = next_pow2(std::max<uint64_t>(2 * heads, 1024));
        TRY(ensure(c, bJnTab, (sizeof(unsigned long long) + sizeof(uint32_t)) * jcap));
        TRY(ensure(c, bJnISlot, 16 * N1));
        TRY(ensure(c, bJnStart, 4 * (jcap + 1)));   // group sizes -> starts, per table slot
        TRY(ensure(c, bJnCur, 4 * (heads + 1)));    // rank of each (unique, segment) in its group
        TRY(ensure(c, bJnBpIdx, 4 * (jcap + 1)));
        B.jn_key = ptr<unsigned long long>(c, bJnTab);
        B.jn_cnt = reinterpret_cast<uint32_t *>(B.jn_key + jcap);
        B.jn_mask = jcap - 1;
        B.jn_islot = ptr<uint32_t>(c, bJnISlot);
        B.jn_start = ptr<uint32_t>(c, bJnStart);
        B.jn_cur = ptr<uint32_t>(c, bJnCur);
        B.jn_bpidx = ptr<uint32_t>(c, bJnBpIdx);
        scan_n = std::max<uint64_t>(scan_n, jcap + 1);
    }
    B.scan_part_cap = scan_part_needed(std::max<uint64_t>(scan_n, 1u << 20));
    TRY(ensure(c, bScanPart, 4 * (size_t)B.scan_part_cap));
    B.vbits = ptr<uint64_t>(c, bVBits); B.jbits = ptr<uint64_t>(c, bJBits);
    B.slot = ptr<uint32_t>(c, bSlot); B.rep_row = ptr<uint32_t>(c, bRepRow);
    B.flag = ptr<uint32_t>(c, bFlag); B.uid_of_row = ptr<uint32_t>(c, bUidOfRow);
    B.row2uid = ptr<uint32_t>(c, bRow2Uid);
    B.table = ptr<uint32_t>(c, bTable); B.tcount = ptr<uint32_t>(c, bTCount);
    B.table_mask = tcap - 1;
    TRY(alloc_call_scratch(c, B, N));
    B.urow = ptr<uint32_t>(c, bURow); B.ucopies = ptr<uint32_t>(c, bUCopies);
    B.ulen = ptr<uint32_t>(c, bULen); B.urep = ptr<uint32_t>(c, bURep);
    B.bin_hist = ptr<uint32_t>(c, bBinHist); B.bin_cursor = ptr<uint32_t>(c, bBinCursor);
    B.sig_and = ptr<unsigned long long>(c, bSigAnd); B.uclass = ptr<uint32_t>(c, bUClass);
    B.bp_count = ptr<uint32_t>(c, bBpCount); B.cls_hist = ptr<uint32_t>(c, bClsHist);
    B.cnt = ptr<uint32_t>(c, bCnt); B.ucore = ptr<uint32_t>(c, bUCore);
    B.parent = ptr<uint32_t>(c, bParent); B.bmin = ptr<uint32_t>(c, bBMin);
    B.rootflag = ptr<uint32_t>(c, bRootFlag); B.uid_first = ptr<uint32_t>(c, bUidFirst);
    B.depth_hist = ptr<uint32_t>(c, bDepth);
    B.scan_part = ptr<uint32_t>(c, bScanPart);
    return IDB_OK;
}

idb_status alloc_entries(Pipeline &pl, uint64_t n_entries) {
    idb_context *c = pl.c;
    pl.P.cap_entries = std::max<uint64_t>(n_entries, 1);
    TRY(ensure(c, bEntUid, 4 * pl.P.cap_entries));
    TRY(ensure(c, bEntRec, (size_t)pl.P.RS * pl.P.cap_entries));
    TRY(ensure(c, bEntMeta, 16 * pl.P.cap_entries));
    pl.B.ent_meta = ptr<uint4>(c, bEntMeta);
    pl.B.ent_uid = ptr<uint32_t>(c, bEntUid);
    pl.B.ent_rec = ptr<uint4>(c, bEntRec);
    return IDB_OK;
}

idb_status alloc_binpairs(Pipeline &pl, uint64_t n_bp) {
    idb_context *c = pl.c;
    pl.P.cap_binpairs = std::max<uint64_t>(n_bp, 1);
    TRY(ensure(c, bBp, sizeof(BinPair) * pl.P.cap_binpairs));
    TRY(ensure(c, bBpSorted, sizeof(BinPair) * pl.P.cap_binpairs));
    TRY(ensure(c, bBpUnits, 4 * (pl.P.cap_binpairs + 1)));
    TRY(ensure(c, bBpSmall, 4 * (pl.P.cap_binpairs + 1)));
    TRY(ensure(c, bPred, 4 * (pl.P.cap_binpairs + 1)));
    const uint64_t need = scan_part_needed(pl.P.cap_binpairs + 1);
    if (need > pl.B.scan_part_cap) {
        pl.B.scan_part_cap = (uint32_t)need;
        TRY(ensure(c, bScanPart, 4 * (size_t)need));
        pl.B.scan_part = ptr<uint32_t>(c, bScanPart);
    }
    pl.B.bp = ptr<BinPair>(c, bBp);
    pl.B.bp_sorted = ptr<BinPair>(c, bBpSorted);
    pl.B.bp_units = ptr<uint32_t>(c, bBpUnits);
    pl.B.bp_small = ptr<uint32_t>(c, bBpSmall);
    pl.B.pred = ptr<float>(c, bPred);
    return IDB_OK;
}

idb_status alloc_edges(Pipeline &pl, uint64_t cap) {
    idb_context *c = pl.c;
    cap = std::max<uint64_t>(cap, 4096);
    if (cap > 0xFFFFFFF0ull) return fail(IDB_ERR_UNSUPPORTED, "more than 2^32 neighbour pairs");
    TRY(ensure(c, bEdges, sizeof(uint2) * cap, true));
    // a list kept from an earlier call may hold more pairs: use all of it (up to
    // the edge-memory budget), so that a call whose pairs fit it sweeps once
    uint64_t held = std::min<uint64_t>(c->buf[bEdges].cap / sizeof(uint2), 0xFFFFFFF0ull);
    if (pl.P.edge_budget) held = std::min<uint64_t>(held, pl.P.edge_budget / sizeof(uint2));
    pl.P.cap_edges = std::max(cap, held);
    pl.B.edges = ptr<uint2>(c, bEdges);
    return IDB_OK;
}

idb_status read_counters(Pipeline &pl) {
    CU(cudaMemcpyAsync(pl.c->h_ctr, pl.B.ctr, sizeof(Counters), cudaMemcpyDeviceToHost, pl.c->stream));
    CU(cudaStreamSynchronize(pl.c->stream));
    return IDB_OK;
}

idb_status device_errors(const Counters &h) {
    if (h.error & kErrHashStall) return fail(IDB_ERR_DEVICE_STALL, "duplicate table probe gave up");
    if (h.error & kErrUnionStall) return fail(IDB_ERR_DEVICE_STALL, "union-find retry bound reached");
    if (h.error & (kErrAlphabet | kErrLength))
        return fail(IDB_ERR_REPLAN, "inputs no longer match the captured plan");
    if (h.error & (kErrEdgeOverflow | kErrUnitOverflow | kErrBinPairOverflow | kErrEntryOverflow))
        return fail(IDB_ERR_CAPACITY, "a plan capacity was exceeded (error bits 0x%x)", h.error);
    return IDB_OK;
}

// Phases after the survey.  With `eager`, sizes are read back and buffers grown
// between phases; otherwise (graph capture) the capacities in P are used as-is.
// Gene bitsets, duplicate collapse and unique numbering, row chunk by row
// chunk: chunk k's kernels wait for its copies (when they are still in flight)
// and nothing else.  With more than one chunk a chunk's representatives and
// unique ids are final once its rows are in the duplicate table, so they are
// numbered (and, for the segment join, inserted into the join table) before
// the next chunk arrives.
idb_status launch_front(Pipeline &pl, cudaStream_t s) {
    const Plan &P = pl.P;
    const Buffers &B = pl.B;
    launch_call_init(P, B, true, s);
    launch_call_init(P, B, false, s);
    launch_dedupe_init(P, B, s);
    if (P.front_join) launch_join_init(P, B, s);
    for (uint32_t k = 0; k < P.nchunks; ++k) {
        if (pl.wait_chunk[k])
            CU(cudaStreamWaitEvent(s, pl.wait_chunk[k], pl.external_waits ? cudaEventWaitExternal : 0));
        // the two gene columns are independent: J on the side stream, joined
        // back before the duplicate collapse (parallel branches in a graph)
        const bool fork = !P.no_v && !P.no_j;
        if (fork) {
            CU(cudaEventRecord(pl.c->ev_fork, s));
            CU(cudaStreamWaitEvent(pl.c->side_stream, pl.c->ev_fork, 0));
        }
        launch_gene_bits(P, B, true, k, s);
        launch_gene_bits(P, B, false, k, fork ? pl.c->side_stream : s);
        if (fork) {
            CU(cudaEventRecord(pl.c->ev_join, pl.c->side_stream));
            CU(cudaStreamWaitEvent(s, pl.c->ev_join, 0));
        }
        launch_dedupe_rows(P, B, k, s);
        if (P.nchunks > 1) launch_uniques_rows(P, B, k, s);
        if (P.front_join) launch_join_insert(P, B, (int)k, s);
    }
    if (P.nchunks > 1) {
        launch_uniques_finish(P, B, s);
    } else {
        launch_dedupe_final(P, B, s);
        launch_uniques(P, B, s);
    }
    // a later run of the phases finds the columns in place
    if (!pl.external_waits)
        for (auto &e : pl.wait_chunk) e = nullptr;
    return IDB_OK;
}

idb_status run_phases(Pipeline &pl, bool eager, bool stop_after_schedule = false) {
    idb_context *c = pl.c;
    Plan &P = pl.P;
    Buffers &B = pl.B;
    cudaStream_t s = c->stream;
    if (!eager) launch_check_plan(P, B, s);
    TRY(launch_front(pl, s));
    if (pl.early_out) {
        launch_outputs(P, B, s, kOutCopies);
        CU(cudaEventRecordWithFlags(c->ev_out[0], s, cudaEventRecordExternal));
    }
    TRY(check_launch());
    record(pl, 1);
    launch_buckets(P, B, s);
    if (eager) {
        TRY(read_counters(pl));
        TRY(alloc_entries(pl, c->h_ctr->n_entries));
    }
    launch_fill(P, B, s);
    launch_binpairs(P, B, s);
    TRY(check_launch());
    if (eager) {
        TRY(read_counters(pl));
        TRY(alloc_binpairs(pl, c->h_ctr->n_binpairs));
    }
    launch_binpairs_fill(P, B, s);
    if (P.schedule == 1) {
        if (!c->has_model) return fail(IDB_ERR_INVALID_ARG, "learned schedule requested but no model loaded (idb_mlp_load)");
        launch_mlp_predict(B, (uint32_t)P.cap_binpairs, c->mlp_bf16, s);
    }
    launch_schedule(P, B, s);
    TRY(check_launch());
    record(pl, 2);
    if (stop_after_schedule) return IDB_OK;
    // The neighbour pairs go to an edge list for the graph phase, unless they
    // would take more than the edge memory allowed (or than the device has):
    // then the streamed mode keeps no list and runs the distance work twice.
    const uint64_t kEdgeBytes = sizeof(uint2);   // one list entry per neighbour pair
    if (eager && !P.streamed && P.cap_edges == 0) {
        uint64_t first = std::max<uint64_t>(4ull * P.N, 1ull << 16);
        if (P.edge_budget) first = std::max<uint64_t>(std::min(first, P.edge_budget / kEdgeBytes), 4096);
        TRY(alloc_edges(pl, first));
    }
    for (int attempt = 0; !P.streamed && attempt < 3; ++attempt) {
        launch_distance(P, B, 0, s);
        TRY(check_launch());
        if (!eager) break;
        TRY(read_counters(pl));
        const Counters &h = *c->h_ctr;
        if (!(h.error & kErrEdgeOverflow)) break;
        // grow to the exact requirement and sweep again, or stream
        const uint64_t need = (uint64_t)h.edge_reserved + 64ull * kEdgeChunk * 1024;
        if ((P.edge_budget && need * kEdgeBytes > P.edge_budget) || need > 0xFFFFFFF0ull) {
            P.streamed = true;
        } else {
            const idb_status st = alloc_edges(pl, need);
            if (st == IDB_ERR_OUT_OF_MEMORY) P.streamed = true;
            else if (st != IDB_OK) return st;
        }
        const uint32_t clear_err = h.error & ~kErrEdgeOverflow;
        CU(cudaMemsetAsync(&B.ctr->unit_cursor, 0, 4, s));
        CU(cudaMemsetAsync(&B.ctr->edge_reserved, 0, 4, s));
        CU(cudaMemsetAsync(&B.ctr->n_edges, 0, 4, s));
        CU(cudaMemsetAsync(&B.ctr->pairs_evaluated, 0, 8, s));
        CU(cudaMemsetAsync(&B.ctr->lev_columns, 0, 8, s));
        CU(cudaMemcpyAsync(&B.ctr->error, &clear_err, 4, cudaMemcpyHostToDevice, s));
        CU(cudaStreamSynchronize(s));
    }
    if (P.streamed) {
        launch_streamed_sweeps(P, B, s);
        TRY(check_launch());
        record(pl, 3);
        launch_streamed_labels(P, B, pl.trees, s);
    } else {
        record(pl, 3);
        launch_graph(P, B, pl.trees, s, pl.early_out ? c->ev_out[1] : nullptr);
    }
    record(pl, 4);
    launch_outputs(P, B, s, pl.early_out ? kOutClone : kOutAll);
    TRY(check_launch());
    record(pl, 5);
    return IDB_OK;
}

idb_status fill_stats(Pipeline &pl, idb_stats *st) {
    if (!st) return IDB_OK;
    const Counters &h = *pl.c->h_ctr;
    std::memset(st, 0, sizeof *st);
    st->n_uniques = h.n_uniques;
    st->n_cores = h.n_cores;
    st->n_clusters = h.n_clusters;
    st->n_noise_rows = h.n_noise_rows;
    st->pairs_evaluated = h.pairs_evaluated;
    st->neighbour_pairs = h.n_edges;
    st->n_entries = h.n_entries;
    st->n_units = h.n_units;
    st->lev_columns = h.lev_columns;
    st->core_edges = h.n_core_edges;
    st->candidates = pl.P.join ? 1u : 0u;
    st->streamed = pl.P.streamed ? 1u : 0u;
    if (pl.timing) {
        phase_times(h, st);
        st->ms_total = h.stamp[5] > h.stamp[0] ? 1e-6 * (double)(h.stamp[5] - h.stamp[0]) : 0.0;
    }
    return IDB_OK;
}

// ---------------------------------------------------------------------------
// idb_cluster's plan cache.  An eager call reads sizes back from the device
// between phases (survey, bucket entries, bin pairs, edge overflow) and so
// waits on the device several times.  When a second call arrives with the same
// shape -- row count, repertoire offsets, gene lists, parameters, which columns
// are present -- its eager run is followed by a capture of the whole launch
// sequence with capacities of the graph path (idb_batch_plan); later calls of
// that shape copy their columns into the same staging buffers and replay the
// graph, with one wait at the end.  The graph starts with the plan check
// (k_check_plan): data whose lengths or byte alphabet fall outside the plan,
// or that outgrows a capacity, reports IDB_ERR_REPLAN / IDB_ERR_CAPACITY and
// the call runs eagerly instead, so a replay never changes an answer.

bool same_params(const idb_params &a, const idb_params &b) {
    uint32_t ta, tb;
    std::memcpy(&ta, &a.threshold, 4);
    std::memcpy(&tb, &b.threshold, 4);
    return ta == tb && a.abs_eps == b.abs_eps && a.min_pts == b.min_pts &&
           a.use_hamming == b.use_hamming && a.schedule == b.schedule && a.tile_rx == b.tile_rx &&
           a.tile_ty == b.tile_ty && a.candidates == b.candidates &&
           a.edge_memory_mb == b.edge_memory_mb && a.row_chunks == b.row_chunks;
}

void gene_key(const char *names, const int64_t *off, uint32_t G, std::vector<char> &b,
              std::vector<int64_t> &o) {
    o.assign((size_t)G + 1, 0);
    const int64_t base = G ? off[0] : 0;
    for (uint32_t g = 0; g <= G; ++g) o[g] = off[g] - base;
    b.assign(G ? names + base : nullptr, G ? names + base + o[G] : nullptr);
}

bool same_genes(const char *names, const int64_t *off, uint32_t G, const std::vector<char> &b,
                const std::vector<int64_t> &o) {
    if (o.size() != (size_t)G + 1) return false;
    const int64_t base = G ? off[0] : 0;
    for (uint32_t g = 0; g <= G; ++g)
        if (off[g] - base != o[g]) return false;
    return !G || std::memcmp(names + base, b.data(), (size_t)o[G]) == 0;
}

// Does this call have the shape of the cached key?
bool host_plan_key_matches(const idb_context *c, const idb_input *in, const idb_params *prm,
                           const idb_output *out) {
    const auto &h = c->hp;
    const uint32_t R = (in->n_repertoires > 0 && in->rep_offsets) ? in->n_repertoires : 1;
    if (h.N != in->n_rows || h.R != R || h.roff.size() != (size_t)R + 1) return false;
    if (h.no_v != (in->v_calls == nullptr) || h.no_j != (in->j_calls == nullptr) ||
        h.no_seq != (in->seqs == nullptr) || h.uniques != (out->uniques != nullptr))
        return false;
    if (!same_params(h.prm, *prm)) return false;
    if (in->n_repertoires > 0 && in->rep_offsets) {
        if (std::memcmp(h.roff.data(), in->rep_offsets, 4 * ((size_t)R + 1)) != 0) return false;
    } else if (h.roff[0] != 0 || h.roff[1] != in->n_rows) {
        return false;
    }
    if (!h.no_v && !same_genes(in->v_genes, in->v_gene_offsets, in->n_v_genes, h.vgenes, h.vgoff))
        return false;
    if (!h.no_j && !same_genes(in->j_genes, in->j_gene_offsets, in->n_j_genes, h.jgenes, h.jgoff))
        return false;
    return true;
}

void host_plan_set_key(idb_context *c, const idb_input *in, const idb_params *prm,
                       const idb_output *out) {
    auto &h = c->hp;
    h.N = in->n_rows;
    h.R = (in->n_repertoires > 0 && in->rep_offsets) ? in->n_repertoires : 1;
    if (in->n_repertoires > 0 && in->rep_offsets) h.roff.assign(in->rep_offsets, in->rep_offsets + h.R + 1);
    else h.roff = {0u, in->n_rows};
    h.no_v = in->v_calls == nullptr;
    h.no_j = in->j_calls == nullptr;
    h.no_seq = in->seqs == nullptr;
    h.uniques = out->uniques != nullptr;
    h.prm = *prm;
    if (!h.no_v) gene_key(in->v_genes, in->v_gene_offsets, in->n_v_genes, h.vgenes, h.vgoff);
    if (!h.no_j) gene_key(in->j_genes, in->j_gene_offsets, in->n_j_genes, h.jgenes, h.jgoff);
    h.valid = true;
}

void host_plan_drop_graph(idb_context *c) {
    auto &h = c->hp;
    if (h.exec) cudaGraphExecDestroy(h.exec);
    if (h.graph) cudaGraphDestroy(h.graph);
    h.exec = nullptr;
    h.graph = nullptr;
}

uint32_t graph_kernel_count(cudaGraph_t g) {
    size_t nn = 0;
    if (cudaGraphGetNodes(g, nullptr, &nn) != cudaSuccess) return 0;
    std::vector<cudaGraphNode_t> nodes(nn);
    if (cudaGraphGetNodes(g, nodes.data(), &nn) != cudaSuccess) return 0;
    uint32_t k = 0;
    for (auto nd : nodes) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nd, &t) == cudaSuccess) k += t == cudaGraphNodeTypeKernel;
    }
    return k;
}

// After a successful eager call of the cached shape: capacities with headroom,
// then the capture of the launch sequence over the staging buffers.
idb_status host_plan_capture(Pipeline &pl) {
    idb_context *c = pl.c;
    auto &h = c->hp;
    host_plan_drop_graph(c);
    const Counters hc = *c->h_ctr;
    TRY(alloc_entries(pl, (uint64_t)hc.n_entries + hc.n_entries / 16 + 1024));
    TRY(alloc_binpairs(pl, (uint64_t)hc.n_binpairs + hc.n_binpairs / 16 + 1024));
    if (!pl.P.streamed)
        TRY(alloc_edges(pl, (uint64_t)hc.edge_reserved + hc.edge_reserved / 8 + 64ull * kEdgeChunk * 1024));
    cudaStream_t s = c->stream;
    CU(cudaStreamSynchronize(s));
    pl.timing = true;
    pl.trees = false;
    // a replay's copies are issued on the copy stream before the graph is
    // launched: the graph waits on their events (external event-wait nodes)
    pl.external_waits = true;
    for (uint32_t k = 0; k < kMaxRowChunks; ++k) pl.wait_chunk[k] = k < pl.P.nchunks ? c->ev_chunk[k] : nullptr;
    pl.early_out = !pl.P.streamed;
    CU(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    cudaMemsetAsync(pl.B.ctr, 0, sizeof(Counters), s);
    cudaMemsetAsync(&pl.B.ctr->lmin, 0xFF, sizeof(uint32_t), s);
    record(pl, 0);
    cudaStreamWaitEvent(s, c->ev_seq, cudaEventWaitExternal);
    launch_survey(pl.P, pl.B, s);
    idb_status st = run_phases(pl, false);
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamEndCapture(s, &g);
    if (st != IDB_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (ce != cudaSuccess) return fail(IDB_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
    h.graph = g;
    CU(cudaGraphInstantiate(&h.exec, g, 0));
    CU(cudaGraphUpload(h.exec, s));   // device-side setup now, not in the first replay
    CU(cudaStreamSynchronize(s));
    h.kernels = graph_kernel_count(g);
    h.P = pl.P;
    h.B = pl.B;
    h.model = c->has_model;
    h.early_out = pl.early_out;
    h.generation = c->generation;
    h.epoch = c->stage_epoch;
    return IDB_OK;
}

// Replay for host inputs of the cached shape.  IDB_ERR_REPLAN / IDB_ERR_CAPACITY
// send the call to the eager path.
idb_status host_plan_run(idb_context *c, const idb_input *in, idb_output *out) {
    auto &h = c->hp;
    const size_t N = h.N;
    // the staging buffers must hold this call's columns without moving
    auto fits = [&](BufId bid, BufId oid, const int64_t *off) {
        return c->buf[bid].cap >= (size_t)off[N] + 16 && c->buf[oid].cap >= 8 * (N + 1);
    };
    if ((!h.no_seq && !fits(bSeq, bSeqOff, in->seq_offsets)) ||
        (!h.no_v && !fits(bV, bVOff, in->v_offsets)) || (!h.no_j && !fits(bJ, bJOff, in->j_offsets)))
        return fail(IDB_ERR_CAPACITY, "columns larger than the cached plan's staging buffers");
    cudaStream_t s = c->stream, cs = c->copy_stream;
    struct CopyGuard {   // no copy from the caller's buffers stays in flight
        cudaStream_t cs;
        ~CopyGuard() { cudaStreamSynchronize(cs); }
    } guard{cs};
    // the copies go first on the copy stream; the graph's event-wait nodes hold
    // each part of the path until the rows it reads have arrived
    TRY(issue_host_copies(c, h.P, in));
    CU(cudaEventRecord(c->ev[0], s));
    CU(cudaGraphLaunch(h.exec, s));
    CU(cudaEventRecord(c->ev[1], s));
    const Buffers &B = h.B;
    if (h.early_out) {
        // the launch records ev_out[0] once the row copies are written and
        // ev_out[1] once the row core flags are: their copies to the host run
        // on the copy stream while the graph goes on
        CU(cudaStreamWaitEvent(cs, c->ev_out[0], 0));
        CU(cudaMemcpyAsync(out->copies, B.copies, 4 * N, cudaMemcpyDeviceToHost, cs));
        CU(cudaStreamWaitEvent(cs, c->ev_out[1], 0));
        CU(cudaMemcpyAsync(out->core, B.core, 4 * N, cudaMemcpyDeviceToHost, cs));
    }
    CU(cudaMemcpyAsync(c->h_ctr, B.ctr, sizeof(Counters), cudaMemcpyDeviceToHost, s));
    CU(cudaMemcpyAsync(out->clone_id, B.clone_id, 4 * N, cudaMemcpyDeviceToHost, s));
    if (!h.early_out) {
        CU(cudaMemcpyAsync(out->core, B.core, 4 * N, cudaMemcpyDeviceToHost, s));
        CU(cudaMemcpyAsync(out->copies, B.copies, 4 * N, cudaMemcpyDeviceToHost, s));
    }
    CU(cudaStreamSynchronize(s));
    CU(cudaStreamSynchronize(cs));
    TRY(device_errors(*c->h_ctr));
    const Counters &hc = *c->h_ctr;
    if (out->uniques) CU(cudaMemcpy(out->uniques, B.uniques, 4 * (size_t)hc.n_uniques, cudaMemcpyDeviceToHost));
    if (out->n_uniques) *out->n_uniques = hc.n_uniques;
    if (out->stats) {
        idb_stats *st = out->stats;
        std::memset(st, 0, sizeof *st);
        st->n_uniques = hc.n_uniques;
        st->n_cores = hc.n_cores;
        st->n_clusters = hc.n_clusters;
        st->n_noise_rows = hc.n_noise_rows;
        st->pairs_evaluated = hc.pairs_evaluated;
        st->neighbour_pairs = hc.n_edges;
        st->n_entries = hc.n_entries;
        st->n_units = hc.n_units;
        st->lev_columns = hc.lev_columns;
        st->core_edges = hc.n_core_edges;
        st->candidates = h.P.join ? 1u : 0u;
        st->streamed = h.P.streamed ? 1u : 0u;
        phase_times(hc, st);
        st->ms_total = hc.stamp[5] > hc.stamp[0] ? 1e-6 * (double)(hc.stamp[5] - hc.stamp[0]) : 0.0;
        st->kernel_launches = h.kernels;
    }
    return IDB_OK;
}

idb_status cluster_impl(idb_context *c, const idb_input *in, const idb_params *prm,
                        idb_output *out, bool host_io) {
    TRY(validate(in, prm, out));
    CU(cudaSetDevice(c->device));
    cudaGetLastError();   // a stale error of an unrelated call must not fail this one
    Pipeline pl;
    pl.c = c;
    pl.trees = prm->eval_trees != 0 && out->tree_depth_hist != nullptr;
    pl.timing = out->stats != nullptr;
    if (in->n_rows == 0) {
        if (out->n_uniques) *out->n_uniques = 0;
        if (out->stats) std::memset(out->stats, 0, sizeof *out->stats);
        return IDB_OK;
    }
    // the plan cache serves host inputs without the tree-depth statistics
    const bool cacheable = host_io && !pl.trees && (prm->schedule != 1 || c->has_model);
    bool seen = false;
    if (cacheable && c->hp.valid && host_plan_key_matches(c, in, prm, out)) {
        seen = true;
        if (c->hp.exec && c->hp.generation == c->generation && c->hp.epoch == c->stage_epoch &&
            c->hp.model == c->has_model) {
            const idb_status st = host_plan_run(c, in, out);
            if (st != IDB_ERR_REPLAN && st != IDB_ERR_CAPACITY) return st;
            host_plan_drop_graph(c);   // the data outgrew the plan: eager, then capture anew
        }
    }
    TRY(stage_inputs_and_survey(pl, in, host_io, prm->row_chunks));
    TRY(derive_plan(pl, prm));
    TRY(alloc_fixed(pl));
    Buffers &B = pl.B;
    const size_t N = pl.P.N;
    if (host_io) {
        TRY(ensure(c, bClone, 4 * N));
        TRY(ensure(c, bCore, 4 * N));
        TRY(ensure(c, bCopies, 4 * N));
        B.clone_id = ptr<uint32_t>(c, bClone);
        B.core = ptr<int32_t>(c, bCore);
        B.copies = ptr<uint32_t>(c, bCopies);
        if (out->uniques) {
            TRY(ensure(c, bUniques, 4 * N));
            B.uniques = ptr<uint32_t>(c, bUniques);
        }
    } else {
        B.clone_id = out->clone_id;
        B.core = out->core;
        B.copies = out->copies;
        B.uniques = out->uniques;
    }
    TRY(run_phases(pl, true));
    cudaStream_t s = c->stream;
    if (host_io) {
        CU(cudaMemcpyAsync(out->clone_id, B.clone_id, 4 * N, cudaMemcpyDeviceToHost, s));
        CU(cudaMemcpyAsync(out->core, B.core, 4 * N, cudaMemcpyDeviceToHost, s));
        CU(cudaMemcpyAsync(out->copies, B.copies, 4 * N, cudaMemcpyDeviceToHost, s));
    }
    CU(cudaMemcpyAsync(c->h_ctr, B.ctr, sizeof(Counters), cudaMemcpyDeviceToHost, s));
    std::vector<uint32_t> hist(kDepthMax + 1);
    if (pl.trees)
        CU(cudaMemcpyAsync(hist.data(), B.depth_hist, 4 * (kDepthMax + 1), cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    TRY(device_errors(*c->h_ctr));
    const uint32_t nu = c->h_ctr->n_uniques;
    if (out->uniques) {
        if (host_io)
            CU(cudaMemcpy(out->uniques, B.uniques, 4 * (size_t)nu, cudaMemcpyDeviceToHost));
    }
    if (out->n_uniques) {
        if (host_io) *out->n_uniques = nu;
        else CU(cudaMemcpy(out->n_uniques, &nu, 4, cudaMemcpyHostToDevice));
    }
    if (pl.trees) std::memcpy(out->tree_depth_hist, hist.data(), 4 * (kDepthMax + 1));
    TRY(fill_stats(pl, out->stats));
    if (cacheable) {
        // the second eager call of a shape captures it; a failed capture only
        // means the next call runs eagerly too
        if (seen && host_plan_capture(pl) != IDB_OK) {
            cudaGetLastError();
            host_plan_drop_graph(c);
        }
        host_plan_set_key(c, in, prm, out);
        g_err.clear();
    }
    return IDB_OK;
}

thread_local idb_context *t_default_ctx = nullptr;

idb_status get_ctx(idb_context **pc) {
    if (*pc) return IDB_OK;
    if (!t_default_ctx) TRY(idb_context_create(0, &t_default_ctx));
    *pc = t_default_ctx;
    return IDB_OK;
}

}  // namespace

namespace idb {
void set_last_error(const char *msg) { g_err = msg ? msg : ""; }

int resident_blocks(const void *kern, int threads, size_t smem) {
    struct Entry { const void *k; int threads; size_t smem; int dev; int blocks; };
    static std::mutex mu;
    static std::vector<Entry> cache;
    int d = 0;
    cudaGetDevice(&d);
    std::lock_guard<std::mutex> lock(mu);
    for (const Entry &e : cache)
        if (e.k == kern && e.threads == threads && e.smem == smem && e.dev == d) return e.blocks;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem) != cudaSuccess)
        per_sm = 0;
    if (per_sm <= 0) per_sm = 1;
    cache.push_back(Entry{kern, threads, smem, d, per_sm});
    return per_sm;
}

int sm_count() {
    static thread_local int dev = -1, n = 0;
    int d = 0;
    cudaGetDevice(&d);
    if (d != dev) {
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, d);
        if (n <= 0) n = 1;
        dev = d;
    }
    return n;
}
}  // namespace idb

// ============================================================================
// C ABI
// ============================================================================
extern "C" {

int idb_abi_version(void) { return IDB_ABI_VERSION; }

const char *idb_status_string(idb_status s) {
    switch (s) {
        case IDB_OK: return "ok";
        case IDB_ERR_INVALID_ARG: return "invalid argument";
        case IDB_ERR_CUDA: return "CUDA error";
        case IDB_ERR_NO_DEVICE: return "no usable CUDA device";
        case IDB_ERR_UNSUPPORTED: return "unsupported input";
        case IDB_ERR_OUT_OF_MEMORY: return "out of device memory";
        case IDB_ERR_CAPACITY: return "plan capacity exceeded";
        case IDB_ERR_DEVICE_STALL: return "bounded device wait gave up";
        case IDB_ERR_REPLAN: return "inputs no longer match the plan";
    }
    return "unknown status";
}

idb_status idb_host_alloc(size_t bytes, void **out) {
    if (!out) return fail(IDB_ERR_INVALID_ARG, "NULL output pointer");
    *out = nullptr;
    const cudaError_t e = cudaMallocHost(out, bytes ? bytes : 1);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *out = nullptr;
        return fail(IDB_ERR_OUT_OF_MEMORY, "page-locked allocation of %zu bytes failed: %s", bytes,
                    cudaGetErrorString(e));
    }
    return IDB_OK;
}

idb_status idb_host_free(void *p) {
    if (p) CU(cudaFreeHost(p));
    return IDB_OK;
}

size_t idb_last_error(char *buf, size_t size) {
    if (buf && size) {
        std::snprintf(buf, size, "%s", g_err.c_str());
    }
    return g_err.size();
}

idb_status idb_context_create(int device, idb_context **out) {
    if (!out) return fail(IDB_ERR_INVALID_ARG, "NULL context pointer");
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return fail(IDB_ERR_NO_DEVICE, "no CUDA device");
    }
    if (device < 0 || device >= n) return fail(IDB_ERR_NO_DEVICE, "device %d not present", device);
    cudaDeviceProp prop;
    CU(cudaGetDeviceProperties(&prop, device));
    if (prop.major * 10 + prop.minor < 100)
        return fail(IDB_ERR_NO_DEVICE, "device %d is sm_%d%d; this library targets sm_103", device,
                    prop.major, prop.minor);
    CU(cudaSetDevice(device));
    idb_context *c = new idb_context();
    c->device = device;
    CU(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    CU(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
    CU(cudaStreamCreateWithFlags(&c->side_stream, cudaStreamNonBlocking));
    CU(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
    CU(cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming));
    CU(cudaEventCreateWithFlags(&c->ev_seq, cudaEventDisableTiming));
    for (auto &e : c->ev_out) CU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    for (auto &e : c->ev_chunk) CU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    CU(cudaMallocHost(&c->h_ctr, sizeof(Counters)));
    for (auto &e : c->ev) CU(cudaEventCreate(&e));
    *out = c;
    return IDB_OK;
}

idb_status idb_context_destroy(idb_context *c) {
    if (!c) return IDB_OK;
    cudaSetDevice(c->device);
    if (c->exec) cudaGraphExecDestroy(c->exec);
    if (c->graph) cudaGraphDestroy(c->graph);
    host_plan_drop_graph(c);
    for (auto &b : c->buf)
        if (b.p) cudaFree(b.p);
    for (auto &e : c->ev)
        if (e) cudaEventDestroy(e);
    if (c->h_ctr) cudaFreeHost(c->h_ctr);
    if (c->mlp_bf16) cudaFree(c->mlp_bf16);
    if (c->ev_seq) cudaEventDestroy(c->ev_seq);
    for (auto e : c->ev_out)
        if (e) cudaEventDestroy(e);
    for (auto e : c->ev_chunk)
        if (e) cudaEventDestroy(e);
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    if (c->side_stream) cudaStreamDestroy(c->side_stream);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->stream) cudaStreamDestroy(c->stream);
    if (c == t_default_ctx) t_default_ctx = nullptr;
    delete c;
    return IDB_OK;
}

idb_status idb_cluster(idb_context *ctx, const idb_input *in, const idb_params *prm,
                       idb_output *out) {
    TRY(get_ctx(&ctx));
    return cluster_impl(ctx, in, prm, out, true);
}

idb_status idb_cluster_device(idb_context *ctx, const idb_input *in, const idb_params *prm,
                              idb_output *out) {
    TRY(get_ctx(&ctx));
    return cluster_impl(ctx, in, prm, out, false);
}

idb_status idb_batch_plan(idb_context *c, const idb_input *in, const idb_params *prm,
                          const idb_output *out) {
    if (!c) return fail(IDB_ERR_INVALID_ARG, "idb_batch_plan needs an explicit context");
    TRY(validate(in, prm, out));
    if (in->n_rows == 0) return fail(IDB_ERR_INVALID_ARG, "empty input");
    CU(cudaSetDevice(c->device));
    if (c->exec) { cudaGraphExecDestroy(c->exec); c->exec = nullptr; }
    if (c->graph) { cudaGraphDestroy(c->graph); c->graph = nullptr; }
    c->planned = false;
    // 1. discovery run (eager) to learn the sizes
    idb_output o = *out;
    o.stats = nullptr;
    o.tree_depth_hist = nullptr;
    o.n_uniques = nullptr;
    Pipeline pl;
    pl.c = c;
    pl.trees = false;
    TRY(stage_inputs_and_survey(pl, in, false));
    TRY(derive_plan(pl, prm));
    TRY(alloc_fixed(pl));
    pl.B.clone_id = o.clone_id;
    pl.B.core = o.core;
    pl.B.copies = o.copies;
    pl.B.uniques = o.uniques;
    TRY(run_phases(pl, true));
    TRY(read_counters(pl));
    TRY(device_errors(*c->h_ctr));
    // 2. capacities with headroom; the buffers keep their addresses from here on
    const Counters h = *c->h_ctr;
    TRY(alloc_entries(pl, (uint64_t)h.n_entries + h.n_entries / 16 + 1024));
    TRY(alloc_binpairs(pl, (uint64_t)h.n_binpairs + h.n_binpairs / 16 + 1024));
    if (!pl.P.streamed)
        TRY(alloc_edges(pl, (uint64_t)h.edge_reserved + h.edge_reserved / 8 + 64ull * kEdgeChunk * 1024));
    // 3. capture the complete launch sequence
    cudaStream_t s = c->stream;
    CU(cudaStreamSynchronize(s));
    CU(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    cudaMemsetAsync(pl.B.ctr, 0, sizeof(Counters), s);
    cudaMemsetAsync(&pl.B.ctr->lmin, 0xFF, sizeof(uint32_t), s);
    pl.timing = true;   // time-stamp kernels between the phases
    record(pl, 0);
    launch_survey(pl.P, pl.B, s);
    idb_status st = run_phases(pl, false);
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamEndCapture(s, &g);
    if (st != IDB_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (ce != cudaSuccess) return fail(IDB_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
    c->graph = g;
    CU(cudaGraphInstantiate(&c->exec, g, 0));
    CU(cudaGraphUpload(c->exec, s));   // device-side setup now, not in the first replay
    CU(cudaStreamSynchronize(s));
    {
        size_t nn = 0;
        CU(cudaGraphGetNodes(g, nullptr, &nn));
        std::vector<cudaGraphNode_t> nodes(nn);
        CU(cudaGraphGetNodes(g, nodes.data(), &nn));
        uint32_t k = 0;
        for (auto nd : nodes) {
            cudaGraphNodeType t;
            CU(cudaGraphNodeGetType(nd, &t));
            k += t == cudaGraphNodeTypeKernel;
        }
        c->graph_kernels = k;
    }
    c->plan = pl.P;
    c->bufs = pl.B;
    c->out_dev = o;
    c->planned = true;
    c->batch_generation = c->generation;
    c->batch_epoch = c->stage_epoch;
    return IDB_OK;
}

idb_status idb_batch_run(idb_context *c, idb_stats *stats) {
    if (!c || !c->planned) return fail(IDB_ERR_INVALID_ARG, "no batch plan");
    if (c->batch_generation != c->generation || c->batch_epoch != c->stage_epoch)
        return fail(IDB_ERR_REPLAN, "another call on this context replaced the staged inputs or "
                                    "moved the workspace since idb_batch_plan: plan again");
    CU(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    CU(cudaEventRecord(c->ev[0], s));
    CU(cudaGraphLaunch(c->exec, s));
    CU(cudaEventRecord(c->ev[1], s));
    CU(cudaMemcpyAsync(c->h_ctr, c->bufs.ctr, sizeof(Counters), cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    TRY(device_errors(*c->h_ctr));
    if (stats) {
        const Counters &h = *c->h_ctr;
        std::memset(stats, 0, sizeof *stats);
        stats->n_uniques = h.n_uniques;
        stats->n_cores = h.n_cores;
        stats->n_clusters = h.n_clusters;
        stats->n_noise_rows = h.n_noise_rows;
        stats->pairs_evaluated = h.pairs_evaluated;
        stats->neighbour_pairs = h.n_edges;
        stats->n_entries = h.n_entries;
        stats->n_units = h.n_units;
        stats->lev_columns = h.lev_columns;
        stats->core_edges = h.n_core_edges;
        stats->candidates = c->plan.join ? 1u : 0u;
        stats->streamed = c->plan.streamed ? 1u : 0u;
        float ms = 0;
        CU(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
        stats->ms_total = ms;
        phase_times(h, stats);
        stats->kernel_launches = c->graph_kernels;
    }
    return IDB_OK;
}

int32_t idb_diag_eps(uint32_t lx, uint32_t ly, float threshold, int32_t abs_eps) {
    return eps_value(lx, ly, threshold, abs_eps);
}

int32_t idb_diag_eps_hops(uint32_t lx, uint32_t ly, float threshold, int32_t hops,
                          int32_t use_hamming) {
    if (hops == 1) return eps_value(lx, ly, threshold, -1);
    if (hops != 2 && hops != 3) return INT32_MIN;
    return eps_hops_value(lx, ly, threshold, hops, use_hamming != 0);
}

idb_status idb_diag_gene_bits(idb_context *c, const char *calls, const int64_t *offsets,
                              uint32_t n_rows, const char *genes, const int64_t *gene_offsets,
                              uint32_t n_genes, uint64_t *words_out) {
    TRY(get_ctx(&c));
    if (!calls || !offsets || !words_out || (n_genes && (!genes || !gene_offsets)))
        return fail(IDB_ERR_INVALID_ARG, "NULL argument");
    if (n_genes > 64u * kMaxGeneWords)
        return fail(IDB_ERR_UNSUPPORTED, "at most %d genes", 64 * kMaxGeneWords);
    if (n_rows == 0) return IDB_OK;
    CU(cudaSetDevice(c->device));
    cudaGetLastError();
    Pipeline pl;
    pl.c = c;
    Plan &P = pl.P;
    Buffers &B = pl.B;
    P.N = n_rows;
    P.no_v = false;
    P.Gv = n_genes;
    P.VW = n_genes > 64 ? (n_genes + 63) / 64 : 1;
    const size_t nbytes = (size_t)offsets[n_rows];
    TRY(ensure(c, bV, nbytes + 16));
    TRY(ensure(c, bVOff, sizeof(int64_t) * ((size_t)n_rows + 1)));
    TRY(ensure(c, bVBits, sizeof(uint64_t) * n_rows * P.VW));
    if (nbytes) CU(cudaMemcpyAsync(c->buf[bV].p, calls, nbytes, cudaMemcpyHostToDevice, c->stream));
    CU(cudaMemcpyAsync(c->buf[bVOff].p, offsets, sizeof(int64_t) * ((size_t)n_rows + 1),
                       cudaMemcpyHostToDevice, c->stream));
    TRY(upload_genes(c, genes, gene_offsets, n_genes, bVGenes, bVGOff, bVTab, &P.gene_bytes_v,
                     &P.vmatch));
    B.vcall = ptr<uint8_t>(c, bV); B.v_off = ptr<int64_t>(c, bVOff);
    B.vgenes = ptr<uint8_t>(c, bVGenes); B.vg_off = ptr<int32_t>(c, bVGOff);
    B.vtab = ptr<GeneEntry>(c, bVTab);
    B.vbits = ptr<uint64_t>(c, bVBits);
    TRY(alloc_call_scratch(c, B, n_rows));
    set_row_chunks(P, false, 1);
    launch_call_init(P, B, true, c->stream);
    launch_gene_bits(P, B, true, 0, c->stream);
    TRY(check_launch());
    CU(cudaMemcpyAsync(words_out, B.vbits, sizeof(uint64_t) * n_rows * P.VW, cudaMemcpyDeviceToHost,
                       c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return IDB_OK;
}

idb_status idb_profile_binpairs(idb_context *c, const idb_input *in, const idb_params *prm,
                                float *features, float *log2_cycles, uint64_t cap,
                                uint64_t *n_out) {
    TRY(get_ctx(&c));
    if (!features || !log2_cycles || !n_out) return fail(IDB_ERR_INVALID_ARG, "NULL output");
    uint32_t dummy = 0;
    idb_output o{};
    o.clone_id = &dummy; o.core = reinterpret_cast<int32_t *>(&dummy); o.copies = &dummy;
    TRY(validate(in, prm, &o));
    *n_out = 0;
    if (in->n_rows == 0) return IDB_OK;
    CU(cudaSetDevice(c->device));
    cudaGetLastError();
    idb_params p0 = *prm;
    p0.schedule = 0;
    Pipeline pl;
    pl.c = c;
    TRY(stage_inputs_and_survey(pl, in, true));
    TRY(derive_plan(pl, &p0));
    TRY(alloc_fixed(pl));
    Plan &P = pl.P;
    Buffers &B = pl.B;
    cudaStream_t s = c->stream;
    TRY(run_phases(pl, true, true));   // up to the static schedule
    TRY(read_counters(pl));
    const uint32_t nbp = c->h_ctr->n_binpairs;
    if (P.cap_edges == 0) TRY(alloc_edges(pl, std::max<uint64_t>(4ull * P.N, 1ull << 16)));
    unsigned long long *cyc = nullptr;
    float *feat = nullptr;
    CU(cudaMalloc(&cyc, sizeof(unsigned long long) * (nbp + 1)));
    cudaError_t e = cudaMalloc(&feat, sizeof(float) * kMlpIn * (nbp + 1));
    if (e != cudaSuccess) { cudaFree(cyc); return fail(IDB_ERR_OUT_OF_MEMORY, "profile buffers"); }
    idb_status st = IDB_OK;
    for (int attempt = 0; attempt < 3; ++attempt) {
        cudaMemsetAsync(cyc, 0, sizeof(unsigned long long) * (nbp + 1), s);
        cudaMemsetAsync(&B.ctr->unit_cursor, 0, 4, s);
        cudaMemsetAsync(&B.ctr->edge_reserved, 0, 4, s);
        B.bp_cycles = cyc;
        launch_distance(P, B, 0, s);
        B.bp_cycles = nullptr;
        st = read_counters(pl);
        if (st != IDB_OK || !(c->h_ctr->error & kErrEdgeOverflow)) break;
        st = alloc_edges(pl, (uint64_t)c->h_ctr->edge_reserved + 64ull * kEdgeChunk * 1024);
        if (st != IDB_OK) break;
        uint32_t clear = 0;
        cudaMemcpyAsync(&B.ctr->error, &clear, 4, cudaMemcpyHostToDevice, s);
    }
    const uint64_t n = std::min<uint64_t>(nbp, cap);
    if (st == IDB_OK) {
        launch_features(B, nbp, feat, s);
        std::vector<unsigned long long> hc(nbp);
        cudaMemcpyAsync(hc.data(), cyc, sizeof(unsigned long long) * nbp, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(features, feat, sizeof(float) * kMlpIn * n, cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) st = fail(IDB_ERR_CUDA, "profile copy failed");
        for (uint64_t i = 0; i < n; ++i) log2_cycles[i] = std::log2(1.0 + (double)hc[i]);
        *n_out = n;
    }
    cudaFree(cyc);
    cudaFree(feat);
    return st;
}

idb_status idb_mlp_train(idb_context *c, const float *features, const float *targets, uint64_t n,
                         int epochs, float lr, float *params, float *final_loss) {
    TRY(get_ctx(&c));
    if (!features || !targets || !params || n == 0 || epochs <= 0)
        return fail(IDB_ERR_INVALID_ARG, "idb_mlp_train: bad arguments");
    CU(cudaSetDevice(c->device));
    cudaGetLastError();
    cudaStream_t s = c->stream;
    float *X = nullptr, *T = nullptr, *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr,
          *loss = nullptr;
    auto cleanup = [&]() {
        cudaFree(X); cudaFree(T); cudaFree(p); cudaFree(g); cudaFree(m); cudaFree(v); cudaFree(loss);
    };
    if (cudaMalloc(&X, sizeof(float) * kMlpIn * n) != cudaSuccess ||
        cudaMalloc(&T, sizeof(float) * n) != cudaSuccess ||
        cudaMalloc(&p, sizeof(float) * kMlpParams) != cudaSuccess ||
        cudaMalloc(&g, sizeof(float) * kMlpParams) != cudaSuccess ||
        cudaMalloc(&m, sizeof(float) * kMlpParams) != cudaSuccess ||
        cudaMalloc(&v, sizeof(float) * kMlpParams) != cudaSuccess ||
        cudaMalloc(&loss, sizeof(float)) != cudaSuccess) {
        cleanup();
        cudaGetLastError();
        return fail(IDB_ERR_OUT_OF_MEMORY, "idb_mlp_train: allocation failed");
    }
    cudaMemcpyAsync(X, features, sizeof(float) * kMlpIn * n, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(T, targets, sizeof(float) * n, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(p, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(m, 0, sizeof(float) * kMlpParams, s);
    cudaMemsetAsync(v, 0, sizeof(float) * kMlpParams, s);
    const uint64_t batch = std::min<uint64_t>(n, 8192);
    int step = 0;
    for (int ep = 0; ep < epochs; ++ep) {
        for (uint64_t b0 = 0; b0 < n; b0 += batch) {
            const uint32_t nb = (uint32_t)std::min<uint64_t>(batch, n - b0);
            cudaMemsetAsync(g, 0, sizeof(float) * kMlpParams, s);
            cudaMemsetAsync(loss, 0, sizeof(float), s);
            launch_mlp_grad(X + kMlpIn * b0, T + b0, nb, p, 1.0f / (float)nb, g, loss, s);
            launch_adam(p, g, m, v, lr, ++step, s);
        }
    }
    // loss over the full set with the final parameters
    cudaMemsetAsync(g, 0, sizeof(float) * kMlpParams, s);
    cudaMemsetAsync(loss, 0, sizeof(float), s);
    launch_mlp_grad(X, T, (uint32_t)n, p, 1.0f / (float)n, g, loss, s);
    float hl = 0;
    cudaMemcpyAsync(params, p, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&hl, loss, sizeof(float), cudaMemcpyDeviceToHost, s);
    const cudaError_t e = cudaStreamSynchronize(s);
    cleanup();
    if (e != cudaSuccess) return fail(IDB_ERR_CUDA, "idb_mlp_train: %s", cudaGetErrorString(e));
    TRY(check_launch());
    if (final_loss) *final_loss = hl / (float)n;
    return IDB_OK;
}

idb_status idb_mlp_load(idb_context *c, const float *params) {
    if (!c) return fail(IDB_ERR_INVALID_ARG, "idb_mlp_load needs an explicit context");
    CU(cudaSetDevice(c->device));
    if (!params) { c->has_model = false; return IDB_OK; }
    float *p = nullptr;
    CU(cudaMalloc(&p, sizeof(float) * kMlpParams));
    if (!c->mlp_bf16) {
        cudaError_t e = cudaMalloc(&c->mlp_bf16, 2 * kMlpParams);
        if (e != cudaSuccess) { cudaFree(p); return fail(IDB_ERR_OUT_OF_MEMORY, "model buffer"); }
    }
    cudaMemcpyAsync(p, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice, c->stream);
    launch_to_bf16(p, c->mlp_bf16, c->stream);
    const cudaError_t e = cudaStreamSynchronize(c->stream);
    cudaFree(p);
    if (e != cudaSuccess) return fail(IDB_ERR_CUDA, "idb_mlp_load: %s", cudaGetErrorString(e));
    c->has_model = true;
    return IDB_OK;
}

idb_status idb_diag_mlp_grad(idb_context *c, const float *params, const float *features,
                             const float *targets, uint32_t n, float *grad_out, float *loss_out) {
    TRY(get_ctx(&c));
    if (!params || !features || !targets || !grad_out || n == 0)
        return fail(IDB_ERR_INVALID_ARG, "idb_diag_mlp_grad: bad arguments");
    CU(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    float *X, *T, *p, *g, *loss;
    CU(cudaMalloc(&X, sizeof(float) * kMlpIn * n));
    CU(cudaMalloc(&T, sizeof(float) * n));
    CU(cudaMalloc(&p, sizeof(float) * kMlpParams));
    CU(cudaMalloc(&g, sizeof(float) * kMlpParams));
    CU(cudaMalloc(&loss, sizeof(float)));
    cudaMemcpyAsync(X, features, sizeof(float) * kMlpIn * n, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(T, targets, sizeof(float) * n, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(p, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(g, 0, sizeof(float) * kMlpParams, s);
    cudaMemsetAsync(loss, 0, sizeof(float), s);
    launch_mlp_grad(X, T, n, p, 1.0f / (float)n, g, loss, s);
    float hl = 0;
    cudaMemcpyAsync(grad_out, g, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&hl, loss, sizeof(float), cudaMemcpyDeviceToHost, s);
    const cudaError_t e = cudaStreamSynchronize(s);
    cudaFree(X); cudaFree(T); cudaFree(p); cudaFree(g); cudaFree(loss);
    if (e != cudaSuccess) return fail(IDB_ERR_CUDA, "idb_diag_mlp_grad: %s", cudaGetErrorString(e));
    if (loss_out) *loss_out = hl / (float)n;
    return IDB_OK;
}

idb_status idb_diag_mlp_predict(idb_context *c, const float *params, const float *features,
                                uint32_t n, float *log2_cycles_out) {
    TRY(get_ctx(&c));
    if (!params || !features || !log2_cycles_out || n == 0)
        return fail(IDB_ERR_INVALID_ARG, "idb_diag_mlp_predict: bad arguments");
    CU(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    float *X = nullptr, *p = nullptr, *y = nullptr;
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&X, sizeof(float) * kMlpIn * n);
    if (e == cudaSuccess) e = cudaMalloc(&p, sizeof(float) * kMlpParams);
    if (e == cudaSuccess) e = cudaMalloc(&y, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMalloc(&q, 2 * kMlpParams);
    if (e == cudaSuccess) {
        cudaMemcpyAsync(X, features, sizeof(float) * kMlpIn * n, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(p, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice, s);
        launch_to_bf16(p, q, s);              // the conversion idb_mlp_load applies
        launch_mlp_forward_rows(X, n, q, y, s);
        cudaMemcpyAsync(log2_cycles_out, y, sizeof(float) * n, cudaMemcpyDeviceToHost, s);
        e = cudaStreamSynchronize(s);
    }
    cudaFree(X); cudaFree(p); cudaFree(y); cudaFree(q);
    if (e != cudaSuccess) return fail(IDB_ERR_CUDA, "idb_diag_mlp_predict: %s", cudaGetErrorString(e));
    return IDB_OK;
}

idb_status idb_autotune(idb_context *c, const idb_input *in, const idb_params *prm,
                        idb_tuning *best) {
    TRY(get_ctx(&c));
    if (!best) return fail(IDB_ERR_INVALID_ARG, "NULL output");
    uint32_t dummy = 0;
    idb_output o{};
    o.clone_id = &dummy; o.core = reinterpret_cast<int32_t *>(&dummy); o.copies = &dummy;
    TRY(validate(in, prm, &o));
    std::memset(best, 0, sizeof *best);
    if (in->n_rows == 0) return IDB_OK;
    CU(cudaSetDevice(c->device));
    cudaGetLastError();
    Pipeline pl;
    pl.c = c;
    TRY(stage_inputs_and_survey(pl, in, true));
    TRY(derive_plan(pl, prm));
    TRY(alloc_fixed(pl));
    Plan &P = pl.P;
    Buffers &B = pl.B;
    cudaStream_t s = c->stream;
    // front and buckets once (independent of the unit shape)
    TRY(launch_front(pl, s));
    launch_buckets(P, B, s);
    TRY(read_counters(pl));
    TRY(alloc_entries(pl, c->h_ctr->n_entries));
    launch_fill(P, B, s);
    TRY(check_launch());
    // candidate shapes
    std::vector<std::pair<int, int>> cand;
    if (!P.fast) {
        cand = {{1, 64}, {1, 256}, {1, 1024}};
    } else if (P.hamming) {
        const int rxs[3] = {2, 4, 8};
        for (int rx : rxs) {
            if (rx != 4 && P.W != 1) continue;
            if (rx == 2 && !P.join) continue;
            for (int ty : {128, 256, 512, 1024})
                if (ty >= 32 * rx) cand.push_back({rx, ty});
        }
    } else {
        for (int rx : {1, 2}) {
            if (rx == 2 && P.W != 1) continue;
            for (int ty : {64, 128, 256, 512, 1024}) cand.push_back({rx, ty});
        }
    }
    if (cand.size() > 16) cand.resize(16);
    if (P.cap_edges == 0) TRY(alloc_edges(pl, std::max<uint64_t>(4ull * P.N, 1ull << 16)));
    // one shape and schedule order: bin pairs, the order, then the distance
    // kernel three times (best of the three)
    auto time_shape = [&](Plan Q, float *ms_out) -> idb_status {
        CU(cudaMemsetAsync(&B.ctr->n_binpairs, 0, 4, s));
        launch_binpairs(Q, B, s);
        TRY(read_counters(pl));
        pl.P = Q;
        TRY(alloc_binpairs(pl, c->h_ctr->n_binpairs));
        Q.cap_binpairs = pl.P.cap_binpairs;
        launch_binpairs_fill(Q, B, s);
        if (Q.schedule == 1) launch_mlp_predict(B, (uint32_t)Q.cap_binpairs, c->mlp_bf16, s);
        launch_schedule(Q, B, s);
        float ms_best = 1e30f;
        for (int rep = 0; rep < 3; ++rep) {
            CU(cudaMemsetAsync(&B.ctr->unit_cursor, 0, 4, s));
            CU(cudaMemsetAsync(&B.ctr->edge_reserved, 0, 4, s));
            CU(cudaMemsetAsync(&B.ctr->n_edges, 0, 4, s));
            CU(cudaMemsetAsync(&B.ctr->pairs_evaluated, 0, 8, s));
            CU(cudaEventRecord(c->ev[0], s));
            Q.cap_edges = pl.P.cap_edges;
            launch_distance(Q, B, 0, s);
            CU(cudaEventRecord(c->ev[1], s));
            TRY(check_launch());
            CU(cudaEventSynchronize(c->ev[1]));
            float ms = 0;
            CU(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
            ms_best = std::min(ms_best, ms);
            TRY(read_counters(pl));
            if (c->h_ctr->error & kErrEdgeOverflow) {   // grow and repeat this shape
                TRY(alloc_edges(pl, (uint64_t)c->h_ctr->edge_reserved + 64ull * kEdgeChunk * 1024));
                uint32_t clear = 0;
                CU(cudaMemcpyAsync(&B.ctr->error, &clear, 4, cudaMemcpyHostToDevice, s));
                --rep;
                ms_best = 1e30f;
            }
        }
        *ms_out = ms_best;
        return IDB_OK;
    };
    double best_ms = 1e30;
    Plan best_plan = P;
    for (auto &cd : cand) {
        Plan Q = P;
        Q.schedule = 0;
        if (P.fast) {
            Q.RX = cd.first;
            Q.TX = 32 * Q.RX;
            Q.TY = cd.second;
        } else {
            Q.TY = cd.second;
        }
        float ms_best = 0;
        TRY(time_shape(Q, &ms_best));
        const int k = best->n_tried++;
        best->tried_rx[k] = Q.RX;
        best->tried_ty[k] = (int)Q.TY;
        best->tried_ms[k] = ms_best;
        if (ms_best < best_ms) {
            best_ms = ms_best;
            best_plan = Q;
            best->tile_rx = Q.RX;
            best->tile_ty = (int)Q.TY;
            best->ms_distance = ms_best;
        }
    }
    // the schedule order for the fastest shape: static heavy-first, or the
    // learned cost when the context holds a model
    best->schedule = 0;
    best->schedule_ms[0] = best_ms;
    if (c->has_model) {
        Plan Q = best_plan;
        Q.schedule = 1;
        float ms_learned = 0;
        TRY(time_shape(Q, &ms_learned));
        best->schedule_ms[1] = ms_learned;
        if (ms_learned < best_ms) best->schedule = 1;
    }
    TRY(device_errors(*c->h_ctr));
    return IDB_OK;
}

idb_status idb_count_admissible(idb_context *c, const idb_input *in, const idb_params *prm,
                                uint64_t *pairs_out) {
    TRY(get_ctx(&c));
    if (!pairs_out) return fail(IDB_ERR_INVALID_ARG, "NULL output");
    uint32_t dummy = 0;
    idb_output o{};
    o.clone_id = &dummy; o.core = reinterpret_cast<int32_t *>(&dummy); o.copies = &dummy;
    TRY(validate(in, prm, &o));
    *pairs_out = 0;
    if (in->n_rows == 0) return IDB_OK;
    CU(cudaSetDevice(c->device));
    Pipeline pl;
    pl.c = c;
    pl.allow_join = false;    // every admissible pair must be enumerated here
    TRY(stage_inputs_and_survey(pl, in, true));
    TRY(derive_plan(pl, prm));
    TRY(alloc_fixed(pl));
    TRY(run_phases(pl, true, true));
    launch_count_admissible(pl.P, pl.B, c->stream);
    TRY(check_launch());
    TRY(read_counters(pl));
    TRY(device_errors(*c->h_ctr));
    *pairs_out = c->h_ctr->admissible_pairs;
    return IDB_OK;
}

}  // extern "C"
