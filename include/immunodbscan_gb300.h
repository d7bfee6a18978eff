/*
 * immunodbscan_gb300.h -- C ABI of the GB300 (sm_103a) DBSCAN clone-collapsing
 * path of immunodbscan.
 *
 * This is the drop-in for the reference's only host<->CUDA boundary, the
 * constructor of InterlinkClass (cuda/Interlink.hpp:54-57, body
 * cuda/Interlink.cu:34-95) and its getters (cuda/Interlink.hpp:59-67), called
 * from TableHolderClass::do_the_clustering (cpp/TableHolder.hpp:340-343).
 *
 * Conventions
 *  - Plain C types only; every entry point returns an idb_status (0 = success)
 *    and never throws.  idb_last_error() returns the calling thread's message.
 *  - Strings are passed as a byte blob plus int64 offsets (n+1 entries, blob
 *    bytes [off[i], off[i+1]) are string i; strings hold no NUL terminator).
 *  - The caller owns all memory.  Host entry points take host pointers and are
 *    synchronous.  Device entry points take device pointers and run on the
 *    context's stream.
 *  - Results follow the reference's rules: same duplicate classes and copies,
 *    same core flags,
 *    same core partition and noise set, clone ids numbered by ascending minimum
 *    core row index.  A border row (non-core, with core neighbours) joins the
 *    cluster of its minimum-index core neighbour; the reference lets the first
 *    of its core neighbours win a race (cuda/PSDBSCAN.hcu:113-122).
 */
#ifndef IMMUNODBSCAN_GB300_H
#define IMMUNODBSCAN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define IDB_ABI_VERSION 1

typedef enum idb_status {
    IDB_OK = 0,
    IDB_ERR_INVALID_ARG = 1,   /* NULL pointer, inconsistent sizes, bad enum      */
    IDB_ERR_CUDA = 2,          /* a CUDA runtime call failed                      */
    IDB_ERR_NO_DEVICE = 3,     /* no CUDA device / device is not sm_103           */
    IDB_ERR_UNSUPPORTED = 4,   /* outside the documented limits                   */
    IDB_ERR_OUT_OF_MEMORY = 5, /* device allocation failed / memory budget hit    */
    IDB_ERR_CAPACITY = 6,      /* a replayed plan's capacities were exceeded      */
    IDB_ERR_DEVICE_STALL = 7,  /* a bounded device-side wait gave up              */
    IDB_ERR_REPLAN = 8         /* input no longer matches a captured plan         */
} idb_status;

typedef enum idb_alphabet {
    IDB_ALPHABET_AUTO = 0,     /* derived from the bytes present (exact, any data) */
} idb_alphabet;

/* Clustering parameters (INFO keys of the reference, cpp/ConfigHolder.hpp:181-205). */
typedef struct idb_params {
    float    threshold;        /* maximum_relative_edit_distance (NaN = unused)    */
    int32_t  abs_eps;          /* absolute eps (new key; < 0 = unused)             */
    uint32_t min_pts;          /* minimum_number_of_neighbors (counts itself)      */
    int32_t  use_hamming;      /* use_hamming                                      */
    int32_t  eval_trees;       /* get_tree_depth_statistics                        */
    int32_t  schedule;         /* 0 = static (pair-count) order, 1 = learned       */
    int32_t  tile_rx;          /* x-entries per lane of a work unit (0 = default)  */
    int32_t  tile_ty;          /* y-entries of a work unit (0 = default)           */
    int32_t  candidates;       /* 0 = automatic (Hamming eps <= 2: segment join),
                                  1 = every admissible pair of the buckets        */
    int32_t  edge_memory_mb;   /* device memory for the neighbour-pair list:
                                  0 = as much as the pairs need; > 0 = at most this
                                  many MiB; < 0 = none.  Neighbour graphs that do
                                  not fit are clustered in streamed mode: the
                                  distance work runs twice (counts, then unions
                                  and border minima) and no pair is stored.  Same
                                  answer either way.                              */
    int32_t  row_chunks;       /* idb_cluster (host columns): number of row chunks
                                  the columns are copied and pre-processed in, so
                                  that copies overlap the gene-bitset and
                                  duplicate work (chunk i of k holds (k-i) parts
                                  of k(k+1)/2); 0 = automatic (8 from 2^20 rows,
                                  else 1), 1..8 = that many.  Same answer.       */
    int32_t  reserved[1];
} idb_params;

/* Input rows (cuda/Interlink.hpp:54-57: zip(V calls, J calls, sequences)). */
typedef struct idb_input {
    uint32_t n_rows;
    /* V and J gene calls; NULL data = column not configured: every row matches
       the single gene "V" (cpp/TableHolder.hpp:293-296, 311-314). */
    const char    *v_calls;
    const int64_t *v_offsets;
    const char    *j_calls;
    const int64_t *j_offsets;
    /* sequences; NULL = every row is "Gene" (cpp/TableHolder.hpp:326-328) */
    const char    *seqs;
    const int64_t *seq_offsets;
    /* reference gene names (cpp/GeneReader.hpp:65-76), host memory always */
    const char    *v_genes;
    const int64_t *v_gene_offsets;
    uint32_t       n_v_genes;
    const char    *j_genes;
    const int64_t *j_gene_offsets;
    uint32_t       n_j_genes;
    /* independent repertoires: rows [rep_offsets[r], rep_offsets[r+1]) form
       repertoire r (n_repertoires+1 entries, host memory); NULL = one.
       Clone ids are numbered per repertoire. */
    uint32_t        n_repertoires;
    const uint32_t *rep_offsets;
} idb_input;

typedef struct idb_stats {
    uint32_t n_uniques;
    uint32_t n_cores;          /* core uniques                                     */
    uint32_t n_clusters;
    uint32_t n_noise_rows;
    uint64_t pairs_evaluated;  /* distance evaluations performed by the kernels    */
    uint64_t neighbour_pairs;  /* unique pairs that are neighbours (graph edges)   */
    uint64_t n_entries;        /* bucket entries (unique x V gene x J gene)        */
    uint64_t n_units;          /* scheduled work units                             */
    double   ms_total;         /* device time of the whole call                    */
    double   ms_distance;      /* device time of the distance kernel               */
    double   ms_phase[8];      /* front+dedupe, buckets+schedule, distance, graph,
                                  outputs (device time; eager calls include waits
                                  on host read-backs, and with host columns the
                                  first phase includes the copies it overlaps)     */
    uint32_t kernel_launches;  /* kernels in the replayed graph; 0 for an eager
                                  call                                             */
    uint32_t core_edges;       /* neighbour pairs with both ends core              */
    uint64_t lev_columns;      /* text columns consumed by live Levenshtein pairs  */
    uint32_t candidates;       /* 0: every admissible pair of the buckets scored;
                                  1: Hamming segment join (eps <= 2 at every
                                  length): only pairs sharing a whole segment    */
    uint32_t streamed;         /* 1: neighbour pairs were not stored (two sweeps;
                                  core_edges is not counted)                      */
} idb_stats;

/* Outputs (cuda/Interlink.hpp:59-67).  clone_id/core/copies are required. */
typedef struct idb_output {
    uint32_t  *clone_id;        /* [n_rows] 0 = noise (get_clusters_iterator)      */
    int32_t   *core;            /* [n_rows] 0/1 (get_cores_iterator)               */
    uint32_t  *copies;          /* [n_rows] class size at the representative,
                                   0 at duplicates (get_copies_iterator)           */
    uint32_t  *uniques;         /* optional [n_rows]: ascending representative rows
                                   (get_uniques_iterator)                          */
    uint32_t  *n_uniques;       /* optional (get_n_uniques)                        */
    uint32_t  *tree_depth_hist; /* optional [51]: union-find depth histogram
                                   (cuda/PSDBSCAN.hcu:1020-1040)                   */
    idb_stats *stats;           /* optional                                        */
} idb_output;

typedef struct idb_context idb_context;

/* Context = device + stream + workspace.  One context per host thread. */
idb_status idb_context_create(int device, idb_context **ctx);
idb_status idb_context_destroy(idb_context *ctx);

/* The InterlinkClass replacement: host inputs, host outputs, synchronous.
   ctx may be NULL (a per-thread default context on device 0 is used, matching
   the reference's implicit device 0, cuda/PSDBSCAN.hcu:977). */
idb_status idb_cluster(idb_context *ctx, const idb_input *in, const idb_params *prm,
                       idb_output *out);

/* Same, with the row columns (calls, sequences and their offsets) and the
   outputs in device memory.  Gene name lists and rep_offsets stay in host
   memory.  Synchronous. */
idb_status idb_cluster_device(idb_context *ctx, const idb_input *in, const idb_params *prm,
                              idb_output *out);

/* Batched, graph-captured path: plan once for a set of repertoires whose
   device-resident columns stay at the same addresses, then replay.  The plan
   sizes the workspace and captures the complete launch sequence (bitsets,
   duplicate collapse, bucketing, one persistent distance launch over all
   repertoires, graph, labels) into a CUDA graph; idb_batch_run replays it and
   recomputes everything from the inputs.  If new data at the same addresses
   exceeds the plan, idb_batch_run returns IDB_ERR_CAPACITY or IDB_ERR_REPLAN
   and the caller plans again. */
idb_status idb_batch_plan(idb_context *ctx, const idb_input *in, const idb_params *prm,
                          const idb_output *out);
idb_status idb_batch_run(idb_context *ctx, idb_stats *stats);

/* No-allocation duplicate collapse.  This entry point has no counterpart in
   the reference; it serves callers that cannot allocate device memory (for
   example a host whose GPU memory is owned by another allocator, or a serving
   loop that may not call cudaMalloc/cudaFree because they synchronise the
   device).  It performs the duplicate-collapse step of the path (rows are
   duplicates iff they have equal length, equal V and J bitsets when given, and
   equal bytes): rep_out[i] = the minimum row of i's class, copies_out[i] = the
   class size at that row and 0 elsewhere -- the copies column idb_cluster
   returns for the same rows.  Inputs and outputs are caller-owned device
   memory; v_bits / j_bits (n_rows x v_words / j_words uint64 words, bit g =
   reference gene g, 1 <= words <= 8, i.e. at most 512 genes a column) may be
   NULL.  Its hash table lives in a fixed ~5 MB
   __device__ array inside the library, which every GPU that loads the library
   holds until the process exits; at most IDB_DEDUPE_NOALLOC_MAX_ROWS rows
   (larger inputs are rejected with IDB_ERR_UNSUPPORTED).  Runs on the calling
   thread's current device and on `stream` (a cudaStream_t, NULL = legacy
   default stream) and returns when the results are complete: it waits on the
   stream and reads an error word back, so it cannot be called while that
   stream is being captured.  The first call on a device resolves the array's
   address (cudaGetSymbolAddress) and keeps it for the life of the process;
   after cudaDeviceReset that address is stale, so the entry point is not for
   use across device resets.  All calls on a device share the
   array, which keeps the last call's contents (each call resets it first):
   calls that overlap on the GPU race and must be serialised by the caller.
   Calls no cudaMalloc, cudaFree or allocating library routine. */
#define IDB_DEDUPE_NOALLOC_MAX_ROWS (1u << 18)
idb_status idb_dedupe_noalloc(const char *seqs, const int64_t *seq_offsets,
                              const uint64_t *v_bits, uint32_t v_words,
                              const uint64_t *j_bits, uint32_t j_words, uint32_t n_rows,
                              uint32_t *rep_out, uint32_t *copies_out, void *stream);

/* Autotuner: builds the buckets of the input once, then times the distance
   kernel for every candidate work-unit shape (x-entries per lane, y-chunk
   length) on this data and returns the fastest in best->tile_rx/tile_ty
   (pass them in idb_params for the real runs).  For that shape it then times
   the bucket-pair schedule orders: the static heavy-first order and, when the
   context holds a model (idb_mlp_load), the learned one; the faster goes in
   best->schedule (pass it as idb_params.schedule).  Host inputs as
   idb_cluster. */
typedef struct idb_tuning {
    int32_t tile_rx, tile_ty;   /* the fastest shape                              */
    double  ms_distance;        /* its distance-kernel time (best of the repeats)  */
    int32_t n_tried;
    int32_t tried_rx[16];
    int32_t tried_ty[16];
    double  tried_ms[16];
    int32_t schedule;           /* the faster order for that shape: 0 static,
                                   1 learned                                       */
    double  schedule_ms[2];     /* distance-kernel time per order (0: not timed)   */
} idb_tuning;
idb_status idb_autotune(idb_context *ctx, const idb_input *in, const idb_params *prm,
                        idb_tuning *best);

/* Learned schedule.  The persistent distance kernel hands out work units of
   heavy bin pairs first.  With idb_params.schedule = 1 "heavy" is the cost a
   small network predicts for the bin pair (16 features -> 64 -> 64 -> 1, ReLU,
   predicting log2 device cycles; BF16 inference), instead of the pair count.
   The schedule never changes the result.  Training data comes from
   idb_profile_binpairs, which runs a clustering with per-bin-pair cycle
   logging; idb_mlp_train fits the network on the device (FP32, Adam) and
   idb_mlp_load installs it in a context. */
#define IDB_MLP_FEATURES 16
#define IDB_MLP_PARAMS (16 * 64 + 64 + 64 * 64 + 64 + 64 + 1)
idb_status idb_profile_binpairs(idb_context *ctx, const idb_input *in, const idb_params *prm,
                                float *features /* cap x IDB_MLP_FEATURES */,
                                float *log2_cycles /* cap */, uint64_t cap, uint64_t *n_out);
idb_status idb_mlp_train(idb_context *ctx, const float *features, const float *targets,
                         uint64_t n, int epochs, float lr, float *params /* in/out */,
                         float *final_loss);
idb_status idb_mlp_load(idb_context *ctx, const float *params /* NULL = unload */);

/* Page-locked host memory for the input columns of idb_cluster (its
   host->device copies then run at the full rate of the host link; pageable
   buffers work too, through the driver's staging).  No counterpart in the
   reference, whose columns are thrust host vectors (cuda/Interlink.hpp:41-43).
   idb_host_alloc returns IDB_ERR_OUT_OF_MEMORY if the memory cannot be had. */
idb_status idb_host_alloc(size_t bytes, void **out);
idb_status idb_host_free(void *p);

/* Thread-local message of the last failing call ("" if none). */
size_t idb_last_error(char *buf, size_t size);
const char *idb_status_string(idb_status s);
int idb_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* IMMUNODBSCAN_GB300_H */
