/*
 * oracle.h -- CPU oracle for the immunodbscan DBSCAN clone-collapsing path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference arm of bench.py may load this library, and only as
 * the checker (or the timed CPU baseline).  The product path never links it.
 *
 * PARITY UNPINNED: the reference ships no tests, no golden vectors and no
 * example data (data/ExampleData.csv is missing from the reference tree), and
 * its CUDA path cannot run in a GPU-less container.  This oracle restates the
 * reference's rules (cuda/PSDBSCAN.hcu, cuda/BitsetVector.inl,
 * cuda/SpecialFunctors.hcu) and is pinned by hand-derived known-answer tests
 * under tests/ instead.
 *
 * All strings are passed as a byte blob plus int64 offsets (n+1 entries).
 * A NULL gene-call blob means "gene column not configured": every row gets
 * the call "V" and the reference list ["V"] (cpp/TableHolder.hpp:293-296).
 * A NULL sequence blob means every row carries the sequence "Gene"
 * (cpp/TableHolder.hpp:326-328).
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ora_params {
    float    threshold;      /* maximum_relative_edit_distance; NaN = not used   */
    int32_t  abs_eps;        /* absolute eps; < 0 = not used                      */
    uint32_t min_pts;        /* minimum_number_of_neighbors                       */
    int32_t  use_hamming;    /* use_hamming                                       */
    int32_t  n_threads;      /* OpenMP threads (<=0: library default)             */
    int32_t  max_candidates; /* K: border candidate labels reported per row       */
    int32_t  indexed;        /* 0: every pair of uniques, full DP (the reference's
                                structure and cost, used as the CPU baseline);
                                1: only pairs within the largest admissible length
                                gap, edit distance with a cutoff at eps -- the same
                                answer, for checking large inputs               */
} ora_params;

typedef struct ora_result {
    /* per row (caller allocated, n_rows entries) */
    uint32_t *clone_id;      /* deterministic rule: min-index core neighbour      */
    int32_t  *core;
    uint32_t *copies;
    /* optional: per row, the labels of all clusters a border row may join under
       the reference's first-wins CAS (PSDBSCAN.hcu:113-122); n_rows*K entries */
    uint32_t *cand;
    uint32_t *n_cand;        /* per row number of candidate labels (may exceed K) */
    /* scalars */
    uint32_t n_uniques;
    uint32_t n_cores;        /* core uniques                                       */
    uint32_t n_clusters;     /* summed over repertoires                            */
    uint64_t admissible_pairs; /* unique pairs with V and J overlap and an
                                  admissible length gap, counted once            */
    uint64_t neighbour_pairs;  /* unique pairs that are neighbours                */
    uint64_t all_pairs;        /* n_u(n_u-1)/2 per repertoire, summed             */
} ora_result;

/* Cluster n_rows rows split into n_rep independent repertoires
   (rep_off[n_rep+1]; NULL = one repertoire).  Returns 0 on success. */
int ora_cluster(uint32_t n_rows,
                const char *v_data, const int64_t *v_off,
                const char *j_data, const int64_t *j_off,
                const char *s_data, const int64_t *s_off,
                const char *vg_data, const int64_t *vg_off, uint32_t n_vg,
                const char *jg_data, const int64_t *jg_off, uint32_t n_jg,
                uint32_t n_rep, const uint32_t *rep_off,
                const ora_params *params, ora_result *out);

/* S1 only: gene bitsets as the reference stores them, int32 words,
   width = ceil(n_genes/32) words per row (cuda/BitsetVector.inl:28-45). */
int ora_gene_bitsets(uint32_t n_rows, const char *c_data, const int64_t *c_off,
                     const char *g_data, const int64_t *g_off, uint32_t n_genes,
                     uint32_t *words_out);

/* S2 only: eps(Lx,Ly) (cuda/SpecialFunctors.hcu:257-261, plus the absolute
   cap); INT32_MIN if neither threshold is in use. */
int32_t ora_eps(uint32_t lx, uint32_t ly, float threshold, int32_t abs_eps);

/* S4 helpers: full-DP Levenshtein (cuda/PSDBSCAN.hcu:246-290) and Hamming
   (cuda/PSDBSCAN.hcu:410-428) on raw bytes. */
int32_t ora_levenshtein(const char *a, uint32_t la, const char *b, uint32_t lb);
int32_t ora_hamming(const char *a, const char *b, uint32_t len);
/* 1 iff the edit distance of a and b is at most e (banded DP, stops once a row
   of the band exceeds e); the indexed mode's test. */
int32_t ora_levenshtein_within(const char *a, uint32_t la, const char *b, uint32_t lb, int32_t e);

#ifdef __cplusplus
}
#endif
