/*
 * immunodbscan_gb300_diag.h -- measurement entry points of libimmunodbscan_gb300.
 *
 * These have no counterpart in the reference (its only boundary is
 * InterlinkClass, cuda/Interlink.hpp:54-57).  They exist so that throughput can
 * be reported against a schedule-independent numerator and a measured peak.
 */
#ifndef IMMUNODBSCAN_GB300_DIAG_H
#define IMMUNODBSCAN_GB300_DIAG_H

#include <stdint.h>

#include "immunodbscan_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Measured 32-bit integer-logic throughput of `device` in Gop/s (lop3/add
   chains, all SMs, best of 5 launches); *ms_out = duration of the best launch.
   Returns 0 on success. */
int idb_diag_int_peak(int device, double *gops_out, double *ms_out);

/* The neighbour threshold the library uses for a pair of lengths: relative
   threshold (NaN = unused) applied as (int)truncf((float)max(lx, ly) * threshold),
   the reference's epsilonOneFunctorClass (cuda/SpecialFunctors.hcu:245-274),
   capped by abs_eps when abs_eps >= 0.  Host-only; needs no device. */
int32_t idb_diag_eps(uint32_t lx, uint32_t ly, float threshold, int32_t abs_eps);

/* The reference's multi-hop distance bounds (epsilonTwoFunctorClass and
   epsilonThreeFunctorClass, cuda/SpecialFunctors.hcu:276-344), which its
   clustering never calls: the most edits between two sequences that are joined
   through hops - 1 intermediate sequences, each step within the relative
   threshold.  hops = 1 is idb_diag_eps without the absolute cap; 2 and 3 follow
   the reference's single-precision expressions (Levenshtein form, or the
   equal-length Hamming form with use_hamming).  INT32_MIN for other hops.
   Host-only. */
int32_t idb_diag_eps_hops(uint32_t lx, uint32_t ly, float threshold, int32_t hops,
                          int32_t use_hamming);

/* Number of admissible unique pairs of the input: pairs of uniques (after the
   duplicate collapse) in one repertoire whose V sets and J sets overlap and
   whose length gap is admissible (equal lengths in Hamming mode, |Lx-Ly| <=
   eps(Lx,Ly) otherwise), each pair counted once.  Host inputs as idb_cluster. */
idb_status idb_count_admissible(idb_context *ctx, const idb_input *in, const idb_params *prm,
                                uint64_t *pairs_out);

/* Gene bitsets alone (rule S1): words_out[i * W + w] (W = max(1, ceil(n_genes/64)))
   has bit g%64 of word g/64 set iff gene name g is a byte-exact substring of
   call i.  Host inputs and output; synchronous. */
idb_status idb_diag_gene_bits(idb_context *ctx, const char *calls, const int64_t *offsets,
                              uint32_t n_rows, const char *genes, const int64_t *gene_offsets,
                              uint32_t n_genes, uint64_t *words_out);

/* Gradient of the learned scheduler's loss (mean squared error) with respect to
   the IDB_MLP_PARAMS parameters, computed by the training kernel (FP32) on n
   samples; for checking against a CPU implementation. */
idb_status idb_diag_mlp_grad(idb_context *ctx, const float *params, const float *features,
                             const float *targets, uint32_t n, float *grad_out, float *loss_out);

/* The learned scheduler's inference on given feature rows: the parameters are
   converted to BF16 as idb_mlp_load converts them, and the forward pass the
   scheduler runs on bin pairs (BF16 inputs, weights and activations, FP32
   accumulation) writes log2_cycles_out[i] for features[i * IDB_MLP_FEATURES ..];
   for checking against a CPU forward pass. */
idb_status idb_diag_mlp_predict(idb_context *ctx, const float *params, const float *features,
                                uint32_t n, float *log2_cycles_out);

#ifdef __cplusplus
}
#endif
#endif /* IMMUNODBSCAN_GB300_DIAG_H */
