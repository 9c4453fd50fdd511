/*
 * oic_gpu.h -- C ABI of the GB300 overlapInCore engine (liboic_gpu.so).
 *
 * The library is the drop-in for canu's overlapInCore hot path: the k-mer hash
 * block, the seed lookup and per-read-pair bucketing, and the banded prefix edit
 * distance extension that turns seeds into ovOverlap records.  All compute runs in
 * hand-written sm_103a CUDA kernels on one GPU; there is no CPU fallback: every
 * entry point returns OIC_ERR_CUDA when the device or the kernels are unavailable.
 *
 * Plain C types only: pointers, sizes, status codes.  All host buffers are owned by
 * the caller.  A context is single-threaded and owns one CUDA stream.
 *
 * Record format: one overlap = six uint32 words, exactly what canu's ovFile writes
 * for an ovFileFullWrite record (src/stores/ovStoreFile.C:262-276):
 *   a_iid, b_iid, dat[0] >> 32, dat[0] & 0xffffffff, dat[1] >> 32, dat[1] & 0xffffffff
 * with the ovOverlapDAT bit layout of AS_MAX_READLEN_BITS == 21
 * (src/stores/ovOverlap.H:55-78).
 */
#ifndef OIC_GPU_H
#define OIC_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  0 is success. */
enum {
  OIC_OK             = 0,
  OIC_ERR_ARG        = 1,   /* bad argument / unsupported option                     */
  OIC_ERR_INPUT      = 2,   /* input the reference rejects (bad base, short read ...) */
  OIC_ERR_CUDA       = 3,   /* CUDA runtime error or no usable device                 */
  OIC_ERR_NOMEM      = 4,   /* device or host allocation failed                       */
  OIC_ERR_OVERFLOW   = 5,   /* a size limit of the engine was exceeded                */
  OIC_ERR_STATE      = 6,   /* call out of order (e.g. no reads / no hash block)      */
  OIC_ERR_DEVICE     = 7    /* a kernel reported an internal error flag               */
};

/* overlapInCore's parameters (overlapInCore.H:367-473; parsing overlapInCore.C:293-411).
 * oic_default_params() gives the reference defaults. */
typedef struct oic_params {
  double      maxErate;          /* --maxerate; callers pass the strtof-rounded value     */
  double      alignNoise;        /* --alignnoise (strtof-rounded)                          */
  int32_t     partial;           /* -partial                                               */
  int32_t     uniqueOlapPerPair; /* -u (1, default) or -m (0)                              */
  int32_t     useHopelessCheck;  /* 0 after -z; the library also clears it when maxErate > 0.06 */
  int32_t     minKmers;          /* --minkmers                                             */
  uint32_t    kmerLen;           /* -k <int>, 1..31                                        */
  uint32_t    hashBits;          /* --hashbits                                             */
  double      maxHashLoad;       /* --hashload                                             */
  uint64_t    maxHashDataLen;    /* --hashdatalen (the library adds AS_MAX_READLEN, overlapInCore.C:454) */
  int32_t     minOlapLen;        /* --minlength                                            */
  uint32_t    numThreads;        /* -t; only its effect on which ref reads a chunked run visits */
  uint32_t    bgnHashID, endHashID, minLibToHash, maxLibToHash;   /* -h, -H               */
  uint32_t    bgnRefID, endRefID, minLibToRef, maxLibToRef;       /* -r, -R               */
} oic_params;

/* The -s stats counters (overlapInCore.C:550-558) plus work counters. */
typedef struct oic_stats {
  uint64_t kmerHitsWithoutOlap, kmerHitsWithOlap, kmerHitsSkipped, multiOverlap;
  uint64_t totalOverlaps, containedOverlaps, dovetailOverlaps;
  uint64_t badShortWindow, badLongWindow;
  uint64_t dpCells, slideBases, extensions, seeds, candidatePairs, nodes, dpRows;
  uint32_t nHashBlocks, reserved;
  double   msHash, msSeed, msAlign, msTotal;       /* device time (CUDA events) of oic_run work */
  double   msReads;                                /* device time of the last oic_set_reads */
  uint64_t kernelLaunches;                         /* kernels launched by oic_run and its parts */
  uint64_t dpCellsNoOverlap;                       /* DP cells spent on pairs that emitted nothing */
  uint64_t filteredPairs;                          /* candidate pairs the learned filter dropped */
  double   msFilter;                               /* device time of features + filter inference */
  double   msNarrow, msWide;                       /* device time of the one-warp and CTA DP bins */
  uint64_t pairsNarrow, pairsWide;                 /* pairs run in each bin (reruns in the CTA bin) */
  uint64_t cellsWide;                              /* DP cells of the CTA bin */
  uint64_t graphLaunches;                          /* batches whose DP stage ran as one captured CUDA graph */
} oic_stats;

typedef struct oic_ctx oic_ctx;

/* Reference defaults (oicParameters::initialize, overlapInCore.H:374-411). */
void oic_default_params(oic_params *p);

/* Create a context on CUDA device `device`.  Replaces main()'s setup and
 * Initialize_Work_Area (overlapInCore.C:113-144, 452-523): validates the parameters,
 * builds the Edit_Match_Limit and Error_Bound tables (prefixEditDistance.C:23-90,
 * Binomial_Bound.C:104-195) on the host and uploads them. */
int  oic_create(const oic_params *p, int device, oic_ctx **out);
void oic_destroy(oic_ctx *ctx);

/* Load the read store: the 1-based read IDs 1..nReads with their library IDs,
 * lengths and bases (A/C/G/T/N, either case) at bases[offset[i] .. offset[i]+length[i]).
 * Replaces sqStore / sqCache_loadReads (overlapInCore.C:166-195).  Reads are packed
 * to 2 bits per base (both strands) plus an N mask on the device. */
int oic_set_reads(oic_ctx *ctx, uint32_t nReads, const uint32_t *libID, const uint32_t *length,
                  const uint64_t *offset, const char *bases, uint64_t nBases);

/* Optional skip list: nKmers k-mers of exactly kmerLen bases each, concatenated
 * (the -k <file> contents, Build_Hash_Index.C:184-257).  Each k-mer and its reverse
 * complement are screened in every hash block built afterwards. */
int oic_set_skip_kmers(oic_ctx *ctx, const char *kmers, uint64_t nKmers);

/* Build one hash block starting at read bgnID and ending at or before endID
 * (Build_Hash_Index, overlapInCore-Build_Hash_Index.C:414-631).  *lastLoaded gets the
 * ID of the last read placed in the block. */
int oic_load_hash_block(oic_ctx *ctx, uint32_t bgnID, uint32_t endID, uint32_t *lastLoaded);

/* Overlap every ref read of [bgnRefID, endRefID] (both strands) against the loaded
 * block (Process_Overlaps / Find_Overlaps / Process_String_Olaps, overlapInCore-
 * Process_Overlaps.C:24-122).  The records are appended to the context's output. */
int oic_run_refs(oic_ctx *ctx, uint32_t bgnRefID, uint32_t endRefID);

/* The whole stage (OverlapDriver, overlapInCore.C:161-277): every hash block of the
 * -h range against the -r range, with the reference's range clamping and chunking
 * rules.  Records are appended to the context's output. */
int oic_run(oic_ctx *ctx);

/* Number of records accumulated so far, and a copy of them (6 uint32 each) into
 * `words` (capacity maxRecords).  oic_clear_overlaps() empties the output. */
int oic_num_overlaps(oic_ctx *ctx, uint64_t *n);
int oic_fetch_overlaps(oic_ctx *ctx, uint32_t *words, uint64_t maxRecords, uint64_t *n);
int oic_clear_overlaps(oic_ctx *ctx);

int oic_get_stats(oic_ctx *ctx, oic_stats *st);

/* No counterpart in the reference (its only report is the -s stats text,
 * overlapInCore.C:550-558).  The counters and device times of *st as one JSON object
 * (keys as the oic_stats field names) plus the derived rates overlapsPerSec
 * (totalOverlaps over msTotal) and dpCellsPerSec (dpCells over msAlign; 0 when a time
 * is 0): the metrics sidecar of a run.  Host code only.  Writes at most cap bytes
 * (NUL included) to buf and sets *len to the text's length without the NUL; returns
 * OIC_ERR_ARG when cap is too small (*len still says how much is needed). */
int oic_stats_json(const oic_stats *st, char *buf, size_t cap, size_t *len);

/* Batched Extend_Alignment (prefixEditDistance-extend.C:36-183) over nAlign
 * independent problems, for direct testing of the DP kernel.  Problem i aligns the
 * exact match (mStart[i] in S, mOffset[i] in T, mLen[i]) of S = read sRead[i] on
 * strand sRev[i] (0 forward, 1 reverse complement) against T = read tRead[i]
 * (forward), all 1-based IDs of the loaded store.  out[5*i .. 5*i+4] = S_Lo, S_Hi,
 * T_Lo, T_Hi, Errors; kind[i] = 0 NONE, 1 LEFT_BRANCH_PT, 2 RIGHT_BRANCH_PT,
 * 3 DOVETAIL; deltaLen[i] = merged Left_Delta length. */
int oic_extend_batch(oic_ctx *ctx, uint32_t nAlign, const uint32_t *sRead, const uint32_t *sRev,
                     const uint32_t *tRead, const int32_t *mStart, const int32_t *mOffset,
                     const int32_t *mLen, int32_t *out, int32_t *kind, int32_t *deltaLen);

/* One problem of oic_extend_batch_noalloc(), in device memory: 0-based read indices
 * (ID - 1) of S (on strand sRev) and T, and the exact match (mStart in S, mOffset in
 * T, mLen). */
typedef struct oic_extend_problem {
  uint32_t sRead, sRev, tRead;
  int32_t  mStart, mOffset, mLen;
} oic_extend_problem;

/* No counterpart in the reference.  oic_extend_batch() for callers that cannot call
 * cudaMalloc when they align: programs whose own allocator holds the whole device
 * memory pool, and plugins given a fixed device-memory budget by their host program.
 * Problems and outputs are caller-owned DEVICE buffers (dOut: 5 per problem, as
 * oic_extend_batch; dStatus: 0, or the capacity/validity flag a problem hit).  The DP's
 * scratch is a static device array of 23,072,768 bytes that every GPU loading the
 * library holds until exit; the call allocates nothing.  Limit: each problem may keep
 * at most 131072 DP cells and 8191 error rows per side of its seed match, otherwise its
 * dStatus is nonzero and the call returns OIC_ERR_OVERFLOW (the other problems' outputs
 * are still exact); a problem naming a read outside the store or a match outside its
 * reads makes the call return OIC_ERR_ARG.  The first call on a device looks up the
 * array's device address (make it before any stream capture; a cudaDeviceReset of that
 * device invalidates the lookup).  Every call shares the array: calls that overlap on
 * the GPU race.  Runs on the context's stream and returns when the kernel has finished. */
int oic_extend_batch_noalloc(oic_ctx *ctx, uint32_t nAlign, const oic_extend_problem *dProblems, int32_t *dOut,
                             int32_t *dKind, int32_t *dDeltaLen, uint32_t *dStatus);

/* ---------------------------------------------------------------------------------
 * Learned candidate filter.  No counterpart in the reference: overlapInCore extends
 * every candidate pair that passes its hopeless check (overlapInCore-Process_String_
 * Overlaps.C:354-547).  With a filter set, a small MLP scores each candidate pair from
 * its seeds before the DP, and pairs scored below the threshold are not extended.
 * Every record still comes from the exact DP, so the output is a subset of the plain
 * output (recall < 1 is possible, wrong records are not).
 *
 * Feature row of a pair (FP16, OIC_FILTER_IN values): 64 bins of seed density over
 * the pair's diagonals (-lenS, lenT) -- seeds in the bin / overlap length along the
 * bin's centre diagonal (at least 64), capped at 4 -- then (ln lenS - 8)/2,
 * (ln lenT - 8)/2, (ln(1 + seeds) - 5)/4, then 13 zeros.
 * Network: 80 -> 128 ReLU -> 128 ReLU -> 1 (logit), FP16 parameters and activations,
 * FP32 accumulation.  Parameter array (OIC_FILTER_NPARAM FP16 values, row-major
 * [out][in]): w1[128][80] | b1[128] | w2[128][128] | b2[128] | w3[128] | b3.
 * --------------------------------------------------------------------------------- */
#define OIC_FILTER_FEATURES 67
#define OIC_FILTER_IN       80
#define OIC_FILTER_HIDDEN   128
#define OIC_FILTER_NPARAM   27009

/* One candidate pair seen by a run while pair collection is on. */
typedef struct oic_pair_info {
  uint32_t aID;        /* ref read (S), 1-based */
  uint32_t bID;        /* hash-block read (T), 1-based */
  uint32_t flags;      /* bit 0: S reverse-complemented; bit 1: dropped by the filter */
  uint32_t seeds;      /* k-mer seeds of the pair (diag_ct) */
  uint32_t nodes;      /* match runs of the pair (its nodes in oic_get_pairs' node array) */
  uint32_t overlaps;   /* records the DP emitted for the pair */
  uint32_t cells;      /* DP cells spent on the pair (saturating) */
  float    score;      /* filter logit (0 when no filter is set) */
  uint32_t extensions; /* Extend_Alignment calls made for the pair */
  int32_t  firstHit;   /* index of the first extension that added an overlap, -1 none */
  uint32_t cellsFirst; /* DP cells of the pair's first extension */
  uint32_t extLimit;   /* 1 when the filter's single-extension tier applied, else 0 */
} oic_pair_info;

/* The overlapInCore parameters a filter network was trained under.  A network scores
 * seed patterns whose meaning depends on them (k-mer size, error rate, minimum overlap),
 * so it is only used on a context with the same values. */
typedef struct oic_filter_domain {
  uint32_t kmerLen;      /* -k */
  int32_t  minOlapLen;   /* --minlength */
  double   maxErate;     /* --maxerate, strtof-rounded as in oic_params */
} oic_filter_domain;

/* Set the filter (params: host array of OIC_FILTER_NPARAM FP16 bit patterns) and its
 * probability thresholds, p = sigmoid(logit):
 *   p <  dropThreshold                  the pair is not extended;
 *   dropThreshold <= p < fullThreshold  the pair stops once extBudget extensions (0
 *                                       means 1) have run without finding an overlap;
 *   p >= fullThreshold                  every match is extended (the reference's rule).
 * fullThreshold <= dropThreshold disables the middle tier.  trainedOn names the
 * parameters the network was trained under; a context whose kmerLen, minOlapLen or
 * maxErate differs (or a NULL trainedOn) is refused with OIC_ERR_ARG.  params NULL
 * turns the filter off. */
int oic_set_filter(oic_ctx *ctx, const uint16_t *params, float dropThreshold, float fullThreshold,
                   uint32_t extBudget, const oic_filter_domain *trainedOn);

/* Pair collection for training and evaluation: mode 0 off, 1 pairs and feature rows,
 * 2 also the match runs (T offset, length, S start per run).  Collected data accumulate
 * over runs until oic_clear_pairs(). */
int oic_collect_pairs(oic_ctx *ctx, int mode);
int oic_num_pairs(oic_ctx *ctx, uint64_t *nPairs, uint64_t *nNodes);
/* Copies up to maxPairs pairs (info, and feat: OIC_FILTER_IN FP16 per pair, when
 * non-NULL) and up to maxNodes runs (3 int32 each, when non-NULL), in collection order. */
int oic_get_pairs(oic_ctx *ctx, oic_pair_info *info, uint16_t *feat, int32_t *nodes, uint64_t maxPairs,
                  uint64_t maxNodes);
int oic_clear_pairs(oic_ctx *ctx);

/* Training and inference kernels of the filter network on caller-owned DEVICE
 * buffers (stream: a cudaStream_t, NULL for the default stream; the calls return
 * after launching).  X: n rows of OIC_FILTER_IN FP16.
 *   oic_mlp_forward:  logit[n]; dH1/dH2 (n x 128 FP16 activations) when non-NULL.
 *   oic_mlp_backward: adds to dGrad (OIC_FILTER_NPARAM FP32, parameter layout) the
 *     gradient of sum_i weight_i * BCE(sigmoid(logit_i), label_i) (dWeight NULL: 1),
 *     using dG1/dG2 (n x 128 FP16) as scratch; adds the loss to *dLoss when non-NULL.
 *   oic_mlp_adam: one Adam step (bias-corrected, step >= 1, decoupled weight decay)
 *     on FP32 master weights with gradient gradScale * dGrad; writes the FP16 copy
 *     dParams and zeroes dGrad. */
int oic_mlp_forward(const uint16_t *dParams, const uint16_t *dX, uint32_t n, float *dLogit, uint16_t *dH1,
                    uint16_t *dH2, void *stream);
int oic_mlp_backward(const uint16_t *dParams, const uint16_t *dX, const uint16_t *dH1, const uint16_t *dH2,
                     const float *dLogit, const float *dLabel, const float *dWeight, uint32_t n, float *dGrad,
                     uint16_t *dG1, uint16_t *dG2, float *dLoss, void *stream);
int oic_mlp_adam(float *dMaster, float *dM, float *dV, float *dGrad, uint16_t *dParams, float lr, float beta1,
                 float beta2, float eps, float gradScale, float weightDecay, uint32_t step, void *stream);

/* ---------------------------------------------------------------------------------
 * DP launch configuration.  No counterpart in the reference (its DP runs one pair per
 * OpenMP thread).  Candidate pairs go to one of two bins:
 *   one-warp bin   one warp per pair, 8 warps per CTA, 512-int shared-memory rows
 *                  (wider bands continue in HBM rows up to 16384), at most narrowArena
 *                  kept DP cells per extension;
 *   CTA bin        one pair per CTA of wideThreads threads (32 x warps per pair); each
 *                  error row is computed by the whole CTA, wideTile diagonals per
 *                  thread per pass (tile width 32 x wideTile per warp), wideBandW-int
 *                  shared-memory rows, wideCtas CTAs, wideArena kept cells per CTA.
 * A pair whose shorter read has at least wideMinLen bases (the length-bin boundary)
 * goes straight to the CTA bin; a one-warp pair that exceeds a one-warp capacity is
 * discarded without side effects and rerun in the CTA bin; a CTA-bin pair that
 * exceeds its capacity is rerun on 8 CTAs holding the rest of the free memory.  Every
 * configuration computes the same records; only the speed changes.  Zero fields take
 * the defaults; oic_autotune() measures a grid and keeps the fastest. */
typedef struct oic_tuning {
  uint32_t narrowArena;   /* kept DP cells per extension in the one-warp bin (default 1 << 20) */
  uint32_t wideMinLen;    /* length-bin boundary, bases of the shorter read (default: none) */
  uint32_t wideThreads;   /* threads per CTA of the CTA bin: 64 .. 512, a multiple of 32 (default 256) */
  uint32_t wideTile;      /* diagonals per thread per pass in the CTA bin: 1, 2 or 4 (default 1) */
  uint32_t wideBandW;     /* shared-memory row width of the CTA bin, ints (default 12288) */
  uint32_t wideCtas;      /* CTAs of the CTA bin (default: 2 per SM) */
  uint64_t wideArena;     /* kept DP cells per CTA of the CTA bin (default: 2^24, less if memory is short) */
  uint32_t forceWide;     /* testing: every pair goes to the CTA bin (0 / 1) */
  uint32_t noGraph;       /* 1: launch the DP stage kernel by kernel with host-read sizes instead of
                             relaunching its captured CUDA graph (same records) */
  uint32_t wideMode;      /* CTA bin kernel: 2 (default) CTA-wide rows (wideThreads, wideTile, wideBandW
                             apply); 1 speculative -- the CTA's 8 warps each extend one of the pair's next
                             alive match nodes with the one-warp DP and warp 0 replays them in the
                             reference's order (wideArena is split between the warps) */
} oic_tuning;

int oic_set_tuning(oic_ctx *ctx, const oic_tuning *t);   /* NULL: defaults */
int oic_get_tuning(oic_ctx *ctx, oic_tuning *t);          /* the configuration in use */

/* Autotuner: runs the seed pass for ref reads [bgnRefID, endRefID] against the loaded
 * hash block once, then times the DP of those candidate pairs under each configuration
 * of a grid -- the speculative CTA bin, then CTA-wide rows with wideTile {1, 2, 4} x
 * warps per pair {2, 4, 8, 16} -- and then the best of those with length-bin boundary
 * {none, 4 quantiles of the pairs' shorter read}, checks that
 * every configuration emits the same records, and sets the fastest (a length bin only
 * when it beats the best configuration without one by more than 5 %).  The sample's
 * DP runs once per configuration (16 times): keep it to a few seconds of DP.  With report
 * non-NULL, fills report[0 .. maxReport) with one line per configuration:
 * (wideTile, wideThreads, wideMinLen, narrow ms, wide ms, total ms, narrow cells,
 * wide cells) as doubles (wideTile 0: the speculative CTA bin), and *nReport with the
 * number of lines. */
int oic_autotune(oic_ctx *ctx, uint32_t bgnRefID, uint32_t endRefID, double *report, uint32_t maxReport,
                 uint32_t *nReport);

/* Frequent k-mers of reads [bgnID, endID]: the counting step that makes overlapInCore's
 * -k skip file (in canu: `meryl count` + `meryl print` of the k-mers at or above a
 * threshold, src/pipelines/canu/Meryl.pm; read back by Build_Hash_Index.C:203-246).
 * A k-mer and its reverse complement count as one (canonical) k-mer; windows with an N
 * are skipped.  Writes up to maxKmers k-mers with count >= minCount -- kmerLen bases
 * each (ACGT), concatenated -- and their counts (saturating at 2^32-1), in ascending
 * order of the canonical 2-bit key; *nKmers gets the number found (larger than
 * maxKmers: OIC_ERR_OVERFLOW, call again with room).  Read sets with more windows than
 * one sort holds (2^32 - 2, or what the free device memory takes) are counted in
 * passes over ranges of the canonical key space. */
int oic_count_kmers(oic_ctx *ctx, uint32_t bgnID, uint32_t endID, uint32_t minCount, char *kmers, uint32_t *counts,
                    uint64_t maxKmers, uint64_t *nKmers);

/* The record pass of the overlap-store build (ovStoreBuild, src/stores/ovStoreBuild.C:
 * 166-255) on CUDA device `device`: every record of words[0 .. 6 * nRecords) is checked
 * (a_iid and b_iid in 1..maxID, else OIC_ERR_INPUT) and filtered as
 * ovStoreFilter::filterOverlap does (src/stores/ovStoreFilter.C:62-160: a record whose
 * evalue exceeds AS_OVS_encodeEvalue(maxErate) loses forUTG, forOBT and forDUP), its
 * ID-swapped copy is made (ovOverlap::swapIDs, src/stores/ovOverlap.C:216-246), the
 * record and the copy are kept when one of the three flags is set, and the kept records
 * are sorted in ovOverlap order (a_iid, b_iid, the two data words) into out (room for
 * 2 * nRecords records).  *nOut gets their number.  perRead (optional, maxID + 2
 * entries): perRead[i] = index in out of the first record with a_iid i, perRead[maxID +
 * 1] = *nOut.  counts (optional, 5): saved unitigging, saved trimming, discarded for
 * the error rate, discarded untrimmed, discarded flipped -- ovStoreFilter's counters.
 * Host buffers; the call allocates its device memory and returns when done. */
int oic_store_sort(int device, const uint32_t *words, uint64_t nRecords, uint32_t maxID, double maxErate,
                   uint32_t *out, uint64_t *nOut, uint64_t *perRead, uint64_t *counts);

/* Edit_Match_Limit / Error_Bound tables the context uses (for testing): copies
 * min(n, table length) entries; *len gets the table length. */
int oic_get_match_limit(oic_ctx *ctx, int32_t *dst, uint32_t n, uint32_t *len);

/* Last CUDA / kernel error text of the context (never NULL). */
const char *oic_last_error(oic_ctx *ctx);

#ifdef __cplusplus
}
#endif

#endif
