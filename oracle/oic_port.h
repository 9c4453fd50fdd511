/*
 * oic_port.h -- CPU restatement of canu's overlapInCore hot path (test infrastructure).
 *
 * This is the ORACLE: plain C, used only by tests/, __graft_entry__.smoke() and the
 * CPU-baseline legs of bench.py, as the checker and the CPU timing baseline of the
 * CUDA path.  The product (canu_gb300/, include/oic_gpu.h) never links it.
 *
 * Parity is pinned by running canu's own overlapInCore sources, compiled unchanged
 * with a shim (oracle/Makefile.ref -> oracle/_ref/oic_ref), on the same inputs and
 * comparing the sorted overlap record sets, the .oc counts and the stats counters
 * (tests/golden/ holds the fixtures and the script that made them).
 */
#ifndef OIC_PORT_H
#define OIC_PORT_H

#include <stdint.h>
#include "oic_seqdb.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Command-line parameters of overlapInCore (overlapInCore.H:367-473, overlapInCore.C:293-411). */
typedef struct oic_port_params {
  double   maxErate;          /* --maxerate, parsed with strtof (overlapInCore.C:380)   */
  double   alignNoise;        /* --alignnoise, strtof (overlapInCore.C:382)             */
  int      partial;           /* -partial                                               */
  uint32_t bgnHashID, endHashID, minLibToHash, maxLibToHash;   /* -h, -H              */
  uint32_t bgnRefID, endRefID, minLibToRef, maxLibToRef;       /* -r, -R              */
  uint32_t kmerLen;           /* -k <int>                                               */
  const char *kmerSkipFile;   /* -k <file> or NULL                                      */
  int      minKmers;          /* --minkmers                                             */
  int      uniqueOlapPerPair; /* -u (default 1) / -m                                    */
  uint32_t hashBits;          /* --hashbits                                             */
  uint64_t maxHashDataLen;    /* --hashdatalen (before the AS_MAX_READLEN increment)     */
  double   maxHashLoad;       /* --hashload (atof)                                      */
  uint32_t numThreads;        /* -t                                                     */
  int32_t  minOlapLen;        /* --minlength                                            */
  int      useHopelessCheck;  /* cleared by -z, and when maxErate > 0.06                */
} oic_port_params;

/* The eight counters of the -s stats file (overlapInCore.C:550-558). */
typedef struct oic_port_stats {
  uint64_t kmerHitsWithoutOlap, kmerHitsWithOlap, kmerHitsSkipped, multiOverlap;
  uint64_t totalOverlaps, containedOverlaps, dovetailOverlaps;
  uint64_t badShortWindow, badLongWindow;
  uint64_t dpCells, slideBases, extensions, seeds, candidatePairs;   /* work counters */
  uint32_t nHashBlocks;
} oic_port_stats;

/* One emitted overlap: the six 32-bit words ovFile writes per record
 * (a_iid, b_iid, dat[0] hi, dat[0] lo, dat[1] hi, dat[1] lo; ovStoreFile.C:262-276). */
typedef struct oic_port_record {
  uint32_t w[6];
} oic_port_record;

void oic_port_default_params(oic_port_params *p);

/* Parse an overlapInCore command line (argv[0] is the program name).  Returns 0 on
 * success; on success *storePath, *outPath and *statsPath point into argv. */
int oic_port_parse_args(int argc, char **argv, oic_port_params *p, const char **storePath,
                        const char **outPath, const char **statsPath);

/* Run the whole stage: hash blocks over [bgnHashID,endHashID], every ref read of
 * [bgnRefID,endRefID] against each block.  Records are appended to *recs (realloc'd,
 * caller frees).  Returns 0 on success, nonzero on an input the reference rejects. */
int oic_port_run(const oic_port_params *p, const oic_seqdb *db, oic_port_record **recs,
                 uint64_t *nRecs, oic_port_stats *stats);

/* Edit_Match_Limit table (Binomial_Bound.C:104-195) for maxAlignErate = erate*noise,
 * maxErrors = 1 + ceil(erate * AS_MAX_READLEN) (prefixEditDistance.C:33). */
int32_t oic_port_max_errors(double maxErate);
void    oic_port_match_limit(int32_t *ml, double maxAlignErate, int32_t maxErrors);

/* One Extend_Alignment (prefixEditDistance-extend.C:36-183) of the exact match
 * (start in S, offset in T, len) between lowercase strings S and T.  Returns the
 * overlap kind (0 NONE, 1 LEFT_BRANCH_PT, 2 RIGHT_BRANCH_PT, 3 DOVETAIL); fills
 * out[0..4] = S_Lo, S_Hi, T_Lo, T_Hi, Errors and *deltaLen, and if delta != NULL the
 * merged Left_Delta (up to maxErrors entries).  cells/slides accumulate work counts. */
typedef struct oic_port_aligner oic_port_aligner;
oic_port_aligner *oic_port_aligner_new(double maxErate, double alignNoise, int partial);
void              oic_port_aligner_free(oic_port_aligner *a);
int oic_port_extend(oic_port_aligner *a, const char *S, int32_t sLen, const char *T, int32_t tLen,
                    int32_t start, int32_t offset, int32_t len, int32_t *out, int32_t *delta,
                    int32_t *deltaLen, uint64_t *cells, uint64_t *slides);

/* A hash block built once (the first block of the -h range) and ref ranges run
 * against it, for timing the CPU path on a sample of ref reads.  *buildSeconds gets the
 * wall time of the block build.  numThreads threads are used throughout. */
typedef struct oic_port_session oic_port_session;
oic_port_session *oic_port_session_new(const oic_port_params *p, const oic_seqdb *db, double *buildSeconds);
uint32_t          oic_port_session_last_loaded(const oic_port_session *s);
int  oic_port_session_refs(oic_port_session *s, uint32_t bgnRef, uint32_t endRef, oic_port_record **recs,
                           uint64_t *nRecs, oic_port_stats *stats);
void oic_port_session_free(oic_port_session *s);

/* Loading and freeing helpers for callers outside C (ctypes). */
oic_seqdb *oic_port_seqdb_load(const char *path);
void       oic_port_seqdb_free(oic_seqdb *db);
void       oic_port_records_free(oic_port_record *r);

#ifdef __cplusplus
}
#endif

#endif
