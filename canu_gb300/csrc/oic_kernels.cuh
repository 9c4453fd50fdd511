// oic_kernels.cuh -- kernel launch wrappers shared between the .cu files and the
// C-ABI layer.  Everything here runs on the context's stream.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "oic_common.cuh"
#include "oic_align.cuh"

// CTAs of the one-warp DP kernel resident per SM (its register budget follows).
#ifndef OIC_ALIGN_MIN_BLOCKS
#define OIC_ALIGN_MIN_BLOCKS 3
#endif

namespace oic {

// ---------------- reads ----------------
// Pack ASCII reads into the 2-bit strand arrays (see oic_common.cuh).  err gets
// kErrBadBase for a character outside ACGTN (either case).
void launch_pack_reads(const char *ascii, const u64 *srcOff, const u32 *len, const u64 *wordOff, u32 nReads,
                       u64 *fwd, u64 *rc, u64 *nfwd, u64 *nrc, unsigned char *hasN, u32 *err, cudaStream_t st);

// ---------------- hash block ----------------
// K-mer keys of every block string; key = 1 << 2K for a window holding an N.
void launch_kmer_emit(ReadsDev R, const u32 *strRead, const u32 *strKmers, const u64 *flatStart, u32 nStr, int K,
                      u64 *keys, u32 *vals, cudaStream_t st);
// newKeys[s] += number of distinct k-mers whose first occurrence is in block string s.
// chunkStr[c] (nFlat / 4096 + 1 entries) = the block string holding flat k-mer index
// c * 4096; string lookups of the two kernels below start there.
void launch_chunk_str(const u64 *flatStart, u32 nStr, u64 nFlat, u32 *chunkStr, cudaStream_t st);
void launch_first_occ(const u64 *keys, const u32 *vals, u64 n, const u64 *flatStart, const u32 *chunkStr, int K,
                      u32 *newKeys, cudaStream_t st);
// flags[p] = 1 when keys[p] is a valid k-mer and vals[p] < flatLimit.
void launch_keep_flags(const u64 *keys, const u32 *vals, u64 n, int K, u32 flatLimit, u32 *flags, cudaStream_t st);
void launch_compact_kv(const u64 *keys, const u32 *vals, const u32 *flags, const u32 *pos, u64 n, u64 *keysOut,
                       u32 *valsOut, cudaStream_t st);
// Open-addressing table of 16-byte slots (key, value) at tKV, capacity mask + 1;
// launch_table_init empties every slot.
void launch_table_init(u64 *tKV, u64 cap, cudaStream_t st);
void launch_table_build(const u64 *keys, u64 n, u64 *tKV, u64 mask, u32 *err, cudaStream_t st);
void launch_occ_convert(const u32 *vals, u64 n, const u64 *flatStart, const u32 *chunkStr, u64 *occ, cudaStream_t st);
void launch_skip_mark(const u64 *skipKeys, u64 nSkip, TableDev T, u64 *tKVMut, unsigned char *lscr,
                      unsigned char *rscr, int K, int hopeless, u32 *err, cudaStream_t st);

// ---------------- seeds ----------------
struct PairRec {
  u32 sRead;      // 0-based read index of S
  u32 tStr;       // block string index of T
  u32 nodeOff;    // first match node in the node output
  u32 nodeCnt;
  int diagCt, diagBgn, diagEnd;
  u32 flags;      // bit0 reverse strand, bit1 consistent, bit2 S left-end screened, bit3 S right-end screened
};

struct PairAcc {   // seed-replay state of one pair (per-warp scratch)
  u32 T;
  int head;
  int diagCt, diagBgn, diagEnd;
  int consistent;
  int slot;
  int pad;
};

struct SeedScratch {
  int     *slotKey;    // per warp: slotCap ints
  int     *slotVal;
  PairAcc *pairs;      // per warp: pairCap
  int4    *nodes;      // per warp: nodeCap (offset, len, start, next)
};

struct SeedCaps {
  int slotCap;   // power of two
  int pairCap;
  int nodeCap;
};

struct SeedOut {
  PairRec *pairs;
  u32      pairCap;
  u32     *pairCount;
  int4    *nodes;       // (offset, len, start, unused)
  u32      nodeCap;
  u32     *nodeCount;
  u32     *overflowSegs;
  u32     *overflowCount;
  unsigned long long *stats;   // [seeds, segments]
  u32     *err;
};

// Segment k is (ref index << 1 | strand) = segList[k], or k when segList is null.
void launch_seed(ReadsDev R, TableDev T, DevParams P, const u32 *segReads, const u32 *segList, u32 nSeg,
                 u32 *segCounter, SeedScratch sc, SeedCaps cap, int nWarps, SeedOut out, cudaStream_t st);

// ---------------- pairs / DP ----------------
struct AlignOut {
  u32 *rec;             // 3 records x 6 words per pair slot
  u32 *cnt;             // records per pair slot
  u32 *overflow;        // pair indices that exceeded a capacity
  u32 *overflowCount;
  unsigned long long *stats;   // see StatIdx
  u32 *err;
  u32 *cells;           // optional: DP cells spent on each pair slot (saturating) ...
  int4 *ext;            // ... and (extensions, first extension with an overlap or -1,
                        //      cells of the first extension, extension limit applied)
  const float *tierLogit;   // optional: pairs scored below tierThr stop once tierBudget
  float        tierThr;     // extensions have run without finding an overlap
  int          tierBudget;
  const u32   *nWorkDev;    // optional: the work list's length, read on the device
  const u32   *workOffDev;  // optional: the work list starts at work + *workOffDev
};

enum StatIdx {
  kStWithoutOlap = 0, kStWithOlap, kStSkipped, kStMulti, kStTotal, kStContained, kStDovetail,
  kStCells, kStSlides, kStExtensions, kStRows, kStCellsNoOlap, kStCount
};

// One pair per warp, 8 warps per CTA, 512-int shared-memory rows (bandW is ignored).
void launch_align(int bandW, ReadsDev R, TableDev T, DevParams P, const int *eml, const PairRec *pairs,
                  const u32 *work, u32 nWork, u32 *workCounter, const int4 *nodes, WarpScratch sc, AlignCaps cap,
                  int nWarps, AlignOut out, cudaStream_t st);

// One pair per CTA of `threads` threads (a multiple of 32, at most 512): warp 0 runs
// the pair logic and the whole CTA runs each error-row loop, U (1, 2, 4) diagonals per
// thread per pass; row buffers of bandW ints in shared memory; scratch per CTA.
void launch_align_group(int threads, int U, int bandW, int ctas, ReadsDev R, TableDev T, DevParams P, const int *eml,
                        const PairRec *pairs, const u32 *work, u32 nWork, u32 *workCounter, const int4 *nodes,
                        WarpScratch sc, AlignCaps cap, AlignOut out, cudaStream_t st);

// Speculative CTA bin: one pair per CTA of align_spec_warps() warps, each warp running
// whole extensions (one-warp DP, 512-int shared-memory rows, HBM rows up to
// cap.rowsGW) of the pair's next alive match nodes, replayed in the reference's order.
// sc/cap describe ctas * align_spec_warps() warp scratches; a pair's alive flags use the
// nodeCap bytes of all its CTA's warps.
void launch_align_spec(int ctas, ReadsDev R, TableDev T, DevParams P, const int *eml, const PairRec *pairs,
                       const u32 *work, u32 nWork, u32 *workCounter, const int4 *nodes, WarpScratch sc, AlignCaps cap,
                       AlignOut out, cudaStream_t st);
int align_spec_warps();

struct ExtendProblem;
void launch_extend_group(int threads, int U, int bandW, int ctas, ReadsDev R, DevParams P, const int *eml,
                         const ExtendProblem *probs, u32 n, WarpScratch sc, AlignCaps cap, int *out, int *kind,
                         int *deltaLen, u32 *status, unsigned long long *stats, cudaStream_t st);

struct ExtendProblem {
  u32 sRead, sRev, tRead;
  int mStart, mOffset, mLen;
};
void launch_extend_batch(int bandW, ReadsDev R, DevParams P, const int *eml, const ExtendProblem *probs, u32 n,
                         WarpScratch sc, AlignCaps cap, int nWarps, int *out, int *kind, int *deltaLen, u32 *status,
                         unsigned long long *stats, cudaStream_t st);

// Sort keys (32 bits) of the work list: by bin -- 0 one-warp DP, 1 CTA DP (shorter read
// >= wideMinLen bases), 2 dropped by the filter (logit non-null, below logitThr) -- and
// inside a bin the pairs with the most match nodes first.  binCount[0..1] (zeroed by
// the caller) get the sizes of bins 0 and 1.
void launch_work_keys(const PairRec *pairs, u32 n, const float *logit, float logitThr, const u32 *readLen,
                      const u32 *strRead, u32 wideMinLen, u32 *binCount, unsigned long long *keys, u32 *vals,
                      cudaStream_t st, const u32 *nDev = nullptr);
// Append the one-warp overflow behind the CTA bin's own pairs on the device (see
// append_overflow_kernel in oic_pairs.cu).
void launch_append_overflow(u32 *work, const u32 *binCount, const u32 *ovf, u32 *ovfCount, u32 *wideN,
                            u32 *workCounter, u32 *err, cudaStream_t st);

// ---------------- learned candidate filter (oic_filter.cu) ----------------
// feat: n x 80 FP16 rows (67 features, 13 zeros) of the candidate pairs.
void launch_pair_features(const PairRec *pairs, u32 n, const int4 *nodes, const u32 *readLen, const u32 *strRead,
                          int K, void *feat, cudaStream_t st);
// logit[i] of every row of X (n x 80 FP16); H1/H2 (n x 128 FP16) written when non-null.
cudaError_t launch_mlp_forward(const void *prm, const void *X, u32 n, float *logit, void *H1, void *H2,
                               cudaStream_t st);

// Sort keys of a list of pair indices: the pairs with the most match nodes first.
void launch_list_keys(const PairRec *pairs, const u32 *list, u32 n, unsigned long long *keys, u32 *vals,
                      cudaStream_t st);

// ---------------- frequent k-mers (oic_kmers.cu) ----------------
// Partitioned count: hist[part] (canon_parts() parts, part = key >> shift) of the valid
// windows of `reads`, then the windows of parts [p0, p1) appended at *counter.
int  canon_parts();
void launch_canon_hist(ReadsDev R, const u32 *reads, u32 nReads, int K, int shift, unsigned long long *hist,
                       unsigned long long *nInvalid, cudaStream_t st);
void launch_canon_emit_part(ReadsDev R, const u32 *reads, u32 nReads, int K, int shift, u32 p0, u32 p1, u64 *keys,
                            u32 *vals, unsigned long long *counter, cudaStream_t st);
void launch_run_starts(const u64 *keys, u64 nValid, u32 *flags, cudaStream_t st);
void launch_run_index(const u32 *flags, const u32 *pos, u64 nValid, u64 *runStart, cudaStream_t st);
void launch_run_select(const u64 *runStart, u32 nRuns, u64 nValid, u32 minCount, u32 *sel, cudaStream_t st);
void launch_run_compact(const u64 *keys, const u64 *runStart, u32 nRuns, u64 nValid, const u32 *sel, const u32 *pos,
                        u64 *outKey, u32 *outCount, cudaStream_t st);

// Compact per-pair record slots into a dense record array.
void launch_compact_records(const u32 *rec, const u32 *cnt, const u32 *pos, u32 nPairs, u32 *dst, cudaStream_t st);

int align_warps_per_block(int bandW);
size_t align_smem_bytes(int bandW);

}  // namespace oic
