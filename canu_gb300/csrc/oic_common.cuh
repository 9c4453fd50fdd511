// oic_common.cuh -- shared device-side definitions of the GB300 overlapInCore engine.
//
// Read layout in HBM: every read is packed 2 bits per base (A=0 C=1 G=2 T=3, base i
// of a read at bits 2*(i%32) of 64-bit word i/32, the same order overlapInCore builds
// its k-mer keys in, Build_Hash_Index.C:347-350) in two strand arrays -- forward and
// reverse complement -- plus a parallel mask array with 0b11 at every N.  Reads start
// on a word boundary and are separated by one zero guard word, so a 32-base window
// that runs off either end of a read stays inside the arrays.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace oic {

typedef unsigned long long u64;
typedef long long          i64;
typedef unsigned int       u32;

constexpr u32 kMaxReadLenBits = 21;                              // AS_MAX_READLEN_BITS
constexpr u32 kMaxReadLen     = (1u << kMaxReadLenBits) - 1;     // AS_MAX_READLEN
constexpr int kHopelessMatch  = 90;                              // overlapInCore.H:78
constexpr int kMaxDistinct    = 3;                               // overlapInCore.H:107
constexpr int kMinIntersect   = 10;                              // overlapInCore.H:120
constexpr int kShiftSlack     = 1;                               // overlapInCore.H:146
constexpr int kEntriesPerBucket = 21;                            // overlapInCore.H:58
constexpr u64 kEmptyKey       = ~0ull;
constexpr u64 kPairMask       = 0x5555555555555555ull;

// Device error flags (bitwise OR into ctx->dErr).  Kernels never trap: they record
// the condition, skip the access and return.
enum : u32 {
  kErrBadBase      = 1u << 0,
  kErrArenaFull    = 1u << 1,   // DP traceback arena of a warp exhausted
  kErrBandWide     = 1u << 2,   // DP band wider than the shared-memory row buffer
  kErrRowsFull     = 1u << 3,   // more DP rows than the row-header capacity
  kErrNodePool     = 1u << 4,   // seed replay: node pool of a warp exhausted
  kErrPairTable    = 1u << 5,   // seed replay: pair table of a warp exhausted
  kErrOutNodes     = 1u << 6,   // global node output full
  kErrOutPairs     = 1u << 7,   // global pair output full
  kErrDeltaFull    = 1u << 8,
  kErrTableFull    = 1u << 9,   // k-mer table probe ran through every slot
  kErrInternal     = 1u << 10,
  kErrNodesPerPair = 1u << 11
};

// Packed reads (device pointers).
struct ReadsDev {
  const u64 *fwd;       // forward strand words
  const u64 *rc;        // reverse-complement strand words
  const u64 *nfwd;      // N masks (0b11 per N) for the forward strand
  const u64 *nrc;
  const u64 *wordOff;   // first word of read i (0-based index = ID-1)
  const u32 *len;
  const u32 *lib;
  const unsigned char *hasN;
  u32 nReads;
};

// One read strand viewed as a base sequence: base i is base i of the read's first word.
struct SeqView {
  const u64 *w;    // the read's first word in its strand array
  const u64 *nm;   // its first N-mask word; nullptr when the read has no N
};

__device__ __forceinline__ SeqView make_view(const ReadsDev &R, u32 readIdx, int rev) {
  SeqView v;
  const u64 wo = R.wordOff[readIdx];
  v.w  = (rev ? R.rc : R.fwd) + wo;
  v.nm = R.hasN[readIdx] ? (rev ? R.nrc : R.nfwd) + wo : nullptr;
  return v;
}

// 32 bases starting at global base index g (base g in bits 0-1).  Both words are
// always read (the arrays end with two spare words), and the high word's shift is
// split in two so that sh = 0 needs no branch: (hi << 1) << 63 is 0.
__device__ __forceinline__ u64 load_win(const u64 *w, i64 g) {
  const i64 wi = g >> 5;
  const int sh = (int)(g & 31) * 2;
  const u64 lo = __ldg(w + wi);
  const u64 hi = __ldg(w + wi + 1);
  return (lo >> sh) | ((hi << 1) << (63 - sh));
}

// The same for base g of one read (w = the read's first word; -32 < g: the guard word
// before every read keeps g - 31 in bounds), in 32-bit index arithmetic.
__device__ __forceinline__ u64 load_win32(const u64 *w, int g) {
  const int wi = g >> 5;
  const int sh = (g & 31) * 2;
  const u64 lo = __ldg(w + wi);
  const u64 hi = __ldg(w + wi + 1);
  return (lo >> sh) | ((hi << 1) << (63 - sh));
}

// 32 bases g, g-1, ..., g-31 of one read (base g in bits 0-1; the two bits of each
// base come out swapped, which equality tests do not see).
__device__ __forceinline__ u64 load_win_rev(const u64 *w, int g) { return __brevll(load_win32(w, g - 31)); }

// Number of leading bases (0..32) that agree between A (from a) and T (from t), with
// N matching anything (prefixEditDistance-forward.C:164 / -reverse.C:186).
template <int STEP>
__device__ __forceinline__ int match_run32(const SeqView &A, int a, const SeqView &T, int t) {
  u64 wa, wt;
  if (STEP > 0) {
    wa = load_win32(A.w, a);
    wt = load_win32(T.w, t);
  } else {
    wa = load_win_rev(A.w, a);
    wt = load_win_rev(T.w, t);
  }
  u64 x  = wa ^ wt;
  u64 mm = (x | (x >> 1)) & kPairMask;
  if (mm && (A.nm || T.nm)) {
    u64 n = 0;
    if (A.nm) n |= (STEP > 0) ? load_win32(A.nm, a) : load_win_rev(A.nm, a);
    if (T.nm) n |= (STEP > 0) ? load_win32(T.nm, t) : load_win_rev(T.nm, t);
    mm &= ~n;
  }
  return mm ? (__ffsll((long long)mm) - 1) >> 1 : 32;
}

// 16 bases starting at base g of one read, from the strand viewed as 32-bit words (base
// i in bits 2*(i%16) of word i/16 on a little-endian device): one funnel shift.  The
// guard word before a read keeps g >= -32 in bounds.
__device__ __forceinline__ u32 load_win16(const u64 *w, int g) {
  const u32 *w32 = reinterpret_cast<const u32 *>(w);
  const int  wi  = g >> 4;
  return __funnelshift_r(__ldg(w32 + wi), __ldg(w32 + wi + 1), (g & 15) * 2);
}

// Number of leading bases (0..16) that agree between A (from a) and T (from t), N
// matching anything: a cheaper first step for slides that are mostly short.
template <int STEP>
__device__ __forceinline__ int match_run16(const SeqView &A, int a, const SeqView &T, int t) {
  u32 wa, wt;
  if (STEP > 0) {
    wa = load_win16(A.w, a);
    wt = load_win16(T.w, t);
  } else {
    wa = __brev(load_win16(A.w, a - 15));
    wt = __brev(load_win16(T.w, t - 15));
  }
  const u32 x  = wa ^ wt;
  u32       mm = (x | (x >> 1)) & 0x55555555u;
  if (mm && (A.nm || T.nm)) {
    u32 n = 0;
    if (A.nm) n |= (STEP > 0) ? load_win16(A.nm, a) : __brev(load_win16(A.nm, a - 15));
    if (T.nm) n |= (STEP > 0) ? load_win16(T.nm, t) : __brev(load_win16(T.nm, t - 15));
    mm &= ~n;
  }
  return mm ? (__ffs((int)mm) - 1) >> 1 : 16;
}

// Whether the DP kernels start slides with the 16-base compare: above a 2 % error rate
// most slides end within a few bases (measured: 11 % less one-warp DP time at 2 % read
// error), while on low-error reads the slides along the alignment run ~100 bases and the
// 32-base first step is cheaper (2 % more with the 16-base one at 0.5 % read error).
__host__ __device__ inline bool slide_first16(double maxErate) { return maxErate > 0.02; }

// Bases that agree from A[step*row] / T[step*(row+d)] on, capped at `lim` (> 0).  The
// first step compares 32 bases, or 16 when FIRST16 (cheaper when most slides end
// within a few bases, as at higher error rates); the rest go 32 at a time.
template <int STEP, bool FIRST16 = false>
__device__ __forceinline__ int slide(const SeqView &A, int a0, const SeqView &T, int t0, int row, int d, int lim,
                                     unsigned long long &slides) {
  int  run  = 0;
  bool more = true;
  if (FIRST16) {
    run  = match_run16<STEP>(A, a0 + STEP * row, T, t0 + STEP * (row + d));
    more = run == 16;
  }
  if (more)
    while (run < lim) {
      int r = match_run32<STEP>(A, a0 + STEP * (row + run), T, t0 + STEP * (row + d + run));
      run += r;
      if (r < 32) break;
    }
  if (run > lim) run = lim;
  slides += (unsigned long long)run;
  return run;
}

__device__ __forceinline__ u64 mix64(u64 x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ull;
  x ^= x >> 33;
  return x;
}

// K-mer table (device): open addressing over 16-byte slots, slot s = (key kv[2s],
// value kv[2s+1]) so that a probe is one 16-byte load.  value: bits 0-31 first
// occurrence, 32-62 count, 63 screened.
struct TableDev {
  const u64 *kv;
  u64        mask;       // capacity - 1
  const u64 *occ;        // (blockString << 32) | offset, ascending within a k-mer
  const unsigned char *lscr, *rscr;   // String_Info l/rfrag_end_screened per block string
  const u32 *slen;       // per block string: length (0 when the string is empty)
  const u32 *sread;      // per block string: 0-based read index
  u32        firstID;    // Hash_String_Num_Offset
  u32        nStrings;
};

__device__ __forceinline__ bool table_find(const TableDev &T, u64 key, u64 &val) {
  u64 s = mix64(key) & T.mask;
  for (u64 probe = 0; probe <= T.mask; probe++) {
    const ulonglong2 e = __ldg((const ulonglong2 *)T.kv + s);
    if (e.x == key) {
      val = e.y;
      return true;
    }
    if (e.x == kEmptyKey) return false;
    s = (s + 1) & T.mask;
  }
  return false;
}

// Parameters every kernel needs (passed by value).
struct DevParams {
  double maxErate;
  double branchMatchValue;     // prefixEditDistance.C:86
  double minBranchTailSlope;   // prefixEditDistance.C:29
  double kmerExpect;           // exp(-K * maxErate), host glibc
  unsigned long long minKmers; // Filter_By_Kmer_Count after overlapInCore.C:410-411 (0 = off)
  int    kmerLen;
  int    partial;
  int    unique;
  int    hopeless;
  int    minOlapLen;
  int    maxErrors;            // MAX_ERRORS (prefixEditDistance.C:27)
};

__device__ __forceinline__ int error_bound(int i, double maxErate) {
  return (int)ceil(__dmul_rn((double)i, maxErate));   // prefixEditDistance.C:60
}

// Warp helpers.
__device__ __forceinline__ int warp_min(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ int warp_max(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ unsigned long long warp_sum64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

}  // namespace oic
