// oic_capi.cu -- the C ABI of liboic_gpu.so (include/oic_gpu.h): context, device
// memory, host-side tables, and the orchestration of the kernels per hash block and
// per batch of ref reads.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "oic_gpu.h"
#include "oic_kernels.cuh"
#include "oic_prims.cuh"
#include "oic_internal.h"

using namespace oic;

namespace {

// ---------------------------------------------------------------------------------
// Growable device buffer.
struct DevBuf {
  void  *p   = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap && p) return cudaSuccess;
    if (p) cudaFree(p);
    p   = nullptr;
    cap = 0;
    size_t want = bytes ? bytes : 256;
    cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) cap = want;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p   = nullptr;
    cap = 0;
  }
  template <typename T> T *as() const { return (T *)p; }
};

// Edit_Match_Limit: the minimum alignment length worth extending with e errors
// (Binomial_Bound.C:36-97 and :104-195, AS_MAX_READLEN_BITS = 21), computed on the
// host with the C library's pow/exp/sqrt like the reference.
int binomial_bound(int e, double p, int start) {
  const double q = 1.0 - p;
  if (start < e) start = e;
  for (int n = start; n < (int)kMaxReadLen; n++) {
    if (n <= 35) {
      double sum = 0.0, pPow = 1.0, qPow = pow(q, n);
      int    coeff = 1, ct = 0;
      for (int k = 0; k < e && 1.0 - sum > 1e-4; k++) {
        sum += coeff * pPow * qPow;
        // The reference's int product overflows (C(n, k) * (n - k) past 2^31 for n near
        // 35 at high error counts) and the table depends on the 32-bit wraparound it
        // gets; the same wraparound, as a defined unsigned product.
        coeff = (int)((uint32_t)coeff * (uint32_t)(n - ct));
        coeff /= ++ct;
        pPow *= p;
        qPow /= q;
      }
      if (1.0 - sum > 1e-4) return n;
    } else {
      const double z = (e - 0.5 - n * p) / sqrt(n * p * q);
      if (z <= 3.62) return n;
      double sum = 0.0, mu = 1.0, fact = 1.0;
      const double pois = exp(-n * p);
      for (int k = 0; k < e; k++) {
        sum += mu * pois / fact;
        mu *= n * p;
        fact *= k + 1;
      }
      if (1.0 - sum > 1e-4) return n;
    }
  }
  return (int)kMaxReadLen;
}

void match_limit(std::vector<int32_t> &ml, double erate, int32_t maxErrors) {
  ml.assign((size_t)maxErrors + 1, 0);
  int32_t e = 0, s = 1;
  const int32_t l = std::min(maxErrors, 2000);
  while (e <= 1) ml[e++] = 0;
  while (e < l) {
    s     = binomial_bound(e - 1, erate, s);
    ml[e] = s - 1;
    e++;
  }
  const double slope = 0.982064188397525 / erate + 0.067835741959926;
  double v = ml[e - 1] + slope;
  for (; e < maxErrors; e++) {
    ml[e] = (int32_t)ceil(v);
    v += slope;
  }
}

int base2(char c) {
  switch (c) {
    case 'A': case 'a': return 0;
    case 'C': case 'c': return 1;
    case 'G': case 'g': return 2;
    case 'T': case 't': return 3;
    default: return -1;
  }
}

}  // namespace

struct oic_ctx {
  oic_params   P;
  DevParams    dp;
  int          device = 0;
  int          nSM    = 0;
  cudaStream_t st     = nullptr;
  std::string  lastErr;
  std::vector<int32_t> eml;
  DevBuf       dEml;

  // reads
  uint32_t              nReads = 0;
  std::vector<uint32_t> len, lib;
  std::vector<uint64_t> wordOff;
  DevBuf dFwd, dRc, dNfwd, dNrc, dWordOff, dLen, dLib, dHasN;
  ReadsDev R{};

  // skip list
  std::vector<uint64_t> skipKeys;
  DevBuf                dSkip;

  // hash block
  bool     haveBlock = false;
  uint32_t blkFirst = 0, blkN = 0;
  uint64_t blkOcc = 0, blkDistinct = 0;
  DevBuf dTable, dOcc, dLscr, dRscr, dSlen, dSread;   // dTable: 16-byte (key, value) slots
  DevBuf dSortK, dSortV, dSortK2, dSortV2, dFlags, dPos, dSortScratch, dStrRead, dStrKmers, dFlat, dNewKeys;
  DevBuf dChunkStr;   // block string of every 4096th flat k-mer index
  TableDev T{};

  // seeds
  DevBuf dSegReads, dPairs, dNodes, dSegOvf, dSegList;
  DevBuf dSeedSlotK, dSeedSlotV, dSeedPairs, dSeedNodes;        // normal configuration
  DevBuf dSeedSlotK2, dSeedSlotV2, dSeedPairs2, dSeedNodes2;    // wide configuration
  uint32_t pairCap = 0, nodeCap = 0;
  // Candidate pairs and match runs per (ref read x block string) of the batches so far,
  // to size the next batch; the demand of the last batch that did not fit.
  double   pairDensity = 0, nodeDensity = 0;
  uint64_t overPairs = 0, overNodes = 0;

  // align
  DevBuf dWork, dRec, dCnt, dRecPos, dRecOut, dAlnOvf, dWorkK, dWorkK2, dWorkV2, dWorkScratch;
  DevBuf dArena, dRowHdr, dDL, dDR, dStack, dAlive, dRowsG;         // normal
  DevBuf dArena2, dRowHdr2, dDL2, dDR2, dStack2, dAlive2, dRowsG2;  // wide
  DevBuf dScanScratch;

  // counters (one small device block): [0..15] u32 counters, [16..] u64 stats
  DevBuf dCtr;

  // learned candidate filter
  bool   filterOn       = false;
  float  filterLogitThr = 0.0f;      // drop below
  float  filterTierThr  = -INFINITY; // extension-budget tier below
  int    filterBudget   = 1;         // extensions without an overlap allowed in that tier
  DevBuf dFilterPrm, dFeat, dLogit, dPairCells, dPairExt;
  cudaEvent_t evF0 = nullptr, evF1 = nullptr;
  int    collect = 0;                      // 0 off, 1 pairs + features, 2 also match runs
  std::vector<oic_pair_info> colInfo;
  std::vector<uint16_t>      colFeat;
  std::vector<int32_t>       colNodes;

  oic_tuning tune{};            // DP launch configuration (zeros: defaults)

  // Captured align stage (see align_stage_graph): the executable graph, the events it
  // records, and the bytes of every parameter baked into it.
  cudaGraphExec_t      gExec = nullptr;
  unsigned             gKernels = 0;   // kernel nodes of the graph
  cudaEvent_t          gEv[3] = {nullptr, nullptr, nullptr};
  std::vector<uint8_t> gKey;

  std::vector<uint32_t> out;   // accumulated records, 6 words each
  oic_stats stats{};
};

namespace {

constexpr int kRetrySmaller = 100;   // run_batch: the batch's output did not fit

enum CtrIdx {   // u32 counters (cKeep and cKeep + 1: the two bin sizes)
  cSegCounter = 0, cPairCount, cNodeCount, cSegOvf, cWorkCounter, cAlnOvf, cErr, cRecTotal, cKeep, cKeep2, cWideN,
  cNumU32 = 16
};
constexpr int kSeedStatBase  = 16;   // u64 index: [seeds, segments]
constexpr int kAlignStatBase = 20;   // u64 index: kStCount entries
constexpr int kExtStatBase   = 40;
constexpr int kCellsSnap     = 60;   // u64 index: DP cells after the one-warp bin of a captured batch
static_assert(kNoAllocStatBase >= kExtStatBase + 3 && kNoAllocStatBase + 3 <= kCellsSnap,
              "the no-allocation entry point's counters overlap another slot");

uint32_t *ctr32(oic_ctx *c) { return c->dCtr.as<uint32_t>(); }
unsigned long long *ctr64(oic_ctx *c) { return (unsigned long long *)c->dCtr.as<uint32_t>(); }

int fail(oic_ctx *c, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (c) c->lastErr = buf;
  if (getenv("OIC_VERBOSE")) fprintf(stderr, "oic: %s\n", buf);
  return code;
}

#define CK(call)                                                                               \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess)                                                                     \
      return fail(ctx, e_ == cudaErrorMemoryAllocation ? OIC_ERR_NOMEM : OIC_ERR_CUDA, "%s: %s", \
                  #call, cudaGetErrorString(e_));                                              \
  } while (0)

bool verbose() { return getenv("OIC_VERBOSE") != nullptr; }

uint32_t read_err(oic_ctx *ctx) {
  uint32_t e = 0;
  cudaMemcpyAsync(&e, ctr32(ctx) + cErr, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->st);
  cudaStreamSynchronize(ctx->st);
  return e;
}

struct SeedConfig {
  int warps;
  SeedCaps caps;
};

// Seed configurations, tried in this order for a ref strand: pair table and node
// pool in HBM scratch on four warps per SM slot; in large HBM scratch on one warp per SM.
SeedConfig seed_normal(const oic_ctx *c) {
  SeedConfig s;
  s.warps           = c->nSM * 8 * 4;
  s.caps.slotCap = 4096;
  s.caps.pairCap = 2048;
  s.caps.nodeCap = 32768;
  return s;
}
SeedConfig seed_wide(const oic_ctx *c) {
  SeedConfig s;
  s.warps        = c->nSM;
  s.caps.slotCap = 1 << 17;
  s.caps.pairCap = 1 << 16;
  s.caps.nodeCap = 1 << 22;
  return s;
}

int ensure_seed_scratch(oic_ctx *ctx, const SeedConfig &sc, bool wide, SeedScratch &out) {
  DevBuf &k = wide ? ctx->dSeedSlotK2 : ctx->dSeedSlotK;
  DevBuf &v = wide ? ctx->dSeedSlotV2 : ctx->dSeedSlotV;
  DevBuf &p = wide ? ctx->dSeedPairs2 : ctx->dSeedPairs;
  DevBuf &n = wide ? ctx->dSeedNodes2 : ctx->dSeedNodes;
  const size_t W = (size_t)((sc.warps + 3) / 4 * 4);
  CK(k.ensure(W * sc.caps.slotCap * sizeof(int)));
  CK(v.ensure(W * sc.caps.slotCap * sizeof(int)));
  CK(p.ensure(W * sc.caps.pairCap * sizeof(PairAcc)));
  CK(n.ensure(W * sc.caps.nodeCap * sizeof(int4)));
  out.slotKey = k.as<int>();
  out.slotVal = v.as<int>();
  out.pairs   = p.as<PairAcc>();
  out.nodes   = n.as<int4>();
  return OIC_OK;
}

struct AlignConfig {
  int bandW;
  int warps;
  AlignCaps caps;
};

AlignConfig align_normal(const oic_ctx *c) {
  AlignConfig a;
  a.bandW         = 512;
  a.warps         = c->nSM * OIC_ALIGN_MIN_BLOCKS * align_warps_per_block(512);
  a.caps.arenaCap = 1 << 20;
  a.caps.rowCap   = 1 << 14;
  a.caps.nodeCap  = 1 << 16;
  a.caps.bandW    = 512;
  a.caps.rowsGW   = 16384;
  return a;
}
int ensure_align_scratch(oic_ctx *ctx, const AlignConfig &ac, bool wide, WarpScratch &s) {
  const size_t W = (size_t)ac.warps;
  DevBuf &ar = wide ? ctx->dArena2 : ctx->dArena;
  DevBuf &rh = wide ? ctx->dRowHdr2 : ctx->dRowHdr;
  DevBuf &rg = wide ? ctx->dRowsG2 : ctx->dRowsG;
  DevBuf &dl = wide ? ctx->dDL2 : ctx->dDL;
  DevBuf &dr = wide ? ctx->dDR2 : ctx->dDR;
  DevBuf &sk = wide ? ctx->dStack2 : ctx->dStack;
  DevBuf &al = wide ? ctx->dAlive2 : ctx->dAlive;
  CK(ar.ensure(W * ac.caps.arenaCap * sizeof(int)));
  CK(rh.ensure(W * ac.caps.rowCap * sizeof(int4)));
  CK(rg.ensure(W * 2 * (size_t)ac.caps.rowsGW * sizeof(int)));
  CK(dl.ensure(W * (ac.caps.rowCap + 8) * sizeof(int)));
  CK(dr.ensure(W * (ac.caps.rowCap + 8) * sizeof(int)));
  CK(sk.ensure(W * (ac.caps.rowCap + 8) * sizeof(int)));
  CK(al.ensure(W * ac.caps.nodeCap));
  s.arena  = ar.as<int>();
  s.rowHdr = rh.as<int4>();
  s.rowsG  = rg.as<int>();
  s.deltaL = dl.as<int>();
  s.deltaR = dr.as<int>();
  s.stack  = sk.as<int>();
  s.alive  = al.as<unsigned char>();
  return OIC_OK;
}

int sync_check(oic_ctx *ctx, const char *where) {
  cudaError_t e = cudaStreamSynchronize(ctx->st);
  if (e != cudaSuccess) return fail(ctx, OIC_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(ctx, OIC_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
  return OIC_OK;
}

// Append the batch's candidate pairs (and their feature rows and match runs) to the
// context's collection.
int collect_batch(oic_ctx *ctx, uint32_t nPairs, uint32_t nNodes, bool filtered) {
  std::vector<PairRec>  pr(nPairs);
  std::vector<uint32_t> cnt(nPairs), cells(nPairs);
  std::vector<float>    logit(nPairs);
  std::vector<int4>     ext(nPairs);
  CK(cudaMemcpyAsync(ext.data(), ctx->dPairExt.p, (size_t)nPairs * sizeof(int4), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaMemcpyAsync(pr.data(), ctx->dPairs.p, (size_t)nPairs * sizeof(PairRec), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaMemcpyAsync(cnt.data(), ctx->dCnt.p, (size_t)nPairs * 4, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaMemcpyAsync(cells.data(), ctx->dPairCells.p, (size_t)nPairs * 4, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaMemcpyAsync(logit.data(), ctx->dLogit.p, (size_t)nPairs * 4, cudaMemcpyDeviceToHost, ctx->st));
  const size_t f0 = ctx->colFeat.size();
  ctx->colFeat.resize(f0 + (size_t)nPairs * OIC_FILTER_IN);
  CK(cudaMemcpyAsync(ctx->colFeat.data() + f0, ctx->dFeat.p, (size_t)nPairs * OIC_FILTER_IN * 2,
                     cudaMemcpyDeviceToHost, ctx->st));
  std::vector<int4> nodes;
  if (ctx->collect >= 2) {
    nodes.resize(nNodes);
    CK(cudaMemcpyAsync(nodes.data(), ctx->dNodes.p, (size_t)nNodes * sizeof(int4), cudaMemcpyDeviceToHost, ctx->st));
  }
  int rc = sync_check(ctx, "pair collection");
  if (rc) return rc;
  const size_t i0 = ctx->colInfo.size();
  ctx->colInfo.resize(i0 + nPairs);
  for (uint32_t p = 0; p < nPairs; p++) {
    oic_pair_info &q = ctx->colInfo[i0 + p];
    q.aID      = pr[p].sRead + 1;
    q.bID      = ctx->blkFirst + pr[p].tStr;
    const bool dropped = filtered && logit[p] < ctx->filterLogitThr;
    q.flags    = (pr[p].flags & 1u) | (dropped ? 2u : 0u);
    q.seeds    = (uint32_t)pr[p].diagCt;
    q.nodes    = pr[p].nodeCnt;
    q.overlaps = cnt[p];
    q.cells    = cells[p];
    q.score    = logit[p];
    q.extensions = (uint32_t)ext[p].x;
    q.firstHit   = ext[p].y;
    q.cellsFirst = (uint32_t)ext[p].z;
    q.extLimit   = (uint32_t)ext[p].w;
    if (ctx->collect >= 2)
      for (uint32_t j = 0; j < pr[p].nodeCnt; j++) {
        const int4 &nd = nodes[pr[p].nodeOff + j];
        ctx->colNodes.push_back(nd.x);
        ctx->colNodes.push_back(nd.y);
        ctx->colNodes.push_back(nd.z);
      }
  }
  return OIC_OK;
}

uint32_t resolved_tuning_ctas(const oic_ctx *c, const oic_tuning &t);

// The DP launch configuration with defaults filled in (include/oic_gpu.h).
oic_tuning resolved_tuning(const oic_ctx *c) {
  oic_tuning t = c->tune;
  if (!t.narrowArena) t.narrowArena = 1u << 20;
  if (!t.wideMinLen) t.wideMinLen = 0xffffffffu;
  if (t.forceWide) t.wideMinLen = 0;
  if (!t.wideThreads) t.wideThreads = 256;
  if (!t.wideTile) t.wideTile = 1;
  if (!t.wideBandW) t.wideBandW = 12288;
  if (!t.wideCtas) t.wideCtas = resolved_tuning_ctas(c, t);
  if (!t.wideMode) t.wideMode = 2;
  return t;
}

// The CTA bin's scratch: `ctas` CTAs, each with an arena of `arena` kept cells (0: a
// share of the free memory).  `huge` is the last-resort rerun: 8 CTAs splitting most of
// the free memory, HBM rows up to 2^20 diagonals.
int ensure_group_scratch(oic_ctx *ctx, const oic_tuning &t, bool huge, uint32_t &ctas, AlignCaps &caps,
                         WarpScratch &ws) {
  caps.rowCap  = 1 << 18;
  caps.nodeCap = 1 << 22;
  caps.bandW   = (int)t.wideBandW;
  caps.rowsGW  = huge ? 1 << 20 : 1 << 18;
  ctas         = huge ? 8u : t.wideCtas;
  size_t freeB = 0, totalB = 0;
  cudaMemGetInfo(&freeB, &totalB);
  freeB += ctx->dArena2.cap;   // released before the arena is reallocated
  const size_t fixedPer = (size_t)caps.rowCap * (16 + 12) + (size_t)caps.rowsGW * 8 + caps.nodeCap + 64;
  uint64_t cells = huge ? 0 : t.wideArena;
  if (!cells) {
    const double share = huge ? 0.7 : 0.4;
    double per = share * (double)freeB / ctas - (double)fixedPer;
    cells      = per > 0 ? (uint64_t)(per / sizeof(int)) : 0;
    cells      = std::min<uint64_t>(cells, huge ? 0x7fff0000ull : (1ull << 24));
  }
  if (cells < (1u << 20)) return fail(ctx, OIC_ERR_NOMEM, "not enough device memory for the CTA-bin DP arena");
  caps.arenaCap = (int)std::min<uint64_t>(cells, 0x7fff0000ull);
  AlignConfig ac;
  ac.bandW = caps.bandW;
  ac.warps = (int)ctas;
  ac.caps  = caps;
  if (ctx->dArena2.cap < (size_t)ctas * caps.arenaCap * sizeof(int)) ctx->dArena2.release();
  return ensure_align_scratch(ctx, ac, true, ws);
}

// The speculative CTA bin's scratch: 2 CTAs per SM (wideCtas when set) of
// align_spec_warps() warps, each warp with the one-warp DP's scratch (512-int shared
// rows, HBM rows up to 16384 diagonals, 32767 error rows) and an arena of the CTA's
// wideArena cells (default: 40 % of the free memory, at most 2^27 cells per CTA) split
// between its warps -- the heavy extensions of long high-error pairs keep millions of
// cells each.
int ensure_spec_scratch(oic_ctx *ctx, const oic_tuning &t, uint32_t &ctas, AlignCaps &caps, WarpScratch &ws) {
  const int sw = align_spec_warps();
  caps.rowCap  = 1 << 15;
  caps.nodeCap = (1 << 22) / sw;   // a pair's alive flags take its CTA's warps' slots
  caps.bandW   = 512;
  caps.rowsGW  = 1 << 14;
  ctas         = ctx->tune.wideCtas ? ctx->tune.wideCtas : (uint32_t)(2 * ctx->nSM);
  size_t freeB = 0, totalB = 0;
  cudaMemGetInfo(&freeB, &totalB);
  freeB += ctx->dArena2.cap;
  const size_t fixedPer = (size_t)sw * ((size_t)caps.rowCap * (16 + 12) + (size_t)caps.rowsGW * 8 + caps.nodeCap + 64);
  uint64_t cells = t.wideArena;
  if (!cells) {
    double per = 0.4 * (double)freeB / ctas - (double)fixedPer;
    cells      = per > 0 ? (uint64_t)(per / sizeof(int)) : 0;
    cells      = std::min<uint64_t>(cells, 1ull << 27);
  }
  if (cells < (uint64_t)sw << 17) return fail(ctx, OIC_ERR_NOMEM, "not enough device memory for the CTA-bin DP arena");
  caps.arenaCap = (int)std::min<uint64_t>(cells / sw, 0x7fff0000ull);
  AlignConfig ac;
  ac.bandW = caps.bandW;
  ac.warps = (int)ctas * sw;
  ac.caps  = caps;
  if (ctx->dArena2.cap < (size_t)ac.warps * caps.arenaCap * sizeof(int)) ctx->dArena2.release();
  return ensure_align_scratch(ctx, ac, true, ws);
}

// The CTA bin of a batch (its first level; the large-arena rerun is always CTA-wide).
struct CtaBin {
  bool        spec;
  uint32_t    ctas;
  AlignCaps   caps;
  WarpScratch ws;
};

int ensure_cta_bin(oic_ctx *ctx, const oic_tuning &t, CtaBin &b) {
  b.spec = t.wideMode != 2;
  return b.spec ? ensure_spec_scratch(ctx, t, b.ctas, b.caps, b.ws)
                : ensure_group_scratch(ctx, t, false, b.ctas, b.caps, b.ws);
}

void launch_cta_bin(oic_ctx *ctx, const oic_tuning &t, const CtaBin &b, uint32_t ctas, const uint32_t *work,
                    uint32_t nWork, const AlignOut &ao, cudaStream_t s) {
  if (b.spec)
    launch_align_spec((int)ctas, ctx->R, ctx->T, ctx->dp, ctx->dEml.as<int>(), ctx->dPairs.as<PairRec>(), work, nWork,
                      ctr32(ctx) + cWorkCounter, ctx->dNodes.as<int4>(), b.ws, b.caps, ao, s);
  else
    launch_align_group((int)t.wideThreads, (int)t.wideTile, b.caps.bandW, (int)ctas, ctx->R, ctx->T, ctx->dp,
                       ctx->dEml.as<int>(), ctx->dPairs.as<PairRec>(), work, nWork, ctr32(ctx) + cWorkCounter,
                       ctx->dNodes.as<int4>(), b.ws, b.caps, ao, s);
}

// Seed stage of a batch: the ref reads' seeds replayed into candidate pairs and match
// runs (dPairs, dNodes), then their filter scores when a filter is set or pairs are
// collected.  Returns OIC_OK, kRetrySmaller when the batch's output did not fit.
// Two CUDA events destroyed with the object, so that every return (the error returns
// included) releases them.  ok() is false when either could not be created.
struct EventPair {
  cudaEvent_t a = nullptr, b = nullptr;
  EventPair() {
    if (cudaEventCreate(&a) != cudaSuccess) a = nullptr;
    if (cudaEventCreate(&b) != cudaSuccess) b = nullptr;
  }
  ~EventPair() {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
  }
  bool ok() const { return a && b; }
  EventPair(const EventPair &)            = delete;
  EventPair &operator=(const EventPair &) = delete;
};

// A named range on the NVTX timeline for the life of the object: the library's stages
// by name in Nsight Systems / Nsight Compute; nothing is recorded without such a tool.
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &)            = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

int seed_stage(oic_ctx *ctx, const uint32_t *refs, uint32_t nRefs, cudaEvent_t evSeed0, cudaEvent_t evSeed1,
               uint32_t &nPairs, uint32_t &nNodes) {
  NvtxRange range("oic seed stage");
  const uint32_t nSeg = nRefs * 2;
  CK(ctx->dSegReads.ensure((size_t)nRefs * sizeof(uint32_t)));
  CK(cudaMemcpyAsync(ctx->dSegReads.p, refs, (size_t)nRefs * sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->st));
  CK(cudaMemsetAsync(ctx->dCtr.p, 0, 64 * sizeof(uint32_t) + 0, ctx->st));
  CK(cudaMemsetAsync(ctr64(ctx) + kSeedStatBase, 0, 2 * sizeof(unsigned long long), ctx->st));
  CK(ctx->dSegOvf.ensure((size_t)nSeg * sizeof(uint32_t)));

  SeedOut so;
  so.pairs         = ctx->dPairs.as<PairRec>();
  so.pairCap       = ctx->pairCap;
  so.pairCount     = ctr32(ctx) + cPairCount;
  so.nodes         = ctx->dNodes.as<int4>();
  so.nodeCap       = ctx->nodeCap;
  so.nodeCount     = ctr32(ctx) + cNodeCount;
  so.overflowSegs  = ctx->dSegOvf.as<uint32_t>();
  so.overflowCount = ctr32(ctx) + cSegOvf;
  so.stats         = ctr64(ctx) + kSeedStatBase;
  so.err           = ctr32(ctx) + cErr;

  CK(cudaEventRecord(evSeed0, ctx->st));
  // Strands whose pair table or node pool overflowed run again in the wide
  // configuration, their ids being the work list of that pass.
  const SeedConfig tiers[2] = {seed_normal(ctx), seed_wide(ctx)};
  uint32_t h[16];
  int      rc    = OIC_OK;
  uint32_t nTodo = nSeg;
  for (int t = 0; t < 2; t++) {
    SeedScratch ss;
    if ((rc = ensure_seed_scratch(ctx, tiers[t], t == 1, ss))) return rc;
    if (t > 0) {
      if (verbose()) fprintf(stderr, "oic: %u ref strands rerun in seed configuration %d\n", nTodo, t);
      CK(ctx->dSegList.ensure((size_t)nTodo * sizeof(uint32_t)));
      CK(cudaMemcpyAsync(ctx->dSegList.p, ctx->dSegOvf.p, nTodo * sizeof(uint32_t), cudaMemcpyDeviceToDevice,
                         ctx->st));
      CK(cudaMemsetAsync(ctr32(ctx) + cSegCounter, 0, sizeof(uint32_t), ctx->st));
      CK(cudaMemsetAsync(ctr32(ctx) + cSegOvf, 0, sizeof(uint32_t), ctx->st));
    }
    launch_seed(ctx->R, ctx->T, ctx->dp, ctx->dSegReads.as<uint32_t>(), t ? ctx->dSegList.as<uint32_t>() : nullptr,
                nTodo, ctr32(ctx) + cSegCounter, ss, tiers[t].caps, tiers[t].warps, so, ctx->st);
    CK(cudaMemcpyAsync(h, ctx->dCtr.p, 16 * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->st));
    if ((rc = sync_check(ctx, "seed kernel"))) return rc;
    if (h[cErr] & (kErrOutNodes | kErrOutPairs)) {
      // Every segment reserved its output with one atomic add, so the counters hold the
      // batch's whole demand.
      ctx->overPairs = h[cPairCount];
      ctx->overNodes = h[cNodeCount];
      return kRetrySmaller;
    }
    if (h[cSegOvf] == 0) break;
    if (t == 1)
      return fail(ctx, OIC_ERR_OVERFLOW, "a ref read has more candidate pairs or match nodes than the engine holds");
    nTodo = h[cSegOvf];
  }
  CK(cudaEventRecord(evSeed1, ctx->st));
  nPairs = h[cPairCount];
  nNodes = h[cNodeCount];

  // Learned filter: feature rows of every candidate pair, then their scores.
  const bool useFilter = ctx->filterOn && nPairs > 0;
  if ((useFilter || ctx->collect) && nPairs) {
    if (!ctx->evF0) {
      CK(cudaEventCreate(&ctx->evF0));
      CK(cudaEventCreate(&ctx->evF1));
    }
    CK(cudaEventRecord(ctx->evF0, ctx->st));
    CK(ctx->dFeat.ensure((size_t)nPairs * OIC_FILTER_IN * 2));
    launch_pair_features(ctx->dPairs.as<PairRec>(), nPairs, ctx->dNodes.as<int4>(), ctx->R.len, ctx->T.sread,
                         ctx->dp.kmerLen, ctx->dFeat.p, ctx->st);
    // Capacity-sized, so the captured align stage's pointer to the scores stays valid.
    CK(ctx->dLogit.ensure((size_t)std::max(nPairs, ctx->pairCap) * sizeof(float)));
    if (useFilter)
      CK(launch_mlp_forward(ctx->dFilterPrm.p, ctx->dFeat.p, nPairs, ctx->dLogit.as<float>(), nullptr, nullptr,
                            ctx->st));
    else
      CK(cudaMemsetAsync(ctx->dLogit.p, 0, (size_t)nPairs * sizeof(float), ctx->st));
    CK(cudaEventRecord(ctx->evF1, ctx->st));
  }
  return OIC_OK;
}

// Per-bin figures of one align stage.
struct AlignTimes {
  float    msNarrow = 0, msWide = 0;
  uint64_t pairsNarrow = 0, pairsWide = 0, cellsWide = 0;
};

// Align stage of a batch: work list by bin, the one-warp bin, the CTA bin (its own
// pairs plus the one-warp overflow), the large-arena rerun, then the records compacted
// into `recOut` (appended) and the counters into ctx->stats.
int align_stage(oic_ctx *ctx, uint32_t nPairs, uint32_t nNodes, const oic_tuning &tn, cudaEvent_t evAln0,
                cudaEvent_t evAln1, std::vector<uint32_t> &recOut, AlignTimes &at) {
  NvtxRange range("oic DP stage");
  int rc = OIC_OK;
  const bool useFilter = ctx->filterOn && nPairs > 0;
  CK(cudaMemsetAsync(ctr32(ctx) + cWorkCounter, 0, 4 * sizeof(uint32_t), ctx->st));   // work, aln ovf, err, rec total
  CK(cudaMemsetAsync(ctr32(ctx) + cKeep, 0, 2 * sizeof(uint32_t), ctx->st));
  CK(cudaMemsetAsync(ctr64(ctx) + kAlignStatBase, 0, kStCount * sizeof(unsigned long long), ctx->st));
  CK(cudaEventRecord(evAln0, ctx->st));
  const size_t np1 = std::max<uint32_t>(nPairs, 1);
  CK(ctx->dWork.ensure(np1 * 2 * sizeof(uint32_t)));
  CK(ctx->dCnt.ensure(np1 * sizeof(uint32_t)));
  CK(ctx->dRecPos.ensure(np1 * sizeof(uint32_t)));
  CK(ctx->dRec.ensure(np1 * 18 * sizeof(uint32_t)));
  CK(ctx->dAlnOvf.ensure(np1 * sizeof(uint32_t)));
  uint32_t nNarrow = 0, nWide = 0;
  if (nPairs) {
    CK(ctx->dWorkK.ensure((size_t)nPairs * 8));
    CK(ctx->dWorkK2.ensure((size_t)nPairs * 8));
    CK(ctx->dWorkV2.ensure((size_t)nPairs * 4));
    CK(ctx->dWorkScratch.ensure(radix_sort_scratch(nPairs) + 256));
    launch_work_keys(ctx->dPairs.as<PairRec>(), nPairs, useFilter ? ctx->dLogit.as<float>() : nullptr,
                     ctx->filterLogitThr, ctx->R.len, ctx->T.sread, tn.wideMinLen, ctr32(ctx) + cKeep,
                     ctx->dWorkK.as<u64>(), ctx->dWork.as<uint32_t>(), ctx->st);
    CK(radix_sort_u64_u32(ctx->dWorkK.as<u64>(), ctx->dWork.as<uint32_t>(), ctx->dWorkK2.as<u64>(),
                          ctx->dWorkV2.as<uint32_t>(), nPairs, 32, ctx->dWorkScratch.p, ctx->st));
    CK(cudaMemsetAsync(ctx->dCnt.p, 0, nPairs * sizeof(uint32_t), ctx->st));
    uint32_t bc[2];
    CK(cudaMemcpyAsync(bc, ctr32(ctx) + cKeep, sizeof(bc), cudaMemcpyDeviceToHost, ctx->st));
    if ((rc = sync_check(ctx, "work list"))) return rc;
    nNarrow = bc[0];
    nWide   = bc[1];
  }
  if (ctx->collect && nPairs) {
    CK(ctx->dPairCells.ensure((size_t)nPairs * sizeof(uint32_t)));
    CK(ctx->dPairExt.ensure((size_t)nPairs * sizeof(int4)));
    CK(cudaMemsetAsync(ctx->dPairCells.p, 0, (size_t)nPairs * sizeof(uint32_t), ctx->st));
    CK(cudaMemsetAsync(ctx->dPairExt.p, 0, (size_t)nPairs * sizeof(int4), ctx->st));
  }
  AlignOut ao;
  ao.rec           = ctx->dRec.as<uint32_t>();
  ao.cnt           = ctx->dCnt.as<uint32_t>();
  ao.overflow      = ctx->dAlnOvf.as<uint32_t>();
  ao.overflowCount = ctr32(ctx) + cAlnOvf;
  ao.stats         = ctr64(ctx) + kAlignStatBase;
  ao.err           = ctr32(ctx) + cErr;
  ao.cells         = (ctx->collect && nPairs) ? ctx->dPairCells.as<uint32_t>() : nullptr;
  ao.ext           = (ctx->collect && nPairs) ? ctx->dPairExt.as<int4>() : nullptr;
  const bool tier  = useFilter && ctx->filterTierThr > ctx->filterLogitThr;
  ao.tierLogit     = tier ? ctx->dLogit.as<float>() : nullptr;
  ao.tierThr       = ctx->filterTierThr;
  ao.tierBudget    = ctx->filterBudget;
  ao.nWorkDev      = nullptr;
  ao.workOffDev    = nullptr;

  cudaEvent_t ev[4];
  for (auto &x : ev) CK(cudaEventCreate(&x));
  struct EvGuard {
    cudaEvent_t *e;
    ~EvGuard() {
      for (int i = 0; i < 4; i++) cudaEventDestroy(e[i]);
    }
  } guard{ev};

  // One-warp bin.
  uint32_t h[16];
  uint32_t nOvf = 0;
  unsigned long long cellsAfterNarrow = 0;
  CK(cudaEventRecord(ev[0], ctx->st));
  if (nNarrow) {
    AlignConfig an = align_normal(ctx);
    an.caps.arenaCap = (int)tn.narrowArena;
    WarpScratch ws;
    if ((rc = ensure_align_scratch(ctx, an, false, ws))) return rc;
    launch_align(an.bandW, ctx->R, ctx->T, ctx->dp, ctx->dEml.as<int>(), ctx->dPairs.as<PairRec>(),
                 ctx->dWork.as<uint32_t>(), nNarrow, ctr32(ctx) + cWorkCounter, ctx->dNodes.as<int4>(), ws, an.caps,
                 an.warps, ao, ctx->st);
    CK(cudaMemcpyAsync(h, ctx->dCtr.p, 16 * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(&cellsAfterNarrow, ctr64(ctx) + kAlignStatBase + kStCells, 8, cudaMemcpyDeviceToHost,
                       ctx->st));
    if ((rc = sync_check(ctx, "align kernel"))) return rc;
    nOvf = h[cAlnOvf];
  }
  CK(cudaEventRecord(ev[1], ctx->st));
  at.pairsNarrow += nNarrow;

  // CTA bin: its own pairs (after the one-warp bin in the sorted list) and the
  // one-warp overflow appended behind them.
  uint32_t nW = nWide + nOvf;
  if (nW) {
    if (nOvf) {
      if (verbose()) fprintf(stderr, "oic: %u pairs moved from the one-warp DP to the CTA DP\n", nOvf);
      CK(cudaMemcpyAsync(ctx->dWork.as<uint32_t>() + nNarrow + nWide, ctx->dAlnOvf.p, nOvf * sizeof(uint32_t),
                         cudaMemcpyDeviceToDevice, ctx->st));
      // The moved pairs arrive in completion order: sort the whole CTA-bin list so the
      // pairs with the most match nodes (the longest chains of extensions) start first.
      uint32_t *lst = ctx->dWork.as<uint32_t>() + nNarrow;
      launch_list_keys(ctx->dPairs.as<PairRec>(), lst, nW, ctx->dWorkK.as<u64>(), ctx->dWorkV2.as<uint32_t>(),
                       ctx->st);
      CK(cudaMemcpyAsync(lst, ctx->dWorkV2.p, (size_t)nW * sizeof(uint32_t), cudaMemcpyDeviceToDevice, ctx->st));
      CK(radix_sort_u64_u32(ctx->dWorkK.as<u64>(), lst, ctx->dWorkK2.as<u64>(), ctx->dWorkV2.as<uint32_t>(), nW, 32,
                            ctx->dWorkScratch.p, ctx->st));
    }
    for (int level = 0; level < 2 && nW; level++) {
      const bool huge = level == 1;
      CK(cudaMemsetAsync(ctr32(ctx) + cWorkCounter, 0, sizeof(uint32_t), ctx->st));
      CK(cudaMemsetAsync(ctr32(ctx) + cAlnOvf, 0, sizeof(uint32_t), ctx->st));
      CK(cudaMemsetAsync(ctr32(ctx) + cErr, 0, sizeof(uint32_t), ctx->st));
      if (!huge) {
        CtaBin b;
        if ((rc = ensure_cta_bin(ctx, tn, b))) return rc;
        launch_cta_bin(ctx, tn, b, std::min<uint32_t>(b.ctas, nW), ctx->dWork.as<uint32_t>() + nNarrow, nW, ao,
                       ctx->st);
      } else {
        uint32_t    ctas = 0;
        AlignCaps   caps;
        WarpScratch ws;
        if ((rc = ensure_group_scratch(ctx, tn, true, ctas, caps, ws))) return rc;
        launch_align_group((int)std::max<uint32_t>(tn.wideThreads, 512), (int)tn.wideTile, caps.bandW,
                           (int)std::min<uint32_t>(ctas, nW), ctx->R, ctx->T, ctx->dp, ctx->dEml.as<int>(),
                           ctx->dPairs.as<PairRec>(), ctx->dWork.as<uint32_t>() + nNarrow, nW,
                           ctr32(ctx) + cWorkCounter, ctx->dNodes.as<int4>(), ws, caps, ao, ctx->st);
      }
      CK(cudaMemcpyAsync(h, ctx->dCtr.p, 16 * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->st));
      if ((rc = sync_check(ctx, huge ? "align kernel (large arena)" : "align kernel (CTA bin)"))) return rc;
      at.pairsWide += nW;
      const uint32_t o = h[cAlnOvf];
      if (o && huge)
        return fail(ctx, OIC_ERR_OVERFLOW,
                    "a read pair needs a wider DP band or deeper traceback than the engine holds (err 0x%x)", h[cErr]);
      if (o) {
        if (verbose()) fprintf(stderr, "oic: %u pairs rerun with the large DP arena\n", o);
        CK(cudaMemcpyAsync(ctx->dWork.as<uint32_t>() + nNarrow, ctx->dAlnOvf.p, o * sizeof(uint32_t),
                           cudaMemcpyDeviceToDevice, ctx->st));
      }
      nW = o;
    }
  }
  CK(cudaEventRecord(ev[2], ctx->st));
  CK(cudaEventRecord(evAln1, ctx->st));

  // Compact the records and bring them home.
  CK(ctx->dScanScratch.ensure(scan_u32_scratch(nPairs) + 256));
  CK(scan_u32(ctx->dCnt.as<uint32_t>(), ctx->dRecPos.as<uint32_t>(), nPairs, ctr32(ctx) + cRecTotal,
              ctx->dScanScratch.p, ctx->st));
  uint32_t nRec = 0;
  CK(cudaMemcpyAsync(&nRec, ctr32(ctx) + cRecTotal, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  if (nRec) {
    CK(ctx->dRecOut.ensure((size_t)nRec * 6 * sizeof(uint32_t)));
    launch_compact_records(ctx->dRec.as<uint32_t>(), ctx->dCnt.as<uint32_t>(), ctx->dRecPos.as<uint32_t>(), nPairs,
                           ctx->dRecOut.as<uint32_t>(), ctx->st);
    size_t old = recOut.size();
    recOut.resize(old + (size_t)nRec * 6);
    CK(cudaMemcpyAsync(recOut.data() + old, ctx->dRecOut.p, (size_t)nRec * 6 * sizeof(uint32_t),
                       cudaMemcpyDeviceToHost, ctx->st));
  }
  unsigned long long st64[2 + kStCount];
  CK(cudaMemcpyAsync(st64, ctr64(ctx) + kSeedStatBase, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaMemcpyAsync(st64 + 2, ctr64(ctx) + kAlignStatBase, kStCount * sizeof(unsigned long long),
                     cudaMemcpyDeviceToHost, ctx->st));
  if ((rc = sync_check(ctx, "record compaction"))) return rc;
  float a0 = 0, a1 = 0;
  cudaEventElapsedTime(&a0, ev[0], ev[1]);
  cudaEventElapsedTime(&a1, ev[1], ev[2]);
  at.msNarrow += a0;
  at.msWide += a1;
  at.cellsWide += st64[2 + kStCells] - cellsAfterNarrow;

  oic_stats &S = ctx->stats;
  S.seeds += st64[0];
  S.candidatePairs += nPairs;
  S.nodes += nNodes;
  S.kmerHitsWithoutOlap += st64[2 + kStWithoutOlap];
  S.kmerHitsWithOlap += st64[2 + kStWithOlap];
  S.kmerHitsSkipped += st64[2 + kStSkipped];
  S.multiOverlap += st64[2 + kStMulti];
  S.totalOverlaps += st64[2 + kStTotal];
  S.containedOverlaps += st64[2 + kStContained];
  S.dovetailOverlaps += st64[2 + kStDovetail];
  S.dpCells += st64[2 + kStCells];
  S.slideBases += st64[2 + kStSlides];
  S.extensions += st64[2 + kStExtensions];
  S.dpRows += st64[2 + kStRows];
  S.dpCellsNoOverlap += st64[2 + kStCellsNoOlap];
  if (useFilter) S.filteredPairs += nPairs - nNarrow - nWide;
  return OIC_OK;
}

template <typename T> void key_add(std::vector<uint8_t> &k, const T &v) {
  const uint8_t *b = (const uint8_t *)&v;
  k.insert(k.end(), b, b + sizeof(T));
}

// The align stage as one captured CUDA graph per context: work keys, the radix sort,
// the one-warp bin, the overflow hand-over, the CTA bin, the record scan and
// compaction, all sized for the batch capacity (pairCap) and reading the batch's pair
// count and bin sizes on the device.  It is captured once and relaunched for every
// batch; a new capture happens only when a baked-in parameter changes (a buffer was
// reallocated, the tuning or the filter changed).  The host reads the counters once
// after the launch; the rare large-arena rerun runs outside the graph.
int align_stage_graph(oic_ctx *ctx, uint32_t nPairs, uint32_t nNodes, const oic_tuning &tn, cudaEvent_t evAln0,
                      cudaEvent_t evAln1, std::vector<uint32_t> &recOut, AlignTimes &at) {
  NvtxRange range("oic DP stage (graph)");
  int rc = OIC_OK;
  const bool     useFilter = ctx->filterOn && nPairs > 0;
  const bool     coll      = ctx->collect != 0;
  const uint32_t cap       = ctx->pairCap;
  CK(ctx->dWork.ensure((size_t)cap * 2 * sizeof(uint32_t)));
  CK(ctx->dCnt.ensure((size_t)cap * sizeof(uint32_t)));
  CK(ctx->dRecPos.ensure((size_t)cap * sizeof(uint32_t)));
  CK(ctx->dRec.ensure((size_t)cap * 18 * sizeof(uint32_t)));
  CK(ctx->dRecOut.ensure((size_t)cap * 18 * sizeof(uint32_t)));
  CK(ctx->dAlnOvf.ensure((size_t)cap * sizeof(uint32_t)));
  CK(ctx->dWorkK.ensure((size_t)cap * 8));
  CK(ctx->dWorkK2.ensure((size_t)cap * 8));
  CK(ctx->dWorkV2.ensure((size_t)cap * 4));
  CK(ctx->dWorkScratch.ensure(radix_sort_scratch(cap) + 256));
  CK(ctx->dScanScratch.ensure(scan_u32_scratch(cap) + 256));
  if (useFilter) CK(ctx->dLogit.ensure((size_t)cap * sizeof(float)));
  if (coll) {
    CK(ctx->dPairCells.ensure((size_t)cap * sizeof(uint32_t)));
    CK(ctx->dPairExt.ensure((size_t)cap * sizeof(int4)));
  }
  AlignConfig an = align_normal(ctx);
  an.caps.arenaCap = (int)tn.narrowArena;
  WarpScratch wsN;
  if ((rc = ensure_align_scratch(ctx, an, false, wsN))) return rc;
  CtaBin bG;
  if ((rc = ensure_cta_bin(ctx, tn, bG))) return rc;
  const uint32_t    ctas  = bG.ctas;
  const AlignCaps   capsG = bG.caps;
  const WarpScratch wsG   = bG.ws;
  for (cudaEvent_t &e : ctx->gEv)
    if (!e) CK(cudaEventCreate(&e));

  AlignOut ao{};
  ao.rec           = ctx->dRec.as<uint32_t>();
  ao.cnt           = ctx->dCnt.as<uint32_t>();
  ao.overflow      = ctx->dAlnOvf.as<uint32_t>();
  ao.overflowCount = ctr32(ctx) + cAlnOvf;
  ao.stats         = ctr64(ctx) + kAlignStatBase;
  ao.err           = ctr32(ctx) + cErr;
  ao.cells         = coll ? ctx->dPairCells.as<uint32_t>() : nullptr;
  ao.ext           = coll ? ctx->dPairExt.as<int4>() : nullptr;
  const bool tier  = useFilter && ctx->filterTierThr > ctx->filterLogitThr;
  ao.tierLogit     = tier ? ctx->dLogit.as<float>() : nullptr;
  ao.tierThr       = ctx->filterTierThr;
  ao.tierBudget    = ctx->filterBudget;
  AlignOut aoN = ao, aoW = ao;
  aoN.nWorkDev   = ctr32(ctx) + cKeep;    // one-warp bin: work[0 .. bin 0)
  aoW.nWorkDev   = ctr32(ctx) + cWideN;   // CTA bin: work[bin 0 .. bin 0 + wideN)
  aoW.workOffDev = ctr32(ctx) + cKeep;
  const float *logit = useFilter ? ctx->dLogit.as<float>() : nullptr;
  std::vector<uint8_t> key;
  key_add(key, aoN);
  key_add(key, aoW);
  key_add(key, logit);
  key_add(key, ctx->filterLogitThr);
  key_add(key, tn);
  key_add(key, cap);
  key_add(key, ctas);
  key_add(key, capsG);
  key_add(key, wsN);
  key_add(key, wsG);
  key_add(key, an);
  key_add(key, ctx->R);
  key_add(key, ctx->T);
  key_add(key, ctx->dp);
  const void *bufs[] = {ctx->dPairs.p, ctx->dNodes.p, ctx->dWork.p, ctx->dRecPos.p, ctx->dRecOut.p, ctx->dWorkK.p,
                        ctx->dWorkK2.p, ctx->dWorkV2.p, ctx->dWorkScratch.p, ctx->dScanScratch.p, ctx->dEml.p,
                        ctx->dCtr.p};
  key_add(key, bufs);

  if (!ctx->gExec || key != ctx->gKey) {
    if (ctx->gExec) {
      cudaGraphExecDestroy(ctx->gExec);
      ctx->gExec = nullptr;
    }
    const unsigned long long launches0 = g_launches;   // capture launches nothing
    CK(cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeThreadLocal));
    cudaStream_t s = ctx->st;
    cudaMemsetAsync(ctr32(ctx) + cWorkCounter, 0, 4 * sizeof(uint32_t), s);   // work, aln ovf, err, rec total
    cudaMemsetAsync(ctr32(ctx) + cKeep, 0, 3 * sizeof(uint32_t), s);          // bins, CTA-bin length
    cudaMemsetAsync(ctr64(ctx) + kAlignStatBase, 0, kStCount * sizeof(unsigned long long), s);
    launch_work_keys(ctx->dPairs.as<PairRec>(), cap, logit, ctx->filterLogitThr, ctx->R.len, ctx->T.sread,
                     tn.wideMinLen, ctr32(ctx) + cKeep, ctx->dWorkK.as<u64>(), ctx->dWork.as<uint32_t>(), s,
                     ctr32(ctx) + cPairCount);
    radix_sort_u64_u32(ctx->dWorkK.as<u64>(), ctx->dWork.as<uint32_t>(), ctx->dWorkK2.as<u64>(),
                       ctx->dWorkV2.as<uint32_t>(), cap, 32, ctx->dWorkScratch.p, s, ctr32(ctx) + cPairCount);
    cudaMemsetAsync(ctx->dCnt.p, 0, (size_t)cap * sizeof(uint32_t), s);
    if (coll) {
      cudaMemsetAsync(ctx->dPairCells.p, 0, (size_t)cap * sizeof(uint32_t), s);
      cudaMemsetAsync(ctx->dPairExt.p, 0, (size_t)cap * sizeof(int4), s);
    }
    cudaEventRecordWithFlags(ctx->gEv[0], s, cudaEventRecordExternal);   // recorded at every replay
    launch_align(an.bandW, ctx->R, ctx->T, ctx->dp, ctx->dEml.as<int>(), ctx->dPairs.as<PairRec>(),
                 ctx->dWork.as<uint32_t>(), 0, ctr32(ctx) + cWorkCounter, ctx->dNodes.as<int4>(), wsN, an.caps,
                 an.warps, aoN, s);
    cudaMemcpyAsync(ctr64(ctx) + kCellsSnap, ctr64(ctx) + kAlignStatBase + kStCells, sizeof(unsigned long long),
                    cudaMemcpyDeviceToDevice, s);
    cudaEventRecordWithFlags(ctx->gEv[1], s, cudaEventRecordExternal);   // recorded at every replay
    launch_append_overflow(ctx->dWork.as<uint32_t>(), ctr32(ctx) + cKeep, ctx->dAlnOvf.as<uint32_t>(),
                           ctr32(ctx) + cAlnOvf, ctr32(ctx) + cWideN, ctr32(ctx) + cWorkCounter, ctr32(ctx) + cErr,
                           s);
    launch_cta_bin(ctx, tn, bG, ctas, ctx->dWork.as<uint32_t>(), 0, aoW, s);
    cudaEventRecordWithFlags(ctx->gEv[2], s, cudaEventRecordExternal);   // recorded at every replay
    scan_u32(ctx->dCnt.as<uint32_t>(), ctx->dRecPos.as<uint32_t>(), cap, ctr32(ctx) + cRecTotal,
             ctx->dScanScratch.p, s);
    launch_compact_records(ctx->dRec.as<uint32_t>(), ctx->dCnt.as<uint32_t>(), ctx->dRecPos.as<uint32_t>(), cap,
                           ctx->dRecOut.as<uint32_t>(), s);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(ctx->st, &g);
    g_launches    = launches0;
    ctx->gKernels = 0;
    if (e == cudaSuccess) {
      size_t nn = 0;
      cudaGraphGetNodes(g, nullptr, &nn);
      std::vector<cudaGraphNode_t> nodes(nn);
      if (nn) cudaGraphGetNodes(g, nodes.data(), &nn);
      for (cudaGraphNode_t nd : nodes) {
        cudaGraphNodeType ty;
        if (cudaGraphNodeGetType(nd, &ty) == cudaSuccess && ty == cudaGraphNodeTypeKernel) ctx->gKernels++;
      }
      e = cudaGraphInstantiate(&ctx->gExec, g, 0);
    }
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      ctx->gExec = nullptr;
      return fail(ctx, OIC_ERR_CUDA, "align graph capture: %s", cudaGetErrorString(e));
    }
    ctx->gKey = key;
  }

  CK(cudaEventRecord(evAln0, ctx->st));
  CK(cudaGraphLaunch(ctx->gExec, ctx->st));
  g_launches += ctx->gKernels;
  uint32_t           h[16];
  unsigned long long snap = 0;
  CK(cudaMemcpyAsync(h, ctx->dCtr.p, 16 * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaMemcpyAsync(&snap, ctr64(ctx) + kCellsSnap, sizeof(snap), cudaMemcpyDeviceToHost, ctx->st));
  if ((rc = sync_check(ctx, "align graph"))) return rc;
  const uint32_t nNarrow = h[cKeep], nWide = h[cKeep2], nW = h[cWideN];
  at.pairsNarrow += nNarrow;
  at.pairsWide += nW;
  float a0 = 0, a1 = 0;
  if (cudaEventElapsedTime(&a0, ctx->gEv[0], ctx->gEv[1]) != cudaSuccess ||
      cudaEventElapsedTime(&a1, ctx->gEv[1], ctx->gEv[2]) != cudaSuccess) {
    a0 = a1 = 0;
    cudaGetLastError();
  }
  at.msNarrow += a0;
  at.msWide += a1;
  uint32_t nRec = h[cRecTotal];
  if (h[cAlnOvf]) {
    // CTA-bin pairs over the CTA arena: the large-arena rerun, then the records again.
    const uint32_t o = h[cAlnOvf];
    if (verbose()) fprintf(stderr, "oic: %u pairs rerun with the large DP arena\n", o);
    CK(cudaMemcpyAsync(ctx->dWork.as<uint32_t>(), ctx->dAlnOvf.p, o * sizeof(uint32_t), cudaMemcpyDeviceToDevice,
                       ctx->st));
    CK(cudaMemsetAsync(ctr32(ctx) + cWorkCounter, 0, sizeof(uint32_t), ctx->st));
    CK(cudaMemsetAsync(ctr32(ctx) + cAlnOvf, 0, sizeof(uint32_t), ctx->st));
    CK(cudaMemsetAsync(ctr32(ctx) + cErr, 0, sizeof(uint32_t), ctx->st));
    uint32_t    ctasH = 0;
    AlignCaps   capsH;
    WarpScratch wsH;
    if ((rc = ensure_group_scratch(ctx, tn, true, ctasH, capsH, wsH))) return rc;
    EventPair hev;
    if (!hev.ok()) return fail(ctx, OIC_ERR_CUDA, "cudaEventCreate failed");
    const cudaEvent_t h0 = hev.a, h1 = hev.b;
    cudaEventRecord(h0, ctx->st);
    launch_align_group((int)std::max<uint32_t>(tn.wideThreads, 512), (int)tn.wideTile, capsH.bandW,
                       (int)std::min<uint32_t>(ctasH, o), ctx->R, ctx->T, ctx->dp, ctx->dEml.as<int>(),
                       ctx->dPairs.as<PairRec>(), ctx->dWork.as<uint32_t>(), o, ctr32(ctx) + cWorkCounter,
                       ctx->dNodes.as<int4>(), wsH, capsH, ao, ctx->st);
    cudaEventRecord(h1, ctx->st);
    CK(scan_u32(ctx->dCnt.as<uint32_t>(), ctx->dRecPos.as<uint32_t>(), cap, ctr32(ctx) + cRecTotal,
                ctx->dScanScratch.p, ctx->st));
    launch_compact_records(ctx->dRec.as<uint32_t>(), ctx->dCnt.as<uint32_t>(), ctx->dRecPos.as<uint32_t>(), cap,
                           ctx->dRecOut.as<uint32_t>(), ctx->st);
    CK(cudaMemcpyAsync(h, ctx->dCtr.p, 16 * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->st));
    rc = sync_check(ctx, "align kernel (large arena)");
    float hm = 0;
    cudaEventElapsedTime(&hm, h0, h1);
    if (rc) return rc;
    at.msWide += hm;
    at.pairsWide += o;
    if (h[cAlnOvf])
      return fail(ctx, OIC_ERR_OVERFLOW,
                  "a read pair needs a wider DP band or deeper traceback than the engine holds (err 0x%x)", h[cErr]);
    nRec = h[cRecTotal];
  }
  CK(cudaEventRecord(evAln1, ctx->st));
  if (nRec) {
    size_t old = recOut.size();
    recOut.resize(old + (size_t)nRec * 6);
    CK(cudaMemcpyAsync(recOut.data() + old, ctx->dRecOut.p, (size_t)nRec * 6 * sizeof(uint32_t),
                       cudaMemcpyDeviceToHost, ctx->st));
  }
  unsigned long long st64[2 + kStCount];
  CK(cudaMemcpyAsync(st64, ctr64(ctx) + kSeedStatBase, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaMemcpyAsync(st64 + 2, ctr64(ctx) + kAlignStatBase, kStCount * sizeof(unsigned long long),
                     cudaMemcpyDeviceToHost, ctx->st));
  if ((rc = sync_check(ctx, "record download"))) return rc;
  at.cellsWide += st64[2 + kStCells] - snap;

  oic_stats &S = ctx->stats;
  S.seeds += st64[0];
  S.candidatePairs += nPairs;
  S.nodes += nNodes;
  S.kmerHitsWithoutOlap += st64[2 + kStWithoutOlap];
  S.kmerHitsWithOlap += st64[2 + kStWithOlap];
  S.kmerHitsSkipped += st64[2 + kStSkipped];
  S.multiOverlap += st64[2 + kStMulti];
  S.totalOverlaps += st64[2 + kStTotal];
  S.containedOverlaps += st64[2 + kStContained];
  S.dovetailOverlaps += st64[2 + kStDovetail];
  S.dpCells += st64[2 + kStCells];
  S.slideBases += st64[2 + kStSlides];
  S.extensions += st64[2 + kStExtensions];
  S.dpRows += st64[2 + kStRows];
  S.dpCellsNoOverlap += st64[2 + kStCellsNoOlap];
  if (useFilter) S.filteredPairs += nPairs - nNarrow - nWide;
  S.graphLaunches++;
  return OIC_OK;
}

// Process one batch of eligible ref reads against the loaded block.  Returns OIC_OK,
// or kRetrySmaller when the batch's output did not fit (caller splits the batch).
int run_batch(oic_ctx *ctx, const uint32_t *refs, uint32_t nRefs, cudaEvent_t evSeed0, cudaEvent_t evSeed1,
              cudaEvent_t evAln1, float &msSeed, float &msAlign) {
  uint32_t nPairs = 0, nNodes = 0;
  int rc = seed_stage(ctx, refs, nRefs, evSeed0, evSeed1, nPairs, nNodes);
  if (rc) return rc;
  const bool useFilter = ctx->filterOn && nPairs > 0;
  const oic_tuning tn = resolved_tuning(ctx);
  AlignTimes at;
  rc = tn.noGraph || nPairs == 0 ? align_stage(ctx, nPairs, nNodes, tn, evSeed1, evAln1, ctx->out, at)
                                 : align_stage_graph(ctx, nPairs, nNodes, tn, evSeed1, evAln1, ctx->out, at);
  if (rc) return rc;
  float a = 0, b = 0;
  cudaEventElapsedTime(&a, evSeed0, evSeed1);
  cudaEventElapsedTime(&b, evSeed1, evAln1);
  msSeed += a;
  msAlign += b;
  oic_stats &S = ctx->stats;
  S.msNarrow += at.msNarrow;
  S.msWide += at.msWide;
  S.pairsNarrow += at.pairsNarrow;
  S.pairsWide += at.pairsWide;
  S.cellsWide += at.cellsWide;
  if ((useFilter || ctx->collect) && nPairs) {
    float f = 0;
    cudaEventElapsedTime(&f, ctx->evF0, ctx->evF1);
    S.msFilter += f;
  }
  if (ctx->collect && nPairs && (rc = collect_batch(ctx, nPairs, nNodes, useFilter))) return rc;
  return OIC_OK;
}

// 0-based indices of the ref reads of [bgnRefID, endRefID] that Process_Overlaps
// scans (Process_Overlaps.C:50-55: library range and minimum overlap length).
int eligible_refs(oic_ctx *ctx, uint32_t bgnRefID, uint32_t endRefID, std::vector<uint32_t> &refs) {
  const oic_params &P = ctx->P;
  if (bgnRefID < 1) bgnRefID = 1;
  if (endRefID > ctx->nReads) endRefID = ctx->nReads;
  for (uint64_t id = bgnRefID; id <= endRefID; id++) {
    const uint32_t r = (uint32_t)id - 1;
    if (ctx->lib[r] < P.minLibToRef || ctx->lib[r] > P.maxLibToRef) continue;
    if ((int64_t)ctx->len[r] < (int64_t)P.minOlapLen) continue;
    if (ctx->len[r] < P.kmerLen) return fail(ctx, OIC_ERR_INPUT, "read %u is shorter than the k-mer size", (uint32_t)id);
    refs.push_back(r);
  }
  return OIC_OK;
}

// Output capacities of a batch, sized once from the free memory.
int ensure_pair_caps(oic_ctx *ctx) {
  if (ctx->pairCap) return OIC_OK;
  size_t freeB = 0, totalB = 0;
  cudaMemGetInfo(&freeB, &totalB);
  // Per pair: the record (32 B), three output slots (72 B) and the work-list, count and
  // position words; per node 16 B.  Take about a fifth of the free memory.
  const size_t budget = freeB / 5;
  size_t pc = std::min<size_t>(32u << 20, budget / 3 / 160), nc = std::min<size_t>(1u << 29, budget * 2 / 3 / 16);
  ctx->pairCap = (uint32_t)std::max<size_t>(pc, 1u << 16);
  ctx->nodeCap = (uint32_t)std::max<size_t>(nc, 1u << 20);
  CK(ctx->dPairs.ensure((size_t)ctx->pairCap * sizeof(PairRec)));
  CK(ctx->dNodes.ensure((size_t)ctx->nodeCap * sizeof(int4)));
  return OIC_OK;
}

// CTAs of the CTA bin: as many per SM (at most 2) as the row buffers leave room for
// in the SM's 227 KB of shared memory.
uint32_t resolved_tuning_ctas(const oic_ctx *c, const oic_tuning &t) {
  const size_t per = (size_t)2 * t.wideBandW * sizeof(int) + 4096;
  const int    k   = (int)std::max<size_t>(1, std::min<size_t>(2, (227u << 10) / per));
  return (uint32_t)(k * c->nSM);
}

}  // namespace

namespace oic {

int ctx_views(oic_ctx *ctx, CtxViews *v) {
  if (!ctx || ctx->nReads == 0) return 1;
  v->R      = ctx->R;
  v->dp     = ctx->dp;
  v->eml    = ctx->dEml.as<int>();
  v->ctr32  = ctr32(ctx);
  v->st     = ctx->st;
  v->device = ctx->device;
  return 0;
}

void ctx_set_error(oic_ctx *ctx, const char *msg) {
  if (ctx) ctx->lastErr = msg;
}

void ctx_add_dp_work(oic_ctx *ctx, unsigned long long cells, unsigned long long slides) {
  if (!ctx) return;
  ctx->stats.dpCells += cells;
  ctx->stats.slideBases += slides;
}

}  // namespace oic

// =================================================================================
extern "C" {

void oic_default_params(oic_params *p) {
  memset(p, 0, sizeof(*p));
  p->maxErate          = 0.06;
  p->alignNoise        = 1.0;
  p->uniqueOlapPerPair = 1;
  p->useHopelessCheck  = 1;
  p->hashBits          = 22;
  p->maxHashLoad       = 0.6;
  p->maxHashDataLen    = 100000000;
  p->numThreads        = 1;
  p->bgnHashID         = 1;
  p->endHashID         = UINT32_MAX;
  p->maxLibToHash      = UINT32_MAX;
  p->bgnRefID          = 1;
  p->endRefID          = UINT32_MAX;
  p->maxLibToRef       = UINT32_MAX;
}

int oic_create(const oic_params *p, int device, oic_ctx **out) {
  if (!p || !out) return OIC_ERR_ARG;
  *out = nullptr;
  if (p->kmerLen < 1 || p->kmerLen > 31) return OIC_ERR_ARG;
  if (p->hashBits < 1 || p->hashBits > 40) return OIC_ERR_ARG;
  if (!(p->maxErate > 0.0) || p->maxErate > 0.65) return OIC_ERR_ARG;
  if (!(p->alignNoise > 0.0)) return OIC_ERR_ARG;

  oic_ctx *ctx = new oic_ctx();
  ctx->P = *p;
  if (ctx->P.maxErate > 0.06) ctx->P.useHopelessCheck = 0;   // overlapInCore.C:400-401
  if (ctx->P.numThreads < 1) ctx->P.numThreads = 1;

  int nDev = 0;
  cudaError_t e = cudaGetDeviceCount(&nDev);
  if (e != cudaSuccess || device < 0 || device >= nDev) {
    int code = fail(ctx, OIC_ERR_CUDA, "no usable CUDA device %d (%s)", device,
                    e == cudaSuccess ? "not present" : cudaGetErrorString(e));
    delete ctx;
    return code;
  }
  ctx->device = device;
  if ((e = cudaSetDevice(device)) != cudaSuccess || (e = cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking)) !=
                                                         cudaSuccess) {
    delete ctx;
    return OIC_ERR_CUDA;
  }
  cudaDeviceGetAttribute(&ctx->nSM, cudaDevAttrMultiProcessorCount, device);
  if (ctx->nSM <= 0) ctx->nSM = 1;

  // prefixEditDistance constructor (prefixEditDistance.C:23-90).
  const double erate     = ctx->P.maxErate;
  const int32_t maxErrors = 1 + (int32_t)ceil(erate * (double)kMaxReadLen);
  match_limit(ctx->eml, erate * ctx->P.alignNoise, maxErrors);
  DevParams &dp        = ctx->dp;
  dp.maxErate          = erate;
  dp.branchMatchValue  = erate / (1 + erate);
  dp.minBranchTailSlope = (erate > 0.06) ? 1.0 : 0.20;
  dp.kmerExpect        = exp(-1.0 * (double)ctx->P.kmerLen * erate);
  dp.minKmers          = 0;
  if (ctx->P.minKmers)   // overlapInCore.C:410-411
    dp.minKmers = (unsigned long long)(int)floor(
        dp.kmerExpect * (double)((uint64_t)(int64_t)ctx->P.minOlapLen - (uint64_t)ctx->P.kmerLen + 1));
  dp.kmerLen    = (int)ctx->P.kmerLen;
  dp.partial    = ctx->P.partial ? 1 : 0;
  dp.unique     = ctx->P.uniqueOlapPerPair ? 1 : 0;
  dp.hopeless   = ctx->P.useHopelessCheck ? 1 : 0;
  dp.minOlapLen = ctx->P.minOlapLen;
  dp.maxErrors  = maxErrors;

  int rc = OIC_OK;
  if ((e = ctx->dEml.ensure(ctx->eml.size() * sizeof(int32_t))) != cudaSuccess ||
      (e = cudaMemcpy(ctx->dEml.p, ctx->eml.data(), ctx->eml.size() * sizeof(int32_t), cudaMemcpyHostToDevice)) !=
          cudaSuccess ||
      (e = ctx->dCtr.ensure(4096)) != cudaSuccess) {
    rc = OIC_ERR_CUDA;
  }
  if (rc) {
    oic_destroy(ctx);
    return rc;
  }
  *out = ctx;
  return OIC_OK;
}

void oic_destroy(oic_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  DevBuf *bufs[] = {&ctx->dEml,      &ctx->dFwd,        &ctx->dRc,         &ctx->dNfwd,      &ctx->dNrc,
                    &ctx->dWordOff,  &ctx->dLen,        &ctx->dLib,        &ctx->dHasN,      &ctx->dSkip,
                    &ctx->dTable,     &ctx->dOcc,        &ctx->dLscr,      &ctx->dRscr,
                    &ctx->dSlen,     &ctx->dSread,      &ctx->dSortK,      &ctx->dSortV,     &ctx->dSortK2,
                    &ctx->dSortV2,   &ctx->dFlags,      &ctx->dPos,        &ctx->dSortScratch, &ctx->dStrRead,
                    &ctx->dStrKmers, &ctx->dFlat,       &ctx->dNewKeys,    &ctx->dChunkStr,    &ctx->dSegReads,  &ctx->dPairs,
                    &ctx->dNodes,    &ctx->dSegOvf,     &ctx->dSeedSlotK,  &ctx->dSeedSlotV, &ctx->dSeedPairs,
                    &ctx->dSeedNodes, &ctx->dSeedSlotK2, &ctx->dSeedSlotV2, &ctx->dSeedPairs2, &ctx->dSeedNodes2,
                    &ctx->dWork,     &ctx->dRec,        &ctx->dCnt,        &ctx->dRecPos,    &ctx->dRecOut,
                    &ctx->dAlnOvf,   &ctx->dArena,      &ctx->dRowHdr,
                    &ctx->dDL,       &ctx->dDR,         &ctx->dStack,      &ctx->dAlive,     &ctx->dArena2,
                    &ctx->dRowHdr2,  &ctx->dDL2,       &ctx->dDR2,
                    &ctx->dStack2,   &ctx->dAlive2,     &ctx->dScanScratch, &ctx->dCtr,
                    &ctx->dWorkK,    &ctx->dWorkK2,     &ctx->dWorkV2,     &ctx->dWorkScratch, &ctx->dSegList,
                    &ctx->dRowsG,    &ctx->dRowsG2,     &ctx->dFilterPrm,  &ctx->dFeat,      &ctx->dLogit,
                    &ctx->dPairCells, &ctx->dPairExt};
  for (DevBuf *b : bufs) b->release();
  if (ctx->gExec) cudaGraphExecDestroy(ctx->gExec);
  for (cudaEvent_t e : ctx->gEv)
    if (e) cudaEventDestroy(e);
  if (ctx->evF0) cudaEventDestroy(ctx->evF0);
  if (ctx->evF1) cudaEventDestroy(ctx->evF1);
  if (ctx->st) cudaStreamDestroy(ctx->st);
  delete ctx;
}

const char *oic_last_error(oic_ctx *ctx) { return ctx ? ctx->lastErr.c_str() : "no context"; }

int oic_get_match_limit(oic_ctx *ctx, int32_t *dst, uint32_t n, uint32_t *len) {
  if (!ctx) return OIC_ERR_ARG;
  if (len) *len = (uint32_t)ctx->eml.size();
  if (dst) memcpy(dst, ctx->eml.data(), sizeof(int32_t) * std::min<size_t>(n, ctx->eml.size()));
  return OIC_OK;
}

int oic_set_reads(oic_ctx *ctx, uint32_t nReads, const uint32_t *libID, const uint32_t *length,
                  const uint64_t *offset, const char *bases, uint64_t nBases) {
  if (!ctx || (nReads && (!length || !offset || !bases))) return OIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  ctx->haveBlock = false;
  ctx->nReads    = nReads;
  ctx->len.assign(length, length + nReads);
  ctx->lib.resize(nReads);
  for (uint32_t i = 0; i < nReads; i++) ctx->lib[i] = libID ? libID[i] : 1;
  ctx->wordOff.resize((size_t)nReads + 1);
  uint64_t w = 1;
  for (uint32_t i = 0; i < nReads; i++) {
    if (length[i] > kMaxReadLen) return fail(ctx, OIC_ERR_INPUT, "read %u is longer than %u bases", i + 1, kMaxReadLen);
    if (offset[i] + length[i] > nBases) return fail(ctx, OIC_ERR_ARG, "read %u lies outside the base buffer", i + 1);
    ctx->wordOff[i] = w;
    w += (length[i] + 31) / 32 + 1;
  }
  ctx->wordOff[nReads] = w;
  const uint64_t nWords = w + 4;   // spare words: 32-base windows and staged tiles past the last read

  EventPair rev;
  if (!rev.ok()) return fail(ctx, OIC_ERR_CUDA, "cudaEventCreate failed");
  const cudaEvent_t r0 = rev.a, r1 = rev.b;
  cudaEventRecord(r0, ctx->st);
  CK(ctx->dFwd.ensure(nWords * 8));
  CK(ctx->dRc.ensure(nWords * 8));
  CK(ctx->dNfwd.ensure(nWords * 8));
  CK(ctx->dNrc.ensure(nWords * 8));
  CK(cudaMemsetAsync(ctx->dFwd.p, 0, nWords * 8, ctx->st));
  CK(cudaMemsetAsync(ctx->dRc.p, 0, nWords * 8, ctx->st));
  CK(cudaMemsetAsync(ctx->dNfwd.p, 0, nWords * 8, ctx->st));
  CK(cudaMemsetAsync(ctx->dNrc.p, 0, nWords * 8, ctx->st));
  CK(ctx->dWordOff.ensure((size_t)(nReads + 1) * 8));
  CK(ctx->dLen.ensure((size_t)(nReads + 1) * 4));
  CK(ctx->dLib.ensure((size_t)(nReads + 1) * 4));
  CK(ctx->dHasN.ensure((size_t)(nReads + 1)));
  if (nReads) {
    CK(cudaMemcpyAsync(ctx->dWordOff.p, ctx->wordOff.data(), (size_t)nReads * 8, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(ctx->dLen.p, length, (size_t)nReads * 4, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(ctx->dLib.p, ctx->lib.data(), (size_t)nReads * 4, cudaMemcpyHostToDevice, ctx->st));
    DevBuf ascii, off;
    CK(ascii.ensure(nBases + 64));
    CK(off.ensure((size_t)nReads * 8));
    CK(cudaMemcpyAsync(ascii.p, bases, nBases, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(off.p, offset, (size_t)nReads * 8, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemsetAsync(ctr32(ctx) + cErr, 0, 4, ctx->st));
    launch_pack_reads(ascii.as<char>(), off.as<u64>(), ctx->dLen.as<uint32_t>(), ctx->dWordOff.as<u64>(),
                      nReads, ctx->dFwd.as<u64>(), ctx->dRc.as<u64>(), ctx->dNfwd.as<u64>(), ctx->dNrc.as<u64>(),
                      ctx->dHasN.as<unsigned char>(), ctr32(ctx) + cErr, ctx->st);
    int rc = sync_check(ctx, "pack reads");
    uint32_t err = read_err(ctx);
    ascii.release();
    off.release();
    if (rc) return rc;
    if (err & kErrBadBase) return fail(ctx, OIC_ERR_INPUT, "a read holds a character other than A, C, G, T or N");
  }
  cudaEventRecord(r1, ctx->st);
  cudaEventSynchronize(r1);
  float msR = 0;
  cudaEventElapsedTime(&msR, r0, r1);
  ctx->stats.msReads = msR;
  ReadsDev &R = ctx->R;
  R.fwd     = ctx->dFwd.as<u64>();
  R.rc      = ctx->dRc.as<u64>();
  R.nfwd    = ctx->dNfwd.as<u64>();
  R.nrc     = ctx->dNrc.as<u64>();
  R.wordOff = ctx->dWordOff.as<u64>();
  R.len     = ctx->dLen.as<uint32_t>();
  R.lib     = ctx->dLib.as<uint32_t>();
  R.hasN    = ctx->dHasN.as<unsigned char>();
  R.nReads  = nReads;
  return OIC_OK;
}

int oic_set_skip_kmers(oic_ctx *ctx, const char *kmers, uint64_t nKmers) {
  if (!ctx || (nKmers && !kmers)) return OIC_ERR_ARG;
  const uint32_t K = ctx->P.kmerLen;
  ctx->skipKeys.clear();
  ctx->skipKeys.reserve(nKmers * 2);
  for (uint64_t i = 0; i < nKmers; i++) {
    const char *s = kmers + i * K;
    uint64_t fw = 0, rc = 0;
    for (uint32_t j = 0; j < K; j++) {
      int c = base2(s[j]);
      if (c < 0) return fail(ctx, OIC_ERR_INPUT, "skip k-mer %lu is not ACGT", (unsigned long)(i + 1));
      fw |= (uint64_t)c << (2 * j);                // Mark_Skip_Kmers, Build_Hash_Index.C:231-232
      rc |= (uint64_t)(3 - c) << (2 * (K - 1 - j));
    }
    ctx->skipKeys.push_back(fw);
    ctx->skipKeys.push_back(rc);
  }
  return OIC_OK;
}

int oic_load_hash_block(oic_ctx *ctx, uint32_t bgnID, uint32_t endID, uint32_t *lastLoaded) {
  NvtxRange range("oic hash block");
  if (!ctx) return OIC_ERR_ARG;
  if (ctx->nReads == 0) return fail(ctx, OIC_ERR_STATE, "no reads loaded");
  cudaSetDevice(ctx->device);
  if (bgnID < 1) bgnID = 1;
  if (endID > ctx->nReads) endID = ctx->nReads;
  if (bgnID > endID) return fail(ctx, OIC_ERR_ARG, "empty hash range %u-%u", bgnID, endID);
  const oic_params &P = ctx->P;
  const uint32_t K = P.kmerLen;
  const uint64_t maxData  = P.maxHashDataLen + kMaxReadLen;                        // overlapInCore.C:454
  const uint64_t tableSz  = (uint64_t)1 << P.hashBits;
  const uint64_t entryLim = (uint64_t)(P.maxHashLoad * (double)tableSz * kEntriesPerBucket);   // :445

  cudaEvent_t ev0, ev1;
  cudaEventCreate(&ev0);
  cudaEventCreate(&ev1);
  cudaEventRecord(ev0, ctx->st);

  // Candidate strings under the data-length limit (Build_Hash_Index.C:504-545).
  std::vector<uint32_t> strRead, strKmers, strLen;
  std::vector<uint64_t> flat(1, 0);
  std::vector<uint8_t>  eligible;
  uint64_t total = 0;
  for (uint32_t cur = bgnID; total < maxData && cur <= endID; cur++) {
    const uint32_t r  = cur - 1;
    const bool     ok = ctx->lib[r] >= P.minLibToHash && ctx->lib[r] <= P.maxLibToHash &&
                    (int64_t)ctx->len[r] >= (int64_t)P.minOlapLen;
    if (ok && ctx->len[r] < K) return fail(ctx, OIC_ERR_INPUT, "read %u is shorter than the k-mer size", cur);
    strRead.push_back(r);
    eligible.push_back(ok ? 1 : 0);
    strLen.push_back(ok ? ctx->len[r] : 0);
    const uint32_t nk = ok ? ctx->len[r] - K + 1 : 0;
    strKmers.push_back(nk);
    flat.push_back(flat.back() + nk);
    if (ok) total += (uint64_t)ctx->len[r] + 1;
  }
  const uint32_t nCand = (uint32_t)strRead.size();
  const uint64_t nFlat = flat.back();
  if (nFlat >= 0xffffffffull) return fail(ctx, OIC_ERR_OVERFLOW, "hash block holds more than 2^32 k-mers");

  CK(ctx->dStrRead.ensure((size_t)nCand * 4 + 4));
  CK(ctx->dStrKmers.ensure((size_t)nCand * 4 + 4));
  CK(ctx->dFlat.ensure((size_t)(nCand + 1) * 8));
  CK(ctx->dNewKeys.ensure((size_t)nCand * 4 + 4));
  CK(ctx->dChunkStr.ensure(((size_t)(nFlat >> 12) + 1) * 4));
  CK(cudaMemcpyAsync(ctx->dStrRead.p, strRead.data(), nCand * 4, cudaMemcpyHostToDevice, ctx->st));
  CK(cudaMemcpyAsync(ctx->dStrKmers.p, strKmers.data(), nCand * 4, cudaMemcpyHostToDevice, ctx->st));
  CK(cudaMemcpyAsync(ctx->dFlat.p, flat.data(), (size_t)(nCand + 1) * 8, cudaMemcpyHostToDevice, ctx->st));
  CK(cudaMemsetAsync(ctx->dNewKeys.p, 0, (size_t)nCand * 4 + 4, ctx->st));
  if (nCand) launch_chunk_str(ctx->dFlat.as<u64>(), nCand, nFlat, ctx->dChunkStr.as<uint32_t>(), ctx->st);

  const size_t n = (size_t)nFlat;
  CK(ctx->dSortK.ensure(n * 8 + 8));
  CK(ctx->dSortV.ensure(n * 4 + 4));
  CK(ctx->dSortK2.ensure(n * 8 + 8));
  CK(ctx->dSortV2.ensure(n * 4 + 4));
  CK(ctx->dFlags.ensure(n * 4 + 4));
  CK(ctx->dPos.ensure(n * 4 + 4));
  CK(ctx->dSortScratch.ensure(std::max(radix_sort_scratch(n), scan_u32_scratch(n)) + 256));

  launch_kmer_emit(ctx->R, ctx->dStrRead.as<uint32_t>(), ctx->dStrKmers.as<uint32_t>(), ctx->dFlat.as<u64>(), nCand,
                   (int)K, ctx->dSortK.as<u64>(), ctx->dSortV.as<uint32_t>(), ctx->st);
  CK(radix_sort_u64_u32(ctx->dSortK.as<u64>(), ctx->dSortV.as<uint32_t>(), ctx->dSortK2.as<u64>(),
                        ctx->dSortV2.as<uint32_t>(), n, 2 * (int)K + 1, ctx->dSortScratch.p, ctx->st));
  launch_first_occ(ctx->dSortK.as<u64>(), ctx->dSortV.as<uint32_t>(), n, ctx->dFlat.as<u64>(),
                   ctx->dChunkStr.as<uint32_t>(), (int)K,
                   ctx->dNewKeys.as<uint32_t>(), ctx->st);
  std::vector<uint32_t> newKeys(nCand);
  CK(cudaMemcpyAsync(newKeys.data(), ctx->dNewKeys.p, (size_t)nCand * 4, cudaMemcpyDeviceToHost, ctx->st));
  int rc = sync_check(ctx, "hash k-mer sort");
  if (rc) return rc;

  // The load loop stops before a read once the data length or the distinct-k-mer
  // count reached its limit (Build_Hash_Index.C:504-506).
  uint32_t cut = 0;
  uint64_t len = 0, distinct = 0;
  for (; cut < nCand; cut++) {
    if (!(len < maxData && distinct < entryLim)) break;
    if (eligible[cut]) len += (uint64_t)strLen[cut] + 1;
    distinct += newKeys[cut];
  }
  const uint32_t nStr = cut;

  // Keep the occurrences of the loaded strings (and drop windows with an N).
  launch_keep_flags(ctx->dSortK.as<u64>(), ctx->dSortV.as<uint32_t>(), n, (int)K, (uint32_t)flat[nStr],
                    ctx->dFlags.as<uint32_t>(), ctx->st);
  CK(scan_u32(ctx->dFlags.as<uint32_t>(), ctx->dPos.as<uint32_t>(), n, ctr32(ctx) + cRecTotal, ctx->dSortScratch.p,
              ctx->st));
  launch_compact_kv(ctx->dSortK.as<u64>(), ctx->dSortV.as<uint32_t>(), ctx->dFlags.as<uint32_t>(),
                    ctx->dPos.as<uint32_t>(), n, ctx->dSortK2.as<u64>(), ctx->dSortV2.as<uint32_t>(), ctx->st);
  uint32_t nOcc = 0;
  CK(cudaMemcpyAsync(&nOcc, ctr32(ctx) + cRecTotal, 4, cudaMemcpyDeviceToHost, ctx->st));
  if ((rc = sync_check(ctx, "hash compaction"))) return rc;

  uint64_t cap = 1024;
  while (cap < 2 * (distinct + ctx->skipKeys.size() + 1)) cap <<= 1;
  // Slots of 16 bytes: empty key (all ones), value 0.
  CK(ctx->dTable.ensure(cap * 16));
  CK(ctx->dOcc.ensure((size_t)nOcc * 8 + 8));
  launch_table_init(ctx->dTable.as<u64>(), cap, ctx->st);
  CK(cudaMemsetAsync(ctr32(ctx) + cErr, 0, 4, ctx->st));
  launch_table_build(ctx->dSortK2.as<u64>(), nOcc, ctx->dTable.as<u64>(), cap - 1, ctr32(ctx) + cErr, ctx->st);
  launch_occ_convert(ctx->dSortV2.as<uint32_t>(), nOcc, ctx->dFlat.as<u64>(), ctx->dChunkStr.as<uint32_t>(),
                     ctx->dOcc.as<u64>(), ctx->st);

  // String_Info (Build_Hash_Index.C:511-536): loaded strings unscreened, skipped ones screened.
  std::vector<uint8_t>  lscr(nStr), rscr(nStr);
  std::vector<uint32_t> slen(nStr), sread(nStr);
  for (uint32_t s = 0; s < nStr; s++) {
    lscr[s] = rscr[s] = eligible[s] ? 0 : 1;
    slen[s]  = strLen[s];
    sread[s] = strRead[s];
  }
  CK(ctx->dLscr.ensure(nStr + 1));
  CK(ctx->dRscr.ensure(nStr + 1));
  CK(ctx->dSlen.ensure((size_t)nStr * 4 + 4));
  CK(ctx->dSread.ensure((size_t)nStr * 4 + 4));
  CK(cudaMemcpyAsync(ctx->dLscr.p, lscr.data(), nStr, cudaMemcpyHostToDevice, ctx->st));
  CK(cudaMemcpyAsync(ctx->dRscr.p, rscr.data(), nStr, cudaMemcpyHostToDevice, ctx->st));
  CK(cudaMemcpyAsync(ctx->dSlen.p, slen.data(), (size_t)nStr * 4, cudaMemcpyHostToDevice, ctx->st));
  CK(cudaMemcpyAsync(ctx->dSread.p, sread.data(), (size_t)nStr * 4, cudaMemcpyHostToDevice, ctx->st));

  TableDev &T = ctx->T;
  T.kv       = ctx->dTable.as<u64>();
  T.mask     = cap - 1;
  T.occ      = ctx->dOcc.as<u64>();
  T.lscr     = ctx->dLscr.as<unsigned char>();
  T.rscr     = ctx->dRscr.as<unsigned char>();
  T.slen     = ctx->dSlen.as<uint32_t>();
  T.sread    = ctx->dSread.as<uint32_t>();
  T.firstID  = bgnID;
  T.nStrings = nStr;

  if (!ctx->skipKeys.empty()) {
    CK(ctx->dSkip.ensure(ctx->skipKeys.size() * 8));
    CK(cudaMemcpyAsync(ctx->dSkip.p, ctx->skipKeys.data(), ctx->skipKeys.size() * 8, cudaMemcpyHostToDevice, ctx->st));
    launch_skip_mark(ctx->dSkip.as<u64>(), ctx->skipKeys.size(), T, ctx->dTable.as<u64>(),
                     ctx->dLscr.as<unsigned char>(), ctx->dRscr.as<unsigned char>(), (int)K, P.useHopelessCheck ? 1 : 0,
                     ctr32(ctx) + cErr, ctx->st);
  }
  cudaEventRecord(ev1, ctx->st);
  if ((rc = sync_check(ctx, "hash table build"))) return rc;
  uint32_t err = read_err(ctx);
  if (err & kErrTableFull) return fail(ctx, OIC_ERR_DEVICE, "k-mer table full");
  float ms = 0;
  cudaEventElapsedTime(&ms, ev0, ev1);
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  ctx->stats.msHash += ms;
  ctx->stats.nHashBlocks++;

  ctx->haveBlock   = true;
  ctx->blkFirst    = bgnID;
  ctx->blkN        = nStr;
  ctx->blkOcc      = nOcc;
  ctx->blkDistinct = distinct;
  if (verbose())
    fprintf(stderr, "oic: hash block %u-%u: %u strings, %lu distinct k-mers, %u occurrences, %.2f ms\n", bgnID,
            bgnID + nStr - 1, nStr, (unsigned long)distinct, nOcc, ms);
  if (lastLoaded) *lastLoaded = bgnID + nStr - 1;
  return OIC_OK;
}

int oic_run_refs(oic_ctx *ctx, uint32_t bgnRefID, uint32_t endRefID) {
  NvtxRange range("oic ref reads");
  if (!ctx) return OIC_ERR_ARG;
  if (!ctx->haveBlock) return fail(ctx, OIC_ERR_STATE, "no hash block loaded");
  cudaSetDevice(ctx->device);
  std::vector<uint32_t> refs;
  int erc = eligible_refs(ctx, bgnRefID, endRefID, refs);
  if (erc) return erc;
  if (refs.empty()) return OIC_OK;
  if ((erc = ensure_pair_caps(ctx))) return erc;

  cudaEvent_t e0, e1, e2;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventCreate(&e2);
  float msSeed = 0, msAlign = 0;
  size_t   pos   = 0;
  int      rc    = OIC_OK;
  // Batch size from the density of earlier batches (any block, scaled by this block's
  // string count), else from 256 candidate pairs and 4096 match runs per ref read;
  // 20 % headroom.
  const double strs = std::max<double>(1.0, ctx->blkN);
  auto size_for = [&](double pairsPerRef, double nodesPerRef) {
    double lim = (double)refs.size();
    if (pairsPerRef > 0) lim = std::min(lim, 0.8 * ctx->pairCap / pairsPerRef);
    if (nodesPerRef > 0) lim = std::min(lim, 0.8 * ctx->nodeCap / nodesPerRef);
    return (uint32_t)std::max(1.0, lim);
  };
  uint32_t batch = ctx->pairDensity > 0 ? size_for(ctx->pairDensity * strs, ctx->nodeDensity * strs)
                                        : size_for(256.0, 4096.0);
  while (pos < refs.size()) {
    const uint32_t nb = (uint32_t)std::min<size_t>(batch, refs.size() - pos);
    const size_t   outMark = ctx->out.size();
    const oic_stats saved  = ctx->stats;
    rc = run_batch(ctx, refs.data() + pos, nb, e0, e1, e2, msSeed, msAlign);
    if (rc == kRetrySmaller && nb > 1) {
      ctx->out.resize(outMark);
      ctx->stats = saved;
      // The failed batch's demand sizes the retry (at most half the failed size).
      batch = std::min<uint32_t>((nb + 1) / 2, size_for((double)ctx->overPairs / nb, (double)ctx->overNodes / nb));
      if (verbose()) fprintf(stderr, "oic: batch output full, retrying with %u ref reads per batch\n", batch);
      continue;
    }
    if (rc) break;
    pos += nb;
    const double pr = (double)(ctx->stats.candidatePairs - saved.candidatePairs) / nb;
    const double nr = (double)(ctx->stats.nodes - saved.nodes) / nb;
    ctx->pairDensity = std::max(ctx->pairDensity, pr / strs);
    ctx->nodeDensity = std::max(ctx->nodeDensity, nr / strs);
    batch            = size_for(std::max(pr, ctx->pairDensity * strs), std::max(nr, ctx->nodeDensity * strs));
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(e2);
  ctx->stats.msSeed += msSeed;
  ctx->stats.msAlign += msAlign;
  if (rc == kRetrySmaller) return fail(ctx, OIC_ERR_OVERFLOW, "a single ref read's output does not fit");
  return rc;
}

int oic_run(oic_ctx *ctx) {
  NvtxRange range("oic run");
  if (!ctx) return OIC_ERR_ARG;
  if (ctx->nReads == 0) return fail(ctx, OIC_ERR_STATE, "no reads loaded");
  oic_params G = ctx->P;
  const uint32_t last = ctx->nReads;
  // OverlapDriver range clamping (overlapInCore.C:179-189).
  if (G.bgnHashID < 1) G.bgnHashID = 1;
  if (last < G.endHashID) G.endHashID = last;
  if (G.bgnRefID < 1) G.bgnRefID = 1;
  if (G.endRefID > last) G.endRefID = last;

  // Every read the reference visits must be at least k long (Find_Overlaps.C:249).
  for (uint32_t r = 0; r < last; r++)
    if ((int64_t)ctx->len[r] >= (int64_t)G.minOlapLen && ctx->len[r] < G.kmerLen)
      return fail(ctx, OIC_ERR_INPUT, "read %u is shorter than the k-mer size", r + 1);

  // Thread chunks start at bgnRef + k * perThread and a chunk starting on endRef is
  // never run (Process_Overlaps.C:33, overlapInCore.C:225).
  uint32_t refEnd = G.endRefID;
  bool     anyRef = G.bgnRefID < G.endRefID;
  if (G.bgnRefID <= G.endRefID) {
    const uint32_t perThread = 1 + (G.endRefID - G.bgnRefID) / G.numThreads / 8;
    if ((G.endRefID - G.bgnRefID) % perThread == 0) refEnd = G.endRefID - 1;
  }

  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  cudaEventRecord(t0, ctx->st);
  const unsigned long long launches0 = g_launches;
  int rc = OIC_OK;
  uint32_t bgnH = G.bgnHashID;
  while (bgnH < G.endHashID) {   // overlapInCore.C:204
    uint32_t lastLoaded = 0;
    if ((rc = oic_load_hash_block(ctx, bgnH, G.endHashID, &lastLoaded))) break;
    if (anyRef && (rc = oic_run_refs(ctx, G.bgnRefID, refEnd))) break;
    bgnH = lastLoaded + 1;
  }
  cudaEventRecord(t1, ctx->st);
  cudaEventSynchronize(t1);
  float ms = 0;
  cudaEventElapsedTime(&ms, t0, t1);
  ctx->stats.msTotal += ms;
  ctx->stats.kernelLaunches += g_launches - launches0;
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  return rc;
}

int oic_num_overlaps(oic_ctx *ctx, uint64_t *n) {
  if (!ctx || !n) return OIC_ERR_ARG;
  *n = ctx->out.size() / 6;
  return OIC_OK;
}

int oic_fetch_overlaps(oic_ctx *ctx, uint32_t *words, uint64_t maxRecords, uint64_t *n) {
  if (!ctx || (!words && maxRecords)) return OIC_ERR_ARG;
  const uint64_t have = ctx->out.size() / 6, k = std::min(have, maxRecords);
  if (k) memcpy(words, ctx->out.data(), (size_t)k * 6 * sizeof(uint32_t));
  if (n) *n = k;
  return OIC_OK;
}

int oic_clear_overlaps(oic_ctx *ctx) {
  if (!ctx) return OIC_ERR_ARG;
  ctx->out.clear();
  const double msReads = ctx->stats.msReads;
  ctx->stats = oic_stats{};
  ctx->stats.msReads = msReads;
  return OIC_OK;
}

int oic_get_stats(oic_ctx *ctx, oic_stats *st) {
  if (!ctx || !st) return OIC_ERR_ARG;
  *st = ctx->stats;
  return OIC_OK;
}

int oic_stats_json(const oic_stats *s, char *buf, size_t cap, size_t *len) {
  if (!s || !len || (!buf && cap)) return OIC_ERR_ARG;
  const double ovps = s->msTotal > 0 ? (double)s->totalOverlaps / (s->msTotal / 1000.0) : 0.0;
  const double dpps = s->msAlign > 0 ? (double)s->dpCells / (s->msAlign / 1000.0) : 0.0;
  const int n = snprintf(
      buf, cap,
      "{\"kmerHitsWithoutOlap\": %llu, \"kmerHitsWithOlap\": %llu, \"kmerHitsSkipped\": %llu, "
      "\"multiOverlap\": %llu, \"totalOverlaps\": %llu, \"containedOverlaps\": %llu, "
      "\"dovetailOverlaps\": %llu, \"badShortWindow\": %llu, \"badLongWindow\": %llu, \"dpCells\": %llu, "
      "\"slideBases\": %llu, \"extensions\": %llu, \"seeds\": %llu, \"candidatePairs\": %llu, \"nodes\": %llu, "
      "\"dpRows\": %llu, \"nHashBlocks\": %u, \"msHash\": %.6f, \"msSeed\": %.6f, \"msAlign\": %.6f, "
      "\"msTotal\": %.6f, \"msReads\": %.6f, \"kernelLaunches\": %llu, \"dpCellsNoOverlap\": %llu, "
      "\"filteredPairs\": %llu, \"msFilter\": %.6f, \"msNarrow\": %.6f, \"msWide\": %.6f, "
      "\"pairsNarrow\": %llu, \"pairsWide\": %llu, \"cellsWide\": %llu, \"graphLaunches\": %llu, "
      "\"overlapsPerSec\": %.3f, \"dpCellsPerSec\": %.3f}",
      (unsigned long long)s->kmerHitsWithoutOlap, (unsigned long long)s->kmerHitsWithOlap,
      (unsigned long long)s->kmerHitsSkipped, (unsigned long long)s->multiOverlap,
      (unsigned long long)s->totalOverlaps, (unsigned long long)s->containedOverlaps,
      (unsigned long long)s->dovetailOverlaps, (unsigned long long)s->badShortWindow,
      (unsigned long long)s->badLongWindow, (unsigned long long)s->dpCells, (unsigned long long)s->slideBases,
      (unsigned long long)s->extensions, (unsigned long long)s->seeds, (unsigned long long)s->candidatePairs,
      (unsigned long long)s->nodes, (unsigned long long)s->dpRows, s->nHashBlocks, s->msHash, s->msSeed,
      s->msAlign, s->msTotal, s->msReads, (unsigned long long)s->kernelLaunches,
      (unsigned long long)s->dpCellsNoOverlap, (unsigned long long)s->filteredPairs, s->msFilter, s->msNarrow,
      s->msWide, (unsigned long long)s->pairsNarrow, (unsigned long long)s->pairsWide,
      (unsigned long long)s->cellsWide, (unsigned long long)s->graphLaunches, ovps, dpps);
  if (n < 0) return OIC_ERR_ARG;
  *len = (size_t)n;
  return (size_t)n < cap ? OIC_OK : OIC_ERR_ARG;
}

int oic_set_filter(oic_ctx *ctx, const uint16_t *params, float threshold, float fullThreshold, uint32_t extBudget,
                   const oic_filter_domain *trainedOn) {
  if (!ctx) return OIC_ERR_ARG;
  if (!params) {
    ctx->filterOn = false;
    return OIC_OK;
  }
  if (!trainedOn) return fail(ctx, OIC_ERR_ARG, "a filter needs the parameters it was trained under");
  if (trainedOn->kmerLen != ctx->P.kmerLen || trainedOn->minOlapLen != ctx->P.minOlapLen ||
      (float)trainedOn->maxErate != (float)ctx->P.maxErate)
    return fail(ctx, OIC_ERR_ARG,
                "the filter was trained for -k %u --minlength %d --maxerate %g; this context runs -k %u "
                "--minlength %d --maxerate %g",
                trainedOn->kmerLen, trainedOn->minOlapLen, (double)(float)trainedOn->maxErate, ctx->P.kmerLen,
                ctx->P.minOlapLen, (double)(float)ctx->P.maxErate);
  if (!(threshold >= 0.0f && threshold < 1.0f) || !(fullThreshold >= 0.0f && fullThreshold < 1.0f))
    return fail(ctx, OIC_ERR_ARG, "filter thresholds must be in [0, 1)");
  cudaSetDevice(ctx->device);
  CK(ctx->dFilterPrm.ensure(OIC_FILTER_NPARAM * sizeof(uint16_t)));
  CK(cudaMemcpyAsync(ctx->dFilterPrm.p, params, OIC_FILTER_NPARAM * sizeof(uint16_t), cudaMemcpyHostToDevice,
                     ctx->st));
  int rc = sync_check(ctx, "filter upload");
  if (rc) return rc;
  // sigmoid(z) < t  <=>  z < ln(t / (1 - t)); t = 0 keeps every pair.
  auto logit = [](float t) {
    return t > 0.0f ? (float)std::log((double)t / (1.0 - (double)t)) : -INFINITY;
  };
  ctx->filterLogitThr = logit(threshold);
  ctx->filterTierThr  = logit(fullThreshold);
  ctx->filterBudget   = extBudget ? (int)extBudget : 1;
  ctx->filterOn       = true;
  return OIC_OK;
}

int oic_collect_pairs(oic_ctx *ctx, int mode) {
  if (!ctx || mode < 0 || mode > 2) return OIC_ERR_ARG;
  ctx->collect = mode;
  return OIC_OK;
}

int oic_num_pairs(oic_ctx *ctx, uint64_t *nPairs, uint64_t *nNodes) {
  if (!ctx) return OIC_ERR_ARG;
  if (nPairs) *nPairs = ctx->colInfo.size();
  if (nNodes) *nNodes = ctx->colNodes.size() / 3;
  return OIC_OK;
}

int oic_get_pairs(oic_ctx *ctx, oic_pair_info *info, uint16_t *feat, int32_t *nodes, uint64_t maxPairs,
                  uint64_t maxNodes) {
  if (!ctx) return OIC_ERR_ARG;
  const uint64_t np = std::min<uint64_t>(maxPairs, ctx->colInfo.size());
  const uint64_t nn = std::min<uint64_t>(maxNodes, ctx->colNodes.size() / 3);
  if (info) memcpy(info, ctx->colInfo.data(), np * sizeof(oic_pair_info));
  if (feat) memcpy(feat, ctx->colFeat.data(), np * OIC_FILTER_IN * sizeof(uint16_t));
  if (nodes) memcpy(nodes, ctx->colNodes.data(), nn * 3 * sizeof(int32_t));
  return OIC_OK;
}

int oic_clear_pairs(oic_ctx *ctx) {
  if (!ctx) return OIC_ERR_ARG;
  std::vector<oic_pair_info>().swap(ctx->colInfo);
  std::vector<uint16_t>().swap(ctx->colFeat);
  std::vector<int32_t>().swap(ctx->colNodes);
  return OIC_OK;
}

int oic_extend_batch(oic_ctx *ctx, uint32_t nAlign, const uint32_t *sRead, const uint32_t *sRev,
                     const uint32_t *tRead, const int32_t *mStart, const int32_t *mOffset, const int32_t *mLen,
                     int32_t *out, int32_t *kind, int32_t *deltaLen) {
  if (!ctx) return OIC_ERR_ARG;
  if (nAlign == 0) return OIC_OK;
  if (!sRead || !sRev || !tRead || !mStart || !mOffset || !mLen || !out || !kind || !deltaLen) return OIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  std::vector<ExtendProblem> pb(nAlign);
  for (uint32_t i = 0; i < nAlign; i++) {
    if (sRead[i] < 1 || sRead[i] > ctx->nReads || tRead[i] < 1 || tRead[i] > ctx->nReads)
      return fail(ctx, OIC_ERR_ARG, "problem %u names a read outside the store", i);
    const int sl = (int)ctx->len[sRead[i] - 1], tl = (int)ctx->len[tRead[i] - 1];
    if (mLen[i] < 1 || mStart[i] < 0 || mOffset[i] < 0 || mStart[i] + mLen[i] > sl || mOffset[i] + mLen[i] > tl)
      return fail(ctx, OIC_ERR_ARG, "problem %u: match outside the reads", i);
    pb[i] = ExtendProblem{sRead[i] - 1, sRev[i] ? 1u : 0u, tRead[i] - 1, mStart[i], mOffset[i], mLen[i]};
  }
  DevBuf dP, dOut, dKind, dDl, dStatus;
  CK(dP.ensure(nAlign * sizeof(ExtendProblem)));
  CK(dOut.ensure((size_t)nAlign * 5 * 4));
  CK(dKind.ensure((size_t)nAlign * 4));
  CK(dDl.ensure((size_t)nAlign * 4));
  CK(dStatus.ensure((size_t)nAlign * 4));
  CK(cudaMemcpyAsync(dP.p, pb.data(), nAlign * sizeof(ExtendProblem), cudaMemcpyHostToDevice, ctx->st));
  CK(cudaMemsetAsync(ctr64(ctx) + kExtStatBase, 0, 2 * sizeof(unsigned long long), ctx->st));
  std::vector<uint32_t> status(nAlign);
  int rc = OIC_OK;
  const oic_tuning tn = resolved_tuning(ctx);
  // Pass 0: one warp per problem; pass 1: one CTA per problem (every problem when the
  // tuning forces the CTA bin, else those that overflowed); pass 2: the large arena.
  DevBuf dSub;
  std::vector<uint32_t> idx;
  for (int pass = tn.forceWide ? 1 : 0; pass < 3 && rc == OIC_OK; pass++) {
    CK(cudaMemsetAsync(ctr64(ctx) + kExtStatBase, 0, 2 * sizeof(unsigned long long), ctx->st));
    if (pass == 0) {
      AlignConfig ac = align_normal(ctx);
      ac.caps.arenaCap = (int)tn.narrowArena;
      WarpScratch ws;
      if ((rc = ensure_align_scratch(ctx, ac, false, ws))) break;
      launch_extend_batch(ac.bandW, ctx->R, ctx->dp, ctx->dEml.as<int>(), dP.as<ExtendProblem>(), nAlign, ws,
                          ac.caps, ac.warps, dOut.as<int>(), dKind.as<int>(), dDl.as<int>(), dStatus.as<uint32_t>(),
                          ctr64(ctx) + kExtStatBase, ctx->st);
    } else {
      // The problems still open run in a compact sub-batch; results are scattered back.
      std::vector<ExtendProblem> sub;
      idx.clear();
      for (uint32_t i = 0; i < nAlign; i++)
        if (pass == 1 ? (tn.forceWide || status[i] != 0) : status[i] != 0) {
          idx.push_back(i);
          sub.push_back(pb[i]);
        }
      const uint32_t ns = (uint32_t)sub.size();
      CK(dSub.ensure((size_t)ns * (sizeof(ExtendProblem) + 8 * 4)));
      ExtendProblem *sp = dSub.as<ExtendProblem>();
      int *so = (int *)(sp + ns), *sk = so + 5 * (size_t)ns, *sd = sk + ns;
      uint32_t *ss = (uint32_t *)(sd + ns);
      CK(cudaMemcpyAsync(sp, sub.data(), ns * sizeof(ExtendProblem), cudaMemcpyHostToDevice, ctx->st));
      uint32_t    ctas = 0;
      AlignCaps   caps;
      WarpScratch ws;
      if ((rc = ensure_group_scratch(ctx, tn, pass == 2, ctas, caps, ws))) break;
      const int threads = pass == 2 ? (int)std::max<uint32_t>(tn.wideThreads, 512) : (int)tn.wideThreads;
      launch_extend_group(threads, (int)tn.wideTile, caps.bandW, (int)std::min<uint32_t>(ctas, ns), ctx->R, ctx->dp,
                          ctx->dEml.as<int>(), sp, ns, ws, caps, so, sk, sd, ss, ctr64(ctx) + kExtStatBase, ctx->st);
      std::vector<int32_t> o5((size_t)ns * 5), ok(ns), od(ns);
      std::vector<uint32_t> os(ns);
      CK(cudaMemcpyAsync(o5.data(), so, (size_t)ns * 20, cudaMemcpyDeviceToHost, ctx->st));
      CK(cudaMemcpyAsync(ok.data(), sk, (size_t)ns * 4, cudaMemcpyDeviceToHost, ctx->st));
      CK(cudaMemcpyAsync(od.data(), sd, (size_t)ns * 4, cudaMemcpyDeviceToHost, ctx->st));
      CK(cudaMemcpyAsync(os.data(), ss, (size_t)ns * 4, cudaMemcpyDeviceToHost, ctx->st));
      if ((rc = sync_check(ctx, "extend batch (CTA bin)"))) break;
      // Scatter into the full-size device outputs.
      std::vector<int32_t> f5((size_t)nAlign * 5), fk(nAlign), fd(nAlign);
      CK(cudaMemcpy(f5.data(), dOut.p, (size_t)nAlign * 20, cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(fk.data(), dKind.p, (size_t)nAlign * 4, cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(fd.data(), dDl.p, (size_t)nAlign * 4, cudaMemcpyDeviceToHost));
      for (uint32_t q = 0; q < ns; q++) {
        const uint32_t i = idx[q];
        for (int k = 0; k < 5; k++) f5[(size_t)i * 5 + k] = o5[(size_t)q * 5 + k];
        fk[i]     = ok[q];
        fd[i]     = od[q];
        status[i] = os[q];
      }
      CK(cudaMemcpy(dOut.p, f5.data(), (size_t)nAlign * 20, cudaMemcpyHostToDevice));
      CK(cudaMemcpy(dKind.p, fk.data(), (size_t)nAlign * 4, cudaMemcpyHostToDevice));
      CK(cudaMemcpy(dDl.p, fd.data(), (size_t)nAlign * 4, cudaMemcpyHostToDevice));
      unsigned long long s2[2];
      CK(cudaMemcpy(s2, ctr64(ctx) + kExtStatBase, sizeof(s2), cudaMemcpyDeviceToHost));
      ctx->stats.dpCells += s2[0];
      ctx->stats.slideBases += s2[1];
      bool any = false;
      for (uint32_t q = 0; q < ns; q++) any |= os[q] != 0;
      if (!any) break;
      if (pass == 2) rc = fail(ctx, OIC_ERR_OVERFLOW, "an alignment exceeds the engine's DP capacity");
      continue;
    }
    CK(cudaMemcpyAsync(status.data(), dStatus.p, (size_t)nAlign * 4, cudaMemcpyDeviceToHost, ctx->st));
    if ((rc = sync_check(ctx, "extend batch"))) break;
    unsigned long long s2[2];
    CK(cudaMemcpy(s2, ctr64(ctx) + kExtStatBase, sizeof(s2), cudaMemcpyDeviceToHost));
    ctx->stats.dpCells += s2[0];
    ctx->stats.slideBases += s2[1];
    bool any = false;
    for (uint32_t i = 0; i < nAlign; i++) any |= status[i] != 0;
    if (!any) break;
  }
  if (rc == OIC_OK) {
    CK(cudaMemcpy(out, dOut.p, (size_t)nAlign * 5 * 4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(kind, dKind.p, (size_t)nAlign * 4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(deltaLen, dDl.p, (size_t)nAlign * 4, cudaMemcpyDeviceToHost));
  }
  dP.release();
  dSub.release();
  dOut.release();
  dKind.release();
  dDl.release();
  dStatus.release();
  return rc;
}

int oic_count_kmers(oic_ctx *ctx, uint32_t bgnID, uint32_t endID, uint32_t minCount, char *kmers, uint32_t *counts,
                    uint64_t maxKmers, uint64_t *nKmers) {
  if (!ctx || !nKmers || (maxKmers && (!kmers || !counts))) return OIC_ERR_ARG;
  if (ctx->nReads == 0) return fail(ctx, OIC_ERR_STATE, "no reads loaded");
  cudaSetDevice(ctx->device);
  const int K = (int)ctx->P.kmerLen;
  if (bgnID < 1) bgnID = 1;
  if (endID > ctx->nReads) endID = ctx->nReads;
  std::vector<uint32_t> reads;
  uint64_t              n = 0;
  for (uint64_t id = bgnID; id <= endID; id++) {
    const uint32_t r = (uint32_t)id - 1;
    if (ctx->len[r] < (uint32_t)K) continue;
    reads.push_back(r);
    n += ctx->len[r] - K + 1;
  }
  *nKmers = 0;
  if (n == 0) return OIC_OK;
  const uint32_t nr = (uint32_t)reads.size();
  DevBuf dReads, dHist, dK, dV, dK2, dV2, dScr, dFlags, dPos, dRun, dSel, dSelPos, dOutK, dOutC;
  auto release = [&]() {
    for (DevBuf *b : {&dReads, &dHist, &dK, &dV, &dK2, &dV2, &dScr, &dFlags, &dPos, &dRun, &dSel, &dSelPos, &dOutK, &dOutC})
      b->release();
  };
  int  rc   = OIC_OK;
  auto step = [&](cudaError_t e) {
    if (e != cudaSuccess && !rc) rc = fail(ctx, OIC_ERR_CUDA, "k-mer count: %s", cudaGetErrorString(e));
    return rc == OIC_OK;
  };

  // Key-space parts: the top 12 bits of the 2K-bit canonical key.  A pass sorts the
  // windows of consecutive parts, at most passMax of them (sized from the free memory:
  // about 48 bytes per window; OIC_KMER_PASS_WINDOWS lowers it for testing).
  const int   P     = canon_parts();
  const int   shift = std::max(0, 2 * K - 12);
  size_t freeB = 0, totalB = 0;
  cudaMemGetInfo(&freeB, &totalB);
  uint64_t passMax = std::min<uint64_t>(0xfffffffeull, (uint64_t)(0.6 * (double)freeB / 48.0));
  if (const char *e = getenv("OIC_KMER_PASS_WINDOWS")) passMax = std::max<uint64_t>(1, strtoull(e, nullptr, 10));
  std::vector<unsigned long long> hist(P, 0);
  unsigned long long              nInvalid = 0;
  if (step(dReads.ensure((size_t)nr * 4)) && step(dHist.ensure((size_t)P * 8)) &&
      step(cudaMemcpyAsync(dReads.p, reads.data(), (size_t)nr * 4, cudaMemcpyHostToDevice, ctx->st)) &&
      step(cudaMemsetAsync(dHist.p, 0, (size_t)P * 8, ctx->st)) &&
      step(cudaMemsetAsync(ctr64(ctx) + kCellsSnap, 0, 8, ctx->st))) {
    launch_canon_hist(ctx->R, dReads.as<uint32_t>(), nr, K, shift, dHist.as<unsigned long long>(),
                      ctr64(ctx) + kCellsSnap, ctx->st);
    if (step(cudaMemcpyAsync(hist.data(), dHist.p, (size_t)P * 8, cudaMemcpyDeviceToHost, ctx->st)) &&
        step(cudaMemcpyAsync(&nInvalid, ctr64(ctx) + kCellsSnap, 8, cudaMemcpyDeviceToHost, ctx->st)))
      rc = sync_check(ctx, "k-mer histogram");
  }
  // Passes: consecutive parts while their windows fit.
  std::vector<std::pair<uint32_t, uint32_t>> passes;
  uint64_t                                   biggest = 0;
  for (int p = 0; !rc && p < P;) {
    uint64_t w = 0;
    int      q = p;
    while (q < P && (q == p || w + hist[q] <= passMax)) w += hist[q++];
    if (w > 0xfffffffeull)
      rc = fail(ctx, OIC_ERR_OVERFLOW, "one k-mer key range holds more than 2^32-2 windows");
    if (w) passes.push_back({(uint32_t)p, (uint32_t)q});
    biggest = std::max(biggest, w);
    p       = q;
  }
  const uint64_t m = biggest;
  std::vector<uint64_t> outKeys;
  std::vector<uint32_t> outCounts;
  if (!rc && m &&
      !(step(dK.ensure(m * 8)) && step(dV.ensure(m * 4)) && step(dK2.ensure(m * 8)) && step(dV2.ensure(m * 4)) &&
        step(dScr.ensure(std::max(radix_sort_scratch(m), scan_u32_scratch(m)) + 256)) && step(dFlags.ensure(m * 4)) &&
        step(dPos.ensure(m * 4))))
    rc = rc ? rc : OIC_ERR_NOMEM;
  for (size_t pi = 0; !rc && pi < passes.size(); pi++) {
    unsigned long long nPass = 0;
    if (!step(cudaMemsetAsync(ctr64(ctx) + kCellsSnap, 0, 8, ctx->st))) break;
    launch_canon_emit_part(ctx->R, dReads.as<uint32_t>(), nr, K, shift, passes[pi].first, passes[pi].second,
                           dK.as<u64>(), dV.as<uint32_t>(), ctr64(ctx) + kCellsSnap, ctx->st);
    if (!step(cudaMemcpyAsync(&nPass, ctr64(ctx) + kCellsSnap, 8, cudaMemcpyDeviceToHost, ctx->st)) ||
        (rc = sync_check(ctx, "k-mer emission")))
      break;
    if (!nPass) continue;
    if (!step(radix_sort_u64_u32(dK.as<u64>(), dV.as<uint32_t>(), dK2.as<u64>(), dV2.as<uint32_t>(), nPass, 2 * K,
                                 dScr.p, ctx->st)))
      break;
    uint32_t nRuns = 0, nSel = 0;
    launch_run_starts(dK.as<u64>(), nPass, dFlags.as<uint32_t>(), ctx->st);
    if (!step(scan_u32(dFlags.as<uint32_t>(), dPos.as<uint32_t>(), nPass, ctr32(ctx) + cRecTotal, dScr.p, ctx->st)) ||
        !step(cudaMemcpyAsync(&nRuns, ctr32(ctx) + cRecTotal, 4, cudaMemcpyDeviceToHost, ctx->st)) ||
        (rc = sync_check(ctx, "k-mer runs")))
      break;
    if (!step(dRun.ensure((size_t)nRuns * 8 + 8)) || !step(dSel.ensure((size_t)nRuns * 4 + 4)) ||
        !step(dSelPos.ensure((size_t)nRuns * 4 + 4)))
      break;
    launch_run_index(dFlags.as<uint32_t>(), dPos.as<uint32_t>(), nPass, dRun.as<u64>(), ctx->st);
    launch_run_select(dRun.as<u64>(), nRuns, nPass, minCount, dSel.as<uint32_t>(), ctx->st);
    if (!step(scan_u32(dSel.as<uint32_t>(), dSelPos.as<uint32_t>(), nRuns, ctr32(ctx) + cRecTotal, dScr.p, ctx->st)) ||
        !step(cudaMemcpyAsync(&nSel, ctr32(ctx) + cRecTotal, 4, cudaMemcpyDeviceToHost, ctx->st)) ||
        (rc = sync_check(ctx, "k-mer selection")))
      break;
    if (!nSel) continue;
    if (!step(dOutK.ensure((size_t)nSel * 8)) || !step(dOutC.ensure((size_t)nSel * 4))) break;
    launch_run_compact(dK.as<u64>(), dRun.as<u64>(), nRuns, nPass, dSel.as<uint32_t>(), dSelPos.as<uint32_t>(),
                       dOutK.as<u64>(), dOutC.as<uint32_t>(), ctx->st);
    const size_t at = outKeys.size();
    outKeys.resize(at + nSel);
    outCounts.resize(at + nSel);
    if (!step(cudaMemcpyAsync(outKeys.data() + at, dOutK.p, (size_t)nSel * 8, cudaMemcpyDeviceToHost, ctx->st)) ||
        !step(cudaMemcpyAsync(outCounts.data() + at, dOutC.p, (size_t)nSel * 4, cudaMemcpyDeviceToHost, ctx->st)) ||
        (rc = sync_check(ctx, "k-mer output")))
      break;
  }
  release();
  if (rc) return rc;
  // Parts ascend with the key, and every pass's output ascends: the concatenation does.
  *nKmers = outKeys.size();
  if (outKeys.size() > maxKmers)
    return fail(ctx, OIC_ERR_OVERFLOW, "%zu k-mers found, room for %lu", outKeys.size(), (unsigned long)maxKmers);
  static const char acgt[4] = {'A', 'C', 'G', 'T'};
  for (size_t i = 0; i < outKeys.size(); i++) {
    for (int b = 0; b < K; b++) kmers[i * K + b] = acgt[(outKeys[i] >> (2 * b)) & 3];
    counts[i] = outCounts[i];
  }
  if (verbose())
    fprintf(stderr, "oic: k-mer count: %lu windows (%llu with N) in %zu passes\n", (unsigned long)n, nInvalid,
            passes.size());
  return OIC_OK;
}

int oic_set_tuning(oic_ctx *ctx, const oic_tuning *t) {
  if (!ctx) return OIC_ERR_ARG;
  if (!t) {
    ctx->tune = oic_tuning{};
    return OIC_OK;
  }
  if (t->wideThreads && (t->wideThreads < 64 || t->wideThreads > 512 || t->wideThreads % 32))
    return fail(ctx, OIC_ERR_ARG, "wideThreads must be a multiple of 32 in [64, 512]");
  if (t->wideTile && t->wideTile != 1 && t->wideTile != 2 && t->wideTile != 4)
    return fail(ctx, OIC_ERR_ARG, "wideTile must be 1, 2 or 4");
  if (t->wideBandW && (t->wideBandW < 512 || (size_t)t->wideBandW * 8 > (200u << 10)))
    return fail(ctx, OIC_ERR_ARG, "wideBandW must be in [512, 25600]");
  if (t->narrowArena && t->narrowArena < (1u << 16))
    return fail(ctx, OIC_ERR_ARG, "narrowArena must be at least 65536 cells");
  if (t->wideArena && (t->wideArena < (1u << 20) || t->wideArena > 0x7fff0000ull))
    return fail(ctx, OIC_ERR_ARG, "wideArena must be in [2^20, 2^31) cells");
  ctx->tune = *t;
  return OIC_OK;
}

int oic_get_tuning(oic_ctx *ctx, oic_tuning *t) {
  if (!ctx || !t) return OIC_ERR_ARG;
  *t = resolved_tuning(ctx);
  return OIC_OK;
}

int oic_autotune(oic_ctx *ctx, uint32_t bgnRefID, uint32_t endRefID, double *report, uint32_t maxReport,
                 uint32_t *nReport) {
  if (!ctx) return OIC_ERR_ARG;
  if (!ctx->haveBlock) return fail(ctx, OIC_ERR_STATE, "no hash block loaded");
  cudaSetDevice(ctx->device);
  std::vector<uint32_t> refs;
  int rc = eligible_refs(ctx, bgnRefID, endRefID, refs);
  if (rc) return rc;
  if (refs.empty()) return fail(ctx, OIC_ERR_ARG, "no eligible ref reads in %u-%u", bgnRefID, endRefID);
  if ((rc = ensure_pair_caps(ctx))) return rc;
  const oic_stats saved   = ctx->stats;
  const size_t    outMark = ctx->out.size();
  cudaEvent_t e0, e1, e2;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventCreate(&e2);
  uint32_t nPairs = 0, nNodes = 0;
  rc = seed_stage(ctx, refs.data(), (uint32_t)refs.size(), e0, e1, nPairs, nNodes);
  if (rc == kRetrySmaller) rc = fail(ctx, OIC_ERR_OVERFLOW, "the autotune sample's candidate pairs do not fit");

  // Length-bin boundaries to try: quantiles of the pairs' shorter read.
  std::vector<uint32_t> minLen;
  if (!rc && nPairs) {
    std::vector<PairRec> pr(nPairs);
    CK(cudaMemcpy(pr.data(), ctx->dPairs.p, (size_t)nPairs * sizeof(PairRec), cudaMemcpyDeviceToHost));
    minLen.resize(nPairs);
    for (uint32_t i = 0; i < nPairs; i++)
      minLen[i] = std::min(ctx->len[pr[i].sRead], ctx->len[ctx->blkFirst - 1 + pr[i].tStr]);
    std::sort(minLen.begin(), minLen.end());
  }

  struct Line {
    oic_tuning t;
    AlignTimes at;
  };
  std::vector<Line>     lines;
  size_t                stage1 = 0;   // lines of stage 1 (no length bin)
  std::vector<uint32_t> ref0;
  bool                  haveRef = false;
  oic_tuning base       = resolved_tuning(ctx);
  base.forceWide        = 0;
  auto measure = [&](oic_tuning t) -> int {
    std::vector<uint32_t> recs;
    AlignTimes at;
    int r = align_stage(ctx, nPairs, nNodes, t, e1, e2, recs, at);
    if (r) return r;
    if (!haveRef) {
      ref0    = recs;
      haveRef = true;
    } else if (recs != ref0) {
      return fail(ctx, OIC_ERR_DEVICE, "DP configurations disagree on the records (threads %u, tile %u)",
                  t.wideThreads, t.wideTile);
    }
    lines.push_back(Line{t, at});
    return OIC_OK;
  };
  auto total = [](const Line &l) { return (double)l.at.msNarrow + l.at.msWide; };
  if (!rc && nPairs) {
    // Stage 1: the speculative CTA bin, then CTA-wide rows with warps per pair x tile
    // width, no length bin.
    {
      oic_tuning t = base;
      t.wideMode   = 1;
      t.wideMinLen = 0xffffffffu;
      rc           = measure(t);
    }
    const uint32_t threadsGrid[] = {64, 128, 256, 512};
    const uint32_t tileGrid[]    = {1, 2, 4};
    for (uint32_t th : threadsGrid)
      for (uint32_t tl : tileGrid) {
        if (rc) break;
        oic_tuning t  = base;
        t.wideMode    = 2;
        t.wideThreads = th;
        t.wideTile    = tl;
        t.wideMinLen  = 0xffffffffu;
        t.wideCtas    = 0;
        t.wideCtas    = resolved_tuning_ctas(ctx, t);
        if ((rc = measure(t))) break;
      }
    // Stage 2: the length-bin boundary with the best CTA configuration.
    if (!rc) {
      size_t best = 0;
      for (size_t i = 1; i < lines.size(); i++)
        if (total(lines[i]) < total(lines[best])) best = i;
      stage1 = lines.size();
      const double qs[] = {0.5, 0.9, 0.99, 0.999};
      for (double q : qs) {
        oic_tuning t = lines[best].t;
        t.wideMinLen = std::max<uint32_t>(1, minLen[(size_t)(q * (minLen.size() - 1))]);
        if ((rc = measure(t))) break;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(e2);
  ctx->stats = saved;
  ctx->out.resize(outMark);
  if (rc) return rc;
  if (!lines.empty()) {
    // Best configuration without a length bin; a length bin is taken only when it is
    // more than 5 % faster (a sample is dominated by its longest pairs, so smaller
    // differences are noise).
    if (!stage1) stage1 = lines.size();
    size_t best = 0;
    for (size_t i = 1; i < stage1; i++)
      if (total(lines[i]) < total(lines[best])) best = i;
    for (size_t i = stage1; i < lines.size(); i++)
      if (total(lines[i]) < 0.95 * total(lines[best])) best = i;
    ctx->tune = lines[best].t;
    if (verbose())
      for (const Line &l : lines)
        fprintf(stderr, "oic: autotune: %s threads %u tile %u length bin %d: one-warp %.1f ms, CTA %.1f ms\n",
                l.t.wideMode == 2 ? "CTA rows" : "speculative", l.t.wideThreads, l.t.wideTile, l.t.wideMinLen == 0xffffffffu ? -1 : (int)l.t.wideMinLen,
                l.at.msNarrow, l.at.msWide);
    if (verbose())
      fprintf(stderr, "oic: autotune: %zu configurations on %u pairs; best: %u threads, tile %u, length bin %u (%.1f ms)\n",
              lines.size(), nPairs, ctx->tune.wideThreads, ctx->tune.wideTile, ctx->tune.wideMinLen,
              total(lines[best]));
  }
  uint32_t k = 0;
  for (const Line &l : lines) {
    if (!report || k >= maxReport) break;
    double *r = report + (size_t)k * 8;
    r[0] = l.t.wideMode == 2 ? l.t.wideTile : 0;
    r[1] = l.t.wideThreads;
    r[2] = l.t.wideMinLen == 0xffffffffu ? -1.0 : (double)l.t.wideMinLen;
    r[3] = l.at.msNarrow;
    r[4] = l.at.msWide;
    r[5] = total(l);
    r[6] = (double)(l.at.pairsNarrow);
    r[7] = (double)l.at.cellsWide;
    k++;
  }
  if (nReport) *nReport = report ? k : (uint32_t)lines.size();
  return OIC_OK;
}

}  // extern "C"
