// oic_pairs.cu -- per-read-pair processing: Process_Matches with the warp DP.
//
// Reference: Process_Matches (overlapInCore-Process_String_Overlaps.C:354-547) takes a
// pair's match list, repeatedly extends its longest remaining exact match with
// Extend_Alignment, keeps dovetail results in at most three distinct overlaps
// (Add_Overlap :175-244), drops the matches that lie on each alignment
// (Lies_On_Alignment :260-281), then keeps one overlap per pair (Combine_Into_One_Olap
// :40-96, or Merge_Intersecting_Olaps :106-162 with -m, Choose_Best_Partial :289-311
// with -partial) and encodes it (Output_Overlap / Output_Partial_Overlap,
// overlapInCore-Output.C:26-264).
//
// Here a persistent warp takes pairs from a queue; the node list is the array the seed
// kernel wrote in list order, with an alive flag per node.  Pairs that exceed a
// capacity of this configuration are queued for a wider configuration and leave no
// output or counts behind.
#include "oic_kernels.cuh"
#include "oic_prims.cuh"
#include "oic_extend.cuh"

namespace oic {

namespace {

constexpr int kAlignWarpsSmall = 8;   // bandW 512

struct Olap {
  int    s_lo, s_hi, t_lo, t_hi;
  double quality;
  int    delta_ct;
  int    slb, srb, tlb, trb;     // s/t left/right boundaries
  int    min_diag, max_diag;
};

// Add_Overlap (Process_String_Overlaps.C:175-244); every lane runs it identically.
__device__ __forceinline__ void add_overlap(int partial, int s_lo, int s_hi, int t_lo, int t_hi, double q, int deltaCt,
                                            Olap *o, int &ct) {
  if (!partial) {
    const int nd = t_lo - s_lo;
    for (int i = 0; i < ct; i++) {
      const int od = o[i].t_lo - o[i].s_lo;
      if ((nd > 0 && od > 0 && o[i].trb - nd - o[i].slb >= kMinIntersect) ||
          (nd <= 0 && od <= 0 && o[i].srb + nd - o[i].tlb >= kMinIntersect)) {
        if (nd < o[i].min_diag) o[i].min_diag = nd;
        if (nd > o[i].max_diag) o[i].max_diag = nd;
        if (s_lo < o[i].slb) o[i].slb = s_lo;
        if (s_hi > o[i].srb) o[i].srb = s_hi;
        if (t_lo < o[i].tlb) o[i].tlb = t_lo;
        if (t_hi > o[i].trb) o[i].trb = t_hi;
        if (q < o[i].quality) {
          o[i].s_lo = s_lo;
          o[i].s_hi = s_hi;
          o[i].t_lo = t_lo;
          o[i].t_hi = t_hi;
          o[i].quality  = q;
          o[i].delta_ct = deltaCt;
        }
        return;
      }
    }
  }
  if (ct >= kMaxDistinct) return;
  Olap &n = o[ct];
  n.s_lo = n.slb = s_lo;
  n.s_hi = n.srb = s_hi;
  n.t_lo = n.tlb = t_lo;
  n.t_hi = n.trb = t_hi;
  n.quality  = q;
  n.delta_ct = deltaCt;
  n.min_diag = n.max_diag = t_lo - s_lo;
  ct++;
}

__device__ __forceinline__ bool lies_on_alignment(const int *delta, int deltaLen, int start, int offset, int s_lo,
                                                  int t_lo) {
  int diag = t_lo - s_lo;
  const int nd = offset - start;
  for (int i = 0; i < deltaLen; i++) {
    const int dl = delta[i];
    s_lo += abs(dl);
    if (start < s_lo) return abs(nd - diag) <= kShiftSlack;
    if (dl < 0) diag++;
    else {
      s_lo++;
      diag--;
    }
  }
  return abs(nd - diag) <= kShiftSlack;
}

__device__ __forceinline__ void combine_into_one(Olap *o, int ct, int *deleted) {
  int best = 0;
  int mnd = o[0].min_diag, mxd = o[0].max_diag, slb = o[0].slb, srb = o[0].srb, tlb = o[0].tlb, trb = o[0].trb;
  for (int i = 1; i < ct; i++) {
    const int li = 1 + min(o[i].s_hi - o[i].s_lo, o[i].t_hi - o[i].t_lo);
    const int lb = 1 + min(o[best].s_hi - o[best].s_lo, o[best].t_hi - o[best].t_lo);
    if (o[i].quality < o[best].quality || (o[i].quality == o[best].quality && li > lb)) best = i;
    mnd = min(mnd, o[i].min_diag);
    mxd = max(mxd, o[i].max_diag);
    slb = min(slb, o[i].slb);
    srb = max(srb, o[i].srb);
    tlb = min(tlb, o[i].tlb);
    trb = max(trb, o[i].trb);
  }
  o[best].min_diag = mnd;
  o[best].max_diag = mxd;
  o[best].slb = slb;
  o[best].srb = srb;
  o[best].tlb = tlb;
  o[best].trb = trb;
  for (int i = 0; i < ct; i++) deleted[i] = (i != best);
}

__device__ __forceinline__ void merge_intersecting(Olap *p, int ct, int *deleted) {
  for (int i = 0; i < ct - 1; i++)
    for (int j = i + 1; j < ct; j++) {
      if (deleted[i] || deleted[j]) continue;
      const int lo = p[i].min_diag, hi = p[i].max_diag;
      if ((lo <= 0 && p[j].min_diag > 0) || (lo > 0 && p[j].min_diag <= 0)) continue;
      if ((lo >= 0 && p[j].trb - lo - p[j].slb >= kMinIntersect) ||
          (lo <= 0 && p[j].srb + lo - p[j].tlb >= kMinIntersect) ||
          (hi >= 0 && p[j].trb - hi - p[j].slb >= kMinIntersect) ||
          (hi <= 0 && p[j].srb + hi - p[j].tlb >= kMinIntersect)) {
        Olap *keep, *disc;
        if (p[i].quality < p[j].quality) { keep = p + i; disc = p + j; deleted[j] = 1; }
        else { keep = p + j; disc = p + i; deleted[i] = 1; }
        keep->min_diag = min(keep->min_diag, disc->min_diag);
        keep->max_diag = max(keep->max_diag, disc->max_diag);
        keep->slb = min(keep->slb, disc->slb);
        keep->srb = max(keep->srb, disc->srb);
        keep->tlb = min(keep->tlb, disc->tlb);
        keep->trb = max(keep->trb, disc->trb);
      }
    }
}

__device__ __forceinline__ void choose_best_partial(const Olap *o, int ct, int *deleted) {
  int best = 0;
  const double mb0 =
      __dmul_rn(__dsub_rn(1.0, o[0].quality), (double)(2 + o[0].s_hi - o[0].s_lo + o[0].t_hi - o[0].t_lo));
  for (int i = 1; i < ct; i++) {
    const double mb =
        __dmul_rn(__dsub_rn(1.0, o[i].quality), (double)(2 + o[i].s_hi - o[i].s_lo + o[i].t_hi - o[i].t_lo));
    if (mb0 < mb || (mb0 == mb && o[i].quality < o[best].quality)) best = i;
  }
  for (int i = 0; i < ct; i++) deleted[i] = (i != best);
}

// AS_OVS_encodeEvalue (ovOverlap.H:35).
__device__ __forceinline__ u32 encode_evalue(double q) {
  return (q < 65535 / 100000.0) ? (u32)__dadd_rn(__dmul_rn(100000.0, q), 0.5) : 65535u;
}

// The span is accumulated in a 21-bit field one term at a time (Output.C:41-45).
__device__ __forceinline__ u32 span21(const Olap &o) {
  const u32 M21 = (1u << 21) - 1;
  u32 sp = (u32)(o.s_hi - o.s_lo) & M21;
  sp     = (sp + (u32)(o.t_hi - o.t_lo)) & M21;
  sp     = (sp + (u32)o.delta_ct) & M21;
  return sp / 2;
}

__device__ __forceinline__ void put_record(u32 *dst, u32 a, u32 b, u32 ahg5, u32 ahg3, u32 bhg5, u32 bhg3, u32 span,
                                           u32 evalue, u32 flipped, u32 forOBT, u32 forDUP, u32 forUTG) {
  const u64 M21 = (1u << 21) - 1;
  const u64 d0 = ((u64)ahg5 & M21) | (((u64)ahg3 & M21) << 21) | (((u64)evalue & 0xffff) << 42) |
                 ((u64)(flipped & 1) << 58) | ((u64)(forOBT & 1) << 59) | ((u64)(forDUP & 1) << 60) |
                 ((u64)(forUTG & 1) << 61);
  const u64 d1 = ((u64)bhg5 & M21) | (((u64)bhg3 & M21) << 21) | (((u64)span & M21) << 42);
  dst[0] = a;
  dst[1] = b;
  dst[2] = (u32)(d0 >> 32);
  dst[3] = (u32)d0;
  dst[4] = (u32)(d1 >> 32);
  dst[5] = (u32)d1;
}

struct PairCounts {
  unsigned long long v[kStCount];
};

// Per-warp shared state of the pair driver (kept out of registers).
struct PairSmem {
  Olap               olap[kMaxDistinct];
  int                nOlap;
  int                nExt;       // extensions run for the pair in flight
  int                firstHit;   // index of its first extension that added an overlap, -1 none
  unsigned long long cellsFirst; // DP cells of its first extension
  PairCounts         pc;    // counts of the pair in flight
  PairCounts         acc;   // committed counts of the warp
};

// Output_Overlap (Output.C:26-191).
__device__ void output_overlap(u32 *dst, u32 sID, int sLen, int rev, u32 tID, int tLen, const Olap &o,
                               PairCounts &pc) {
  const int  sRH = sLen - o.s_hi - 1, tRH = tLen - o.t_hi - 1;
  const bool sLeft = (o.s_lo > o.t_lo) || (o.s_lo == o.t_lo && sRH > tRH);
  const u32  a = sLeft ? sID : tID, b = sLeft ? tID : sID;
  char orient;
  int  ahg, bhg;
  if (sLeft) {
    orient = rev ? 'O' : 'N';
    ahg    = o.s_lo;
    bhg    = tRH - sRH;
  } else {
    orient = rev ? 'I' : 'N';
    ahg    = o.t_lo;
    bhg    = sRH - tRH;
  }
  if (orient == 'O' && sRH >= tRH) {
    orient = 'I';
    ahg    = -(tRH - sRH);
    bhg    = -(o.s_lo);
  }
  int ah, bh;
  u32 flipped;
  if (orient == 'O') { ah = -bhg; bh = -ahg; flipped = 1; }
  else { ah = ahg; bh = bhg; flipped = (orient == 'I'); }
  const u32 ahg5 = ah < 0 ? 0 : (u32)ah, bhg5 = ah < 0 ? (u32)(-ah) : 0;
  const u32 bhg3 = bh < 0 ? 0 : (u32)bh, ahg3 = bh < 0 ? (u32)(-bh) : 0;
  put_record(dst, a, b, ahg5, ahg3, bhg5, bhg3, span21(o), encode_evalue(o.quality), flipped, 0, 0, 1);
  pc.v[kStTotal]++;
  if (bhg <= 0) pc.v[kStContained]++;
  else pc.v[kStDovetail]++;
}

// Output_Partial_Overlap (Output.C:195-264).
__device__ void output_partial(u32 *dst, u32 sID, u32 tID, int rev, const Olap &o, int sLen, int tLen,
                               PairCounts &pc) {
  u32 ahg5, ahg3, bhg5, bhg3;
  if (!rev) {
    ahg5 = (u32)o.s_lo;
    ahg3 = (u32)(sLen - (o.s_hi + 1));
    bhg5 = (u32)o.t_lo;
    bhg3 = (u32)(tLen - (o.t_hi + 1));
  } else {
    ahg5 = (u32)(sLen - (o.s_hi + 1));
    ahg3 = (u32)o.s_lo;
    bhg5 = (u32)(tLen - (o.t_hi + 1));
    bhg3 = (u32)o.t_lo;
  }
  put_record(dst, sID, tID, ahg5, ahg3, bhg5, bhg3, span21(o), encode_evalue(o.quality), rev ? 1u : 0u, 1, 1, 0);
  pc.v[kStTotal]++;
}


// Process_Matches for one pair.  Counts go to ps.pc, records (lane 0) to recOut.
// Returns false on a capacity overflow: the caller then discards ps.pc and the records.
template <bool GROUP, bool FIRST16 = false>
__device__ bool process_pair(WarpDP &w, PairSmem &ps, const ReadsDev &R, const TableDev &Tb, const PairRec &pr,
                             const int4 *nodesAll, u32 *recOut, u32 &nRec, int extLimit) {
  const int lane = threadIdx.x & 31;
  const DevParams &P = w.P;
  if (lane == 0) {
#pragma unroll
    for (int i = 0; i < kStCount; i++) ps.pc.v[i] = 0;
    ps.nOlap      = 0;
    ps.nExt       = 0;
    ps.firstHit   = -1;
    ps.cellsFirst = 0;
  }
  __syncwarp();
  nRec = 0;

  const u32 sRead = pr.sRead;
  const int rev   = pr.flags & 1;
  const int cons  = (pr.flags >> 1) & 1;
  const bool segL = (pr.flags >> 2) & 1, segR = (pr.flags >> 3) & 1;
  const int sLen  = (int)R.len[sRead];
  const u32 tRead = Tb.sread[pr.tStr];
  const int tLen  = (int)R.len[tRead];

  // --minkmers (computeMinimumKmers, Process_String_Overlaps.C:21-33, :618-621)
  if (P.minKmers) {
    double ol = (double)(pr.diagEnd - pr.diagBgn);
    if (ol < 0) ol = -ol;
    unsigned long long ex = 0;
    if (!(ol < (double)P.kmerLen))
      ex = (unsigned long long)(long long)(int)floor(
          __dmul_rn(P.kmerExpect, __dadd_rn(__dsub_rn(ol, (double)P.kmerLen), 1.0)));
    const unsigned long long need = P.minKmers > ex ? P.minKmers : ex;
    if (need > (unsigned long long)(long long)pr.diagCt) {
      if (lane == 0) ps.pc.v[kStSkipped] = 1;
      __syncwarp();
      return true;
    }
  }

  const int4 *nodes = nodesAll + pr.nodeOff;
  const int   cnt   = (int)pr.nodeCnt;
  if (cnt <= 0) {
    if (lane == 0) ps.pc.v[kStWithoutOlap] = 1;
    __syncwarp();
    return true;
  }

  // Hopeless check for a single match (:384-415).
  if (P.hopeless && cnt == 1 && !P.partial) {
    const int4 m = nodes[0];   // x offset, y len, z start
    const bool tLs = Tb.lscr[pr.tStr] != 0, tRs = Tb.rscr[pr.tStr] != 0;
    bool hopeless = false;
    const int sHead = m.z, tHead = m.x;
    if (sHead <= tHead) {
      if (sHead > kHopelessMatch && !segL) hopeless = true;
    } else {
      if (tHead > kHopelessMatch && !tLs) hopeless = true;
    }
    const int sTail = sLen - sHead - m.y + 1, tTail = tLen - tHead - m.y + 1;
    if (sTail <= tTail) {
      if (sTail > kHopelessMatch && !segR) hopeless = true;
    } else {
      if (tTail > kHopelessMatch && !tRs) hopeless = true;
    }
    if (hopeless) {
      if (lane == 0) ps.pc.v[kStWithoutOlap] = 1;
      __syncwarp();
      return true;
    }
  }

  if (cnt > w.cap.nodeCap) {
    w.err |= kErrNodesPerPair;
    return false;
  }
  for (int i = lane; i < cnt; i += 32) w.sc.alive[i] = 1;
  __syncwarp();

  const SeqView S = make_view(R, sRead, rev);
  const SeqView T = make_view(R, tRead, 0);
  const unsigned long long cells0 = w.cells, slides0 = w.slides, rows0 = w.rows;

  while (true) {
    // Longest remaining match, first in list order on ties (:424-431).
    int myLen = -1, myIdx = INT_MAX;
    for (int i = lane; i < cnt; i += 32)
      if (w.sc.alive[i]) {
        const int len = nodes[i].y;
        if (len > myLen) {
          myLen = len;
          myIdx = i;
        }
      }
    const int maxLen = __reduce_max_sync(0xffffffffu, myLen);
    if (maxLen < 0) break;
    const int li = __reduce_min_sync(0xffffffffu, myLen == maxLen ? myIdx : INT_MAX);
    const int4 lm = nodes[li];

    int sLo = 0, sHi = 0, tLo = 0, tHi = 0, errors = 0;
    const int kind = warp_extend<GROUP, FIRST16>(w, S, sLen, T, tLen, lm.z, lm.x, lm.y, sLo, sHi, tLo, tHi, errors);
    if (w.err) {
      w.cells  = cells0;
      w.slides = slides0;
      w.rows   = rows0;
      return false;
    }
    const bool dov = (kind == kDovetail) || P.partial;
    if (lane == 0) {
      ps.pc.v[kStExtensions]++;
      bool added = false;
      if (dov && 1 + sHi - sLo >= P.minOlapLen && 1 + tHi - tLo >= P.minOlapLen) {
        const int    olapLen = 1 + min(sHi - sLo, tHi - tLo);
        const double quality = __ddiv_rn((double)errors, (double)olapLen);
        if (errors <= error_bound(olapLen, P.maxErate)) {
          add_overlap(P.partial, sLo, sHi, tLo, tHi, quality, w.leftLen, ps.olap, ps.nOlap);
          added = true;
        }
      }
      if (ps.nExt == 0) ps.cellsFirst = w.cells - cells0;
      if (added && ps.firstHit < 0) ps.firstHit = ps.nExt;
      ps.nExt++;
    }
    if (cons) break;
    // Early exit (learned filter's single-extension tier): stop once extLimit
    // extensions have run without an overlap.
    if (extLimit > 0) {
      __syncwarp();
      if (ps.nExt >= extLimit && ps.nOlap == 0) break;
    }

    // Drop the longest match and every match that lies on the alignment (:476-490).
    for (int i = lane; i < cnt; i += 32) {
      if (!w.sc.alive[i]) continue;
      const int4 q = nodes[i];
      bool rm = (i == li);
      if (!rm && dov && sLo - kShiftSlack <= q.z && q.z + q.y <= (sHi + 1) + kShiftSlack - 1 &&
          lies_on_alignment(w.sc.deltaL, w.leftLen, q.z, q.x, sLo, tLo))
        rm = true;
      if (rm) w.sc.alive[i] = 0;
    }
    __syncwarp();
  }

  if (lane == 0) {
    const u32 sID = sRead + 1, tID = tRead + 1;
    int nOut = 0;
    const int nOlap = ps.nOlap;
    if (nOlap > 0) {
      int deleted[kMaxDistinct] = {0, 0, 0};
      if (P.partial) {
        if (P.unique) choose_best_partial(ps.olap, nOlap, deleted);
      } else {
        if (P.unique) combine_into_one(ps.olap, nOlap, deleted);
        else merge_intersecting(ps.olap, nOlap, deleted);
      }
      for (int i = 0; i < nOlap; i++)
        if (!deleted[i]) {
          if (P.partial) output_partial(recOut + nOut * 6, sID, tID, rev, ps.olap[i], sLen, tLen, ps.pc);
          else output_overlap(recOut + nOut * 6, sID, sLen, rev, tID, tLen, ps.olap[i], ps.pc);
          nOut++;
        }
    }
    if (nOut == 0) ps.pc.v[kStWithoutOlap]++;
    else {
      ps.pc.v[kStWithOlap]++;
      if (nOut > 1) ps.pc.v[kStMulti]++;
    }
    nRec = (u32)nOut;
  }
  __syncwarp();
  return true;
}

// The work loop of one warp: pairs from the shared work list until it is empty.
template <bool GROUP, bool FIRST16 = false>
static __device__ __forceinline__ void align_loop(WarpDP &w, PairSmem &ps, const ReadsDev &R, const TableDev &Tb,
                                                  const PairRec *pairs, const u32 *work, u32 nWork, u32 *workCounter,
                                                  const int4 *nodes, const AlignOut &out) {
  const int lane = threadIdx.x & 31;
  // Inside a captured graph the list's length and start are known only on the device.
  if (out.nWorkDev) nWork = *out.nWorkDev;
  if (out.workOffDev) work += *out.workOffDev;
  if (lane == 0)
    for (int i = 0; i < kStCount; i++) ps.acc.v[i] = 0;
  __syncwarp();

  while (true) {
    u32 k = 0;
    if (lane == 0) k = atomicAdd(workCounter, 1u);
    k = __shfl_sync(0xffffffffu, k, 0);
    if (k >= nWork) break;
    const u32 pi = work[k];
    const PairRec pr = pairs[pi];
    u32 nRec = 0;
    w.err = 0;
    const unsigned long long cellsBefore = w.cells;
    int extLimit = 0;   // 0: every match node may be extended (the reference's rule)
    if (out.tierLogit && out.tierLogit[pi] < out.tierThr) extLimit = out.tierBudget;
    const bool ok = process_pair<GROUP, FIRST16>(w, ps, R, Tb, pr, nodes, out.rec + (u64)pi * 18, nRec, extLimit);
    if (lane == 0) {
      if (ok) {
        if (nRec == 0) ps.pc.v[kStCellsNoOlap] += w.cells - cellsBefore;
        out.cnt[pi] = nRec;
        if (out.cells) {
          const unsigned long long c = w.cells - cellsBefore;
          out.cells[pi] = c > 0xffffffffull ? 0xffffffffu : (u32)c;
          out.ext[pi]   = make_int4(ps.nExt, ps.firstHit,
                                    ps.cellsFirst > 0x7fffffffull ? 0x7fffffff : (int)ps.cellsFirst, extLimit);
        }
        for (int i = 0; i < kStCount; i++) ps.acc.v[i] += ps.pc.v[i];
      } else {
        out.cnt[pi] = 0;
        u32 slot = atomicAdd(out.overflowCount, 1u);
        out.overflow[slot] = pi;
        atomicOr(out.err, w.err);
      }
    }
    __syncwarp();
  }
  // Cells and rows are warp-uniform; slides are counted per lane.
  const unsigned long long slidesWarp = warp_sum64(w.slides);
  if (lane == 0) {
    ps.acc.v[kStCells] += w.cells;
    ps.acc.v[kStSlides] += slidesWarp;
    ps.acc.v[kStRows] += w.rows;
    for (int i = 0; i < kStCount; i++)
      if (ps.acc.v[i]) atomicAdd(&out.stats[i], ps.acc.v[i]);
  }
}

// One pair per warp, WARPS warps per CTA; FIRST16: slides start with a 16-base compare.
template <int BANDW, int WARPS, bool FIRST16>
__global__ void __launch_bounds__(WARPS * 32, (WARPS > 1 ? OIC_ALIGN_MIN_BLOCKS : 1)) align_kernel(ReadsDev R, TableDev Tb, DevParams P, const int *eml,
                                                           const PairRec *pairs, const u32 *work, u32 nWork,
                                                           u32 *workCounter, const int4 *nodes, WarpScratch scBase,
                                                           AlignCaps cap, AlignOut out) {
  extern __shared__ int smemRows[];
  __shared__ PairSmem pairSmem[WARPS];
  const int wib = threadIdx.x >> 5;
  const u64 gw  = (u64)blockIdx.x * WARPS + wib;
  WarpDP w;
  int *smA = smemRows + (size_t)wib * 2 * BANDW;
  warp_dp_init(w, warp_scratch(scBase, cap, gw), cap, smA, smA + BANDW, eml, P);
  align_loop<false, FIRST16>(w, pairSmem[wib], R, Tb, pairs, work, nWork, workCounter, nodes, out);
}

// One pair per CTA (the wide bins): warp 0 runs the pair logic, and every error-row
// loop runs on all blockDim.x threads (group_rows, U diagonals per thread per pass);
// the other warps wait for row loops in group_worker.  The row buffers are
// cap.bandW ints each in dynamic shared memory.  Scratch is per CTA.
__global__ void __launch_bounds__(512, 1) align_group_kernel(ReadsDev R, TableDev Tb, DevParams P, const int *eml,
                                                              const PairRec *pairs, const u32 *work, u32 nWork,
                                                              u32 *workCounter, const int4 *nodes, WarpScratch scBase,
                                                              AlignCaps cap, AlignOut out, int U) {
  extern __shared__ int smemRows[];
  __shared__ PairSmem    pairSmem;
  __shared__ GroupShared gs;
  const WarpScratch sc = warp_scratch(scBase, cap, blockIdx.x);
  if (threadIdx.x >= 32) {
    unsigned long long slides = 0;
    group_worker(gs, sc, cap, eml, slides);
    slides = warp_sum64(slides);
    if ((threadIdx.x & 31) == 0 && slides) atomicAdd(&out.stats[kStSlides], slides);
    return;
  }
  WarpDP w;
  warp_dp_init(w, sc, cap, smemRows, smemRows + cap.bandW, eml, P);
  w.gs       = &gs;
  w.gThreads = blockDim.x;
  w.gU       = U;
  align_loop<true>(w, pairSmem, R, Tb, pairs, work, nWork, workCounter, nodes, out);
  if (threadIdx.x == 0) gs.cmd = kGroupExit;
  __syncwarp();
  group_bar(1, blockDim.x);
}

// ---------------------------------------------------------------------------------
// Speculative CTA bin: one pair per CTA of kSpecWarps warps, each warp running whole
// extensions with the one-warp DP.  Process_Matches extends, one after another, the
// longest alive match node (first in list order on ties) and then removes the nodes
// that lie on its alignment (Process_String_Overlaps.C:420-491).  An extension depends
// only on its own node, and removal only ever takes nodes away, so the order of
// extensions is the order of the nodes by (length descending, list index ascending),
// skipping removed nodes.  Each round, warp 0 picks the next kSpecWarps alive nodes in
// that order, every warp extends one of them, and warp 0 replays the round in order:
// a node removed by an earlier extension of the round is skipped (its result is
// discarded), the others are committed exactly as the sequential loop commits them.
// Only committed extensions count as DP work.  Consistent pairs (a single extension)
// and pairs under the filter's extension budget take one node per round.
constexpr int kSpecWarps = 8;
enum { kSpecExtend = 1, kSpecExit = 2 };

struct SpecRes {
  int sLo, sHi, tLo, tHi, errors, kind, leftLen;
  u32 err;
  unsigned long long cells, slides, rows;
};

struct SpecShared {
  int         cmd;
  int         nCand;
  int         cand[kSpecWarps];
  SeqView     S, T;
  int         sLen, tLen;
  const int4 *nodes;
  SpecRes     res[kSpecWarps];
};

// Warp `wib` extends node cand[wib] of the posted pair into res[wib]; its deltas stay
// in its scratch (sc.deltaL) until the next round.
static __device__ __forceinline__ void spec_work(WarpDP &w, SpecShared &ss, int wib) {
  const int lane = threadIdx.x & 31;
  if (wib >= ss.nCand) return;
  const int4 lm = ss.nodes[ss.cand[wib]];
  const unsigned long long c0 = w.cells, r0 = w.rows, s0 = w.slides;
  w.err = 0;
  int sLo = 0, sHi = 0, tLo = 0, tHi = 0, errors = 0;
  const int kind = warp_extend<false>(w, ss.S, ss.sLen, ss.T, ss.tLen, lm.z, lm.x, lm.y, sLo, sHi, tLo, tHi, errors);
  const unsigned long long sl = warp_sum64(w.slides - s0);
  if (lane == 0) {
    SpecRes &r = ss.res[wib];
    r.sLo = sLo; r.sHi = sHi; r.tLo = tLo; r.tHi = tHi; r.errors = errors; r.kind = kind;
    r.leftLen = w.leftLen;
    r.err     = w.err;
    r.cells   = w.cells - c0;
    r.rows    = w.rows - r0;
    r.slides  = sl;
  }
  __syncwarp();
}

// Process_Matches for one pair on warp 0 of a speculative CTA (same rules and outputs as
// process_pair); wsc[j] is warp j's scratch (for its deltas).  Committed DP work is
// added to ps.pc.  Returns false on a capacity overflow.
__device__ bool process_pair_spec(WarpDP &w, PairSmem &ps, SpecShared &ss, const WarpScratch *wsc, int nThr,
                                  const ReadsDev &R, const TableDev &Tb, const PairRec &pr, const int4 *nodesAll,
                                  u32 *recOut, u32 &nRec, int extLimit, unsigned long long &cellsPair) {
  const int lane = threadIdx.x & 31;
  const DevParams &P = w.P;
  if (lane == 0) {
#pragma unroll
    for (int i = 0; i < kStCount; i++) ps.pc.v[i] = 0;
    ps.nOlap      = 0;
    ps.nExt       = 0;
    ps.firstHit   = -1;
    ps.cellsFirst = 0;
  }
  __syncwarp();
  nRec      = 0;
  cellsPair = 0;

  const u32 sRead = pr.sRead;
  const int rev   = pr.flags & 1;
  const int cons  = (pr.flags >> 1) & 1;
  const bool segL = (pr.flags >> 2) & 1, segR = (pr.flags >> 3) & 1;
  const int sLen  = (int)R.len[sRead];
  const u32 tRead = Tb.sread[pr.tStr];
  const int tLen  = (int)R.len[tRead];

  // --minkmers (computeMinimumKmers, Process_String_Overlaps.C:21-33, :618-621)
  if (P.minKmers) {
    double ol = (double)(pr.diagEnd - pr.diagBgn);
    if (ol < 0) ol = -ol;
    unsigned long long ex = 0;
    if (!(ol < (double)P.kmerLen))
      ex = (unsigned long long)(long long)(int)floor(
          __dmul_rn(P.kmerExpect, __dadd_rn(__dsub_rn(ol, (double)P.kmerLen), 1.0)));
    const unsigned long long need = P.minKmers > ex ? P.minKmers : ex;
    if (need > (unsigned long long)(long long)pr.diagCt) {
      if (lane == 0) ps.pc.v[kStSkipped] = 1;
      __syncwarp();
      return true;
    }
  }

  const int4 *nodes = nodesAll + pr.nodeOff;
  const int   cnt   = (int)pr.nodeCnt;
  if (cnt <= 0) {
    if (lane == 0) ps.pc.v[kStWithoutOlap] = 1;
    __syncwarp();
    return true;
  }

  // Hopeless check for a single match (:384-415).
  if (P.hopeless && cnt == 1 && !P.partial) {
    const int4 m = nodes[0];
    const bool tLs = Tb.lscr[pr.tStr] != 0, tRs = Tb.rscr[pr.tStr] != 0;
    bool hopeless = false;
    const int sHead = m.z, tHead = m.x;
    if (sHead <= tHead) {
      if (sHead > kHopelessMatch && !segL) hopeless = true;
    } else {
      if (tHead > kHopelessMatch && !tLs) hopeless = true;
    }
    const int sTail = sLen - sHead - m.y + 1, tTail = tLen - tHead - m.y + 1;
    if (sTail <= tTail) {
      if (sTail > kHopelessMatch && !segR) hopeless = true;
    } else {
      if (tTail > kHopelessMatch && !tRs) hopeless = true;
    }
    if (hopeless) {
      if (lane == 0) ps.pc.v[kStWithoutOlap] = 1;
      __syncwarp();
      return true;
    }
  }

  if (cnt > w.cap.nodeCap) {
    w.err |= kErrNodesPerPair;
    return false;
  }
  // alive: 1 alive, 2 alive and picked for the current round, 0 removed.
  unsigned char *alive = w.sc.alive;
  for (int i = lane; i < cnt; i += 32) alive[i] = 1;
  if (lane == 0) {
    ss.S     = make_view(R, sRead, rev);
    ss.T     = make_view(R, tRead, 0);
    ss.sLen  = sLen;
    ss.tLen  = tLen;
    ss.nodes = nodes;
  }
  __syncwarp();
  const int want = (cons || extLimit > 0) ? 1 : kSpecWarps;
  bool done = false, failed = false;

  while (!done) {
    // The next `want` alive nodes by (length descending, list index ascending).
    int nC = 0;
    for (; nC < want; nC++) {
      int myLen = -1, myIdx = INT_MAX;
      for (int i = lane; i < cnt; i += 32)
        if (alive[i] == 1) {
          const int len = nodes[i].y;
          if (len > myLen) {
            myLen = len;
            myIdx = i;
          }
        }
      const int maxLen = __reduce_max_sync(0xffffffffu, myLen);
      if (maxLen < 0) break;
      const int li = __reduce_min_sync(0xffffffffu, myLen == maxLen ? myIdx : INT_MAX);
      if (lane == 0) {
        alive[li]   = 2;
        ss.cand[nC] = li;
      }
      __syncwarp();
    }
    if (nC == 0) break;
    if (lane == 0) {
      ss.nCand = nC;
      ss.cmd   = kSpecExtend;
    }
    __syncwarp();
    group_bar(1, nThr);
    spec_work(w, ss, 0);
    group_bar(2, nThr);

    for (int j = 0; j < nC; j++) {
      const int li = ss.cand[j];
      if (alive[li] != 2) continue;            // removed by an earlier extension of the round
      const SpecRes &r = ss.res[j];
      if (r.err) {
        w.err |= r.err;
        failed = true;
        done   = true;
        break;
      }
      cellsPair += r.cells;
      const bool dov = (r.kind == kDovetail) || P.partial;
      if (lane == 0) {
        ps.pc.v[kStExtensions]++;
        ps.pc.v[kStCells] += r.cells;
        ps.pc.v[kStSlides] += r.slides;
        ps.pc.v[kStRows] += r.rows;
        bool added = false;
        if (dov && 1 + r.sHi - r.sLo >= P.minOlapLen && 1 + r.tHi - r.tLo >= P.minOlapLen) {
          const int    olapLen = 1 + min(r.sHi - r.sLo, r.tHi - r.tLo);
          const double quality = __ddiv_rn((double)r.errors, (double)olapLen);
          if (r.errors <= error_bound(olapLen, P.maxErate)) {
            add_overlap(P.partial, r.sLo, r.sHi, r.tLo, r.tHi, quality, r.leftLen, ps.olap, ps.nOlap);
            added = true;
          }
        }
        if (ps.nExt == 0) ps.cellsFirst = r.cells;
        if (added && ps.firstHit < 0) ps.firstHit = ps.nExt;
        ps.nExt++;
      }
      __syncwarp();
      if (cons) { done = true; break; }
      if (extLimit > 0 && ps.nExt >= extLimit && ps.nOlap == 0) { done = true; break; }
      // Drop the extended node and every node that lies on its alignment (:476-490).
      const int *dl = wsc[j].deltaL;
      for (int i = lane; i < cnt; i += 32) {
        if (!alive[i]) continue;
        const int4 q = nodes[i];
        bool rm = (i == li);
        if (!rm && dov && r.sLo - kShiftSlack <= q.z && q.z + q.y <= (r.sHi + 1) + kShiftSlack - 1 &&
            lies_on_alignment(dl, r.leftLen, q.z, q.x, r.sLo, r.tLo))
          rm = true;
        if (rm) alive[i] = 0;
      }
      __syncwarp();
    }
  }
  if (failed) return false;

  if (lane == 0) {
    const u32 sID = sRead + 1, tID = tRead + 1;
    int nOut = 0;
    const int nOlap = ps.nOlap;
    if (nOlap > 0) {
      int deleted[kMaxDistinct] = {0, 0, 0};
      if (P.partial) {
        if (P.unique) choose_best_partial(ps.olap, nOlap, deleted);
      } else {
        if (P.unique) combine_into_one(ps.olap, nOlap, deleted);
        else merge_intersecting(ps.olap, nOlap, deleted);
      }
      for (int i = 0; i < nOlap; i++)
        if (!deleted[i]) {
          if (P.partial) output_partial(recOut + nOut * 6, sID, tID, rev, ps.olap[i], sLen, tLen, ps.pc);
          else output_overlap(recOut + nOut * 6, sID, sLen, rev, tID, tLen, ps.olap[i], ps.pc);
          nOut++;
        }
    }
    if (nOut == 0) ps.pc.v[kStWithoutOlap]++;
    else {
      ps.pc.v[kStWithOlap]++;
      if (nOut > 1) ps.pc.v[kStMulti]++;
    }
    nRec = (u32)nOut;
  }
  __syncwarp();
  return true;
}

// The speculative CTA bin (see above): warp 0 takes pairs from the work list and runs
// their pair logic; all kSpecWarps warps run the extensions of each round.  Warp j's
// scratch is scBase's warp blockIdx.x * kSpecWarps + j; the pair's alive flags are in
// the nodeCap * kSpecWarps bytes that start at warp 0's.
__global__ void __launch_bounds__(kSpecWarps * 32, OIC_ALIGN_MIN_BLOCKS) align_spec_kernel(
    ReadsDev R, TableDev Tb, DevParams P, const int *eml, const PairRec *pairs, const u32 *work, u32 nWork,
    u32 *workCounter, const int4 *nodes, WarpScratch scBase, AlignCaps cap, AlignOut out) {
  extern __shared__ int smemRows[];
  __shared__ PairSmem    ps;
  __shared__ SpecShared  ss;
  __shared__ WarpScratch wsc[kSpecWarps];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nThr = blockDim.x;
  const u64 gw = (u64)blockIdx.x * kSpecWarps + wib;
  WarpDP w;
  int *smA = smemRows + (size_t)wib * 2 * 512;
  warp_dp_init(w, warp_scratch(scBase, cap, gw), cap, smA, smA + 512, eml, P);
  if (lane == 0) wsc[wib] = w.sc;
  w.cap.nodeCap = cap.nodeCap * kSpecWarps;   // warp 0's alive flags span the CTA's slots
  __syncthreads();

  if (wib != 0) {
    while (true) {
      group_bar(1, nThr);
      if (ss.cmd != kSpecExtend) break;
      spec_work(w, ss, wib);
      group_bar(2, nThr);
    }
    return;
  }

  // Warp 0: the pairs.
  if (out.nWorkDev) nWork = *out.nWorkDev;
  if (out.workOffDev) work += *out.workOffDev;
  if (lane == 0)
    for (int i = 0; i < kStCount; i++) ps.acc.v[i] = 0;
  __syncwarp();
  while (true) {
    u32 k = 0;
    if (lane == 0) k = atomicAdd(workCounter, 1u);
    k = __shfl_sync(0xffffffffu, k, 0);
    if (k >= nWork) break;
    const u32 pi = work[k];
    const PairRec pr = pairs[pi];
    u32 nRec = 0;
    w.err = 0;
    int extLimit = 0;
    if (out.tierLogit && out.tierLogit[pi] < out.tierThr) extLimit = out.tierBudget;
    unsigned long long cellsPair = 0;
    const bool ok = process_pair_spec(w, ps, ss, wsc, nThr, R, Tb, pr, nodes, out.rec + (u64)pi * 18, nRec, extLimit,
                                      cellsPair);
    if (lane == 0) {
      if (ok) {
        if (nRec == 0) ps.pc.v[kStCellsNoOlap] += cellsPair;
        out.cnt[pi] = nRec;
        if (out.cells) {
          out.cells[pi] = cellsPair > 0xffffffffull ? 0xffffffffu : (u32)cellsPair;
          out.ext[pi]   = make_int4(ps.nExt, ps.firstHit,
                                    ps.cellsFirst > 0x7fffffffull ? 0x7fffffff : (int)ps.cellsFirst, extLimit);
        }
        for (int i = 0; i < kStCount; i++) ps.acc.v[i] += ps.pc.v[i];
      } else {
        out.cnt[pi] = 0;
        u32 slot = atomicAdd(out.overflowCount, 1u);
        out.overflow[slot] = pi;
        atomicOr(out.err, w.err);
      }
    }
    __syncwarp();
  }
  if (lane == 0) {
    ss.cmd = kSpecExit;
    for (int i = 0; i < kStCount; i++)
      if (ps.acc.v[i]) atomicAdd(&out.stats[i], ps.acc.v[i]);
  }
  __syncwarp();
  group_bar(1, nThr);
}

// Work list order: key = bin << 30 | (2^30 - 1 - match nodes), value = pair index, so
// the pairs sort by bin and, inside a bin, the pairs with the most match nodes (the most
// extensions) come first.  Bin 0: the one-warp DP; bin 1: the CTA DP, for pairs whose
// shorter read has at least wideMinLen bases; bin 2: dropped by the filter (logit
// non-null and below logitThr).  binCount[0..1] (zeroed by the caller) get the sizes
// of bins 0 and 1.
__global__ void work_keys_kernel(const PairRec *pairs, u32 n, const float *logit, float logitThr, const u32 *readLen,
                                 const u32 *strRead, u32 wideMinLen, u32 *binCount, unsigned long long *keys,
                                 u32 *vals, const u32 *nDev) {
  if (nDev && *nDev < n) n = *nDev;
  const u32 stride = gridDim.x * blockDim.x;
  const int lane   = threadIdx.x & 31;
  for (u32 i0 = blockIdx.x * blockDim.x; i0 < n; i0 += stride) {
    const u32 i   = i0 + threadIdx.x;
    u32       bin = 3;
    if (i < n) {
      const PairRec pr = pairs[i];
      if (logit && logit[i] < logitThr) bin = 2;
      else {
        const u32 ls = readLen[pr.sRead], lt = readLen[strRead[pr.tStr]];
        bin          = (ls < lt ? ls : lt) >= wideMinLen ? 1 : 0;
      }
      const u32 nc = pr.nodeCnt < 0x3fffffffu ? pr.nodeCnt : 0x3fffffffu;
      keys[i]      = ((unsigned long long)bin << 30) | (0x3fffffffu - nc);
      vals[i]      = i;
    }
    const unsigned b0 = __ballot_sync(0xffffffffu, bin == 0), b1 = __ballot_sync(0xffffffffu, bin == 1);
    if (lane == 0) {
      if (b0) atomicAdd(&binCount[0], (u32)__popc(b0));
      if (b1) atomicAdd(&binCount[1], (u32)__popc(b1));
    }
  }
}

// The CTA-bin list of a captured batch: the one-warp overflow (ovf[0 .. *ovfCount))
// appended behind the bin's own pairs (work[b0 .. b0 + b1), b0/b1 = binCount[0..1]);
// its length goes to *wideN, and the counters the CTA pass uses are cleared.  One block.
__global__ void append_overflow_kernel(u32 *work, const u32 *binCount, const u32 *ovf, u32 *ovfCount, u32 *wideN,
                                       u32 *workCounter, u32 *err) {
  __shared__ u32 n;
  if (threadIdx.x == 0) n = *ovfCount;
  __syncthreads();
  const u32 b0 = binCount[0], b1 = binCount[1];
  for (u32 i = threadIdx.x; i < n; i += blockDim.x) work[b0 + b1 + i] = ovf[i];
  __syncthreads();
  if (threadIdx.x == 0) {
    *wideN       = b1 + n;
    *ovfCount    = 0;
    *workCounter = 0;
    *err         = 0;
  }
}

// keys[i] = 2^30 - 1 - match nodes of pair list[i], vals[i] = list[i]: the order that
// puts a list's pairs with the most match nodes first.
__global__ void list_keys_kernel(const PairRec *pairs, const u32 *list, u32 n, unsigned long long *keys, u32 *vals) {
  for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const u32 pi = list[i];
    const u32 nc = pairs[pi].nodeCnt < 0x3fffffffu ? pairs[pi].nodeCnt : 0x3fffffffu;
    keys[i]      = 0x3fffffffu - nc;
    vals[i]      = pi;
  }
}

__global__ void compact_records_kernel(const u32 *rec, const u32 *cnt, const u32 *pos, u32 nPairs, u32 *dst) {
  for (u32 p = blockIdx.x * blockDim.x + threadIdx.x; p < nPairs; p += gridDim.x * blockDim.x) {
    const u32 c = cnt[p];
    for (u32 j = 0; j < c * 6; j++) dst[(u64)pos[p] * 6 + j] = rec[(u64)p * 18 + j];
  }
}

}  // namespace

int align_warps_per_block(int) { return kAlignWarpsSmall; }

size_t align_smem_bytes(int) { return (size_t)kAlignWarpsSmall * 2 * 512 * sizeof(int); }

void launch_align(int, ReadsDev R, TableDev T, DevParams P, const int *eml, const PairRec *pairs, const u32 *work,
                  u32 nWork, u32 *workCounter, const int4 *nodes, WarpScratch sc, AlignCaps cap, int nWarps,
                  AlignOut out, cudaStream_t st) {
  if (nWork == 0 && !out.nWorkDev) return;
  const int    blocks = (nWarps + kAlignWarpsSmall - 1) / kAlignWarpsSmall;
  const size_t smem   = align_smem_bytes(512);
  cap.bandW           = 512;
  auto k = slide_first16(P.maxErate) ? align_kernel<512, kAlignWarpsSmall, true>
                                     : align_kernel<512, kAlignWarpsSmall, false>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k<<<blocks, kAlignWarpsSmall * 32, smem, st>>>(R, T, P, eml, pairs, work, nWork, workCounter, nodes, sc, cap, out);
  g_launches++;
}

void launch_align_group(int threads, int U, int bandW, int ctas, ReadsDev R, TableDev T, DevParams P, const int *eml,
                        const PairRec *pairs, const u32 *work, u32 nWork, u32 *workCounter, const int4 *nodes,
                        WarpScratch sc, AlignCaps cap, AlignOut out, cudaStream_t st) {
  if (nWork == 0 && !out.nWorkDev) return;
  cap.bandW         = bandW;
  const size_t smem = (size_t)2 * bandW * sizeof(int);
  cudaFuncSetAttribute(align_group_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  align_group_kernel<<<ctas, threads, smem, st>>>(R, T, P, eml, pairs, work, nWork, workCounter, nodes, sc, cap, out,
                                                  U);
  g_launches++;
}

void launch_align_spec(int ctas, ReadsDev R, TableDev T, DevParams P, const int *eml, const PairRec *pairs,
                       const u32 *work, u32 nWork, u32 *workCounter, const int4 *nodes, WarpScratch sc, AlignCaps cap,
                       AlignOut out, cudaStream_t st) {
  if (nWork == 0 && !out.nWorkDev) return;
  cap.bandW         = 512;
  cap.rowsGW        = cap.rowsGW < 512 ? 512 : cap.rowsGW;
  const size_t smem = (size_t)kSpecWarps * 2 * 512 * sizeof(int);
  cudaFuncSetAttribute(align_spec_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  align_spec_kernel<<<ctas, kSpecWarps * 32, smem, st>>>(R, T, P, eml, pairs, work, nWork, workCounter, nodes, sc, cap,
                                                        out);
  g_launches++;
}

int align_spec_warps() { return kSpecWarps; }

void launch_extend_batch(int, ReadsDev R, DevParams P, const int *eml, const ExtendProblem *probs, u32 n,
                         WarpScratch sc, AlignCaps cap, int nWarps, int *out, int *kind, int *deltaLen, u32 *status,
                         unsigned long long *stats, cudaStream_t st) {
  if (n == 0) return;
  const int    blocks = (nWarps + kAlignWarpsSmall - 1) / kAlignWarpsSmall;
  const size_t smem   = align_smem_bytes(512);
  cap.bandW           = 512;
  auto k = extend_batch_kernel<512, kAlignWarpsSmall>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k<<<blocks, kAlignWarpsSmall * 32, smem, st>>>(R, P, eml, probs, n, sc, cap, out, kind, deltaLen, status, stats);
  g_launches++;
}

void launch_extend_group(int threads, int U, int bandW, int ctas, ReadsDev R, DevParams P, const int *eml,
                         const ExtendProblem *probs, u32 n, WarpScratch sc, AlignCaps cap, int *out, int *kind,
                         int *deltaLen, u32 *status, unsigned long long *stats, cudaStream_t st) {
  if (n == 0) return;
  cap.bandW         = bandW;
  const size_t smem = (size_t)2 * bandW * sizeof(int);
  auto k = extend_group_kernel<false>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k<<<ctas, threads, smem, st>>>(R, P, eml, probs, n, sc, cap, out, kind, deltaLen, status, stats, U);
  g_launches++;
}

void launch_work_keys(const PairRec *pairs, u32 n, const float *logit, float logitThr, const u32 *readLen,
                      const u32 *strRead, u32 wideMinLen, u32 *binCount, unsigned long long *keys, u32 *vals,
                      cudaStream_t st, const u32 *nDev) {
  if (n == 0) return;
  unsigned g = (n + 255) / 256;
  if (g > 65535u * 8) g = 65535u * 8;
  work_keys_kernel<<<g, 256, 0, st>>>(pairs, n, logit, logitThr, readLen, strRead, wideMinLen, binCount, keys, vals,
                                      nDev);
  g_launches++;
}

void launch_append_overflow(u32 *work, const u32 *binCount, const u32 *ovf, u32 *ovfCount, u32 *wideN,
                            u32 *workCounter, u32 *err, cudaStream_t st) {
  append_overflow_kernel<<<1, 1024, 0, st>>>(work, binCount, ovf, ovfCount, wideN, workCounter, err);
  g_launches++;
}

void launch_list_keys(const PairRec *pairs, const u32 *list, u32 n, unsigned long long *keys, u32 *vals,
                      cudaStream_t st) {
  if (n == 0) return;
  unsigned g = (n + 255) / 256;
  if (g > 65535u * 8) g = 65535u * 8;
  list_keys_kernel<<<g, 256, 0, st>>>(pairs, list, n, keys, vals);
  g_launches++;
}

void launch_compact_records(const u32 *rec, const u32 *cnt, const u32 *pos, u32 nPairs, u32 *dst, cudaStream_t st) {
  if (nPairs == 0) return;
  unsigned g = (nPairs + 255) / 256;
  if (g > 65535u * 8) g = 65535u * 8;
  compact_records_kernel<<<g, 256, 0, st>>>(rec, cnt, pos, nPairs, dst);
  g_launches++;
}

}  // namespace oic
