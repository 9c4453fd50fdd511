// oic_seed.cu -- seed lookup and per-read-pair match lists, one warp per (ref read, strand).
//
// Reference: Find_Overlaps (overlapInCore-Find_Overlaps.C:234-336) walks the ref read's
// k-mers in order, looks each one up, and for every occurrence in a read with a larger
// ID calls Add_Ref (:104-163), which appends the seed to that read pair's match list
// with Add_Match (:25-96).  The list rules are order dependent (runs extend only when
// found before the walk stops; move-to-front), so a pair must see its seeds in exactly
// the reference order: ref offsets ascending, and for one offset the occurrences newest
// first.
//
// Here a warp takes 32 k-mer offsets at a time (one lookup per lane), flattens their
// occurrences into seeds in reference order, and applies them 32 per round: lanes are
// grouped by partner read with match_any, and the lowest lane of each group replays its
// group's seeds in lane order.  Different partners advance in parallel; one partner's
// seeds stay in order.  The pair table and node pool live in the warp's HBM scratch.
//
// A table probe is one 16-byte load of a (key, value) slot.  The qualifying
// occurrences of a k-mer (partner ID above the ref read's) are the tail of its run,
// which ascends by partner: runs of up to kScanMax entries are counted by a backward
// scan, four entries per step -- the entries the replay reads next -- and longer runs
// by binary search.
#include "oic_kernels.cuh"
#include "oic_prims.cuh"

namespace oic {

namespace {

constexpr int kSeedThreads = 128;
constexpr int kSeedWarps   = kSeedThreads / 32;
constexpr int kScanMax     = 64;   // occurrence runs up to this long are scanned backwards

struct SeedSmem {
  u32 incl[32];
  u32 qEnd[32];
  int seedS[32];
  int seedO[32];
  int nPairs;
  int nNodes;
  int overflow;
};

__device__ __forceinline__ u32 warp_incl_scan_u32(u32 v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    u32 t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Add_Match (Find_Overlaps.C:25-96) on the node pool; head is the pair's list head.
__device__ __forceinline__ bool add_match(int4 *nodes, SeedSmem &sm, int nodeCap, int &head, int tOff, int sOff,
                                          int &consistent, int K) {
  int diag = 0, expected = 0, checked = 0;
  const int newDiag = tOff - sOff;
  bool mtf = false;
  int  link = -1;   // -1: the list head; otherwise the node whose .w (next) links `cur`
  int  cur  = head;
  while (cur != 0) {
    int4 nd  = nodes[cur];   // x offset, y len, z start, w next
    expected = nd.z + nd.y - K + 1;
    diag     = nd.x - nd.z;
    if (expected < sOff) break;
    if (expected == sOff) {
      if (newDiag == diag) {
        nodes[cur].y = nd.y + 1;
        if (mtf) {
          // unlink cur (its predecessor exists because mtf was set on an earlier node)
          nodes[link].w = nd.w;
          nodes[cur].w  = head;
          head          = cur;
        }
        return true;
      } else
        mtf = true;
    }
    checked++;
    link = cur;
    cur  = nd.w;
  }
  if (head != 0 && (checked > 0 || abs(diag - newDiag) > 3 || sOff < expected + K - 2)) consistent = 0;
  int id = atomicAdd(&sm.nNodes, 1);
  if (id >= nodeCap) {
    sm.overflow = 1;
    return false;
  }
  nodes[id] = make_int4(tOff, K, sOff, head);
  head      = id;
  return true;
}

__global__ void __launch_bounds__(kSeedThreads) seed_kernel(ReadsDev R, TableDev T, DevParams P, const u32 *segReads,
                                                            const u32 *segList, u32 nSeg, u32 *segCounter,
                                                            SeedScratch sc, SeedCaps cap, SeedOut out) {
  __shared__ SeedSmem smem[kSeedWarps];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  SeedSmem &sm   = smem[wib];
  const u64 gw   = (u64)blockIdx.x * kSeedWarps + wib;
  int     *slotKey = sc.slotKey + gw * cap.slotCap;
  int     *slotVal = sc.slotVal + gw * cap.slotCap;
  PairAcc *pairs   = sc.pairs + gw * cap.pairCap;
  int4    *nodes   = sc.nodes + gw * cap.nodeCap;
  const int K      = P.kmerLen;
  const u64 kmask  = (K >= 32) ? ~0ull : ((1ull << (2 * K)) - 1);
  unsigned long long nSeeds = 0, nSegs = 0;

  for (int i = lane; i < cap.slotCap; i += 32) slotKey[i] = -1;
  __syncwarp();

  while (true) {
    u32 k = 0;
    if (lane == 0) k = atomicAdd(segCounter, 1u);
    k = __shfl_sync(0xffffffffu, k, 0);
    if (k >= nSeg) break;
    const u32 seg = segList ? segList[k] : k;   // segment = (ref index << 1) | strand
    nSegs++;

    const u32 sRead = segReads[seg >> 1];
    const int dir   = seg & 1;
    const SeqView S = make_view(R, sRead, dir);
    const int sLen  = (int)R.len[sRead];
    const int nK    = sLen - K + 1;
    const i64 thr   = (i64)(sRead + 1) - (i64)T.firstID;   // T qualifies iff tStr > thr
    if (lane == 0) {
      sm.nPairs   = 0;
      sm.nNodes   = 1;
      sm.overflow = 0;
    }
    bool lscr = false, rscr = false;
    unsigned long long segSeeds = 0;   // counted once the segment completes in this configuration
    __syncwarp();

    for (int i0 = 0; i0 < nK; i0 += 32) {
      const int i = i0 + lane;
      u32 n = 0, qEnd = 0;
      if (i < nK) {
        u64 key = load_win32(S.w, i) & kmask;
        bool ok = !(S.nm && (load_win32(S.nm, i) & kmask));
        u64 val;
        if (ok && table_find(T, key, val)) {
          if (val >> 63) {
            // hi_hits (Find_Overlaps.C:274-276 for offset 0, :310-317 otherwise)
            if (i == 0) lscr = true;
            else {
              if (i < kHopelessMatch) lscr = true;
              if (sLen - i - K + 1 < kHopelessMatch) rscr = true;
            }
          } else {
            const u32 start = (u32)(val & 0xffffffffull);
            const u32 cnt   = (u32)((val >> 32) & 0x7fffffffull);
            const u32 end   = start + cnt;
            if (cnt <= (u32)kScanMax) {
              while (n < cnt) {
                u64 o[4];
#pragma unroll
                for (int k = 0; k < 4; k++) o[k] = (n + k < cnt) ? __ldg(T.occ + (end - 1 - n - k)) : 0ull;
                u32 q = 0;
#pragma unroll
                for (int k = 0; k < 4; k++)
                  if (q == (u32)k && n + k < cnt && (i64)(o[k] >> 32) > thr) q++;
                n += q;
                if (q < 4) break;
              }
            } else {
              // first occurrence whose string is past thr
              u32 lo = start, hi = end;
              while (lo < hi) {
                u32 mid = (lo + hi) >> 1;
                if ((i64)(T.occ[mid] >> 32) > thr) hi = mid;
                else lo = mid + 1;
              }
              n = end - lo;
            }
            qEnd = end;
          }
        }
      }
      const u32 incl  = warp_incl_scan_u32(n);
      const u32 total = __shfl_sync(0xffffffffu, incl, 31);
      sm.incl[lane]   = incl;
      sm.qEnd[lane]   = qEnd;
      __syncwarp();
      segSeeds += (lane == 0) ? total : 0;

      for (u32 b = 0; b < total; b += 32) {
        const u32  s     = b + lane;
        const bool valid = s < total;
        u32 gkey = 0x80000000u | lane;
        if (valid) {
          int lo = 0, hi = 31;   // first lane with incl > s
          while (lo < hi) {
            int mid = (lo + hi) >> 1;
            if (sm.incl[mid] > s) hi = mid;
            else lo = mid + 1;
          }
          const u32 ex   = (lo ? sm.incl[lo - 1] : 0);
          const u32 j    = s - ex;
          const u64 o    = T.occ[sm.qEnd[lo] - 1 - j];   // newest occurrence first
          sm.seedO[lane] = (int)(u32)o;
          sm.seedS[lane] = i0 + lo;
          gkey           = (u32)(o >> 32);
        }
        __syncwarp();
        const unsigned peers = __match_any_sync(0xffffffffu, gkey);
        if (valid && lane == __ffs(peers) - 1 && !sm.overflow) {
          // Find or create the pair (Add_Ref, Find_Overlaps.C:104-150).
          const u32 tStr = gkey;
          int slot = (int)(mix64(tStr) & (u64)(cap.slotCap - 1));
          int pi   = -1;
          for (int probe = 0; probe < cap.slotCap; probe++) {
            int old = atomicCAS(&slotKey[slot], -1, (int)tStr);
            if (old == -1) {
              pi = atomicAdd(&sm.nPairs, 1);
              if (pi >= cap.pairCap) {
                sm.overflow = 1;
                pi          = -1;
                break;
              }
              PairAcc &pa   = pairs[pi];
              pa.T          = tStr;
              pa.head       = 0;
              pa.diagCt     = 0;
              pa.diagBgn    = (int)kMaxReadLen;
              pa.diagEnd    = 0;
              pa.consistent = 1;
              pa.slot       = slot;
              slotVal[slot] = pi;
              break;
            }
            if (old == (int)tStr) {
              pi = slotVal[slot];
              break;
            }
            slot = (slot + 1) & (cap.slotCap - 1);
          }
          if (pi < 0) sm.overflow = 1;
          else {
            PairAcc pa = pairs[pi];
            unsigned m = peers;
            while (m) {
              const int q = __ffs(m) - 1;
              m &= m - 1;
              const int sOff = sm.seedS[q];
              pa.diagCt++;
              if (pa.diagBgn > sOff) pa.diagBgn = sOff;
              if (pa.diagEnd < sOff) pa.diagEnd = sOff;
              if (!add_match(nodes, sm, cap.nodeCap, pa.head, sm.seedO[q], sOff, pa.consistent, K)) break;
            }
            pairs[pi].head       = pa.head;
            pairs[pi].diagCt     = pa.diagCt;
            pairs[pi].diagBgn    = pa.diagBgn;
            pairs[pi].diagEnd    = pa.diagEnd;
            pairs[pi].consistent = pa.consistent;
          }
        }
        __syncwarp();
        if (sm.overflow) break;
      }
      __syncwarp();
      if (sm.overflow) break;
    }

    lscr = __any_sync(0xffffffffu, lscr);
    rscr = __any_sync(0xffffffffu, rscr);
    __syncwarp();
    const int nPairs = min(sm.nPairs, cap.pairCap);
    const bool ovf   = sm.overflow != 0;
    if (!ovf) nSeeds += segSeeds;

    if (!ovf && nPairs > 0) {
      // Node counts per pair, then one global allocation for the segment.
      u32 nodeTotal = 0;
      for (int p0 = 0; p0 < nPairs; p0 += 32) {
        const int p = p0 + lane;
        u32 c = 0;
        if (p < nPairs)
          for (int q = pairs[p].head; q != 0; q = nodes[q].w) c++;
        nodeTotal += __reduce_add_sync(0xffffffffu, c);
      }
      u32 nodeBase = 0, pairBase = 0;
      if (lane == 0) {
        nodeBase = atomicAdd(out.nodeCount, nodeTotal);
        pairBase = atomicAdd(out.pairCount, (u32)nPairs);
      }
      nodeBase = __shfl_sync(0xffffffffu, nodeBase, 0);
      pairBase = __shfl_sync(0xffffffffu, pairBase, 0);
      const bool fits = (u64)nodeBase + nodeTotal <= out.nodeCap && (u64)pairBase + nPairs <= out.pairCap;
      if (!fits) {
        if (lane == 0) atomicOr(out.err, kErrOutNodes);
      } else {
        u32 run = nodeBase;
        for (int p0 = 0; p0 < nPairs; p0 += 32) {
          const int p = p0 + lane;
          u32 c = 0;
          if (p < nPairs)
            for (int q = pairs[p].head; q != 0; q = nodes[q].w) c++;
          const u32 inc = warp_incl_scan_u32(c);
          const u32 my  = run + inc - c;
          if (p < nPairs) {
            u32 k = my;
            for (int q = pairs[p].head; q != 0; q = nodes[q].w) {
              int4 nd = nodes[q];
              out.nodes[k++] = make_int4(nd.x, nd.y, nd.z, 0);
            }
            PairRec rec;
            rec.sRead   = sRead;
            rec.tStr    = pairs[p].T;
            rec.nodeOff = my;
            rec.nodeCnt = c;
            rec.diagCt  = pairs[p].diagCt;
            rec.diagBgn = pairs[p].diagBgn;
            rec.diagEnd = pairs[p].diagEnd;
            rec.flags   = (u32)dir | ((u32)(pairs[p].consistent != 0) << 1) | ((u32)lscr << 2) | ((u32)rscr << 3);
            out.pairs[pairBase + p] = rec;
          }
          run += __shfl_sync(0xffffffffu, inc, 31);
        }
      }
    } else if (ovf && lane == 0) {
      u32 k = atomicAdd(out.overflowCount, 1u);
      out.overflowSegs[k] = seg;
    }
    // Reset the slots this segment used (all of them after an overflow, whose
    // abandoned claims are not all recorded in the pair list).
    if (ovf)
      for (int i = lane; i < cap.slotCap; i += 32) slotKey[i] = -1;
    else
      for (int p = lane; p < nPairs; p += 32) slotKey[pairs[p].slot] = -1;
    __syncwarp();
  }
  if (lane == 0) {
    atomicAdd(&out.stats[0], nSeeds);
    atomicAdd(&out.stats[1], nSegs);
  }
}

}  // namespace

void launch_seed(ReadsDev R, TableDev T, DevParams P, const u32 *segReads, const u32 *segList, u32 nSeg,
                 u32 *segCounter, SeedScratch sc, SeedCaps cap, int nWarps, SeedOut out, cudaStream_t st) {
  if (nSeg == 0) return;
  int blocks = (nWarps + kSeedWarps - 1) / kSeedWarps;
  seed_kernel<<<blocks, kSeedThreads, 0, st>>>(R, T, P, segReads, segList, nSeg, segCounter, sc, cap, out);
  g_launches++;
}

}  // namespace oic
