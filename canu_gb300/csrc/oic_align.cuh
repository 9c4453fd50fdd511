// oic_align.cuh -- warp-cooperative banded prefix edit distance (furthest-reaching
// diagonals) and the per-read-pair driver around it.
//
// One warp owns one read pair.  Lanes own diagonals of the current error row (lane l
// takes d = Lc + l, Lc + l + 32, ...); the previous row lives in a shared-memory
// buffer, every kept row is appended to the warp's traceback arena in HBM, and the
// slides compare 32 bases per step on the 2-bit packed reads.  The arithmetic is the
// reference's exactly -- integer rows, the same band pruning against Edit_Match_Limit,
// the same first-index tie breaks, and the branch-point test in IEEE double with
// explicitly rounded multiply / subtract / divide (no FMA contraction), as an x86-64
// build of canu computes it.
#pragma once

#include "oic_common.cuh"

namespace oic {

// Per-warp global scratch.
struct WarpScratch {
  int  *arena;       // kept DP rows, band-compacted
  int4 *rowHdr;      // per error row: (arena offset, kept band left, kept band right, unused)
  int  *rowsG;       // two row buffers of rowsGW ints in HBM, used once a band outgrows shared memory
  int  *deltaL;      // Left_Delta (merged delta of the last extension)
  int  *deltaR;      // Right_Delta
  int  *stack;       // Delta_Stack
  unsigned char *alive;   // match-node alive flags of the current pair
};

struct AlignCaps {
  int arenaCap;   // ints per warp
  int rowCap;     // error rows per warp (also bounds the delta arrays)
  int nodeCap;    // match nodes per pair
  int bandW;      // ints per shared-memory row buffer
  int rowsGW;     // ints per HBM row buffer (bands wider than bandW - 4 up to rowsGW - 4)
};

struct WarpDP {
  WarpScratch        sc;
  AlignCaps          cap;
  int               *smA, *smB;     // shared-memory row buffers (bandW ints each)
  const int         *eml;           // Edit_Match_Limit
  DevParams          P;
  unsigned long long cells, slides, rows;
  u32                err;           // capacity error of the current pair (0 = ok)
  int                leftLen, rightLen;
  struct GroupShared *gs;           // non-null: warp 0 of a group CTA (row loops on all warps)
  int                gThreads;      // threads of the group CTA
  int                gU;            // diagonals per thread per pass in the group row loop
};

// The scratch of global warp gw inside the base allocations of a configuration.
static __device__ __forceinline__ WarpScratch warp_scratch(const WarpScratch &base, const AlignCaps &cap, u64 gw) {
  WarpScratch s;
  s.arena  = base.arena + gw * (u64)cap.arenaCap;
  s.rowHdr = base.rowHdr + gw * (u64)cap.rowCap;
  s.rowsG  = base.rowsG ? base.rowsG + gw * (u64)(2 * cap.rowsGW) : nullptr;
  s.deltaL = base.deltaL + gw * (u64)(cap.rowCap + 8);
  s.deltaR = base.deltaR + gw * (u64)(cap.rowCap + 8);
  s.stack  = base.stack + gw * (u64)(cap.rowCap + 8);
  s.alive  = base.alive + gw * (u64)cap.nodeCap;
  return s;
}

// Row-0 exact slide shared by the warp: each lane tests one 32-base window per step.
template <int STEP>
__device__ __forceinline__ int warp_slide0(const SeqView &A, int a0, const SeqView &T, int t0, int m,
                                           unsigned long long &slides) {
  const int lane = threadIdx.x & 31;
  int       base = 0;
  while (base < m) {
    int off = base + lane * 32;
    int r   = 32;
    if (off < m) r = match_run32<STEP>(A, a0 + STEP * off, T, t0 + STEP * off);
    unsigned short_ = __ballot_sync(0xffffffffu, off < m && r < 32);
    if (short_) {
      int first = __ffs(short_) - 1;
      int rr    = __shfl_sync(0xffffffffu, r, first);
      int run   = base + first * 32 + rr;
      run       = min(run, m);
      if (lane == 0) slides += (unsigned long long)run;
      return run;
    }
    base += 32 * 32;
  }
  if (lane == 0) slides += (unsigned long long)m;
  return m;
}

// Traceback of Set_Right_Delta / Set_Left_Delta (prefixEditDistance-forward.C:32-71,
// -reverse.C:36-93) from row e, diagonal d whose value is `last`.  Lane 0 only.
// Pushes one entry per indel into out[]; returns the value reached on row 0.
static __device__ __noinline__ int trace_rows(const WarpDP &w, int e, int d, int last, int *out, int &nOut) {
  // Pointers and the entry count in registers; the next row's header is loaded one
  // step ahead (it does not depend on the path), so only the arena reads stay on the
  // step-to-step dependency chain.
  const int4 *const rowHdr = w.sc.rowHdr;
  const int *const  arena  = w.sc.arena;
  int  n     = 0;
  int4 hNext = e > 0 ? rowHdr[e - 1] : make_int4(0, 0, 0, 0);
  for (int k = e; k > 0; k--) {
    const int4 h = hNext;
    if (k > 1) hNext = rowHdr[k - 2];
    const int off = h.x, L = h.y, R = h.z;
    const int g0 = (d >= L && d <= R) ? arena[off + d - L] : -2;
    const int gm = (d - 1 >= L && d - 1 <= R) ? arena[off + d - 1 - L] : -2;
    const int gp = (d + 1 >= L && d + 1 <= R) ? arena[off + d + 1 - L] : -2;
    int from = d, mx = 1 + g0;
    if (gm > mx) { from = d - 1; mx = gm; }
    if (1 + gp > mx) { from = d + 1; mx = 1 + gp; }
    if (from == d - 1) {
      out[n++] = mx - last - 1;
      last     = gm;
      d--;
    } else if (from == d + 1) {
      out[n++] = last - (mx - 1);
      last     = gp;
      d++;
    }
  }
  nOut = n;
  return last;
}

__device__ __forceinline__ int arena_get(const WarpDP &w, int e, int d) {
  const int4 h = w.sc.rowHdr[e];
  return (d >= h.y && d <= h.z) ? w.sc.arena[h.x + d - h.y] : -2;
}

// Set_Right_Delta (forward.C:32-71) into sc.deltaR; lane 0.
static __device__ __noinline__ void set_right_delta(WarpDP &w, int e, int d, int last) {
  int n;
  int l = trace_rows(w, e, d, last, w.sc.stack, n);
  w.sc.stack[n++] = l + 1;
  int k           = 0;
  for (int i = n - 1; i > 0; i--) {
    int s = w.sc.stack[i - 1];
    w.sc.deltaR[k++] = abs(w.sc.stack[i]) * ((s > 0) - (s < 0));
  }
  w.rightLen = n - 1;
}

// Set_Left_Delta (reverse.C:36-93) into sc.deltaL; lane 0.
static __device__ __noinline__ void set_left_delta(WarpDP &w, int e, int d, int last, int &leftover, int &tEnd, int tLen) {
  int n;
  leftover  = trace_rows(w, e, d, last, w.sc.deltaL, n);
  int *ld   = w.sc.deltaL;
  if (n > 1 && ld[0] == 1 && tEnd + tLen > 0) {
    ld[0] = (ld[1] > 0) ? ld[1] + 1 : ld[1] - 1;
    for (int i = 2; i < n; i++) ld[i - 1] = ld[i];
    n--;
    tEnd--;
    if (n == 0) leftover++;
  }
  w.leftLen = n;
}

// Max_Score bookkeeping of forward()/reverse() (prefixEditDistance-forward.C:284-296,
// -reverse.C:300-312), replayed once after the rows instead of on every row.  Row e
// (1..eLast) stored its largest kept value in rowHdr[e].w.  Walking the rows in order,
// the reference scores a row only when that value passes every earlier row's
// (Longest grows) and keeps the first row whose score fl(fl(value * BMV) - e) is the
// strict maximum above the initial 0.0.  Here lane i takes rows i+1, i+33, ...; a warp
// max-scan finds the rows where Longest grows, each lane scores its rows in IEEE double
// (the same two roundings), and a warp arg-max with the smallest row on ties picks the
// reference's row.  msD is the first diagonal of that row's kept band holding msLen.
static __device__ __noinline__ void max_score_rows(const WarpDP &w, int eLast, double &maxScore, int &msLen,
                                                   int &msD, int &msE) {
  const int    lane = threadIdx.x & 31;
  const double BMV  = w.P.branchMatchValue;
  double best  = 0.0;
  int    bestE = INT_MAX;
  int    carry = 0;   // Longest before the current block of 32 rows
  for (int base = 1; base <= eLast; base += 32) {
    const int e = base + lane;
    const int v = e <= eLast ? w.sc.rowHdr[e].w : INT_MIN;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl = max(incl, t);
    }
    int excl = __shfl_up_sync(0xffffffffu, incl, 1);
    if (lane == 0) excl = INT_MIN;
    if (e <= eLast && v > max(carry, excl)) {
      const double s = __dsub_rn(__dmul_rn((double)v, BMV), (double)e);
      if (s > best) {
        best  = s;
        bestE = e;
      }
    }
    carry = max(carry, __shfl_sync(0xffffffffu, incl, 31));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double ob = __shfl_xor_sync(0xffffffffu, best, o);
    const int    oe = __shfl_xor_sync(0xffffffffu, bestE, o);
    if (ob > best || (ob == best && oe < bestE)) {
      best  = ob;
      bestE = oe;
    }
  }
  if (bestE == INT_MAX) {
    maxScore = 0.0;
    msLen = msD = msE = 0;
    return;
  }
  maxScore     = best;
  msE          = bestE;
  const int4 h = w.sc.rowHdr[msE];
  msLen        = h.w;
  int myD = INT_MAX;
  for (int d = h.y + lane; d <= h.z; d += 32)
    if (w.sc.arena[h.x + d - h.y] == msLen) {
      myD = d;
      break;
    }
  msD = __reduce_min_sync(0xffffffffu, myD);
}

// ---------------------------------------------------------------------------------
// Row loop of forward()/reverse() (prefixEditDistance-forward.C:131-304,
// -reverse.C:151-320): error rows e = 1, 2, ... with the band pruned against
// Edit_Match_Limit.  It stops at the first row where a diagonal reaches the end of A
// or T (kRowsEnd), when every diagonal is pruned or the error limit is reached
// (kRowsDone), or on a capacity limit (kRowsErr).  Every kept row goes to the arena
// with its largest value in the row header (see max_score_rows).
enum { kRowsDone = 0, kRowsEnd = 1, kRowsErr = 2 };

struct RowsOut {
  int  status;
  u32  err;
  int  e, dEnd, eDone;       // end row, first diagonal reaching an end, last kept row
  int  Lc, Rc, prevBase;     // band of row e and the base of row e-1
  int *prev, *cur;           // row e-1 and row e buffers
  unsigned long long cells, rows;
};

// Several warps of one CTA on one pair (the wide bins): warp 0 runs the pair logic and
// hands each extension's row loop to the whole CTA through GroupShared.
struct GroupJob {
  SeqView A, T;
  int     a0, t0;
  int     m, n, errorLimit, step, u;
  int     first16;           // slides start with the 16-base compare (slide_first16)
  int    *rowA, *rowB;       // row buffers (rowA holds row 0)
};
struct GroupShared {
  GroupJob job;
  int      cmd;              // kGroupRows or kGroupExit, posted by warp 0 before barrier 1
  int      red[32][4];       // per-warp partial reductions of a row
};
enum { kGroupRows = 1, kGroupExit = 2 };

// Named barrier over the CTA's nThr threads (id 1: hand-off, id 2: rows).
__device__ __forceinline__ void group_bar(int id, int nThr) {
  asm volatile("bar.sync %0, %1;\n" ::"r"(id), "r"(nThr) : "memory");
}

// The row loop by one warp.  Row 0 (value r0) is in prev[2].  FIRST16: slides start
// with a 16-base compare (see slide()).
template <int STEP, bool FIRST16>
__device__ __forceinline__ RowsOut warp_rows(WarpDP &w, const SeqView &Aref, int a0, int m, const SeqView &Tref,
                                             int t0, int n, int errorLimit) {
  const SeqView A = Aref, T = Tref;   // in registers for the slides
  const int lane = threadIdx.x & 31;
  RowsOut o;
  o.status = kRowsDone;
  o.err = 0;
  o.e = o.dEnd = o.eDone = 0;
  o.cells = o.rows = 0;
  // Row buffers hold diagonal d at index d - base + 2.  Before a row is computed the
  // two diagonals on each side of the previous row's kept band are set to -2, as the
  // reference does (forward.C:150-153), so the neighbour reads need no bounds tests.
  // Loop invariants and the slide counter in registers: the loop stores through
  // generic pointers, which the compiler cannot tell apart from the WarpDP on the stack.
  int *const         arena    = w.sc.arena;
  int4 *const        rowHdr   = w.sc.rowHdr;
  int *const         rowsG    = w.sc.rowsG;
  const int *const   eml      = w.eml;
  const int          rowCap   = w.cap.rowCap;
  const int          rowsGW   = w.cap.rowsGW;
  const int          arenaCap = w.cap.arenaCap;
  unsigned long long slides   = 0;
  int *prev = w.smA, *cur = w.smB;
  int  bufW = w.cap.bandW;
  int  used = 1, prevBase = 0, L = 0, R = 0;
  for (int e = 1; e <= errorLimit; e++) {
    if (e >= rowCap) { o.status = kRowsErr; o.err = kErrRowsFull; break; }
    const int Lc = max(L - 1, -e), Rc = min(R + 1, e);
    const int width = Rc - Lc + 1;
    if (width + 4 > bufW) {
      // The band outgrew the shared-memory rows: continue in the warp's HBM rows.
      if (bufW == rowsGW || width + 4 > rowsGW || !rowsG) { o.status = kRowsErr; o.err = kErrBandWide; break; }
      int *gA = rowsG, *gB = rowsG + rowsGW;
      for (int i = lane; i < bufW; i += 32) gA[i] = prev[i];
      __syncwarp();
      prev = gA;
      cur  = gB;
      bufW = rowsGW;
    }

    const int lim = eml[e];
    if (lane < 4) prev[(lane < 2 ? L - 2 + lane : R - 1 + lane) - prevBase + 2] = -2;
    __syncwarp();
    const int *pv = prev + (2 - prevBase);   // pv[d] = row e-1 at diagonal d
    int       *cv = cur + (2 - Lc);          // cv[d] = row e at diagonal d
    int myEnd = INT_MAX, myL = INT_MAX, myR = INT_MIN;
    for (int d = Lc + lane; d <= Rc; d += 32) {
      const int p0 = pv[d], pm = pv[d - 1], pp = pv[d + 1];
      int row = 1 + p0;
      if (pm > row) row = pm;
      if (1 + pp > row) row = 1 + pp;
      const int room = min(m - row, n - row - d);
      if (room > 0) row += slide<STEP, FIRST16>(A, a0, T, t0, row, d, room, slides);
      cv[d] = row;
      if ((row == m || row + d == n) && d < myEnd) myEnd = d;
      // pruneAlign (prefixEditDistance.H:249-258): extra = max(d, 0) on both band edges
      if (!(row + max(d, 0) < lim)) {
        if (myL == INT_MAX) myL = d;
        myR = d;
      }
    }
    __syncwarp();
    o.rows++;
    const int dEnd = __reduce_min_sync(0xffffffffu, myEnd);
    if (dEnd != INT_MAX) {
      o.cells += (unsigned long long)(dEnd - Lc + 1);
      o.status   = kRowsEnd;
      o.e        = e;
      o.dEnd     = dEnd;
      o.Lc       = Lc;
      o.Rc       = Rc;
      o.prevBase = prevBase;
      o.prev     = prev;
      o.cur      = cur;
      break;
    }
    o.cells += (unsigned long long)width;

    // The kept band is [first, last] unpruned diagonal (forward.C:245-280).
    const int L2 = __reduce_min_sync(0xffffffffu, myL);
    if (L2 == INT_MAX) break;
    const int R2 = __reduce_max_sync(0xffffffffu, myR);

    // Keep the band for the traceback, and take its largest value on the way
    // (forward.C:284-289); the Max_Score test that uses it runs once after the rows
    // (max_score_rows).
    const int cnt = R2 - L2 + 1;
    if (used + cnt > arenaCap) { o.status = kRowsErr; o.err = kErrArenaFull; break; }
    int myV = -1;
    for (int d = L2 + lane; d <= R2; d += 32) {
      const int v = cv[d];
      myV         = max(myV, v);
      arena[used + d - L2] = v;
    }
    const int rowMax = __reduce_max_sync(0xffffffffu, myV);
    if (lane == 0) rowHdr[e] = make_int4(used, L2, R2, rowMax);
    used += cnt;
    int *t = prev;
    prev   = cur;
    cur    = t;
    prevBase = Lc;
    L        = L2;
    R        = R2;
    o.eDone  = e;
    __syncwarp();
  }
  w.slides += slides;
  return o;
}

// The row loop by every thread of the CTA (nThr threads, tid = threadIdx.x).  Thread t
// takes U consecutive diagonals per pass, d0 = Lc + U*t + U*nThr*k, so the U+2
// neighbour values of row e-1 are read once for U cells and U slides are in flight.
// Every decision is made on CTA-reduced values, so all threads take the same path and
// meet the same barriers.
template <int STEP, int U, bool FIRST16>
static __device__ __noinline__ RowsOut group_rows(const GroupJob &j, const WarpScratch &sc, const AlignCaps &cap,
                                                  const int *eml, int tid, int nThr, int (*red)[4],
                                                  unsigned long long &slides) {
  const int lane = tid & 31, wid = tid >> 5, nW = nThr >> 5;
  const SeqView A = j.A, T = j.T;   // in registers for the slides
  const int     a0 = j.a0, t0 = j.t0;
  const int     m = j.m, n = j.n;
  RowsOut o;
  o.status = kRowsDone;
  o.err = 0;
  o.e = o.dEnd = o.eDone = 0;
  o.cells = o.rows = 0;
  // Every thread has read the job before warp 0 can post the next one.
  group_bar(2, nThr);
  int *prev = j.rowA, *cur = j.rowB;
  int  bufW = cap.bandW;
  int  used = 1, prevBase = 0, L = 0, R = 0;
  for (int e = 1; e <= j.errorLimit; e++) {
    if (e >= cap.rowCap) { o.status = kRowsErr; o.err = kErrRowsFull; break; }
    const int Lc = max(L - 1, -e), Rc = min(R + 1, e);
    const int width = Rc - Lc + 1;
    if (width + 4 > bufW) {
      if (bufW == cap.rowsGW || width + 4 > cap.rowsGW || !sc.rowsG) { o.status = kRowsErr; o.err = kErrBandWide; break; }
      int *gA = sc.rowsG, *gB = sc.rowsG + cap.rowsGW;
      for (int i = tid; i < bufW; i += nThr) gA[i] = prev[i];
      group_bar(2, nThr);
      prev = gA;
      cur  = gB;
      bufW = cap.rowsGW;
    }
    const int lim = eml[e];
    if (tid < 4) prev[(tid < 2 ? L - 2 + tid : R - 1 + tid) - prevBase + 2] = -2;
    group_bar(2, nThr);
    const int *pv = prev + (2 - prevBase);
    int       *cv = cur + (2 - Lc);
    int myEnd = INT_MAX, myL = INT_MAX, myR = INT_MIN;
    for (int d0 = Lc + tid * U; d0 <= Rc; d0 += nThr * U) {
      int q[U + 2];   // row e-1 at d0-1 .. d0+U
#pragma unroll
      for (int k = 0; k < U + 2; k++) q[k] = (d0 - 1 + k <= Rc + 1) ? pv[d0 - 1 + k] : -2;
#pragma unroll
      for (int k = 0; k < U; k++) {
        const int d = d0 + k;
        if (d <= Rc) {
          int row = 1 + q[k + 1];
          if (q[k] > row) row = q[k];
          if (1 + q[k + 2] > row) row = 1 + q[k + 2];
          const int room = min(m - row, n - row - d);
          if (room > 0) row += slide<STEP, FIRST16>(A, a0, T, t0, row, d, room, slides);
          cv[d] = row;
          if ((row == m || row + d == n) && d < myEnd) myEnd = d;
          if (!(row + max(d, 0) < lim)) {
            if (myL == INT_MAX) myL = d;
            myR = d;
          }
        }
      }
    }
    {
      const int wEnd = __reduce_min_sync(0xffffffffu, myEnd);
      const int wL   = __reduce_min_sync(0xffffffffu, myL);
      const int wR   = __reduce_max_sync(0xffffffffu, myR);
      if (lane == 0) {
        red[wid][0] = wEnd;
        red[wid][1] = wL;
        red[wid][2] = wR;
      }
    }
    group_bar(2, nThr);
    int dEnd = INT_MAX, L2 = INT_MAX, R2 = INT_MIN;
    for (int i = 0; i < nW; i++) {
      dEnd = min(dEnd, red[i][0]);
      L2   = min(L2, red[i][1]);
      R2   = max(R2, red[i][2]);
    }
    o.rows++;
    if (dEnd != INT_MAX) {
      o.cells += (unsigned long long)(dEnd - Lc + 1);
      o.status   = kRowsEnd;
      o.e        = e;
      o.dEnd     = dEnd;
      o.Lc       = Lc;
      o.Rc       = Rc;
      o.prevBase = prevBase;
      o.prev     = prev;
      o.cur      = cur;
      break;
    }
    o.cells += (unsigned long long)width;
    if (L2 == INT_MAX) break;

    // Keep the band for the traceback and take its largest value on the way.
    const int cnt = R2 - L2 + 1;
    if (used + cnt > cap.arenaCap) { o.status = kRowsErr; o.err = kErrArenaFull; break; }
    int myV = -1;
    for (int d = L2 + tid; d <= R2; d += nThr) {
      const int v = cv[d];
      myV         = max(myV, v);
      sc.arena[used + d - L2] = v;
    }
    {
      const int wV = __reduce_max_sync(0xffffffffu, myV);
      if (lane == 0) red[wid][3] = wV;
    }
    group_bar(2, nThr);
    int rowMax = -1;
    for (int i = 0; i < nW; i++) rowMax = max(rowMax, red[i][3]);
    if (tid == 0) sc.rowHdr[e] = make_int4(used, L2, R2, rowMax);
    used += cnt;
    int *t = prev;
    prev   = cur;
    cur    = t;
    prevBase = Lc;
    L        = L2;
    R        = R2;
    o.eDone  = e;
    group_bar(2, nThr);
  }
  return o;
}

// The job a GroupJob names, with its compile-time step and tile.
static __device__ __forceinline__ RowsOut group_rows_any(const GroupJob &j, const WarpScratch &sc,
                                                         const AlignCaps &cap, const int *eml, int tid, int nThr,
                                                         int (*red)[4], unsigned long long &slides) {
#define OIC_GROUP_ROWS(S, U)                                                                  \
  return j.first16 ? group_rows<S, U, true>(j, sc, cap, eml, tid, nThr, red, slides)          \
                   : group_rows<S, U, false>(j, sc, cap, eml, tid, nThr, red, slides)
  if (j.step > 0) {
    if (j.u == 4) OIC_GROUP_ROWS(+1, 4);
    if (j.u == 2) OIC_GROUP_ROWS(+1, 2);
    OIC_GROUP_ROWS(+1, 1);
  }
  if (j.u == 4) OIC_GROUP_ROWS(-1, 4);
  if (j.u == 2) OIC_GROUP_ROWS(-1, 2);
  OIC_GROUP_ROWS(-1, 1);
#undef OIC_GROUP_ROWS
}

// Worker warps of a group CTA: run the row loops warp 0 posts until it posts exit.
static __device__ __noinline__ void group_worker(GroupShared &gs, const WarpScratch &sc, const AlignCaps &cap,
                                                 const int *eml, unsigned long long &slides) {
  const int tid = threadIdx.x, nThr = blockDim.x;
  while (true) {
    group_bar(1, nThr);
    if (gs.cmd != kGroupRows) break;
    const GroupJob j = gs.job;
    group_rows_any(j, sc, cap, eml, tid, nThr, gs.red, slides);
  }
}

// forward() (prefixEditDistance-forward.C:94-314) for STEP = +1 and reverse()
// (prefixEditDistance-reverse.C:114-330) for STEP = -1.  A[STEP*i] is base a0+STEP*i of
// view A, T likewise.  The row loop runs on this warp, or on the whole CTA when w.gs is
// set (warp 0 of a group CTA); the rest runs on this warp.  Returns the error count;
// the outputs are warp-uniform.  On a capacity overflow sets w.err and returns 0.
template <int STEP, bool GROUP, bool FIRST16 = false>
static __device__ __noinline__ int warp_prefix_dp(WarpDP &w, const SeqView &A, int a0, int m, const SeqView &T, int t0, int n,
                              int errorLimit, int &aEnd, int &tEnd, int &leftover, bool &toEnd) {
  const int lane = threadIdx.x & 31;
  const double BMV = w.P.branchMatchValue;

  if (STEP > 0) w.rightLen = 0;
  else w.leftLen = 0;

  const int r0 = warp_slide0<STEP>(A, a0, T, t0, m, w.slides);
  if (r0 == m) {
    aEnd = tEnd = STEP * m;
    if (STEP < 0) leftover = m;
    toEnd = true;
    return 0;
  }

  if (lane == 0) {
    w.sc.arena[0]  = r0;
    w.sc.rowHdr[0] = make_int4(0, 0, 0, 0);
    w.smA[2]       = r0;
  }
  __syncwarp();

  RowsOut o;
  if (GROUP) {
    if (lane == 0) {
      GroupJob &j  = w.gs->job;
      j.A          = A;
      j.T          = T;
      j.a0         = a0;
      j.t0         = t0;
      j.m          = m;
      j.n          = n;
      j.errorLimit = errorLimit;
      j.step       = STEP;
      j.u          = w.gU;
      j.first16    = slide_first16(w.P.maxErate);
      j.rowA       = w.smA;
      j.rowB       = w.smB;
      w.gs->cmd    = kGroupRows;
    }
    __syncwarp();
    group_bar(1, w.gThreads);
    const GroupJob j = w.gs->job;
    o = group_rows_any(j, w.sc, w.cap, w.eml, lane, w.gThreads, w.gs->red, w.slides);
  } else {
    o = warp_rows<STEP, FIRST16>(w, A, a0, m, T, t0, n, errorLimit);
  }
  w.cells += o.cells;
  w.rows += o.rows;
  if (o.status == kRowsErr) {
    w.err |= o.err;
    return 0;
  }

  double maxScore = 0.0;
  int    msLen = 0, msD = 0, msE = 0;
  max_score_rows(w, o.eDone, maxScore, msLen, msD, msE);

  if (o.status == kRowsEnd) {
    const int  e   = o.e;
    const int *pv  = o.prev + (2 - o.prevBase);
    const int *cv  = o.cur + (2 - o.Lc);
    const int  row = cv[o.dEnd];
    // Branch-point test in IEEE double on lane 0 (the FP64 pipe is narrow); the other
    // lanes take its decision.
    int abort_ = 0;
    if (lane == 0) {
      const double score   = __dsub_rn(__dmul_rn((double)row, BMV), (double)e);
      const int    tailLen = row - msLen;
      const double slope   = __ddiv_rn(__dsub_rn(maxScore, score), (double)tailLen);
      abort_ = (w.P.partial && score < maxScore) ||
               (e > 20 / 2 && tailLen >= 20 && slope >= w.P.minBranchTailSlope);
    }
    abort_ = __shfl_sync(0xffffffffu, abort_, 0);
    if (!abort_) {
      int d = o.dEnd;
      if (STEP > 0) {
        // Force the last error to be a mismatch (forward.C:215-221).
        if (row == m && 1 + pv[d + 1] == row && d < o.Rc) d++;
        aEnd = row;
        tEnd = row + d;
        if (lane == 0) set_right_delta(w, e, d, row);
        w.rightLen = __shfl_sync(0xffffffffu, w.rightLen, 0);
      } else {
        aEnd = -row;
        tEnd = -row - d;
        if (lane == 0) set_left_delta(w, e, d, row, leftover, tEnd, n);
        w.leftLen = __shfl_sync(0xffffffffu, w.leftLen, 0);
        leftover  = __shfl_sync(0xffffffffu, leftover, 0);
        tEnd      = __shfl_sync(0xffffffffu, tEnd, 0);
      }
      toEnd = true;
      __syncwarp();
      return e;
    }
  }

  // Branch point, errors exhausted, or every diagonal pruned (forward.C:197-212,
  // 306-313): the alignment ends at the Max_Score row.
  aEnd = STEP * msLen;
  tEnd = STEP * (msLen + msD);
  __syncwarp();
  if (lane == 0) {
    const int last = arena_get(w, msE, msD);
    if (STEP > 0) set_right_delta(w, msE, msD, last);
    else set_left_delta(w, msE, msD, last, leftover, tEnd, n);
  }
  if (STEP > 0) w.rightLen = __shfl_sync(0xffffffffu, w.rightLen, 0);
  else {
    w.leftLen = __shfl_sync(0xffffffffu, w.leftLen, 0);
    leftover  = __shfl_sync(0xffffffffu, leftover, 0);
    tEnd      = __shfl_sync(0xffffffffu, tEnd, 0);
  }
  toEnd = false;
  __syncwarp();
  return msE;
}

static __device__ __forceinline__ void warp_dp_init(WarpDP &w, const WarpScratch &sc, const AlignCaps &cap, int *smA,
                                                    int *smB, const int *eml, const DevParams &P) {
  w.sc       = sc;
  w.cap      = cap;
  w.smA      = smA;
  w.smB      = smB;
  w.eml      = eml;
  w.P        = P;
  w.cells    = 0;
  w.slides   = 0;
  w.rows     = 0;
  w.err      = 0;
  w.leftLen  = w.rightLen = 0;
  w.gs       = nullptr;
  w.gThreads = 32;
  w.gU       = 1;
}

enum { kNone = 0, kLeftBranch = 1, kRightBranch = 2, kDovetail = 3 };

// Extend_Alignment (prefixEditDistance-extend.C:36-183), one warp.  The merged delta
// ends up in sc.deltaL[0 .. leftLen).  Outputs are warp-uniform.
template <bool GROUP, bool FIRST16 = false>
static __device__ __noinline__ int warp_extend(WarpDP &w, const SeqView &S, int sLen, const SeqView &T, int tLen, int mStart,
                           int mOffset, int mLen, int &sLo, int &sHi, int &tLo, int &tHi, int &errors) {
  const int lane = threadIdx.x & 31;
  int  rightErrors = 0, leftErrors = 0, leftover = 0;
  bool rToEnd = true, lToEnd = true;
  const int sLeftBegin = mStart - 1, sRightBegin = mStart + mLen, sRightLen = sLen - sRightBegin;
  const int tLeftBegin = mOffset - 1, tRightBegin = mOffset + mLen, tRightLen = tLen - tRightBegin;
  int totalOlap = min(mStart, mOffset) + mLen + min(sRightLen, tRightLen);
  if (totalOlap < 0) totalOlap = 0;
  if (totalOlap > (int)kMaxReadLen) totalOlap = (int)kMaxReadLen;
  const int errorLimit = error_bound(totalOlap, w.P.maxErate);

  w.leftLen = w.rightLen = 0;

  if (sRightLen == 0 || tRightLen == 0) {
    sHi = tHi = 0;
    rToEnd    = true;
  } else if (sRightLen <= tRightLen) {
    rightErrors = warp_prefix_dp<+1, GROUP, FIRST16>(w, S, sRightBegin, sRightLen, T, tRightBegin, tRightLen, errorLimit, sHi, tHi,
                                     leftover, rToEnd);
    if (w.err) return kNone;
    for (int i = lane; i < w.rightLen; i += 32) w.sc.deltaR[i] = -w.sc.deltaR[i];
  } else {
    rightErrors = warp_prefix_dp<+1, GROUP, FIRST16>(w, T, tRightBegin, tRightLen, S, sRightBegin, sRightLen, errorLimit, tHi, sHi,
                                     leftover, rToEnd);
    if (w.err) return kNone;
  }
  __syncwarp();
  sHi += sRightBegin - 1;
  tHi += tRightBegin - 1;

  leftover = 0;
  if (sLeftBegin < 0 || tLeftBegin < 0) {
    sLo = tLo = 0;
    lToEnd    = true;
  } else if (sRightBegin <= tRightBegin) {
    leftErrors = warp_prefix_dp<-1, GROUP, FIRST16>(w, S, sLeftBegin, sLeftBegin + 1, T, tLeftBegin, tLeftBegin + 1,
                                    errorLimit - rightErrors, sLo, tLo, leftover, lToEnd);
    if (w.err) return kNone;
  } else {
    leftErrors = warp_prefix_dp<-1, GROUP, FIRST16>(w, T, tLeftBegin, tLeftBegin + 1, S, sLeftBegin, sLeftBegin + 1,
                                    errorLimit - rightErrors, tLo, sLo, leftover, lToEnd);
    if (w.err) return kNone;
    for (int i = lane; i < w.leftLen; i += 32) w.sc.deltaL[i] = -w.sc.deltaL[i];
  }
  __syncwarp();
  sLo += sLeftBegin + 1;
  tLo += tLeftBegin + 1;
  errors = leftErrors + rightErrors;

  const int kind = (!rToEnd) ? ((!lToEnd) ? kNone : kRightBranch) : ((!lToEnd) ? kLeftBranch : kDovetail);

  // Merge the right delta into the left one (extend.C:164-175).
  if (w.leftLen + w.rightLen + 1 > w.cap.rowCap) { w.err |= kErrDeltaFull; return kNone; }
  if (w.rightLen > 0) {
    const int base = w.leftLen;
    if (lane == 0) {
      const int r0 = w.sc.deltaR[0];
      w.sc.deltaL[base] = (r0 > 0) ? -(r0 + leftover + mLen) : -(r0 - leftover - mLen);
    }
    for (int i = 1 + lane; i < w.rightLen; i += 32) w.sc.deltaL[base + i] = -w.sc.deltaR[i];
    w.leftLen = base + w.rightLen;
  }
  w.rightLen = 0;
  __syncwarp();
  return kind;
}

}  // namespace oic
