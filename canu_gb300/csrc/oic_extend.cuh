// oic_extend.cuh -- the batched Extend_Alignment kernel (one warp per problem),
// shared by the allocating entry point (oic_pairs.cu) and the one that runs on a
// static scratch array (oic_noalloc.cu).
#pragma once

#include "oic_kernels.cuh"

namespace oic {

// Problems i = first, first + stride, ... by one warp (the pair logic of a group CTA).
template <bool CHECK, bool GROUP>
static __device__ __forceinline__ void extend_loop(WarpDP &w, const ReadsDev &R, const ExtendProblem *probs, u32 n,
                                                   u64 first, u64 stride, int *out, int *kind, int *deltaLen,
                                                   u32 *status, unsigned long long *stats) {
  const int lane = threadIdx.x & 31;
  for (u64 i = first; i < n; i += stride) {
    const ExtendProblem pb = probs[i];
    // Problems are checked here too: a caller may hand them over in device memory.
    if (CHECK && (pb.sRead >= R.nReads || pb.tRead >= R.nReads || pb.mLen < 1 || pb.mStart < 0 || pb.mOffset < 0 ||
        (u64)pb.mStart + pb.mLen > R.len[pb.sRead] || (u64)pb.mOffset + pb.mLen > R.len[pb.tRead])) {
      if (lane == 0) {
        status[i] = kErrInternal;
        kind[i]   = 0;
        atomicOr((u32 *)(stats + 2), kErrInternal);
      }
      continue;
    }
    const SeqView S = make_view(R, pb.sRead, pb.sRev ? 1 : 0);
    const SeqView T = make_view(R, pb.tRead, 0);
    const int sLen = (int)R.len[pb.sRead], tLen = (int)R.len[pb.tRead];
    int sLo = 0, sHi = 0, tLo = 0, tHi = 0, errors = 0;
    w.err = 0;
    const int k = warp_extend<GROUP>(w, S, sLen, T, tLen, pb.mStart, pb.mOffset, pb.mLen, sLo, sHi, tLo, tHi, errors);
    if (lane == 0) {
      out[5 * i + 0] = sLo;
      out[5 * i + 1] = sHi;
      out[5 * i + 2] = tLo;
      out[5 * i + 3] = tHi;
      out[5 * i + 4] = errors;
      kind[i]        = k;
      deltaLen[i]    = w.leftLen;
      status[i]      = w.err;
      if (CHECK && w.err) atomicOr((u32 *)(stats + 2), w.err);
    }
    __syncwarp();
  }
}

// CHECK: validate each problem on the device (for problems the host has not seen)
// and OR capacity flags into stats[2].
template <int BANDW, int WARPS, bool CHECK = false>
static __global__ void __launch_bounds__(WARPS * 32, (WARPS > 1 ? 3 : 1)) extend_batch_kernel(ReadsDev R, DevParams P, const int *eml,
                                                                  const ExtendProblem *probs, u32 n, WarpScratch scBase,
                                                                  AlignCaps cap, int *out, int *kind, int *deltaLen,
                                                                  u32 *status, unsigned long long *stats) {
  extern __shared__ int smemRows[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const u64 gw   = (u64)blockIdx.x * WARPS + wib;
  const u64 nw   = (u64)gridDim.x * WARPS;

  WarpDP w;
  int *smA = smemRows + (size_t)wib * 2 * BANDW;
  warp_dp_init(w, warp_scratch(scBase, cap, gw), cap, smA, smA + BANDW, eml, P);
  extend_loop<CHECK, false>(w, R, probs, n, gw, nw, out, kind, deltaLen, status, stats);
  const unsigned long long slidesWarp = warp_sum64(w.slides);
  if (lane == 0) {
    atomicAdd(&stats[0], w.cells);
    atomicAdd(&stats[1], slidesWarp);
  }
}

// One problem per CTA: warp 0 runs Extend_Alignment and the whole CTA runs each
// error-row loop (group_rows, U diagonals per thread per pass), as in the wide bins of
// the pair DP.  Row buffers: cap.bandW ints each in dynamic shared memory.
template <bool CHECK = false>
static __global__ void __launch_bounds__(512, 1) extend_group_kernel(ReadsDev R, DevParams P, const int *eml,
                                                                      const ExtendProblem *probs, u32 n,
                                                                      WarpScratch scBase, AlignCaps cap, int *out,
                                                                      int *kind, int *deltaLen, u32 *status,
                                                                      unsigned long long *stats, int U) {
  extern __shared__ int smemRows[];
  __shared__ GroupShared gs;
  const WarpScratch sc = warp_scratch(scBase, cap, blockIdx.x);
  if (threadIdx.x >= 32) {
    unsigned long long slides = 0;
    group_worker(gs, sc, cap, eml, slides);
    slides = warp_sum64(slides);
    if ((threadIdx.x & 31) == 0 && slides) atomicAdd(&stats[1], slides);
    return;
  }
  WarpDP w;
  warp_dp_init(w, sc, cap, smemRows, smemRows + cap.bandW, eml, P);
  w.gs       = &gs;
  w.gThreads = blockDim.x;
  w.gU       = U;
  extend_loop<CHECK, true>(w, R, probs, n, blockIdx.x, gridDim.x, out, kind, deltaLen, status, stats);
  const unsigned long long slidesWarp = warp_sum64(w.slides);
  if (threadIdx.x == 0) {
    atomicAdd(&stats[0], w.cells);
    atomicAdd(&stats[1], slidesWarp);
    gs.cmd = kGroupExit;
  }
  __syncwarp();
  group_bar(1, blockDim.x);
}

}  // namespace oic
