// oic_extend.cuh -- the batched Extend_Alignment kernel (one warp per problem).
#pragma once

#include "oic_kernels.cuh"

namespace oic {

template <int BANDW, int WARPS>
static __global__ void __launch_bounds__(WARPS * 32, (WARPS > 1 ? 3 : 1)) extend_batch_kernel(ReadsDev R, DevParams P, const int *eml,
                                                                  const ExtendProblem *probs, u32 n, WarpScratch scBase,
                                                                  AlignCaps cap, int *out, int *kind, int *deltaLen,
                                                                  u32 *status, unsigned long long *stats) {
  extern __shared__ int smemRows[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const u64 gw   = (u64)blockIdx.x * WARPS + wib;
  const u64 nw   = (u64)gridDim.x * WARPS;

  WarpDP w;
  w.sc     = warp_scratch(scBase, cap, gw);
  w.cap    = cap;
  w.smA    = smemRows + (size_t)wib * 2 * BANDW;
  w.smB    = w.smA + BANDW;
  w.eml    = eml;
  w.P      = P;
  w.cells  = 0;
  w.slides = 0;
  w.rows   = 0;
  w.err    = 0;
  w.leftLen = w.rightLen = 0;

  for (u64 i = gw; i < n; i += nw) {
    const ExtendProblem pb = probs[i];
    const SeqView S = make_view(R, pb.sRead, pb.sRev ? 1 : 0);
    const SeqView T = make_view(R, pb.tRead, 0);
    const int sLen = (int)R.len[pb.sRead], tLen = (int)R.len[pb.tRead];
    int sLo = 0, sHi = 0, tLo = 0, tHi = 0, errors = 0;
    w.err = 0;
    const int k = warp_extend(w, S, sLen, T, tLen, pb.mStart, pb.mOffset, pb.mLen, sLo, sHi, tLo, tHi, errors);
    if (lane == 0) {
      out[5 * i + 0] = sLo;
      out[5 * i + 1] = sHi;
      out[5 * i + 2] = tLo;
      out[5 * i + 3] = tHi;
      out[5 * i + 4] = errors;
      kind[i]        = k;
      deltaLen[i]    = w.leftLen;
      status[i]      = w.err;
    }
    __syncwarp();
  }
  const unsigned long long slidesWarp = warp_sum64(w.slides);
  if (lane == 0) {
    atomicAdd(&stats[0], w.cells);
    atomicAdd(&stats[1], slidesWarp);
  }
}


}  // namespace oic
