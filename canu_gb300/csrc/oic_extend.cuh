// oic_extend.cuh -- the batched Extend_Alignment kernel (one warp per problem),
// shared by the allocating entry point (oic_pairs.cu) and the one that runs on a
// static scratch array (oic_noalloc.cu).
#pragma once

#include "oic_kernels.cuh"

namespace oic {

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
      if (CHECK && w.err) atomicOr((u32 *)(stats + 2), w.err);
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
