// oic_noalloc.cu -- batched Extend_Alignment for callers that cannot allocate GPU memory.
//
// Some callers of this library cannot call cudaMalloc at the point where they want to
// align: programs whose own allocator has reserved the whole device memory pool up
// front (a cudaMalloc from the library would then fail or fragment that pool), and
// plugins that were handed a fixed device-memory budget by their host application and
// must not grow it.  For them, oic_extend_batch_noalloc() runs the same warp DP as
// oic_extend_batch() on problems and outputs the caller already holds in device
// memory, and keeps the DP's working rows, traceback arena and delta lists in one
// file-scope device array (g_dpScratch, kScratchBytes bytes).  Every GPU that loads
// the library holds that array until the process exits.  The entry point itself calls
// no cudaMalloc, no cudaFree and no allocating library routine.
//
// Limits, fixed by the array: 32 warps share it, and each problem may keep at most
// 131072 DP cells and 8191 error rows on each side of its seed match.  A problem that
// needs more gets a nonzero status and the call returns OIC_ERR_OVERFLOW; the
// allocating oic_extend_batch() handles such problems.
//
// Set-up: the first call on a device, with that device current, looks up the array's
// device address with cudaGetSymbolAddress and keeps it for later calls on that device
// (host code cannot use the symbol itself: on the host it names a stand-in, not device
// memory).  Make that first call before any stream capture.  A cudaDeviceReset() ends
// the context the address belongs to; a process that resets a device must not call
// this entry point on that device afterwards.
//
// The array is shared by every call and keeps the previous call's contents; the DP
// writes each cell before it reads it, so nothing needs clearing between calls, and
// the call clears its own counters.  Calls that overlap on the GPU (two streams, or two
// host threads) race on the array and must be serialised by the caller.
#include <mutex>

#include "oic_gpu.h"
#include "oic_extend.cuh"
#include "oic_internal.h"
#include "oic_prims.cuh"

namespace oic {
namespace {

constexpr int    kNaBandW    = 512;
constexpr int    kNaWarps    = 32;                // 4 blocks of 8 warps
constexpr int    kNaArenaCap = 1 << 17;           // kept DP cells per warp
constexpr int    kNaRowCap   = 8192;              // error rows per warp
constexpr size_t kNaArenaBytes = (size_t)kNaWarps * kNaArenaCap * sizeof(int);
constexpr size_t kNaRowBytes   = (size_t)kNaWarps * kNaRowCap * sizeof(int4);
constexpr size_t kNaDeltaBytes = (size_t)kNaWarps * (kNaRowCap + 8) * sizeof(int);
constexpr size_t kScratchBytes = kNaArenaBytes + kNaRowBytes + 3 * kNaDeltaBytes;   // 23,072,768 bytes

static __device__ __align__(256) unsigned char g_dpScratch[kScratchBytes];

// Device address of g_dpScratch per device, looked up once with that device current.
constexpr int kMaxDevices = 64;
std::mutex    g_mu;
void         *g_addr[kMaxDevices];

}  // namespace
}  // namespace oic

using namespace oic;

extern "C" int oic_extend_batch_noalloc(oic_ctx *ctx, uint32_t nAlign, const oic_extend_problem *dProblems,
                                        int32_t *dOut, int32_t *dKind, int32_t *dDeltaLen, uint32_t *dStatus) {
  static_assert(sizeof(oic_extend_problem) == sizeof(ExtendProblem), "problem layout");
  CtxViews v;
  if (ctx_views(ctx, &v)) return OIC_ERR_STATE;
  if (nAlign == 0) return OIC_OK;
  if (!dProblems || !dOut || !dKind || !dDeltaLen || !dStatus) return OIC_ERR_ARG;
  if (v.device < 0 || v.device >= kMaxDevices) return OIC_ERR_ARG;
  if (cudaSetDevice(v.device) != cudaSuccess) return OIC_ERR_CUDA;

  void *base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[v.device]) {
      void *p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_dpScratch);
      if (e != cudaSuccess || !p) {
        ctx_set_error(ctx, "cudaGetSymbolAddress of the static DP scratch failed");
        return OIC_ERR_CUDA;
      }
      g_addr[v.device] = p;
    }
    base = g_addr[v.device];
  }

  unsigned char *b = (unsigned char *)base;
  WarpScratch    sc;
  sc.arena  = (int *)b;
  sc.rowHdr = (int4 *)(b + kNaArenaBytes);
  sc.deltaL = (int *)(b + kNaArenaBytes + kNaRowBytes);
  sc.deltaR = (int *)(b + kNaArenaBytes + kNaRowBytes + kNaDeltaBytes);
  sc.stack  = (int *)(b + kNaArenaBytes + kNaRowBytes + 2 * kNaDeltaBytes);
  sc.alive  = nullptr;
  sc.rowsG  = nullptr;
  AlignCaps cap;
  cap.arenaCap = kNaArenaCap;
  cap.rowCap   = kNaRowCap;
  cap.nodeCap  = 0;
  cap.bandW    = kNaBandW;
  cap.rowsGW   = kNaBandW;

  // Counters in the context's preallocated block: [cells, slides, error flags].
  unsigned long long *stats = (unsigned long long *)v.ctr32 + kNoAllocStatBase;
  if (cudaMemsetAsync(stats, 0, 3 * sizeof(unsigned long long), v.st) != cudaSuccess) return OIC_ERR_CUDA;
  constexpr int wpb = 8;
  extend_batch_kernel<kNaBandW, wpb, true><<<kNaWarps / wpb, wpb * 32, (size_t)wpb * 2 * kNaBandW * sizeof(int), v.st>>>(
      v.R, v.dp, v.eml, (const ExtendProblem *)dProblems, nAlign, sc, cap, dOut, dKind, dDeltaLen, dStatus, stats);
  g_launches++;
  unsigned long long counters[3] = {0, 0, 0};
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(counters, stats, sizeof(counters), cudaMemcpyDeviceToHost, v.st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(v.st);
  if (e != cudaSuccess) {
    ctx_set_error(ctx, cudaGetErrorString(e));
    return OIC_ERR_CUDA;
  }
  ctx_add_dp_work(ctx, counters[0], counters[1]);
  const uint32_t flags = (uint32_t)counters[2];
  if (flags & kErrInternal) {
    ctx_set_error(ctx, "a problem names a read outside the store or a match outside its reads");
    return OIC_ERR_ARG;
  }
  if (flags) {
    ctx_set_error(ctx, "a problem exceeds the static scratch (131072 kept DP cells or 8191 error rows per side)");
    return OIC_ERR_OVERFLOW;
  }
  return OIC_OK;
}
