// oic_internal.h -- device views of a context for entry points outside oic_capi.cu.
#pragma once

#include <cuda_runtime.h>

#include "oic_common.cuh"

struct oic_ctx;

namespace oic {

struct CtxViews {
  ReadsDev            R;
  DevParams           dp;
  const int          *eml;      // Edit_Match_Limit on the device
  unsigned int       *ctr32;    // the context's small counter block (device)
  cudaStream_t        st;
  int                 device;
};

// u64 slots of the context's counter block (CtxViews::ctr32 viewed as u64) that
// oic_extend_batch_noalloc uses: [DP cells, slide bases, error flags].
constexpr int kNoAllocStatBase = 48;

// Fills *v; returns 0, or nonzero when the context has no reads loaded.
int ctx_views(oic_ctx *ctx, CtxViews *v);
void ctx_set_error(oic_ctx *ctx, const char *msg);
// Adds DP work done outside oic_capi.cu to the context's statistics.
void ctx_add_dp_work(oic_ctx *ctx, unsigned long long cells, unsigned long long slides);

}  // namespace oic
