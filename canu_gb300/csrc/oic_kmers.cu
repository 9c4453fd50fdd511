// oic_kmers.cu -- frequent k-mers of the loaded reads on the GPU: the counting step
// that produces overlapInCore's -k skip file.
//
// In canu the list comes from meryl (src/pipelines/canu/Meryl.pm: `meryl count` over the
// reads, then `meryl print` of the k-mers at or above a threshold); overlapInCore reads
// the first token of each line (overlapInCore-Build_Hash_Index.C:203-246) and screens
// the k-mer and its reverse complement.  Here every k-mer window of the reads (both
// strands folded into one canonical key: the smaller of the window's key and its
// reverse complement's, in the 2-bit encoding of oic_common.cuh) is emitted, radix
// sorted, and the runs of equal keys are counted; runs of at least minCount are kept.
// Windows holding an N are skipped.  Read sets with more windows than one sort holds are
// counted in passes over ranges of the key space: a histogram of the keys' top bits
// (4096 parts) splits the key space into ranges of at most a pass's windows, and each
// pass emits only the windows whose key falls in its range.
#include "oic_kernels.cuh"
#include "oic_prims.cuh"

namespace oic {

namespace {

// Canonical key of window o of read r (base offset g0 of its words), or `invalid` for a
// window with an N.
__device__ __forceinline__ u64 canon_key(const ReadsDev &R, i64 g0, u32 L, u32 o, int K, bool hn, u64 kmask,
                                         u64 invalid) {
  const u64 fk = load_win(R.fwd, g0 + o) & kmask;
  const u64 rk = load_win(R.rc, g0 + (i64)(L - K - o)) & kmask;
  if (hn && (load_win(R.nfwd, g0 + o) & kmask)) return invalid;
  return fk < rk ? fk : rk;
}

// hist[key >> shift] for every valid window (kParts parts), via a block histogram.
constexpr int kParts = 4096;
__global__ void canon_hist_kernel(ReadsDev R, const u32 *reads, u32 nReads, int K, int shift, unsigned long long *hist,
                                  unsigned long long *nInvalid) {
  __shared__ unsigned int h[kParts];
  for (int i = threadIdx.x; i < kParts; i += blockDim.x) h[i] = 0;
  __syncthreads();
  const u64 kmask   = (K >= 32) ? ~0ull : ((1ull << (2 * K)) - 1);
  const u64 invalid = 1ull << (2 * K);
  unsigned long long bad = 0;
  for (u32 s = blockIdx.x; s < nReads; s += gridDim.x) {
    const u32 r = reads[s];
    const u32 L = R.len[r];
    if (L < (u32)K) continue;
    const i64  g0 = (i64)R.wordOff[r] * 32;
    const bool hn = R.hasN[r] != 0;
    for (u32 o = threadIdx.x; o < L - K + 1; o += blockDim.x) {
      const u64 key = canon_key(R, g0, L, o, K, hn, kmask, invalid);
      if (key == invalid) bad++;
      else atomicAdd(&h[key >> shift], 1u);
    }
    // Flush before a block's counters could wrap (a read has < 2^21 windows).
    if (((s / gridDim.x) & 1023) == 1023) {
      __syncthreads();
      for (int i = threadIdx.x; i < kParts; i += blockDim.x)
        if (h[i]) {
          atomicAdd(&hist[i], (unsigned long long)h[i]);
          h[i] = 0;
        }
      __syncthreads();
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kParts; i += blockDim.x)
    if (h[i]) atomicAdd(&hist[i], (unsigned long long)h[i]);
  if (bad) atomicAdd(nInvalid, bad);
}

// The valid windows whose key's part lies in [p0, p1), appended at counter positions
// (one atomic per warp and step).
__global__ void canon_emit_part_kernel(ReadsDev R, const u32 *reads, u32 nReads, int K, int shift, u32 p0, u32 p1,
                                       u64 *keys, u32 *vals, unsigned long long *counter) {
  const u64 kmask   = (K >= 32) ? ~0ull : ((1ull << (2 * K)) - 1);
  const u64 invalid = 1ull << (2 * K);
  const int lane    = threadIdx.x & 31;
  for (u32 s = blockIdx.x; s < nReads; s += gridDim.x) {
    const u32 r = reads[s];
    const u32 L = R.len[r];
    if (L < (u32)K) continue;   // uniform across the block
    const i64  g0 = (i64)R.wordOff[r] * 32;
    const bool hn = R.hasN[r] != 0;
    const u32  nk = L - K + 1;
    for (u32 o0 = threadIdx.x & ~31u; o0 < nk; o0 += blockDim.x) {
      const u32 o = o0 + lane;
      u64  key  = invalid;
      bool take = false;
      if (o < nk) {
        key = canon_key(R, g0, L, o, K, hn, kmask, invalid);
        if (key != invalid) {
          const u32 part = (u32)(key >> shift);
          take           = part >= p0 && part < p1;
        }
      }
      const unsigned m = __ballot_sync(0xffffffffu, take);
      if (!m) continue;
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(counter, (unsigned long long)__popc(m));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (take) {
        const u64 at = base + __popc(m & ((1u << lane) - 1));
        keys[at] = key;
        vals[at] = 0;
      }
    }
  }
}

// flags[i] = 1 where a run of equal valid keys starts (i < nValid).
__global__ void run_start_kernel(const u64 *keys, u64 nValid, u32 *flags) {
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < nValid; i += (u64)gridDim.x * blockDim.x)
    flags[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1u : 0u;
}

// runStart[pos[i]] = i for every run start i.
__global__ void run_index_kernel(const u32 *flags, const u32 *pos, u64 nValid, u64 *runStart) {
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < nValid; i += (u64)gridDim.x * blockDim.x)
    if (flags[i]) runStart[pos[i]] = i;
}

// sel[j] = 1 when run j (keys[runStart[j] .. next run)) has at least minCount keys.
__global__ void run_select_kernel(const u64 *runStart, u32 nRuns, u64 nValid, u32 minCount, u32 *sel) {
  for (u32 j = blockIdx.x * blockDim.x + threadIdx.x; j < nRuns; j += gridDim.x * blockDim.x) {
    const u64 e = j + 1 < nRuns ? runStart[j + 1] : nValid;
    sel[j]      = (e - runStart[j] >= minCount) ? 1u : 0u;
  }
}

__global__ void run_compact_kernel(const u64 *keys, const u64 *runStart, u32 nRuns, u64 nValid, const u32 *sel,
                                   const u32 *pos, u64 *outKey, u32 *outCount) {
  for (u32 j = blockIdx.x * blockDim.x + threadIdx.x; j < nRuns; j += gridDim.x * blockDim.x) {
    if (!sel[j]) continue;
    const u64 e   = j + 1 < nRuns ? runStart[j + 1] : nValid;
    const u64 c   = e - runStart[j];
    outKey[pos[j]]   = keys[runStart[j]];
    outCount[pos[j]] = c > 0xffffffffull ? 0xffffffffu : (u32)c;
  }
}

unsigned grid_for(u64 n, unsigned per = 256) {
  u64 g = (n + per - 1) / per;
  if (g < 1) g = 1;
  if (g > 65535u * 8) g = 65535u * 8;
  return (unsigned)g;
}

}  // namespace

int canon_parts() { return kParts; }

void launch_canon_hist(ReadsDev R, const u32 *reads, u32 nReads, int K, int shift, unsigned long long *hist,
                       unsigned long long *nInvalid, cudaStream_t st) {
  if (nReads == 0) return;
  canon_hist_kernel<<<nReads < 152u * 8 ? nReads : 152u * 8, 256, 0, st>>>(R, reads, nReads, K, shift, hist, nInvalid);
  g_launches++;
}

void launch_canon_emit_part(ReadsDev R, const u32 *reads, u32 nReads, int K, int shift, u32 p0, u32 p1, u64 *keys,
                            u32 *vals, unsigned long long *counter, cudaStream_t st) {
  if (nReads == 0) return;
  canon_emit_part_kernel<<<nReads < 65535u * 4 ? nReads : 65535u * 4, 256, 0, st>>>(R, reads, nReads, K, shift, p0, p1,
                                                                                   keys, vals, counter);
  g_launches++;
}

void launch_run_starts(const u64 *keys, u64 nValid, u32 *flags, cudaStream_t st) {
  if (nValid == 0) return;
  run_start_kernel<<<grid_for(nValid), 256, 0, st>>>(keys, nValid, flags);
  g_launches++;
}

void launch_run_index(const u32 *flags, const u32 *pos, u64 nValid, u64 *runStart, cudaStream_t st) {
  if (nValid == 0) return;
  run_index_kernel<<<grid_for(nValid), 256, 0, st>>>(flags, pos, nValid, runStart);
  g_launches++;
}

void launch_run_select(const u64 *runStart, u32 nRuns, u64 nValid, u32 minCount, u32 *sel, cudaStream_t st) {
  if (nRuns == 0) return;
  run_select_kernel<<<grid_for(nRuns), 256, 0, st>>>(runStart, nRuns, nValid, minCount, sel);
  g_launches++;
}

void launch_run_compact(const u64 *keys, const u64 *runStart, u32 nRuns, u64 nValid, const u32 *sel, const u32 *pos,
                        u64 *outKey, u32 *outCount, cudaStream_t st) {
  if (nRuns == 0) return;
  run_compact_kernel<<<grid_for(nRuns), 256, 0, st>>>(keys, runStart, nRuns, nValid, sel, pos, outKey, outCount);
  g_launches++;
}

}  // namespace oic
