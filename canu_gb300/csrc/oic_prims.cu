// oic_prims.cu -- exclusive scan and stable LSD radix sort (hand-written, no library).
//
// Scan: three-phase (per-tile reduce, recursive scan of tile sums, per-tile scan).
// Sort: 8-bit digits; per pass an upsweep histogram per 4096-key tile (digit-major,
// so one exclusive scan gives every (digit, tile) its output base), then a downsweep
// that ranks keys stably inside the tile with warp match_any, groups the tile by digit
// in shared memory and writes each digit's run out with coalesced stores.
#include "oic_prims.cuh"

namespace oic {

thread_local unsigned long long g_launches = 0;

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems   = 16;
constexpr int kScanTile    = kScanThreads * kScanItems;

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Block-wide exclusive scan of one value per thread; returns the exclusive prefix and
// sets blockTotal (same value in every thread).
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t &blockTotal) {
  constexpr int NW = kScanThreads / 32;
  __shared__ uint32_t warpSums[NW + 1];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t incl = warp_incl_scan(v);
  if (lane == 31) warpSums[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    uint32_t s  = (lane < NW) ? warpSums[lane] : 0;
    uint32_t si = warp_incl_scan(s);
    if (lane < NW) warpSums[lane] = si - s;
    if (lane == NW - 1) warpSums[NW] = si;
  }
  __syncthreads();
  blockTotal = warpSums[NW];
  uint32_t r = warpSums[wid] + incl - v;
  __syncthreads();
  return r;
}

__global__ void scan_reduce_kernel(const uint32_t *in, uint64_t n, uint32_t *blockSums) {
  const uint64_t base = (uint64_t)blockIdx.x * kScanTile;
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    uint64_t i = base + (uint64_t)k * kScanThreads + threadIdx.x;
    if (i < n) s += in[i];
  }
  uint32_t tot;
  block_excl_scan(s, tot);
  if (threadIdx.x == 0) blockSums[blockIdx.x] = tot;
}

__global__ void scan_tile_kernel(const uint32_t *in, uint32_t *out, uint64_t n, const uint32_t *blockOffsets,
                                 uint32_t *total) {
  const uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    uint64_t i = base + k;
    v[k]       = (i < n) ? in[i] : 0;
    s += v[k];
  }
  uint32_t tot;
  uint32_t pre = block_excl_scan(s, tot);
  uint32_t off = (blockOffsets ? blockOffsets[blockIdx.x] : 0) + pre;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    uint64_t i = base + k;
    if (i < n) out[i] = off;
    off += v[k];
  }
  if (total && blockOffsets == nullptr && threadIdx.x == 0) *total = tot;
}

}  // namespace

size_t scan_u32_scratch(uint64_t n) {
  uint64_t nb = (n + kScanTile - 1) / kScanTile;
  if (nb <= 1) return 0;
  size_t here = ((nb * sizeof(uint32_t)) + 255) & ~(size_t)255;
  return here + scan_u32_scratch(nb);
}

cudaError_t scan_u32(const uint32_t *in, uint32_t *out, uint64_t n, uint32_t *total, void *scratch, cudaStream_t st) {
  if (n == 0) {
    if (total) return cudaMemsetAsync(total, 0, sizeof(uint32_t), st);
    return cudaSuccess;
  }
  uint64_t nb = (n + kScanTile - 1) / kScanTile;
  if (nb == 1) {
    scan_tile_kernel<<<1, kScanThreads, 0, st>>>(in, out, n, nullptr, total);
    g_launches++;
    return cudaGetLastError();
  }
  uint32_t *sums = (uint32_t *)scratch;
  size_t    here = ((nb * sizeof(uint32_t)) + 255) & ~(size_t)255;
  scan_reduce_kernel<<<(unsigned)nb, kScanThreads, 0, st>>>(in, n, sums);
    g_launches++;
  cudaError_t e = scan_u32(sums, sums, nb, total, (char *)scratch + here, st);
  if (e != cudaSuccess) return e;
  // The recursive call scans `sums` in place into block offsets.
  scan_tile_kernel<<<(unsigned)nb, kScanThreads, 0, st>>>(in, out, n, sums, nullptr);
    g_launches++;
  return cudaGetLastError();
}

// ------------------------------------------------------------------------------------
// Radix sort.

namespace {

constexpr int kSortThreads = 256;
constexpr int kSortWarps   = kSortThreads / 32;
constexpr int kSortItems   = 16;
constexpr int kSortTile    = kSortThreads * kSortItems;   // 4096
constexpr int kDigits      = 256;

__global__ void __launch_bounds__(kSortThreads) radix_upsweep_kernel(const unsigned long long *keys, uint64_t n, int shift,
                                                                     uint32_t *hist, uint32_t nTiles,
                                                                     const uint32_t *nDev) {
  __shared__ uint32_t h[kSortWarps][kDigits];
  if (nDev && *nDev < n) n = *nDev;
  const int wid = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < kSortWarps * kDigits; i += kSortThreads) (&h[0][0])[i] = 0;
  __syncthreads();
  const uint64_t base = (uint64_t)blockIdx.x * kSortTile;
#pragma unroll 4
  for (int k = 0; k < kSortItems; k++) {
    uint64_t i = base + (uint64_t)k * kSortThreads + threadIdx.x;
    if (i < n) atomicAdd(&h[wid][(keys[i] >> shift) & 0xff], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < kDigits; d += kSortThreads) {
    uint32_t s = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; w++) s += h[w][d];
    hist[(uint64_t)d * nTiles + blockIdx.x] = s;
  }
}

// Downsweep of one 4096-key tile: rank every key inside the tile (stable: warp order,
// then item order, then lane order) with warp match_any, place the tile in shared
// memory grouped by digit, then write each digit's run to its output range -- the
// writes of consecutive threads go to consecutive addresses.
__global__ void __launch_bounds__(kSortThreads) radix_downsweep_kernel(const unsigned long long *keysIn, const uint32_t *valsIn,
                                                                       unsigned long long *keysOut, uint32_t *valsOut, uint64_t n,
                                                                       int shift, const uint32_t *offsets,
                                                                       uint32_t nTiles, const uint32_t *nDev) {
  extern __shared__ __align__(16) unsigned char sortDyn[];
  unsigned long long *sk = (unsigned long long *)sortDyn;           // kSortTile keys
  uint32_t           *sv = (uint32_t *)(sk + kSortTile);             // kSortTile values
  __shared__ uint32_t cnt[kSortWarps][kDigits];
  __shared__ uint32_t tileBase[kDigits];     // output position of the tile's first key of each digit
  __shared__ uint32_t localStart[kDigits];   // position of that key inside the tile
  if (nDev && *nDev < n) n = *nDev;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < kSortWarps * kDigits; i += kSortThreads) (&cnt[0][0])[i] = 0;
  for (int d = threadIdx.x; d < kDigits; d += kSortThreads) tileBase[d] = offsets[(uint64_t)d * nTiles + blockIdx.x];
  __syncthreads();

  const uint64_t base = (uint64_t)blockIdx.x * kSortTile + (uint64_t)wid * (32 * kSortItems);
  const unsigned ltMask = (1u << lane) - 1;
  unsigned long long k[kSortItems];
  uint32_t v[kSortItems];
  uint32_t rank[kSortItems];
  int      dig[kSortItems];
#pragma unroll
  for (int it = 0; it < kSortItems; it++) {
    uint64_t i = base + (uint64_t)it * 32 + lane;
    bool     ok = i < n;
    k[it]       = ok ? keysIn[i] : 0;
    v[it]       = ok ? valsIn[i] : 0;
  }
#pragma unroll
  for (int it = 0; it < kSortItems; it++) {
    const bool ok = base + (uint64_t)it * 32 + lane < n;
    int d       = ok ? (int)((k[it] >> shift) & 0xff) : kDigits;
    dig[it]     = d;
    unsigned peers  = __match_any_sync(0xffffffffu, d);
    int      leader = __ffs(peers) - 1;
    uint32_t b      = 0;
    if (lane == leader && ok) b = cnt[wid][d];
    b         = __shfl_sync(0xffffffffu, b, leader);
    rank[it]  = b + __popc(peers & ltMask);
    __syncwarp();
    if (lane == leader && ok) cnt[wid][d] = b + __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // Per digit: the warps' exclusive prefix, then the digit's start inside the tile.
  uint32_t tot = 0;
  {
    const int d = threadIdx.x;   // kSortThreads == kDigits
    uint32_t s = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; w++) {
      uint32_t c = cnt[w][d];
      cnt[w][d]  = s;
      s += c;
    }
    uint32_t all;
    const uint32_t start = block_excl_scan(s, all);
    localStart[d] = start;
#pragma unroll
    for (int w = 0; w < kSortWarps; w++) cnt[w][d] += start;
    tot = all;
  }
  __syncthreads();
#pragma unroll
  for (int it = 0; it < kSortItems; it++) {
    if (dig[it] < kDigits) {
      const uint32_t p = cnt[wid][dig[it]] + rank[it];
      sk[p] = k[it];
      sv[p] = v[it];
    }
  }
  __syncthreads();
  for (uint32_t p = threadIdx.x; p < tot; p += kSortThreads) {
    const unsigned long long key = sk[p];
    const int d = (int)((key >> shift) & 0xff);
    const uint64_t pos = (uint64_t)tileBase[d] + (p - localStart[d]);
    keysOut[pos] = key;
    valsOut[pos] = sv[p];
  }
}

constexpr size_t kDownsweepDyn = (size_t)kSortTile * (sizeof(unsigned long long) + sizeof(uint32_t));
static_assert(kSortThreads == kDigits && kSortThreads == kScanThreads, "one digit per thread in the downsweep");

}  // namespace

size_t radix_sort_scratch(uint64_t n) {
  uint64_t nTiles = (n + kSortTile - 1) / kSortTile;
  uint64_t nh     = nTiles * kDigits;
  size_t   here   = ((nh * sizeof(uint32_t)) + 255) & ~(size_t)255;
  return here + scan_u32_scratch(nh);
}

cudaError_t radix_sort_u64_u32(unsigned long long *keys, uint32_t *vals, unsigned long long *keysAlt, uint32_t *valsAlt, uint64_t n,
                               int bits, void *scratch, cudaStream_t st, const uint32_t *nDev) {
  if (n <= 1 || bits <= 0) return cudaSuccess;
  uint64_t  nTiles = (n + kSortTile - 1) / kSortTile;
  uint64_t  nh     = nTiles * kDigits;
  uint32_t *hist   = (uint32_t *)scratch;
  void     *scanSc = (char *)scratch + (((nh * sizeof(uint32_t)) + 255) & ~(size_t)255);
  unsigned long long *ks = keys, *kd = keysAlt;
  uint32_t *vs = vals, *vd = valsAlt;
  int       passes = 0;
  static bool attrSet = false;   // opt in to the downsweep's 48 KB of dynamic shared memory (per process)
  if (!attrSet) {
    cudaError_t e = cudaFuncSetAttribute(radix_downsweep_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kDownsweepDyn);
    if (e != cudaSuccess) return e;
    attrSet = true;
  }
  for (int shift = 0; shift < bits; shift += 8, passes++) {
    radix_upsweep_kernel<<<(unsigned)nTiles, kSortThreads, 0, st>>>(ks, n, shift, hist, (uint32_t)nTiles, nDev);
    g_launches++;
    cudaError_t e = scan_u32(hist, hist, nh, nullptr, scanSc, st);
    if (e != cudaSuccess) return e;
    radix_downsweep_kernel<<<(unsigned)nTiles, kSortThreads, kDownsweepDyn, st>>>(ks, vs, kd, vd, n, shift, hist,
                                                                                   (uint32_t)nTiles, nDev);
    g_launches++;
    unsigned long long *tk = ks; ks = kd; kd = tk;
    uint32_t *tv = vs; vs = vd; vd = tv;
  }
  if (ks != keys) {
    cudaMemcpyAsync(keys, ks, n * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(vals, vs, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st);
  }
  return cudaGetLastError();
}

}  // namespace oic
