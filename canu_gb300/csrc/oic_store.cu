// oic_store.cu -- the record pass of the overlap-store build on the GPU.
//
// Reference: ovStoreBuild (src/stores/ovStoreBuild.C:166-255) reads every overlapper
// record, runs ovStoreFilter::filterOverlap on it (src/stores/ovStoreFilter.C:62-160:
// IDs must lie in 1..maxID; a record whose evalue exceeds the encoded --e error rate
// loses its forUTG/forOBT/forDUP flags; the ID-swapped copy is made by
// ovOverlap::swapIDs, src/stores/ovOverlap.C:216-246), keeps each of the record and its
// copy that still has one of the three flags, and sorts the kept records with
// ovOverlap::operator< (a_iid, b_iid, then the two data words; ovOverlap.H:264-277).
// The sorted array is what its store writer lays out per a_iid.
//
// Here: one thread per input record writes both copies and their keep flags; a scan
// compacts the kept copies; the library's radix sort orders them by (a_iid, b_iid) as
// one 64-bit key (stable); the rare runs of equal (a_iid, b_iid) are then ordered by the
// data words; a gather writes the records in that order, and a histogram + scan of
// a_iid gives the first record of every read.
//
// Record words (ovFile's full record): a_iid, b_iid, dat0 >> 32, dat0, dat1 >> 32,
// dat1; dat0 = ahg5:21 | ahg3:21 | evalue:16 | flipped | forOBT | forDUP | forUTG,
// dat1 = bhg5:21 | bhg3:21 | span:21 (ovOverlap.H:55-70, AS_MAX_READLEN_BITS 21).
#include <algorithm>
#include <vector>

#include "oic_gpu.h"
#include "oic_common.cuh"
#include "oic_prims.cuh"

namespace oic {
namespace {

constexpr u64 kM21 = (1ull << 21) - 1;

// counters: [saved unitigging, saved trimming, discarded erate, bad IDs]
__global__ void store_expand_kernel(const u32 *in, u64 n, u32 maxID, u32 maxEvalue, u32 *rec, u64 *keys, u32 *keep,
                                    unsigned long long *counters) {
  unsigned long long utg = 0, obt = 0, erate = 0, bad = 0;
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
    const u32 *w = in + 6 * i;
    const u32 a = w[0], b = w[1];
    u64 d0 = ((u64)w[2] << 32) | w[3];
    u64 d1 = ((u64)w[4] << 32) | w[5];
    if (a == 0 || b == 0 || a > maxID || b > maxID) bad++;
    const u32 ev = (u32)((d0 >> 42) & 0xffff);
    if (ev > maxEvalue) {
      d0 &= ~(7ull << 59);   // forOBT, forDUP, forUTG
      erate += 2;
    }
    // swapIDs: A and B hangs exchanged; 5' and 3' exchanged too when flipped.
    const u64 ahg5 = d0 & kM21, ahg3 = (d0 >> 21) & kM21, bhg5 = d1 & kM21, bhg3 = (d1 >> 21) & kM21;
    const bool flip = (d0 >> 58) & 1;
    const u64 ra5 = flip ? bhg3 : bhg5, ra3 = flip ? bhg5 : bhg3, rb5 = flip ? ahg3 : ahg5, rb3 = flip ? ahg5 : ahg3;
    const u64 r0 = (d0 & ~(kM21 | (kM21 << 21))) | ra5 | (ra3 << 21);
    const u64 r1 = (d1 & ~(kM21 | (kM21 << 21))) | rb5 | (rb3 << 21);
    const bool k = ((d0 >> 59) & 7) != 0;   // the copy carries the same flags
    const u32 fw[6] = {a, b, (u32)(d0 >> 32), (u32)d0, (u32)(d1 >> 32), (u32)d1};
    const u32 rw[6] = {b, a, (u32)(r0 >> 32), (u32)r0, (u32)(r1 >> 32), (u32)r1};
#pragma unroll
    for (int j = 0; j < 6; j++) {
      rec[12 * i + j]     = fw[j];
      rec[12 * i + 6 + j] = rw[j];
    }
    keys[2 * i]     = ((u64)a << 32) | b;
    keys[2 * i + 1] = ((u64)b << 32) | a;
    keep[2 * i]     = k;
    keep[2 * i + 1] = k;
    const u64 fUTG = (d0 >> 61) & 1, fOBT = (d0 >> 59) & 1;
    utg += 2 * fUTG;
    obt += 2 * fOBT;
  }
  if (utg) atomicAdd(&counters[0], utg);
  if (obt) atomicAdd(&counters[1], obt);
  if (erate) atomicAdd(&counters[2], erate);
  if (bad) atomicAdd(&counters[3], bad);
}

__global__ void store_compact_kernel(const u64 *keys, const u32 *keep, const u32 *pos, u64 n, u64 *keysOut,
                                     u32 *idxOut) {
  for (u64 p = (u64)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (u64)gridDim.x * blockDim.x)
    if (keep[p]) {
      keysOut[pos[p]] = keys[p];
      idxOut[pos[p]]  = (u32)p;
    }
}

__device__ __forceinline__ bool data_less(const u32 *rec, u32 x, u32 y) {
  const u32 *a = rec + 6 * (u64)x, *b = rec + 6 * (u64)y;
#pragma unroll
  for (int j = 2; j < 6; j++)
    if (a[j] != b[j]) return a[j] < b[j];
  return false;
}

// Runs of equal (a_iid, b_iid) ordered by the data words (insertion sort by the run's
// first thread; runs hold the few overlaps of one read pair).
__global__ void store_ties_kernel(const u64 *keys, u32 *idx, const u32 *rec, u64 m) {
  for (u64 p = (u64)blockIdx.x * blockDim.x + threadIdx.x; p < m; p += (u64)gridDim.x * blockDim.x) {
    if (p > 0 && keys[p - 1] == keys[p]) continue;
    if (p + 1 >= m || keys[p + 1] != keys[p]) continue;
    u64 e = p + 1;
    while (e < m && keys[e] == keys[p]) e++;
    for (u64 i = p + 1; i < e; i++) {
      const u32 v = idx[i];
      u64 j = i;
      while (j > p && data_less(rec, v, idx[j - 1])) {
        idx[j] = idx[j - 1];
        j--;
      }
      idx[j] = v;
    }
  }
}

__global__ void store_gather_kernel(const u32 *rec, const u32 *idx, u64 m, u32 *out, u32 *aCount) {
  for (u64 p = (u64)blockIdx.x * blockDim.x + threadIdx.x; p < m; p += (u64)gridDim.x * blockDim.x) {
    const u32 *s = rec + 6 * (u64)idx[p];
#pragma unroll
    for (int j = 0; j < 6; j++) out[6 * p + j] = s[j];
    atomicAdd(&aCount[s[0]], 1u);
  }
}

unsigned grid_of(u64 n) {
  u64 g = (n + 255) / 256;
  if (g > 65535ull * 8) g = 65535ull * 8;
  return (unsigned)(g ? g : 1);
}

// A device buffer freed on scope exit.
struct Buf {
  void *p = nullptr;
  ~Buf() {
    if (p) cudaFree(p);
  }
  cudaError_t get(size_t n) { return cudaMalloc(&p, n ? n : 16); }
  template <class T> T *as() const { return (T *)p; }
};

}  // namespace
}  // namespace oic

using namespace oic;

extern "C" int oic_store_sort(int device, const uint32_t *words, uint64_t nRecords, uint32_t maxID, double maxErate,
                              uint32_t *out, uint64_t *nOut, uint64_t *perRead, uint64_t *counts) {
  if (!nOut || (nRecords && (!words || !out))) return OIC_ERR_ARG;
  *nOut = 0;
  if (nRecords > 0x7fffffffull) return OIC_ERR_OVERFLOW;   // record indices are 32-bit
  if (cudaSetDevice(device) != cudaSuccess) return OIC_ERR_CUDA;
  // AS_OVS_encodeEvalue (ovOverlap.H:35): double arithmetic, rounded to nearest.
  const double   maxQ      = 65535 / 100000.0;
  const uint32_t maxEvalue = (maxErate < maxQ) ? (uint32_t)(100000.0 * maxErate + 0.5) : 65535u;
  const uint64_t n2        = 2 * nRecords;
  cudaStream_t   st        = nullptr;
  Buf dIn, dRec, dKeys, dKeep, dPos, dK2, dIdx, dK3, dIdx2, dScr, dCnt, dOut, dA, dAOff;
  const size_t scr =
      std::max(std::max(scan_u32_scratch(n2 + 1), radix_sort_scratch(n2)), scan_u32_scratch((uint64_t)maxID + 2)) + 256;
#define TRY(x)                                                                                  \
  do {                                                                                          \
    cudaError_t e_ = (x);                                                                       \
    if (e_ != cudaSuccess) return e_ == cudaErrorMemoryAllocation ? OIC_ERR_NOMEM : OIC_ERR_CUDA; \
  } while (0)
  TRY(dIn.get(nRecords * 24));
  TRY(dRec.get(n2 * 24));
  TRY(dKeys.get(n2 * 8));
  TRY(dKeep.get((n2 + 1) * 4));
  TRY(dPos.get((n2 + 1) * 4));
  TRY(dK2.get(n2 * 8));
  TRY(dIdx.get(n2 * 4));
  TRY(dK3.get(n2 * 8));
  TRY(dIdx2.get(n2 * 4));
  TRY(dScr.get(scr));
  TRY(dCnt.get(8 * 8 + 4 * 4));   // 8 u64 counters, then the compaction total
  TRY(dA.get(((size_t)maxID + 2) * 4));
  TRY(dAOff.get(((size_t)maxID + 2) * 4));
  unsigned long long *cnt   = dCnt.as<unsigned long long>();
  uint32_t           *total = (uint32_t *)(cnt + 8);
  TRY(cudaMemsetAsync(dCnt.p, 0, 8 * 8 + 4 * 4, st));
  TRY(cudaMemsetAsync(dA.p, 0, ((size_t)maxID + 2) * 4, st));
  TRY(cudaMemsetAsync(dKeep.as<uint32_t>() + n2, 0, 4, st));
  if (nRecords) TRY(cudaMemcpyAsync(dIn.p, words, nRecords * 24, cudaMemcpyHostToDevice, st));

  if (nRecords) {
    store_expand_kernel<<<grid_of(nRecords), 256, 0, st>>>(dIn.as<uint32_t>(), nRecords, maxID, maxEvalue,
                                                           dRec.as<uint32_t>(), dKeys.as<u64>(), dKeep.as<uint32_t>(),
                                                           cnt);
    g_launches++;
  }
  unsigned long long hc[4] = {0, 0, 0, 0};
  TRY(cudaMemcpyAsync(hc, cnt, sizeof(hc), cudaMemcpyDeviceToHost, st));
  TRY(cudaStreamSynchronize(st));
  if (hc[3]) return OIC_ERR_INPUT;   // an overlap names a read outside 1..maxID
  uint32_t m = 0;
  if (n2) {
    TRY(scan_u32(dKeep.as<uint32_t>(), dPos.as<uint32_t>(), n2, total, dScr.p, st));
    store_compact_kernel<<<grid_of(n2), 256, 0, st>>>(dKeys.as<u64>(), dKeep.as<uint32_t>(), dPos.as<uint32_t>(), n2,
                                                      dK2.as<u64>(), dIdx.as<uint32_t>());
    g_launches++;
    TRY(cudaMemcpyAsync(&m, total, 4, cudaMemcpyDeviceToHost, st));
    TRY(cudaStreamSynchronize(st));
  }
  if (m) {
    TRY(radix_sort_u64_u32((unsigned long long *)dK2.p, dIdx.as<uint32_t>(), (unsigned long long *)dK3.p,
                           dIdx2.as<uint32_t>(), m, 64, dScr.p, st));
    store_ties_kernel<<<grid_of(m), 256, 0, st>>>(dK2.as<u64>(), dIdx.as<uint32_t>(), dRec.as<uint32_t>(), m);
    g_launches++;
    TRY(dOut.get((size_t)m * 24));
    store_gather_kernel<<<grid_of(m), 256, 0, st>>>(dRec.as<uint32_t>(), dIdx.as<uint32_t>(), m, dOut.as<uint32_t>(),
                                                    dA.as<uint32_t>());
    g_launches++;
    TRY(cudaMemcpyAsync(out, dOut.p, (size_t)m * 24, cudaMemcpyDeviceToHost, st));
  }
  if (perRead) {
    // First record of each a_iid: exclusive scan of the per-read counts.
    TRY(scan_u32(dA.as<uint32_t>(), dAOff.as<uint32_t>(), (uint64_t)maxID + 2, nullptr, dScr.p, st));
    std::vector<uint32_t> off((size_t)maxID + 2);
    TRY(cudaMemcpyAsync(off.data(), dAOff.p, ((size_t)maxID + 2) * 4, cudaMemcpyDeviceToHost, st));
    TRY(cudaStreamSynchronize(st));
    for (size_t i = 0; i <= maxID; i++) perRead[i] = off[i];
    perRead[(size_t)maxID + 1] = m;
  }
  TRY(cudaStreamSynchronize(st));
  TRY(cudaGetLastError());
#undef TRY
  *nOut = m;
  if (counts) {
    counts[0] = hc[0];   // saved unitigging
    counts[1] = hc[1];   // saved trimming
    counts[2] = hc[2];   // discarded: error rate
    counts[3] = 0;       // discarded: read not trimmed (no read is marked, ovStoreFilter.C:38-55)
    counts[4] = 0;       // discarded: flipped (not compiled in, ovStoreFilter.C:103-114)
  }
  return OIC_OK;
}
