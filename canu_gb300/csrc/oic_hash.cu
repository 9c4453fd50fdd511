// oic_hash.cu -- read packing and the k-mer hash block on the GPU.
//
// The reference (overlapInCore-Build_Hash_Index.C:414-631) inserts every ACGT-only
// k-mer of the block's reads one at a time into a bucketed hash table whose chains
// list each k-mer's occurrences newest first.  Here the block is built data-parallel:
// every k-mer window is emitted with its position, the (key, position) pairs are
// sorted stably by key, and one open-addressing table maps each distinct key to its
// run of occurrences (ascending position; the probe walks it backwards to get the
// reference's chain order).  The distinct-k-mer load limit that ends a block
// (:445, :504-506) is found from the first occurrence of every key.
#include "oic_kernels.cuh"
#include "oic_prims.cuh"

namespace oic {

namespace {

__device__ __forceinline__ int base_code(unsigned char c, bool &isN, bool &bad) {
  switch (c) {
    case 'A': case 'a': return 0;
    case 'C': case 'c': return 1;
    case 'G': case 'g': return 2;
    case 'T': case 't': return 3;
    case 'N': case 'n': isN = true; return 0;
    default: isN = true; bad = true; return 0;
  }
}

// Block per read, thread per 32-base word of both strands.
__global__ void pack_reads_kernel(const char *ascii, const u64 *srcOff, const u32 *len, const u64 *wordOff, u32 nReads,
                                  u64 *fwd, u64 *rc, u64 *nfwd, u64 *nrc, unsigned char *hasN, u32 *err) {
  for (u32 r = blockIdx.x; r < nReads; r += gridDim.x) {
    const u32  L   = len[r];
    const u64  w0  = wordOff[r];
    const u32  nw  = (L + 31) / 32;
    const char *s  = ascii + srcOff[r];
    bool anyN = false, anyBad = false;
    for (u32 w = threadIdx.x; w < nw; w += blockDim.x) {
      u64 f = 0, fm = 0, b = 0, bm = 0;
      for (int j = 0; j < 32; j++) {
        u32 p = w * 32 + j;
        if (p >= L) break;
        bool n1 = false, bad1 = false, n2 = false, bad2 = false;
        int  c1 = base_code((unsigned char)s[p], n1, bad1);
        int  c2 = base_code((unsigned char)s[L - 1 - p], n2, bad2);   // RC base p
        f |= (u64)c1 << (2 * j);
        if (n1) fm |= 3ull << (2 * j);
        b |= (u64)(n2 ? 0 : (3 - c2)) << (2 * j);
        if (n2) bm |= 3ull << (2 * j);
        anyN |= n1;
        anyBad |= bad1;
      }
      fwd[w0 + w]  = f;
      nfwd[w0 + w] = fm;
      rc[w0 + w]   = b;
      nrc[w0 + w]  = bm;
    }
    anyN   = __syncthreads_or(anyN);
    anyBad = __syncthreads_or(anyBad);
    if (threadIdx.x == 0) {
      hasN[r] = anyN ? 1 : 0;
      if (anyBad) atomicOr(err, kErrBadBase);
    }
  }
}

__global__ void kmer_emit_kernel(ReadsDev R, const u32 *strRead, const u32 *strKmers, const u64 *flatStart, u32 nStr,
                                 int K, u64 *keys, u32 *vals) {
  const u64 kmask   = (K >= 32) ? ~0ull : ((1ull << (2 * K)) - 1);
  const u64 invalid = 1ull << (2 * K);
  for (u32 s = blockIdx.x; s < nStr; s += gridDim.x) {
    const u32 nk = strKmers[s];
    if (nk == 0) continue;
    const u32 r   = strRead[s];
    const i64 g0  = (i64)R.wordOff[r] * 32;
    const bool hn = R.hasN[r] != 0;
    const u64 f0  = flatStart[s];
    for (u32 o = threadIdx.x; o < nk; o += blockDim.x) {
      u64 key = load_win(R.fwd, g0 + o) & kmask;
      if (hn && (load_win(R.nfwd, g0 + o) & kmask)) key = invalid;
      keys[f0 + o] = key;
      vals[f0 + o] = (u32)(f0 + o);
    }
  }
}

// Block string holding flat k-mer index `flat` (< flatStart[nStr]): the last s with
// flatStart[s] <= flat.  chunkStr[c] is that string for flat index c << kChunkBits, so
// the walk from it passes at most the strings that start inside one chunk.
constexpr int kChunkBits = 12;
__device__ __forceinline__ u32 string_of(const u64 *flatStart, const u32 *chunkStr, u64 flat) {
  u32 s = __ldg(chunkStr + (flat >> kChunkBits));
  while (__ldg(flatStart + s + 1) <= flat) s++;
  return s;
}

__device__ __forceinline__ u32 string_of_search(const u64 *flatStart, u32 nStr, u64 flat) {
  // last s with flatStart[s] <= flat
  u32 lo = 0, hi = nStr;
  while (hi - lo > 1) {
    u32 mid = (lo + hi) >> 1;
    if (flatStart[mid] <= flat) lo = mid;
    else hi = mid;
  }
  return lo;
}

__global__ void first_occ_kernel(const u64 *keys, const u32 *vals, u64 n, const u64 *flatStart, const u32 *chunkStr,
                                 int K, u32 *newKeys) {
  const u64 invalid = 1ull << (2 * K);
  for (u64 p = (u64)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (u64)gridDim.x * blockDim.x) {
    u64 k = keys[p];
    if (k >= invalid) continue;
    if (p == 0 || keys[p - 1] != k) atomicAdd(&newKeys[string_of(flatStart, chunkStr, vals[p])], 1u);
  }
}

__global__ void keep_flags_kernel(const u64 *keys, const u32 *vals, u64 n, int K, u32 flatLimit, u32 *flags) {
  const u64 invalid = 1ull << (2 * K);
  for (u64 p = (u64)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (u64)gridDim.x * blockDim.x)
    flags[p] = (keys[p] < invalid && vals[p] < flatLimit) ? 1u : 0u;
}

__global__ void compact_kv_kernel(const u64 *keys, const u32 *vals, const u32 *flags, const u32 *pos, u64 n,
                                  u64 *keysOut, u32 *valsOut) {
  for (u64 p = (u64)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (u64)gridDim.x * blockDim.x)
    if (flags[p]) {
      keysOut[pos[p]] = keys[p];
      valsOut[pos[p]] = vals[p];
    }
}

__device__ __forceinline__ bool table_slot(const u64 *tKV, u64 mask, u64 key, u64 &slot) {
  u64 s = mix64(key) & mask;
  for (u64 probe = 0; probe <= mask; probe++) {
    u64 k = tKV[2 * s];
    if (k == key) { slot = s; return true; }
    if (k == kEmptyKey) return false;
    s = (s + 1) & mask;
  }
  return false;
}

// Every slot empty: key all ones, value 0 (one 16-byte store per slot).
__global__ void table_init_kernel(u64 *tKV, u64 cap) {
  for (u64 s = (u64)blockIdx.x * blockDim.x + threadIdx.x; s < cap; s += (u64)gridDim.x * blockDim.x)
    ((ulonglong2 *)tKV)[s] = make_ulonglong2(kEmptyKey, 0ull);
}

// Run starts claim a slot; the occurrence run begins at p.
__global__ void table_starts_kernel(const u64 *keys, u64 n, u64 *tKV, u64 mask, u32 *err) {
  for (u64 p = (u64)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (u64)gridDim.x * blockDim.x) {
    u64 k = keys[p];
    if (p > 0 && keys[p - 1] == k) continue;
    u64  s    = mix64(k) & mask;
    bool done = false;
    for (u64 probe = 0; probe <= mask; probe++) {
      u64 old = atomicCAS(&tKV[2 * s], kEmptyKey, k);
      if (old == kEmptyKey || old == k) {
        tKV[2 * s + 1] = p;
        done     = true;
        break;
      }
      s = (s + 1) & mask;
    }
    if (!done) atomicOr(err, kErrTableFull);
  }
}

// Run ends fill in the count.
__global__ void table_counts_kernel(const u64 *keys, u64 n, u64 *tKV, u64 mask) {
  for (u64 p = (u64)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (u64)gridDim.x * blockDim.x) {
    u64 k = keys[p];
    if (p + 1 < n && keys[p + 1] == k) continue;
    u64 s;
    if (table_slot(tKV, mask, k, s)) {
      u64 start      = tKV[2 * s + 1] & 0xffffffffull;
      tKV[2 * s + 1] = start | ((p + 1 - start) << 32);
    }
  }
}

__global__ void occ_convert_kernel(const u32 *vals, u64 n, const u64 *flatStart, const u32 *chunkStr, u64 *occ) {
  for (u64 p = (u64)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (u64)gridDim.x * blockDim.x) {
    u64 flat = vals[p];
    u32 s    = string_of(flatStart, chunkStr, flat);
    occ[p]   = ((u64)s << 32) | (u64)(flat - flatStart[s]);
  }
}

// Mark_Skip_Kmers / Hash_Mark_Empty (Build_Hash_Index.C:130-257): screen the k-mer;
// screen the read ends near its occurrences (Mark_Screened_Ends_Chain, :96-121); with
// the hopeless check on, an absent k-mer gets an empty entry of its own
// (Add_Extra_Hash_String, :26-86) so that probes still see it as screened.
__global__ void skip_mark_kernel(const u64 *skipKeys, u64 nSkip, TableDev T, u64 *tKV,
                                 unsigned char *lscr, unsigned char *rscr, int K, int hopeless, u32 *err) {
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < nSkip; i += (u64)gridDim.x * blockDim.x) {
    const u64 key = skipKeys[i];
    u64       s   = mix64(key) & T.mask;
    bool      done = false;
    for (u64 probe = 0; probe <= T.mask && !done; probe++) {
      u64 k = tKV[2 * s];
      if (k == kEmptyKey) {
        if (!hopeless) { done = true; break; }
        k = atomicCAS(&tKV[2 * s], kEmptyKey, key);
        if (k == kEmptyKey) {
          atomicOr(&tKV[2 * s + 1], 1ull << 63);   // count 0, screened
          done = true;
          break;
        }
      }
      if (k == key) {
        u64 v = atomicOr(&tKV[2 * s + 1], 1ull << 63);
        u32 start = (u32)(v & 0xffffffffull);
        u32 cnt   = (u32)((v >> 32) & 0x7fffffffull);
        for (u32 j = 0; j < cnt; j++) {
          u64 o   = T.occ[start + j];
          u32 str = (u32)(o >> 32);
          u64 off = (u32)o;
          if (off < (u64)kHopelessMatch) lscr[str] = 1;
          if ((u64)T.slen[str] - off - (u64)K + 1 < (u64)kHopelessMatch) rscr[str] = 1;
        }
        done = true;
        break;
      }
      s = (s + 1) & T.mask;
    }
    if (!done) atomicOr(err, kErrTableFull);
  }
}

inline unsigned grid_for(u64 n, int threads) {
  u64 g = (n + threads - 1) / threads;
  if (g > 65535ull * 16) g = 65535ull * 16;
  if (g == 0) g = 1;
  return (unsigned)g;
}

}  // namespace

void launch_pack_reads(const char *ascii, const u64 *srcOff, const u32 *len, const u64 *wordOff, u32 nReads, u64 *fwd,
                       u64 *rc, u64 *nfwd, u64 *nrc, unsigned char *hasN, u32 *err, cudaStream_t st) {
  if (nReads == 0) return;
  unsigned g = nReads < 65535u * 4 ? nReads : 65535u * 4;
  pack_reads_kernel<<<g, 128, 0, st>>>(ascii, srcOff, len, wordOff, nReads, fwd, rc, nfwd, nrc, hasN, err);
  g_launches++;
}

void launch_kmer_emit(ReadsDev R, const u32 *strRead, const u32 *strKmers, const u64 *flatStart, u32 nStr, int K,
                      u64 *keys, u32 *vals, cudaStream_t st) {
  if (nStr == 0) return;
  unsigned g = nStr < 65535u * 4 ? nStr : 65535u * 4;
  kmer_emit_kernel<<<g, 256, 0, st>>>(R, strRead, strKmers, flatStart, nStr, K, keys, vals);
  g_launches++;
}

// chunkStr[c] = block string holding flat k-mer index c << 12 (see string_of).
__global__ void chunk_str_kernel(const u64 *flatStart, u32 nStr, u64 nChunks, u32 *chunkStr) {
  for (u64 c = (u64)blockIdx.x * blockDim.x + threadIdx.x; c < nChunks; c += (u64)gridDim.x * blockDim.x)
    chunkStr[c] = string_of_search(flatStart, nStr, c << kChunkBits);
}

void launch_chunk_str(const u64 *flatStart, u32 nStr, u64 nFlat, u32 *chunkStr, cudaStream_t st) {
  const u64 nChunks = (nFlat >> kChunkBits) + 1;
  chunk_str_kernel<<<grid_for(nChunks, 256), 256, 0, st>>>(flatStart, nStr, nChunks, chunkStr);
  g_launches++;
}

void launch_first_occ(const u64 *keys, const u32 *vals, u64 n, const u64 *flatStart, const u32 *chunkStr, int K,
                      u32 *newKeys,
                      cudaStream_t st) {
  if (n == 0) return;
  first_occ_kernel<<<grid_for(n, 256), 256, 0, st>>>(keys, vals, n, flatStart, chunkStr, K, newKeys);
  g_launches++;
}

void launch_keep_flags(const u64 *keys, const u32 *vals, u64 n, int K, u32 flatLimit, u32 *flags, cudaStream_t st) {
  if (n == 0) return;
  keep_flags_kernel<<<grid_for(n, 256), 256, 0, st>>>(keys, vals, n, K, flatLimit, flags);
  g_launches++;
}

void launch_compact_kv(const u64 *keys, const u32 *vals, const u32 *flags, const u32 *pos, u64 n, u64 *keysOut,
                       u32 *valsOut, cudaStream_t st) {
  if (n == 0) return;
  compact_kv_kernel<<<grid_for(n, 256), 256, 0, st>>>(keys, vals, flags, pos, n, keysOut, valsOut);
  g_launches++;
}

void launch_table_init(u64 *tKV, u64 cap, cudaStream_t st) {
  table_init_kernel<<<grid_for(cap, 256), 256, 0, st>>>(tKV, cap);
  g_launches++;
}

void launch_table_build(const u64 *keys, u64 n, u64 *tKV, u64 mask, u32 *err, cudaStream_t st) {
  if (n == 0) return;
  table_starts_kernel<<<grid_for(n, 256), 256, 0, st>>>(keys, n, tKV, mask, err);
  g_launches++;
  table_counts_kernel<<<grid_for(n, 256), 256, 0, st>>>(keys, n, tKV, mask);
  g_launches++;
}

void launch_occ_convert(const u32 *vals, u64 n, const u64 *flatStart, const u32 *chunkStr, u64 *occ, cudaStream_t st) {
  if (n == 0) return;
  occ_convert_kernel<<<grid_for(n, 256), 256, 0, st>>>(vals, n, flatStart, chunkStr, occ);
  g_launches++;
}

void launch_skip_mark(const u64 *skipKeys, u64 nSkip, TableDev T, u64 *tKVMut, unsigned char *lscr,
                      unsigned char *rscr, int K, int hopeless, u32 *err, cudaStream_t st) {
  if (nSkip == 0) return;
  skip_mark_kernel<<<grid_for(nSkip, 128), 128, 0, st>>>(skipKeys, nSkip, T, tKVMut, lscr, rscr, K, hopeless, err);
  g_launches++;
}

}  // namespace oic
