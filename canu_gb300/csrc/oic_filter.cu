// oic_filter.cu -- the learned candidate filter: per-pair features and a small MLP
// (67 -> 128 -> 128 -> 1) run on the FP16 tensor cores, for inference before the DP
// and for training on labels the exact path produces.
//
// No counterpart in the reference: overlapInCore extends every candidate pair that
// passes the hopeless check (overlapInCore-Process_String_Overlaps.C:354-547).  Here a
// pair whose filter score is below a threshold is not extended; every record that is
// emitted still comes from the exact DP.
//
// Parameters: one FP16 array (IEEE binary16 bit patterns) of kNParam values,
//   w1[128][80] | b1[128] | w2[128][128] | b2[128] | w3[128] | b3
// with weights row-major [out][in].  Layer 1 reads 80 inputs: the 67 features and 13
// zero columns, so that K is a multiple of the MMA's 16.  Activations are rounded to
// FP16 after bias + ReLU (h1, h2); every product accumulates in FP32.
//
// Features of a candidate pair (S = ref read strand, T = hash-block read), from its
// match runs (Match_Node_t: T offset, length, S start; runs of len L hold L-K+1 seeds):
//   f[0..63]  seed density over the pair's diagonals.  Diagonal d = tOff - sOff spans
//             (-lenS, lenT); bin b = floor((d + lenS) * 64 / (lenS + lenT)).  The value
//             is (seeds in the bin) / (overlap length along the bin's centre diagonal,
//             at least 64), capped at 4: a true overlap puts ~(1-e)^K seeds per base of
//             its whole overlap length on one diagonal, a shared repeat only along the
//             repeat.
//   f[64]     (ln lenS - 8) / 2
//   f[65]     (ln lenT - 8) / 2
//   f[66]     (ln(1 + seeds) - 5) / 4
//
// Tensor-core use: mma.sync.m16n8k16 (FP16 in, FP32 accumulate) with ldmatrix
// fragment loads from shared memory.  One warp owns 16 samples at a time; layer 1's
// accumulator fragments are repacked in registers as layer 2's A fragments.
#include <cuda_fp16.h>

#include "oic_gpu.h"
#include "oic_kernels.cuh"
#include "oic_prims.cuh"

namespace oic {

namespace {

constexpr int kIn   = 80;
constexpr int kHid  = 128;
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kHid * kIn;
constexpr int kOffW2 = kOffB1 + kHid;
constexpr int kOffB2 = kOffW2 + kHid * kHid;
constexpr int kOffW3 = kOffB2 + kHid;
constexpr int kOffB3 = kOffW3 + kHid;
constexpr int kNParam = kOffB3 + 1;
static_assert(kNParam == OIC_FILTER_NPARAM, "parameter layout");
static_assert(kIn == OIC_FILTER_IN && kHid == OIC_FILTER_HIDDEN, "layer sizes");

// Shared-memory row strides (halves): 176 B and 272 B rows put the 8 rows of an
// ldmatrix 8x8 block in 8 different 16-byte bank groups.
constexpr int kXS = 88;
constexpr int kHS = 136;

// ---------------------------------------------------------------- MMA helpers
__device__ __forceinline__ u32 smem_addr(const void *p) { return (u32)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void ldsm_x4(u32 (&r)[4], const void *p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_addr(p)));
}
__device__ __forceinline__ void ldsm_x4_t(u32 (&r)[4], const void *p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_addr(p)));
}
// D += A * B, A 16x16 (row), B 16x8 (col), FP16 in, FP32 accumulate.
__device__ __forceinline__ void mma16816(float (&d)[4], const u32 (&a)[4], u32 b0, u32 b1) {
  asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
               "{%0,%1,%2,%3};\n"
               : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
               : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
__device__ __forceinline__ u32 pack_h2(float lo, float hi) {
  __half2 h = __floats2half2_rn(lo, hi);
  return *reinterpret_cast<u32 *>(&h);
}
__device__ __forceinline__ float2 unpack_h2(u32 v) {
  __half2 h = *reinterpret_cast<__half2 *>(&v);
  return __half22float2(h);
}

// Copy rows x 8-half chunks of a row-major global matrix (row length `cols` halves)
// into shared memory with row stride `ss`; rows at or past `nRows` read as zero.
__device__ __forceinline__ void stage_rows(__half *dst, int ss, const __half *src, int cols, u64 row0, int rows,
                                           u64 nRows, int tid, int nThreads) {
  const int cpr = cols / 8;
  for (int c = tid; c < rows * cpr; c += nThreads) {
    const int r = c / cpr, k = c - r * cpr;
    int4 v = make_int4(0, 0, 0, 0);
    if (row0 + r < nRows) v = *reinterpret_cast<const int4 *>(src + (row0 + r) * cols + k * 8);
    *reinterpret_cast<int4 *>(dst + r * ss + k * 8) = v;
  }
}

// ---------------------------------------------------------------- features
constexpr int kFeatWarps = 8;

__global__ void __launch_bounds__(kFeatWarps * 32) pair_features_kernel(const PairRec *pairs, u32 n,
                                                                      const int4 *nodes, const u32 *readLen,
                                                                      const u32 *strRead, int K, __half *feat) {
  __shared__ int hist[kFeatWarps][64];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const u64 nw   = (u64)gridDim.x * kFeatWarps;
  for (u64 p = (u64)blockIdx.x * kFeatWarps + wib; p < n; p += nw) {
    const PairRec pr = pairs[p];
    const int lenS   = (int)readLen[pr.sRead];
    const int lenT   = (int)readLen[strRead[pr.tStr]];
    const long long span = (long long)lenS + lenT;
    hist[wib][lane]      = 0;
    hist[wib][lane + 32] = 0;
    __syncwarp();
    for (u32 i = lane; i < pr.nodeCnt; i += 32) {
      const int4 nd = nodes[pr.nodeOff + i];   // T offset, length, S start
      long long b   = ((long long)nd.x - nd.z + lenS) * 64 / span;
      b             = b < 0 ? 0 : (b > 63 ? 63 : b);
      atomicAdd(&hist[wib][b], nd.y - K + 1);
    }
    __syncwarp();
    __half *f = feat + p * kIn;
    for (int b = lane; b < 64; b += 32) {
      const long long dc = ((2 * b + 1) * span) / 128 - lenS;   // centre diagonal of the bin
      long long ol       = (lenS < lenT - dc ? (long long)lenS : lenT - dc) - (dc < 0 ? -dc : 0);
      if (ol < 64) ol = 64;
      float v = (float)hist[wib][b] / (float)ol;
      f[b]    = __float2half_rn(v < 4.0f ? v : 4.0f);
    }
    if (lane < 16) {
      float v = 0.0f;
      if (lane == 0) v = (logf((float)lenS) - 8.0f) * 0.5f;
      if (lane == 1) v = (logf((float)lenT) - 8.0f) * 0.5f;
      if (lane == 2) v = (logf(1.0f + (float)pr.diagCt) - 5.0f) * 0.25f;
      f[64 + lane] = __float2half_rn(v);
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------- forward
constexpr int kFwdWarps = 8;

struct FwdSmem {   // FP16 arrays first: every row starts on a 16-byte boundary
  __half w1[kHid * kXS];
  __half w2[kHid * kHS];
  __half x[kFwdWarps][16 * kXS];
  float  b1[kHid], b2[kHid], w3[kHid];
  float  b3;
};

__device__ __forceinline__ void load_params(FwdSmem &s, const __half *prm, int tid, int nt) {
  stage_rows(s.w1, kXS, prm + kOffW1, kIn, 0, kHid, kHid, tid, nt);
  stage_rows(s.w2, kHS, prm + kOffW2, kHid, 0, kHid, kHid, tid, nt);
  for (int i = tid; i < kHid; i += nt) {
    s.b1[i] = __half2float(prm[kOffB1 + i]);
    s.b2[i] = __half2float(prm[kOffB2 + i]);
    s.w3[i] = __half2float(prm[kOffW3 + i]);
  }
  if (tid == 0) s.b3 = __half2float(prm[kOffB3]);
}

// Layer-1 output of one 16-row tile as layer-2 A fragments (FP16 after bias + ReLU).
__device__ __forceinline__ void layer1(const FwdSmem &s, const __half *xs, int lane, u32 (&h1)[8][4]) {
  float acc[16][4];
#pragma unroll
  for (int i = 0; i < 16; i++) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.0f;
#pragma unroll
  for (int ks = 0; ks < kIn / 16; ks++) {
    u32 a[4];
    ldsm_x4(a, xs + (lane & 15) * kXS + ks * 16 + (lane >> 4) * 8);
#pragma unroll
    for (int np = 0; np < 8; np++) {
      u32 b[4];
      ldsm_x4(b, s.w1 + (np * 16 + (lane & 7) + (lane >> 4) * 8) * kXS + ks * 16 + ((lane >> 3) & 1) * 8);
      mma16816(acc[2 * np], a, b[0], b[1]);
      mma16816(acc[2 * np + 1], a, b[2], b[3]);
    }
  }
  const int t = lane & 3;
#pragma unroll
  for (int nt = 0; nt < 16; nt++) {
    const int   c  = nt * 8 + 2 * t;
    const float b0 = s.b1[c], b1 = s.b1[c + 1];
    const u32 lo = pack_h2(fmaxf(acc[nt][0] + b0, 0.0f), fmaxf(acc[nt][1] + b1, 0.0f));
    const u32 hi = pack_h2(fmaxf(acc[nt][2] + b0, 0.0f), fmaxf(acc[nt][3] + b1, 0.0f));
    h1[nt >> 1][(nt & 1) * 2 + 0] = lo;
    h1[nt >> 1][(nt & 1) * 2 + 1] = hi;
  }
}

// Layer 2 (+ bias, ReLU, FP16) and the output unit.  h2 gets the FP16 activations in
// accumulator layout (rows g and g+8, columns nt*8 + 2t, +1).
__device__ __forceinline__ void layer2(const FwdSmem &s, const u32 (&h1)[8][4], int lane, u32 (&h2)[16][2],
                                       float &logit0, float &logit1) {
  float acc[16][4];
#pragma unroll
  for (int i = 0; i < 16; i++) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.0f;
#pragma unroll
  for (int j = 0; j < 8; j++) {
#pragma unroll
    for (int np = 0; np < 8; np++) {
      u32 b[4];
      ldsm_x4(b, s.w2 + (np * 16 + (lane & 7) + (lane >> 4) * 8) * kHS + j * 16 + ((lane >> 3) & 1) * 8);
      mma16816(acc[2 * np], h1[j], b[0], b[1]);
      mma16816(acc[2 * np + 1], h1[j], b[2], b[3]);
    }
  }
  const int t = lane & 3;
  float s0 = 0.0f, s1 = 0.0f;
#pragma unroll
  for (int nt = 0; nt < 16; nt++) {
    const int   c  = nt * 8 + 2 * t;
    const float b0 = s.b2[c], b1 = s.b2[c + 1];
    h2[nt][0] = pack_h2(fmaxf(acc[nt][0] + b0, 0.0f), fmaxf(acc[nt][1] + b1, 0.0f));
    h2[nt][1] = pack_h2(fmaxf(acc[nt][2] + b0, 0.0f), fmaxf(acc[nt][3] + b1, 0.0f));
    const float2 lo = unpack_h2(h2[nt][0]), hi = unpack_h2(h2[nt][1]);
    s0 += lo.x * s.w3[c] + lo.y * s.w3[c + 1];
    s1 += hi.x * s.w3[c] + hi.y * s.w3[c + 1];
  }
  s0 += __shfl_xor_sync(0xffffffffu, s0, 1);
  s0 += __shfl_xor_sync(0xffffffffu, s0, 2);
  s1 += __shfl_xor_sync(0xffffffffu, s1, 1);
  s1 += __shfl_xor_sync(0xffffffffu, s1, 2);
  logit0 = s0 + s.b3;
  logit1 = s1 + s.b3;
}

// logit[i] for every sample; h1/h2 (FP16, n x 128) are written when non-null.
__global__ void __launch_bounds__(kFwdWarps * 32) mlp_forward_kernel(const __half *prm, const __half *X, u32 n,
                                                                    float *logit, __half *H1, __half *H2) {
  extern __shared__ __align__(16) unsigned char fwdRaw[];
  FwdSmem &s     = *reinterpret_cast<FwdSmem *>(fwdRaw);
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  load_params(s, prm, threadIdx.x, blockDim.x);
  __syncthreads();
  const int g = lane >> 2, t = lane & 3;
  __half *xs  = s.x[wib];
  const u64 nTiles = ((u64)n + 15) / 16;
  for (u64 tile = (u64)blockIdx.x * kFwdWarps + wib; tile < nTiles; tile += (u64)gridDim.x * kFwdWarps) {
    const u64 r0 = tile * 16;
    stage_rows(xs, kXS, X, kIn, r0, 16, n, lane, 32);
    __syncwarp();
    u32 h1[8][4];
    layer1(s, xs, lane, h1);
    if (H1) {
#pragma unroll
      for (int nt = 0; nt < 16; nt++) {
        const int c = nt * 8 + 2 * t;
        if (r0 + g < n) *reinterpret_cast<u32 *>(H1 + (r0 + g) * kHid + c) = h1[nt >> 1][(nt & 1) * 2];
        if (r0 + g + 8 < n) *reinterpret_cast<u32 *>(H1 + (r0 + g + 8) * kHid + c) = h1[nt >> 1][(nt & 1) * 2 + 1];
      }
    }
    u32 h2[16][2];
    float l0, l1;
    layer2(s, h1, lane, h2, l0, l1);
    if (H2) {
#pragma unroll
      for (int nt = 0; nt < 16; nt++) {
        const int c = nt * 8 + 2 * t;
        if (r0 + g < n) *reinterpret_cast<u32 *>(H2 + (r0 + g) * kHid + c) = h2[nt][0];
        if (r0 + g + 8 < n) *reinterpret_cast<u32 *>(H2 + (r0 + g + 8) * kHid + c) = h2[nt][1];
      }
    }
    if (t == 0) {
      if (r0 + g < n) logit[r0 + g] = l0;
      if (r0 + g + 8 < n) logit[r0 + g + 8] = l1;
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------- backward
// Loss: sum over samples of weight * BCE(sigmoid(logit), label) (no 1/n: the optimizer
// scales), so dlogit = weight * (sigmoid(logit) - label).
//   dz2 = fp16(dlogit * w3 * [h2 > 0])           (written, n x 128)
//   dz1 = fp16((dz2 . W2) * [h1 > 0])             (written, n x 128)
//   grad w3 += sum dlogit * h2;  grad b3 += sum dlogit
// The weight gradients of layers 1-2 and their biases come from mlp_wgrad_kernel.
constexpr int kBwdWarps = 8;

struct BwdSmem {
  __half w2[kHid * kHS];
  float  w3[kHid];
  float  dw3[kHid];
  float  db3;
  float  loss;
};

__global__ void __launch_bounds__(kBwdWarps * 32) mlp_bwd_hidden_kernel(const __half *prm, const __half *H1,
                                                                       const __half *H2, const float *logit,
                                                                       const float *label, const float *weight,
                                                                       u32 n, __half *G2, __half *G1, float *grad,
                                                                       float *loss) {
  extern __shared__ __align__(16) unsigned char bwdRaw[];
  BwdSmem &s     = *reinterpret_cast<BwdSmem *>(bwdRaw);
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  stage_rows(s.w2, kHS, prm + kOffW2, kHid, 0, kHid, kHid, threadIdx.x, blockDim.x);
  for (int i = threadIdx.x; i < kHid; i += blockDim.x) {
    s.w3[i]  = __half2float(prm[kOffW3 + i]);
    s.dw3[i] = 0.0f;
  }
  if (threadIdx.x == 0) s.db3 = s.loss = 0.0f;
  __syncthreads();
  const int g = lane >> 2, t = lane & 3;
  float dw3[8][4];   // columns 16j + 2t + {0,1,8,9}
#pragma unroll
  for (int j = 0; j < 8; j++) dw3[j][0] = dw3[j][1] = dw3[j][2] = dw3[j][3] = 0.0f;
  float db3 = 0.0f, lsum = 0.0f;

  const u64 nTiles = ((u64)n + 15) / 16;
  for (u64 tile = (u64)blockIdx.x * kBwdWarps + wib; tile < nTiles; tile += (u64)gridDim.x * kBwdWarps) {
    const u64  r0 = tile * 16;
    const bool v0 = r0 + g < n, v1 = r0 + g + 8 < n;
    float dl[2] = {0.0f, 0.0f};
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const u64 r = r0 + g + 8 * h;
      if (r < n) {
        const float z = logit[r], y = label[r], wt = weight ? weight[r] : 1.0f;
        const float p = 1.0f / (1.0f + expf(-z));
        dl[h]         = wt * (p - y);
        if (t == 0) lsum += wt * (fmaxf(z, 0.0f) - z * y + log1pf(expf(-fabsf(z))));
      }
    }
    if (t == 0) db3 += dl[0] + dl[1];
    // dz2 as A fragments (k = hidden unit of layer 2).
    u32 a2[8][4];
#pragma unroll
    for (int j = 0; j < 8; j++) {
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int  row = g + (q & 1) * 8;
        const int  c   = 16 * j + 2 * t + (q >> 1) * 8;
        const bool ok  = (q & 1) ? v1 : v0;
        u32 hv = 0;
        if (ok) hv = *reinterpret_cast<const u32 *>(H2 + (r0 + row) * kHid + c);
        const float2 h = unpack_h2(hv);
        const float  d = dl[q & 1];
        dw3[j][(q >> 1) * 2 + 0] += d * h.x;
        dw3[j][(q >> 1) * 2 + 1] += d * h.y;
        a2[j][q] = pack_h2(h.x > 0.0f ? d * s.w3[c] : 0.0f, h.y > 0.0f ? d * s.w3[c + 1] : 0.0f);
        if (ok) *reinterpret_cast<u32 *>(G2 + (r0 + row) * kHid + c) = a2[j][q];
      }
    }
    // dh1 = dz2 . W2  (B[k = j][n = i] = W2[j][i], stored [j][i]: transposed ldmatrix)
    float acc[16][4];
#pragma unroll
    for (int i = 0; i < 16; i++) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.0f;
#pragma unroll
    for (int j = 0; j < 8; j++) {
#pragma unroll
      for (int np = 0; np < 8; np++) {
        u32 b[4];
        ldsm_x4_t(b, s.w2 + (j * 16 + (lane & 7) + ((lane >> 3) & 1) * 8) * kHS + np * 16 + (lane >> 4) * 8);
        mma16816(acc[2 * np], a2[j], b[0], b[1]);
        mma16816(acc[2 * np + 1], a2[j], b[2], b[3]);
      }
    }
#pragma unroll
    for (int nt = 0; nt < 16; nt++) {
      const int c = nt * 8 + 2 * t;
      if (v0) {
        const float2 h = unpack_h2(*reinterpret_cast<const u32 *>(H1 + (r0 + g) * kHid + c));
        *reinterpret_cast<u32 *>(G1 + (r0 + g) * kHid + c) =
            pack_h2(h.x > 0.0f ? acc[nt][0] : 0.0f, h.y > 0.0f ? acc[nt][1] : 0.0f);
      }
      if (v1) {
        const float2 h = unpack_h2(*reinterpret_cast<const u32 *>(H1 + (r0 + g + 8) * kHid + c));
        *reinterpret_cast<u32 *>(G1 + (r0 + g + 8) * kHid + c) =
            pack_h2(h.x > 0.0f ? acc[nt][2] : 0.0f, h.y > 0.0f ? acc[nt][3] : 0.0f);
      }
    }
  }
  // Reduce dw3 over the 8 row groups (g), then over warps in shared memory.
#pragma unroll
  for (int j = 0; j < 8; j++)
#pragma unroll
    for (int q = 0; q < 4; q++) {
      float v = dw3[j][q];
      v += __shfl_xor_sync(0xffffffffu, v, 4);
      v += __shfl_xor_sync(0xffffffffu, v, 8);
      v += __shfl_xor_sync(0xffffffffu, v, 16);
      if (g == 0) atomicAdd(&s.dw3[16 * j + 2 * t + (q >> 1) * 8 + (q & 1)], v);
    }
  if (t == 0) {
    atomicAdd(&s.db3, db3);
    atomicAdd(&s.loss, lsum);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kHid; i += blockDim.x) atomicAdd(&grad[kOffW3 + i], s.dw3[i]);
  if (threadIdx.x == 0) {
    atomicAdd(&grad[kOffB3], s.db3);
    if (loss) atomicAdd(loss, s.loss);
  }
}

// grad W[m][c] += sum_s G[s][m] * H[s][c]   (M = 128, N = NC columns of H)
// grad b[m]    += sum_s G[s][m]
// Each block takes a contiguous range of samples in steps of 32.
constexpr int kWgWarps = 8;
constexpr int kWgRows  = 32;

template <int NC>
struct WgSmem {
  __half g[kWgRows * kHS];
  __half h[kWgRows * kHS];
  float  bsum[kHid];
};

template <int NC>
__global__ void __launch_bounds__(kWgWarps * 32) mlp_wgrad_kernel(const __half *G, const __half *H, u32 n,
                                                                 u32 perBlock, float *gradW, float *gradB) {
  __shared__ __align__(16) WgSmem<NC> s;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  constexpr int NT = NC / 8;
  float acc[NT][4];
#pragma unroll
  for (int i = 0; i < NT; i++) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.0f;
  float bs = 0.0f;
  const u64 s0 = (u64)blockIdx.x * perBlock;
  const u64 s1 = s0 + perBlock < n ? s0 + perBlock : n;
  const int m0 = wib * 16;
  for (u64 r = s0; r < s1; r += kWgRows) {
    __syncthreads();
    const u64 lim = s1;
    stage_rows(s.g, kHS, G, kHid, r, kWgRows, lim, threadIdx.x, blockDim.x);
    stage_rows(s.h, kHS, H, NC, r, kWgRows, lim, threadIdx.x, blockDim.x);
    __syncthreads();
    if (threadIdx.x < kHid)
      for (int q = 0; q < kWgRows; q++) bs += __half2float(s.g[q * kHS + threadIdx.x]);
#pragma unroll
    for (int ks = 0; ks < kWgRows / 16; ks++) {
      // A[m][k] = G[k][m]: stored [k][m], transposed ldmatrix.
      u32 a[4];
      ldsm_x4_t(a, s.g + (ks * 16 + (lane & 7) + (lane >> 4) * 8) * kHS + m0 + ((lane >> 3) & 1) * 8);
#pragma unroll
      for (int np = 0; np < NT / 2; np++) {
        u32 b[4];
        ldsm_x4_t(b, s.h + (ks * 16 + (lane & 7) + ((lane >> 3) & 1) * 8) * kHS + np * 16 + (lane >> 4) * 8);
        mma16816(acc[2 * np], a, b[0], b[1]);
        mma16816(acc[2 * np + 1], a, b[2], b[3]);
      }
    }
  }
  const int g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int nt = 0; nt < NT; nt++) {
    const int c = nt * 8 + 2 * t;
    atomicAdd(&gradW[(m0 + g) * NC + c], acc[nt][0]);
    atomicAdd(&gradW[(m0 + g) * NC + c + 1], acc[nt][1]);
    atomicAdd(&gradW[(m0 + g + 8) * NC + c], acc[nt][2]);
    atomicAdd(&gradW[(m0 + g + 8) * NC + c + 1], acc[nt][3]);
  }
  if (threadIdx.x < kHid) atomicAdd(&gradB[threadIdx.x], bs);
}

// Adam on FP32 master weights; writes the FP16 copy and clears the gradient.
__global__ void mlp_adam_kernel(float *master, float *m, float *v, float *grad, __half *prm, u32 nParam, float lr,
                                float b1, float b2, float eps, float scale, float wd, float c1, float c2) {
  for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < nParam; i += gridDim.x * blockDim.x) {
    const float gi = grad[i] * scale;
    grad[i]        = 0.0f;
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i]           = mi;
    v[i]           = vi;
    float w        = master[i];
    w -= lr * ((mi / c1) / (sqrtf(vi / c2) + eps) + wd * w);
    master[i] = w;
    prm[i]    = __float2half_rn(w);
  }
}

int blocks_for(u64 items, int perBlock, int cap) {
  u64 b = (items + perBlock - 1) / perBlock;
  if (b < 1) b = 1;
  if (b > (u64)cap) b = cap;
  return (int)b;
}

int g_nSM = 0;
int num_sms() {
  if (!g_nSM) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_nSM, cudaDevAttrMultiProcessorCount, dev);
    if (g_nSM <= 0) g_nSM = 1;
  }
  return g_nSM;
}

}  // namespace

void launch_pair_features(const PairRec *pairs, u32 n, const int4 *nodes, const u32 *readLen, const u32 *strRead,
                          int K, void *feat, cudaStream_t st) {
  if (n == 0) return;
  const int blocks = blocks_for(n, kFeatWarps * 4, num_sms() * 8);
  pair_features_kernel<<<blocks, kFeatWarps * 32, 0, st>>>(pairs, n, nodes, readLen, strRead, K, (__half *)feat);
  g_launches++;
}

cudaError_t launch_mlp_forward(const void *prm, const void *X, u32 n, float *logit, void *H1, void *H2,
                               cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const size_t smem = sizeof(FwdSmem);
  cudaError_t e = cudaFuncSetAttribute(mlp_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int blocks = blocks_for(((u64)n + 15) / 16, kFwdWarps * 4, num_sms() * 2);
  mlp_forward_kernel<<<blocks, kFwdWarps * 32, smem, st>>>((const __half *)prm, (const __half *)X, n, logit,
                                                           (__half *)H1, (__half *)H2);
  g_launches++;
  return cudaGetLastError();
}

cudaError_t launch_mlp_backward(const void *prm, const void *X, const void *H1, const void *H2, const float *logit,
                                const float *label, const float *weight, u32 n, float *grad, void *G1, void *G2,
                                float *loss, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const size_t smem = sizeof(BwdSmem);
  cudaError_t e = cudaFuncSetAttribute(mlp_bwd_hidden_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int blocks = blocks_for(((u64)n + 15) / 16, kBwdWarps * 4, num_sms() * 2);
  mlp_bwd_hidden_kernel<<<blocks, kBwdWarps * 32, smem, st>>>((const __half *)prm, (const __half *)H1,
                                                              (const __half *)H2, logit, label, weight, n,
                                                              (__half *)G2, (__half *)G1, grad, loss);
  g_launches++;
  // Weight gradients: blocks of at least 1024 samples keep the FP32 atomics few.
  u32 per = 1024;
  while ((u64)per * num_sms() * 2 < n) per *= 2;
  const int wb = (int)(((u64)n + per - 1) / per);
  mlp_wgrad_kernel<kHid><<<wb, kWgWarps * 32, 0, st>>>((const __half *)G2, (const __half *)H1, n, per,
                                                       grad + kOffW2, grad + kOffB2);
  g_launches++;
  mlp_wgrad_kernel<kIn><<<wb, kWgWarps * 32, 0, st>>>((const __half *)G1, (const __half *)X, n, per, grad + kOffW1,
                                                      grad + kOffB1);
  g_launches++;
  return cudaGetLastError();
}

cudaError_t launch_mlp_adam(float *master, float *m, float *v, float *grad, void *prm, float lr, float b1, float b2,
                            float eps, float scale, float wd, u32 step, cudaStream_t st) {
  const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
  mlp_adam_kernel<<<blocks_for(kNParam, 256, 1024), 256, 0, st>>>(master, m, v, grad, (__half *)prm, kNParam, lr, b1,
                                                                  b2, eps, scale, wd, c1, c2);
  g_launches++;
  return cudaGetLastError();
}

}  // namespace oic

using namespace oic;

extern "C" int oic_mlp_forward(const uint16_t *dParams, const uint16_t *dX, uint32_t n, float *dLogit, uint16_t *dH1,
                               uint16_t *dH2, void *stream) {
  if (n && (!dParams || !dX || !dLogit)) return OIC_ERR_ARG;
  return launch_mlp_forward(dParams, dX, n, dLogit, dH1, dH2, (cudaStream_t)stream) == cudaSuccess ? OIC_OK
                                                                                                   : OIC_ERR_CUDA;
}

extern "C" int oic_mlp_backward(const uint16_t *dParams, const uint16_t *dX, const uint16_t *dH1, const uint16_t *dH2,
                                const float *dLogit, const float *dLabel, const float *dWeight, uint32_t n,
                                float *dGrad, uint16_t *dG1, uint16_t *dG2, float *dLoss, void *stream) {
  if (n && (!dParams || !dX || !dH1 || !dH2 || !dLogit || !dLabel || !dGrad || !dG1 || !dG2)) return OIC_ERR_ARG;
  return launch_mlp_backward(dParams, dX, dH1, dH2, dLogit, dLabel, dWeight, n, dGrad, dG1, dG2, dLoss,
                             (cudaStream_t)stream) == cudaSuccess
             ? OIC_OK
             : OIC_ERR_CUDA;
}

extern "C" int oic_mlp_adam(float *dMaster, float *dM, float *dV, float *dGrad, uint16_t *dParams, float lr,
                            float beta1, float beta2, float eps, float gradScale, float weightDecay, uint32_t step,
                            void *stream) {
  if (!dMaster || !dM || !dV || !dGrad || !dParams || step == 0) return OIC_ERR_ARG;
  return launch_mlp_adam(dMaster, dM, dV, dGrad, dParams, lr, beta1, beta2, eps, gradScale, weightDecay, step,
                         (cudaStream_t)stream) == cudaSuccess
             ? OIC_OK
             : OIC_ERR_CUDA;
}
