// learn.cu -- learned acceleration of source iteration: a small MLP that
// predicts, per zone and group, how far the scalar flux still is from its
// converged value, as a multiple of the last iteration's change.
//
// No counterpart in the reference: Teton accelerates source iteration only
// with grey transport (rt/GTASolver.F90).  The learned step sits beside it in
// the same loop (umt103_source_iterate) and is kept only when the next full
// sweep shows that the iteration residual dropped.
//
// Network: F inputs (4G + 4 per-zone features, padded to K1, a multiple of
// 16) -> 128 -> 128 -> 128 (ReLU) -> G outputs o_g; the correction multiplier
// is m_g = exp(clamp(o_g, MLP_OLO, MLP_OHI)) and the corrected flux of every
// corner c of the zone is phi_c,g + m_g (phi_c,g - phi_prev_c,g).
//
// Every product runs on the 5th-generation tensor cores: BF16 operands in
// shared memory (K-major canonical tiles, tc_util.cuh), FP32 accumulators in
// tensor memory, tcgen05.mma issued by one thread and completed through an
// mbarrier, results read back with tcgen05.ld for the epilogues (bias, ReLU,
// BF16 rounding).  Kernels:
//   k_mlp_forward   128-row tiles, all four layers fused, weights staged once
//                   per CTA; in training also writes the activations in both
//                   layouts for the weight gradients;
//   k_mlp_backward  dZ3 = (dO W4) * [H3>0], dZ2, dZ1, fused per 128-row tile;
//   k_mlp_wgrad     dW_l = dZ_l^T X_l, accumulated over 128-row K steps in
//                   tensor memory, one CTA per (layer, chunk of the batch);
// plus element-wise kernels for features, loss, bias gradients, Adam and the
// BF16 weight packing.  Master weights and Adam moments are FP32.
#include "umt_common.cuh"
#include "tc_util.cuh"
#include "../../include/umt103.h"

#include <cmath>
#include <cstring>
#include <algorithm>

namespace umt {

constexpr int MLP_H = 128;
constexpr int MLP_NT = 128;                 // 4 warps: one quarter of the tensor-memory lanes each
constexpr float MLP_OLO = -12.f, MLP_OHI = 8.f;
constexpr int MLP_MAXG = 60;                // 4G + 4 <= 244 -> K1 <= 256

__host__ __device__ constexpr int mlp_features(int G) { return 4 * G + 4; }
__host__ __device__ constexpr int round16(int x) { return (x + 15) / 16 * 16; }

struct MlpNet {                             // device view of the network
  int G, F, K1, N4;
  const __nv_bfloat16 *W1, *W2, *W3, *W4;  // [128][K1], [128][128], [128][128], [N4][128]
  const __nv_bfloat16 *W2T, *W3T, *W4T;    // [128][128], [128][128], [128][N4]
  const float *b1, *b2, *b3, *b4;          // FP32 biases (inside the master parameters)
};

struct MlpAct {                             // activations of one batch of rows
  int rows, ld;                             // rows (a multiple of 128 when training); ld: transposed row stride
  const __nv_bfloat16 *X;                   // [rows][K1]
  __nv_bfloat16 *XT;                        // [K1][ld]
  __nv_bfloat16 *H[3], *HT[3];              // post-ReLU hidden activations [rows][128], [128][ld]
  float *O;                                 // [rows][N4]
  __nv_bfloat16 *dO, *dOT;                  // [rows][N4], [N4][ld]
  __nv_bfloat16 *dZT[3];                    // [128][ld] gradients of layers 1..3 before the ReLU
};

// ---------------------------------------------------------------------------
// Forward: one CTA of 128 threads per 128-row tile (persistent over tiles).
// ---------------------------------------------------------------------------
static size_t forward_smem(int K1, int N4) {
  const int KA = K1 > MLP_H ? K1 : MLP_H;
  return (size_t)MLP_H * K1 * 2 + 2 * (size_t)MLP_H * MLP_H * 2 + (size_t)N4 * MLP_H * 2 + (size_t)MLP_H * KA * 2 + 16;
}

template <bool TRAIN>
__global__ void __launch_bounds__(MLP_NT, 1) k_mlp_forward(MlpNet net, MlpAct act, unsigned *status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  const int K1 = net.K1, N4 = net.N4, KA = K1 > MLP_H ? K1 : MLP_H;
  unsigned char *sW1 = smem;
  unsigned char *sW2 = sW1 + (size_t)MLP_H * K1 * 2;
  unsigned char *sW3 = sW2 + (size_t)MLP_H * MLP_H * 2;
  unsigned char *sW4 = sW3 + (size_t)MLP_H * MLP_H * 2;
  unsigned char *sA = sW4 + (size_t)N4 * MLP_H * 2;
  uint64_t *mbar = reinterpret_cast<uint64_t *>(sA + (size_t)MLP_H * KA * 2);
  uint32_t *slot = reinterpret_cast<uint32_t *>(mbar + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 0) tmem_alloc(slot, 128);
  if (tid == 0) mbar_init(mbar, 1);
  load_tile_km(sW1, net.W1, MLP_H, K1, K1, tid, MLP_NT);
  load_tile_km(sW2, net.W2, MLP_H, MLP_H, MLP_H, tid, MLP_NT);
  load_tile_km(sW3, net.W3, MLP_H, MLP_H, MLP_H, tid, MLP_NT);
  load_tile_km(sW4, net.W4, N4, MLP_H, MLP_H, tid, MLP_NT);
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *slot;
  const uint32_t tl = tmem + ((uint32_t)(warp * 32) << 16);
  const int r = warp * 32 + lane;
  uint32_t phase = 0;
  bool ok = true;
  const int tiles = (act.rows + 127) / 128;
  for (int t = blockIdx.x; t < tiles && ok; t += gridDim.x) {
    {
      const int c8 = K1 >> 3;
      for (int q = tid; q < MLP_H * c8; q += MLP_NT) {
        const int rr = q / c8, k8 = q - rr * c8;
        const int g = t * 128 + rr;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (g < act.rows) v = *reinterpret_cast<const uint4 *>(act.X + (size_t)g * K1 + k8 * 8);
        *reinterpret_cast<uint4 *>(sA + (rr >> 3) * K1 * 16 + k8 * 128 + (rr & 7) * 16) = v;
      }
    }
    fence_async_smem();
    __syncthreads();
    const int grow = t * 128 + r;
    for (int l = 0; l < 4; ++l) {
      const int K = l == 0 ? K1 : MLP_H, N = l == 3 ? N4 : MLP_H;
      const unsigned char *sB = l == 0 ? sW1 : (l == 1 ? sW2 : (l == 2 ? sW3 : sW4));
      if (tid == 0) {
        tc_fence_after();
        umma_tile(tmem, smem_u32(sA), smem_u32(sB), N, K, mbar, false);
      }
      const bool done = mbar_wait_bounded(mbar, phase);
      phase ^= 1u;
      ok = __syncthreads_and(done) != 0;
      if (!ok) break;
      tc_fence_after();
      if (l < 3) {
        const float *b = l == 0 ? net.b1 : (l == 1 ? net.b2 : net.b3);
        for (int j0 = 0; j0 < MLP_H; j0 += 16) {
          float v[16];
          tmem_ld16(tl + (uint32_t)j0, v);
          __align__(16) __nv_bfloat16 h[16];
#pragma unroll
          for (int i = 0; i < 16; ++i) h[i] = __float2bfloat16_rn(fmaxf(v[i] + b[j0 + i], 0.f));
          *reinterpret_cast<uint4 *>(sA + km_off(r, j0, MLP_H)) = *reinterpret_cast<const uint4 *>(&h[0]);
          *reinterpret_cast<uint4 *>(sA + km_off(r, j0 + 8, MLP_H)) = *reinterpret_cast<const uint4 *>(&h[8]);
          if constexpr (TRAIN) {
            if (grow < act.rows) {
              __nv_bfloat16 *Hr = act.H[l] + (size_t)grow * MLP_H + j0;
              *reinterpret_cast<uint4 *>(Hr) = *reinterpret_cast<const uint4 *>(&h[0]);
              *reinterpret_cast<uint4 *>(Hr + 8) = *reinterpret_cast<const uint4 *>(&h[8]);
#pragma unroll
              for (int i = 0; i < 16; ++i) act.HT[l][(size_t)(j0 + i) * act.ld + grow] = h[i];
            }
          }
        }
      } else {
        for (int j0 = 0; j0 < N4; j0 += 16) {
          float v[16];
          tmem_ld16(tl + (uint32_t)j0, v);
          if (grow < act.rows) {
#pragma unroll
            for (int i = 0; i < 16; ++i)
              act.O[(size_t)grow * N4 + j0 + i] = v[i] + (j0 + i < net.G ? net.b4[j0 + i] : 0.f);
          }
        }
      }
      fence_async_smem();
      tc_fence_before();
      __syncthreads();
    }
  }
  if (!ok) {
    if (tid == 0) atomicOr(status, UMT_DEV_TIMEOUT);
    mbar_wait_bounded(mbar, phase ^ 1u);       // the MMAs of the abandoned step, before the release
    tc_fence_before();
    __syncthreads();
  }
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, 128);
  }
}

// ---------------------------------------------------------------------------
// Backward through the layers: dZ3 = (dO W4) * [H3 > 0], dZ2 = (dZ3 W3) *
// [H2 > 0], dZ1 = (dZ2 W2) * [H1 > 0]; the transposed copies feed the weight
// gradients.
// ---------------------------------------------------------------------------
static size_t backward_smem(int N4) {
  return (size_t)MLP_H * N4 * 2 + 2 * (size_t)MLP_H * MLP_H * 2 + (size_t)MLP_H * MLP_H * 2 + 16;
}

__global__ void __launch_bounds__(MLP_NT, 1) k_mlp_backward(MlpNet net, MlpAct act, unsigned *status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  const int N4 = net.N4;
  unsigned char *sB4 = smem;                                   // W4^T [128][N4]
  unsigned char *sB3 = sB4 + (size_t)MLP_H * N4 * 2;          // W3^T [128][128]
  unsigned char *sB2 = sB3 + (size_t)MLP_H * MLP_H * 2;       // W2^T
  unsigned char *sA = sB2 + (size_t)MLP_H * MLP_H * 2;
  uint64_t *mbar = reinterpret_cast<uint64_t *>(sA + (size_t)MLP_H * MLP_H * 2);
  uint32_t *slot = reinterpret_cast<uint32_t *>(mbar + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 0) tmem_alloc(slot, 128);
  if (tid == 0) mbar_init(mbar, 1);
  load_tile_km(sB4, net.W4T, MLP_H, N4, N4, tid, MLP_NT);
  load_tile_km(sB3, net.W3T, MLP_H, MLP_H, MLP_H, tid, MLP_NT);
  load_tile_km(sB2, net.W2T, MLP_H, MLP_H, MLP_H, tid, MLP_NT);
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *slot;
  const uint32_t tl = tmem + ((uint32_t)(warp * 32) << 16);
  const int r = warp * 32 + lane;
  uint32_t phase = 0;
  bool ok = true;
  const int tiles = act.rows / 128;
  for (int t = blockIdx.x; t < tiles && ok; t += gridDim.x) {
    load_tile_km(sA, act.dO + (size_t)t * 128 * N4, MLP_H, N4, N4, tid, MLP_NT);
    fence_async_smem();
    __syncthreads();
    const int grow = t * 128 + r;
    for (int l = 2; l >= 0; --l) {           // produces dZ of hidden layer l (0-based)
      const int K = l == 2 ? N4 : MLP_H;
      const unsigned char *sB = l == 2 ? sB4 : (l == 1 ? sB3 : sB2);
      if (tid == 0) {
        tc_fence_after();
        umma_tile(tmem, smem_u32(sA), smem_u32(sB), MLP_H, K, mbar, false);
      }
      const bool done = mbar_wait_bounded(mbar, phase);
      phase ^= 1u;
      ok = __syncthreads_and(done) != 0;
      if (!ok) break;
      tc_fence_after();
      const __nv_bfloat16 *Hr = act.H[l] + (size_t)grow * MLP_H;
      for (int j0 = 0; j0 < MLP_H; j0 += 16) {
        float v[16];
        tmem_ld16(tl + (uint32_t)j0, v);
        __align__(16) __nv_bfloat16 hm[16];
        *reinterpret_cast<uint4 *>(&hm[0]) = *reinterpret_cast<const uint4 *>(Hr + j0);
        *reinterpret_cast<uint4 *>(&hm[8]) = *reinterpret_cast<const uint4 *>(Hr + j0 + 8);
        __align__(16) __nv_bfloat16 d[16];
#pragma unroll
        for (int i = 0; i < 16; ++i)
          d[i] = __float2bfloat16_rn(__bfloat162float(hm[i]) > 0.f ? v[i] : 0.f);
#pragma unroll
        for (int i = 0; i < 16; ++i) act.dZT[l][(size_t)(j0 + i) * act.ld + grow] = d[i];
        if (l > 0) {
          *reinterpret_cast<uint4 *>(sA + km_off(r, j0, MLP_H)) = *reinterpret_cast<const uint4 *>(&d[0]);
          *reinterpret_cast<uint4 *>(sA + km_off(r, j0 + 8, MLP_H)) = *reinterpret_cast<const uint4 *>(&d[8]);
        }
      }
      fence_async_smem();
      tc_fence_before();
      __syncthreads();
    }
  }
  if (!ok) {
    if (tid == 0) atomicOr(status, UMT_DEV_TIMEOUT);
    mbar_wait_bounded(mbar, phase ^ 1u);
    tc_fence_before();
    __syncthreads();
  }
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, 128);
  }
}

// ---------------------------------------------------------------------------
// Weight gradients: for layer l (blockIdx.y) and a chunk of the batch
// (blockIdx.x), D = A B^T over the chunk's rows, stored as the chunk's
// partial tile; k_mlp_wreduce sums the chunks in chunk order, so a gradient
// does not depend on the order in which CTAs finish:
//   l = 0..2: A = dZ_l^T [128 out][rows], B = X_l^T [in][rows]  -> dW_l[out][in]
//   l = 3:    A = H3^T  [128 in][rows],   B = dO^T [N4][rows]  -> dW4[o][h] transposed
// Partial tile (l, chunk) holds D[m][n] at ((l*nchunk + chunk)*128 + m)*MLP_WPN + n.
// ---------------------------------------------------------------------------
constexpr int MLP_WPN = 256;                   // widest B operand (rows of sB)
constexpr int MLP_WCHUNKS = 32;                // most chunks per layer
static size_t wgrad_smem() { return (size_t)MLP_H * MLP_H * 2 + (size_t)256 * MLP_H * 2 + 16; }

struct MlpGradOff { long w[4], b[4]; };

__global__ void __launch_bounds__(MLP_NT, 1) k_mlp_wgrad(MlpNet net, MlpAct act, float *part, int chunk,
                                                         unsigned *status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char *sA = smem;
  unsigned char *sB = sA + (size_t)MLP_H * MLP_H * 2;
  uint64_t *mbar = reinterpret_cast<uint64_t *>(sB + (size_t)256 * MLP_H * 2);
  uint32_t *slot = reinterpret_cast<uint32_t *>(mbar + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int l = blockIdx.y;
  const __nv_bfloat16 *AT = l < 3 ? act.dZT[l] : act.HT[2];
  const __nv_bfloat16 *BT = l == 0 ? act.XT : (l < 3 ? act.HT[l - 1] : act.dOT);
  const int N = l == 0 ? net.K1 : (l < 3 ? MLP_H : net.N4);
  const int r0 = blockIdx.x * chunk, r1 = min(act.rows, r0 + chunk);
  if (r0 >= r1) return;                     // uniform across the CTA, before any allocation
  if (warp == 0) tmem_alloc(slot, 256);
  if (tid == 0) mbar_init(mbar, 1);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *slot;
  uint32_t phase = 0;
  bool ok = true;
  for (int b0 = r0; b0 < r1 && ok; b0 += 128) {
    load_tile_km(sA, AT + b0, MLP_H, MLP_H, act.ld, tid, MLP_NT);
    load_tile_km(sB, BT + b0, N, MLP_H, act.ld, tid, MLP_NT);
    fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      umma_tile(tmem, smem_u32(sA), smem_u32(sB), N, MLP_H, mbar, b0 > r0);
    }
    const bool done = mbar_wait_bounded(mbar, phase);
    phase ^= 1u;
    ok = __syncthreads_and(done) != 0;
  }
  if (ok) {
    tc_fence_after();
    const uint32_t tl = tmem + ((uint32_t)(warp * 32) << 16);
    const int m = warp * 32 + lane;
    float *dst = part + ((size_t)(l * gridDim.x + blockIdx.x) * MLP_H + m) * MLP_WPN;
    for (int j0 = 0; j0 < N; j0 += 16) {
      float v[16];
      tmem_ld16(tl + (uint32_t)j0, v);
#pragma unroll
      for (int i = 0; i < 16; i += 4)
        *reinterpret_cast<float4 *>(dst + j0 + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
    }
  } else {
    if (tid == 0) atomicOr(status, UMT_DEV_TIMEOUT);
    mbar_wait_bounded(mbar, phase ^ 1u);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, 256);
  }
}

// bias gradients: row sums of dZ_l^T (l < 3) and of dO^T (the output layer)
// grad (weights) = sum over the chunks' partial tiles, in chunk order
__global__ void k_mlp_wreduce(MlpNet net, MlpGradOff off, const float *part, int nchunk, float *grad) {
  const long total = 4l * MLP_H * MLP_WPN;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    const int l = (int)(t / ((long)MLP_H * MLP_WPN));
    const int m = (int)(t / MLP_WPN % MLP_H), n = (int)(t % MLP_WPN);
    float *dst;
    if (l == 0) dst = n < net.F ? grad + off.w[0] + (long)m * net.F + n : nullptr;
    else if (l < 3) dst = n < MLP_H ? grad + off.w[l] + (long)m * MLP_H + n : nullptr;
    else dst = n < net.G ? grad + off.w[3] + (long)n * MLP_H + m : nullptr;
    if (!dst) continue;
    float s = 0.f;
    for (int c = 0; c < nchunk; ++c) s += part[((size_t)(l * nchunk + c) * MLP_H + m) * MLP_WPN + n];
    *dst = s;
  }
}

__global__ void k_mlp_bgrad(MlpNet net, MlpAct act, MlpGradOff off, float *grad) {
  const int warpsPer = blockDim.x / 32;
  const int w = blockIdx.x * warpsPer + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  const int nrow = 3 * MLP_H + net.G;
  if (w >= nrow) return;
  const __nv_bfloat16 *row;
  float *dst;
  if (w < 3 * MLP_H) {
    const int l = w / MLP_H, o = w - l * MLP_H;
    row = act.dZT[l] + (size_t)o * act.ld;
    dst = grad + off.b[l] + o;
  } else {
    const int o = w - 3 * MLP_H;
    row = act.dOT + (size_t)o * act.ld;
    dst = grad + off.b[3] + o;
  }
  float s = 0.f;
  for (int b = lane; b < act.rows; b += 32) s += __bfloat162float(row[b]);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) *dst = s;
}

// ---------------------------------------------------------------------------
// Element-wise pieces.
// ---------------------------------------------------------------------------
struct MlpParamOff { long W1, b1, W2, b2, W3, b3, W4, b4, n; };

static MlpParamOff param_offsets(int G) {
  const int F = mlp_features(G);
  MlpParamOff p;
  long o = 0;
  p.W1 = o; o += (long)MLP_H * F;
  p.b1 = o; o += MLP_H;
  p.W2 = o; o += (long)MLP_H * MLP_H;
  p.b2 = o; o += MLP_H;
  p.W3 = o; o += (long)MLP_H * MLP_H;
  p.b3 = o; o += MLP_H;
  p.W4 = o; o += (long)G * MLP_H;
  p.b4 = o; o += G;
  p.n = o;
  return p;
}

// BF16 copies of the master weights, padded, and the transposed copies the
// backward pass multiplies by.
__global__ void k_mlp_pack(int G, int F, int K1, int N4, MlpParamOff po, const float *p, __nv_bfloat16 *W1,
                           __nv_bfloat16 *W2, __nv_bfloat16 *W3, __nv_bfloat16 *W4, __nv_bfloat16 *W2T,
                           __nv_bfloat16 *W3T, __nv_bfloat16 *W4T) {
  const int i0 = blockIdx.x * blockDim.x + threadIdx.x, st = gridDim.x * blockDim.x;
  for (int i = i0; i < MLP_H * K1; i += st) {
    const int o = i / K1, k = i - o * K1;
    W1[i] = __float2bfloat16_rn(k < F ? p[po.W1 + (long)o * F + k] : 0.f);
  }
  for (int i = i0; i < MLP_H * MLP_H; i += st) {
    const int o = i / MLP_H, k = i - o * MLP_H;
    W2[i] = __float2bfloat16_rn(p[po.W2 + i]);
    W3[i] = __float2bfloat16_rn(p[po.W3 + i]);
    W2T[(long)k * MLP_H + o] = __float2bfloat16_rn(p[po.W2 + i]);
    W3T[(long)k * MLP_H + o] = __float2bfloat16_rn(p[po.W3 + i]);
  }
  for (int i = i0; i < N4 * MLP_H; i += st) {
    const int o = i / MLP_H, k = i - o * MLP_H;
    const float v = o < G ? p[po.W4 + (long)o * MLP_H + k] : 0.f;
    W4[i] = __float2bfloat16_rn(v);
    W4T[(long)k * N4 + o] = __float2bfloat16_rn(v);
  }
}

template <int NV>
__device__ void block_sum(double (&v)[NV], double *out) {
  __shared__ double sh[NV][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double x = v[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sh[k][w] = x;
  }
  __syncthreads();
  if (w == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double x = lane < (int)(blockDim.x >> 5) ? sh[k][lane] : 0.0;
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if (lane == 0) atomicAdd(out + k, x);
    }
  }
}

// Loss of a batch: sum_r w_r sum_g (m_rg delta_rg - e_rg)^2 with
// m = exp(clamp(o)); out[0] += that sum, out[1] += sum w e^2 (the loss of no
// correction).  dO = d(loss)/d(o), in both layouts.
__global__ void k_mlp_loss(int rows, int G, int N4, int ld, const float *O, const float *delta, const float *target,
                           const float *w, __nv_bfloat16 *dO, __nv_bfloat16 *dOT, double *out) {
  double v[2] = {0.0, 0.0};
  const long n = (long)rows * N4;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const int r = (int)(i / N4), j = (int)(i - (long)r * N4);
    float d = 0.f;
    if (j < G) {
      const float o = O[i];
      const float oc = fminf(fmaxf(o, MLP_OLO), MLP_OHI);
      const float m = __expf(oc);
      const float dl = delta[(long)r * G + j], e = target[(long)r * G + j], wr = w[r];
      const float res = m * dl - e;
      v[0] += (double)wr * res * res;
      v[1] += (double)wr * e * e;
      d = (o == oc) ? 2.f * wr * res * dl * m : 0.f;
    }
    const __nv_bfloat16 b = __float2bfloat16_rn(d);
    dO[i] = b;
    dOT[(long)j * ld + r] = b;
  }
  block_sum<2>(v, out);
}

// dO from a caller-given dY [rows][G] (the gradient-check entry point)
__global__ void k_mlp_dy(int rows, int G, int N4, int ld, const float *dY, __nv_bfloat16 *dO, __nv_bfloat16 *dOT) {
  const long n = (long)rows * N4;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const int r = (int)(i / N4), j = (int)(i - (long)r * N4);
    const __nv_bfloat16 b = __float2bfloat16_rn(j < G ? dY[(long)r * G + j] : 0.f);
    dO[i] = b;
    dOT[(long)j * ld + r] = b;
  }
}

// X^T from X (rows x K1 -> K1 x ld)
__global__ void k_mlp_transpose_x(int rows, int K1, int ld, const __nv_bfloat16 *X, __nv_bfloat16 *XT) {
  const long n = (long)rows * K1;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const int k = (int)(i / rows), r = (int)(i - (long)k * rows);
    XT[(long)k * ld + r] = X[(long)r * K1 + k];
  }
}

// float inputs -> padded BF16 rows
__global__ void k_mlp_x_from_float(int rows, int F, int K1, const float *Xf, __nv_bfloat16 *X) {
  const long n = (long)rows * K1;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const int r = (int)(i / K1), k = (int)(i - (long)r * K1);
    X[i] = __float2bfloat16_rn(k < F ? Xf[(long)r * F + k] : 0.f);
  }
}

__global__ void k_mlp_adam(long n, float *p, const float *g, float *m, float *v, float lr, float b1, float b2,
                           float eps, float bc1, float bc2, float clip) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const float gi = fminf(fmaxf(g[i], -clip), clip);
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  }
}

// Random rows of the training set into the batch (X, X^T, delta, target, w).
__host__ __device__ __forceinline__ uint32_t mix32(uint32_t x) {
  x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16;
  return x;
}

__global__ void k_mlp_gather(int B, int K1, int G, int ld, long nrows, uint32_t seed, const __nv_bfloat16 *Xd,
                             const float *Dd, const float *Td, const float *Wd, __nv_bfloat16 *X, __nv_bfloat16 *XT,
                             float *D, float *T, float *W) {
  const long n = (long)B * K1;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const int k = (int)(i / B), r = (int)(i - (long)k * B);
    const long src = (long)(((uint64_t)mix32(seed ^ mix32((uint32_t)r * 0x9E3779B9u)) * (uint64_t)nrows) >> 32);
    const __nv_bfloat16 x = Xd[src * K1 + k];
    X[(long)r * K1 + k] = x;
    XT[(long)k * ld + r] = x;
    if (k < G) {
      D[(long)r * G + k] = Dd[src * G + k];
      T[(long)r * G + k] = Td[src * G + k];
    }
    if (k == 0) W[r] = Wd[src];
  }
}

// ---------------------------------------------------------------------------
// Features of each zone (one thread per zone), from the current iterate Phi,
// its last change Delta and the change before DeltaPrev (all [nc][G]):
//   [g]        ln(sigma_t,g h) / 8, h = V_zone^(1/3) (zone optical size)
//   [G+g]      -ln(1 - sigma_s,g / sigma_t,g) / 8
//   [2G+g]     zone change ratio Delta / DeltaPrev, clamped to [-1.5, 1.5]
//   [3G+g]     asinh(1e3 Delta / phi) / 8 (signed relative change)
//   [4G..4G+3] ln(h / hmean), corners / 8, corner-volume spread, 1
// Zone values are volume-weighted corner means.  Also writes the zone means
// of Delta and Phi (dz, pz: [nz][G]) when those are given.
// ---------------------------------------------------------------------------
__global__ void k_mlp_features(int nz, int G, int K1, double hmean, const int *numCorner, const int *cOffSet,
                               const double *Volume, const double *Sigt, const double *SigS, const double *Phi,
                               const double *Delta, const double *DeltaPrev, __nv_bfloat16 *X, float *dz,
                               float *pz) {
  for (int z = blockIdx.x * blockDim.x + threadIdx.x; z < nz; z += gridDim.x * blockDim.x) {
    const int c0 = cOffSet[z], nC = numCorner[z];
    double vz = 0.0, v2 = 0.0;
    for (int k = 0; k < nC; ++k) { vz += Volume[c0 + k]; v2 += Volume[c0 + k] * Volume[c0 + k]; }
    const double h = cbrt(vz), vm = vz / nC;
    const double spread = sqrt(fmax(v2 / nC - vm * vm, 0.0)) / vm;
    __nv_bfloat16 *row = X + (size_t)z * K1;
    for (int g = 0; g < G; ++g) {
      double dk = 0.0, dk1 = 0.0, p = 0.0;
      for (int k = 0; k < nC; ++k) {
        const size_t e = (size_t)(c0 + k) * G + g;
        const double V = Volume[c0 + k];
        dk += V * Delta[e];
        dk1 += V * DeltaPrev[e];
        p += V * Phi[e];
      }
      dk /= vz; dk1 /= vz; p /= vz;
      const double st = Sigt[(size_t)z * G + g], ss = SigS[(size_t)z * G + g];
      const double ratio = fabs(dk1) > 1e-300 ? fmin(fmax(dk / dk1, -1.5), 1.5) : 0.0;
      row[g] = __float2bfloat16_rn((float)(log(st * h) / 8.0));
      row[G + g] = __float2bfloat16_rn((float)(-log(fmax(1.0 - ss / st, 1e-6)) / 8.0));
      row[2 * G + g] = __float2bfloat16_rn((float)ratio);
      row[3 * G + g] = __float2bfloat16_rn((float)(asinh(1e3 * dk / (fabs(p) + 1e-300)) / 8.0));
      if (dz) dz[(size_t)z * G + g] = (float)dk;
      if (pz) pz[(size_t)z * G + g] = (float)p;
    }
    row[4 * G] = __float2bfloat16_rn((float)log(h / hmean));
    row[4 * G + 1] = __float2bfloat16_rn((float)nC / 8.f);
    row[4 * G + 2] = __float2bfloat16_rn((float)spread);
    row[4 * G + 3] = __float2bfloat16_rn(1.f);
    for (int k = 4 * G + 4; k < K1; ++k) row[k] = __float2bfloat16_rn(0.f);
  }
}

// Phi_c,g += m_z,g Delta_c,g over every corner (z its zone)
__global__ void k_mlp_apply(int nc, int G, int N4, const int *cToZone, const float *O, const double *Delta,
                            double *Phi) {
  const size_t n = (size_t)nc * G;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(i / G), g = (int)(i - (size_t)c * G);
    const float o = O[(size_t)cToZone[c] * N4 + g];
    const double m = exp((double)fminf(fmaxf(o, MLP_OLO), MLP_OHI));
    Phi[i] += m * Delta[i];
  }
}

// targets of a snapshot: zone mean of PhiStar minus the stored zone mean of
// the iterate; out += sum of squared targets
__global__ void k_mlp_targets(int nz, int G, const int *numCorner, const int *cOffSet, const double *Volume,
                              const double *PhiStar, const float *pz, float *T, double *out) {
  double v[1] = {0.0};
  for (int z = blockIdx.x * blockDim.x + threadIdx.x; z < nz; z += gridDim.x * blockDim.x) {
    const int c0 = cOffSet[z], nC = numCorner[z];
    double vz = 0.0;
    for (int k = 0; k < nC; ++k) vz += Volume[c0 + k];
    for (int g = 0; g < G; ++g) {
      double s = 0.0;
      for (int k = 0; k < nC; ++k) s += Volume[c0 + k] * PhiStar[(size_t)(c0 + k) * G + g];
      const float e = (float)(s / vz - (double)pz[(size_t)z * G + g]);
      T[(size_t)z * G + g] = e;
      v[0] += (double)e * e;
    }
  }
  block_sum<1>(v, out);
}

__global__ void k_fill_f(long n, float *x, float v) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) x[i] = v;
}

// ---------------------------------------------------------------------------
// Host side: one network per process (the library's learned model), its
// training set, and a batch workspace.
// ---------------------------------------------------------------------------
template <typename T>
static int malloc_n(T **p, size_t n) {
  *p = nullptr;
  cudaError_t e = cudaMalloc((void **)p, std::max<size_t>(n, 1) * sizeof(T));
  if (e != cudaSuccess) { *p = nullptr; cudaGetLastError(); return set_error(UMT_ERR_NOMEM, "learned model: allocation of %zu bytes failed", n * sizeof(T)); }
  return 0;
}
template <typename T>
static void free_n(T *&p) { if (p) cudaFree((void *)p); p = nullptr; }

struct Mlp {
  bool ready = false;
  int G = 0, F = 0, K1 = 0, N4 = 0;
  MlpParamOff po{};
  float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
  float *wpart = nullptr;                       // weight-gradient partial tiles [4][chunks][128][MLP_WPN]
  __nv_bfloat16 *W1 = nullptr, *W2 = nullptr, *W3 = nullptr, *W4 = nullptr, *W2T = nullptr, *W3T = nullptr, *W4T = nullptr;
  long step = 0;
  // batch workspace
  int cap = 0;
  __nv_bfloat16 *X = nullptr, *XT = nullptr, *H[3] = {}, *HT[3] = {}, *dO = nullptr, *dOT = nullptr, *dZT[3] = {};
  float *O = nullptr, *bD = nullptr, *bT = nullptr, *bW = nullptr;
  float *Xf = nullptr, *dYf = nullptr;
  double *red = nullptr;
  unsigned *status = nullptr;
  // training set
  long nrows = 0, rowCap = 0, pendingFrom = 0;
  int pendingNz = 0;
  __nv_bfloat16 *Xd = nullptr;
  float *Dd = nullptr, *Pd = nullptr, *Td = nullptr, *Wd = nullptr;
  cudaStream_t stream = nullptr;
};

static Mlp g_mlp;

static void mlp_free_workspace(Mlp &n) {
  free_n(n.X); free_n(n.XT); free_n(n.dO); free_n(n.dOT); free_n(n.O); free_n(n.bD); free_n(n.bT); free_n(n.bW);
  free_n(n.Xf); free_n(n.dYf);
  for (int i = 0; i < 3; ++i) { free_n(n.H[i]); free_n(n.HT[i]); free_n(n.dZT[i]); }
  n.cap = 0;
}

static void mlp_free(Mlp &n) {
  mlp_free_workspace(n);
  free_n(n.p); free_n(n.g); free_n(n.m); free_n(n.v); free_n(n.wpart);
  free_n(n.W1); free_n(n.W2); free_n(n.W3); free_n(n.W4); free_n(n.W2T); free_n(n.W3T); free_n(n.W4T);
  free_n(n.red); free_n(n.status);
  free_n(n.Xd); free_n(n.Dd); free_n(n.Pd); free_n(n.Td); free_n(n.Wd);
  if (n.stream) cudaStreamDestroy(n.stream);
  n = Mlp();
}

// workspace for `rows` rows (rounded up to 128)
static int mlp_workspace(Mlp &n, int rows) {
  const int need = (rows + 127) / 128 * 128;
  if (n.cap >= need) return 0;
  mlp_free_workspace(n);
  const size_t c = (size_t)need;
  int rc = 0;
  rc = rc ? rc : malloc_n(&n.X, c * n.K1);
  rc = rc ? rc : malloc_n(&n.XT, c * n.K1);
  for (int i = 0; i < 3 && !rc; ++i) {
    rc = malloc_n(&n.H[i], c * MLP_H);
    if (!rc) rc = malloc_n(&n.HT[i], c * MLP_H);
    if (!rc) rc = malloc_n(&n.dZT[i], c * MLP_H);
  }
  rc = rc ? rc : malloc_n(&n.dO, c * n.N4);
  rc = rc ? rc : malloc_n(&n.dOT, c * n.N4);
  rc = rc ? rc : malloc_n(&n.O, c * n.N4);
  rc = rc ? rc : malloc_n(&n.bD, c * n.G);
  rc = rc ? rc : malloc_n(&n.bT, c * n.G);
  rc = rc ? rc : malloc_n(&n.bW, c);
  rc = rc ? rc : malloc_n(&n.Xf, c * n.F);
  rc = rc ? rc : malloc_n(&n.dYf, c * n.G);
  if (rc) { mlp_free_workspace(n); return rc; }
  n.cap = need;
  UMT_CUDA(cudaMemsetAsync(n.X, 0, c * n.K1 * 2, n.stream));
  return 0;
}

static MlpNet net_view(const Mlp &n) {
  MlpNet v;
  v.G = n.G; v.F = n.F; v.K1 = n.K1; v.N4 = n.N4;
  v.W1 = n.W1; v.W2 = n.W2; v.W3 = n.W3; v.W4 = n.W4; v.W2T = n.W2T; v.W3T = n.W3T; v.W4T = n.W4T;
  v.b1 = n.p + n.po.b1; v.b2 = n.p + n.po.b2; v.b3 = n.p + n.po.b3; v.b4 = n.p + n.po.b4;
  return v;
}

static MlpAct act_view(const Mlp &n, int rows) {
  MlpAct a;
  a.rows = rows; a.ld = n.cap;
  a.X = n.X; a.XT = n.XT;
  for (int i = 0; i < 3; ++i) { a.H[i] = n.H[i]; a.HT[i] = n.HT[i]; a.dZT[i] = n.dZT[i]; }
  a.O = n.O; a.dO = n.dO; a.dOT = n.dOT;
  return a;
}

static MlpGradOff grad_off(const Mlp &n) {
  MlpGradOff o;
  o.w[0] = n.po.W1; o.w[1] = n.po.W2; o.w[2] = n.po.W3; o.w[3] = n.po.W4;
  o.b[0] = n.po.b1; o.b[1] = n.po.b2; o.b[2] = n.po.b3; o.b[3] = n.po.b4;
  return o;
}

static int mlp_pack(Mlp &n) {
  k_mlp_pack<<<152, 256, 0, n.stream>>>(n.G, n.F, n.K1, n.N4, n.po, n.p, n.W1, n.W2, n.W3, n.W4, n.W2T, n.W3T, n.W4T);
  UMT_CUDA(cudaGetLastError());
  return 0;
}

static int set_smem(const void *fn, size_t bytes) {
  UMT_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  return 0;
}

static int mlp_check_status(Mlp &n) {
  unsigned st = 0;
  UMT_CUDA(cudaMemcpyAsync(&st, n.status, sizeof(st), cudaMemcpyDeviceToHost, n.stream));
  UMT_CUDA(cudaStreamSynchronize(n.stream));
  if (st) {
    UMT_CUDA(cudaMemset(n.status, 0, sizeof(unsigned)));
    return set_error(UMT_ERR_TIMEOUT, "learned model: a tensor-core wait gave up");
  }
  return 0;
}

// forward over the workspace rows (X already there)
static int mlp_forward(Mlp &n, int rows, bool train, cudaStream_t st) {
  const MlpNet net = net_view(n);
  const MlpAct act = act_view(n, rows);
  const int tiles = (rows + 127) / 128;
  const int grid = std::max(1, std::min(tiles, 152));
  const size_t sm = forward_smem(n.K1, n.N4);
  if (train) k_mlp_forward<true><<<grid, MLP_NT, sm, st>>>(net, act, n.status);
  else k_mlp_forward<false><<<grid, MLP_NT, sm, st>>>(net, act, n.status);
  UMT_CUDA(cudaGetLastError());
  return 0;
}

// backward of a batch whose dO is set: grad = d(loss)/d(params)
static int mlp_backward(Mlp &n, int rows) {
  const MlpNet net = net_view(n);
  const MlpAct act = act_view(n, rows);
  const int tiles = rows / 128;
  k_mlp_backward<<<std::max(1, std::min(tiles, 152)), MLP_NT, backward_smem(n.N4), n.stream>>>(net, act, n.status);
  if (!n.wpart) {
    int rc = malloc_n(&n.wpart, (size_t)4 * MLP_WCHUNKS * MLP_H * MLP_WPN);
    if (rc) return rc;
  }
  const int chunk = std::max(128, (rows / 128 + MLP_WCHUNKS - 1) / MLP_WCHUNKS * 128);
  const int nchunk = (rows + chunk - 1) / chunk;
  dim3 grid(nchunk, 4);
  k_mlp_wgrad<<<grid, MLP_NT, wgrad_smem(), n.stream>>>(net, act, n.wpart, chunk, n.status);
  k_mlp_wreduce<<<512, 256, 0, n.stream>>>(net, grad_off(n), n.wpart, nchunk, n.g);
  const int nrow = 3 * MLP_H + n.G;
  k_mlp_bgrad<<<(nrow + 7) / 8, 256, 0, n.stream>>>(net, act, grad_off(n), n.g);
  UMT_CUDA(cudaGetLastError());
  return 0;
}

// ---- used by the source iteration (capi.cu) ----
bool mlp_ready_for(int G) { return g_mlp.ready && g_mlp.G == G; }

// Zone features of the context's iterate, the network's multipliers, and
// Phi += m * Delta on every corner (on the context's stream).
int mlp_correct(Ctx &c, double *Target, const double *Delta, const double *DeltaPrev) {
  Mlp &n = g_mlp;
  if (!mlp_ready_for(c.G)) return set_error(UMT_ERR_STATE, "learned model: none for G=%d (umt103_mlp_init)", c.G);
  int rc = mlp_workspace(n, c.nz);
  if (rc) return rc;
  if (!(c.hMean > 0.0)) {                       // mean zone size, once per context
    std::vector<double> vz(c.nz);
    UMT_CUDA(cudaMemcpy(vz.data(), c.VolumeZone, c.nz * sizeof(double), cudaMemcpyDeviceToHost));
    double vt = 0.0;
    for (double x : vz) vt += x;
    c.hMean = std::cbrt(vt / c.nz);
  }
  k_mlp_features<<<(c.nz + 127) / 128, 128, 0, c.stream>>>(c.nz, c.G, n.K1, c.hMean, c.numCorner, c.cOffSet, c.Volume,
                                                           c.Sigt, c.SigS, Target, Delta, DeltaPrev, n.X, nullptr,
                                                           nullptr);
  UMT_CUDA(cudaGetLastError());
  rc = mlp_forward(n, c.nz, false, c.stream);
  if (rc) return rc;
  k_mlp_apply<<<152 * 4, 256, 0, c.stream>>>(c.nc, c.G, n.N4, c.cToZone, n.O, Delta, Target);
  UMT_CUDA(cudaGetLastError());
  return 0;
}

int mlp_status() { return mlp_check_status(g_mlp); }

}  // namespace umt

using namespace umt;

#define LTRY(x) do { int rc_ = (x); if (rc_) return rc_; } while (0)

extern "C" {

int umt103_mlp_init(int ngr, unsigned seed) {
  if (ngr < 1 || ngr > MLP_MAXG) return set_error(UMT_ERR_ARG, "learned model: groups must be 1..%d", MLP_MAXG);
  mlp_free(g_mlp);
  Mlp &n = g_mlp;
  n.G = ngr; n.F = mlp_features(ngr); n.K1 = round16(n.F); n.N4 = round16(ngr);
  n.po = param_offsets(ngr);
  UMT_CUDA(cudaStreamCreateWithFlags(&n.stream, cudaStreamNonBlocking));
  LTRY(malloc_n(&n.p, n.po.n)); LTRY(malloc_n(&n.g, n.po.n)); LTRY(malloc_n(&n.m, n.po.n)); LTRY(malloc_n(&n.v, n.po.n));
  LTRY(malloc_n(&n.W1, (size_t)MLP_H * n.K1)); LTRY(malloc_n(&n.W2, (size_t)MLP_H * MLP_H));
  LTRY(malloc_n(&n.W3, (size_t)MLP_H * MLP_H)); LTRY(malloc_n(&n.W4, (size_t)n.N4 * MLP_H));
  LTRY(malloc_n(&n.W2T, (size_t)MLP_H * MLP_H)); LTRY(malloc_n(&n.W3T, (size_t)MLP_H * MLP_H));
  LTRY(malloc_n(&n.W4T, (size_t)MLP_H * n.N4));
  LTRY(malloc_n(&n.red, 4)); LTRY(malloc_n(&n.status, 1));
  UMT_CUDA(cudaMemset(n.status, 0, sizeof(unsigned)));
  // He-uniform weights from a seeded generator (host), zero biases; the
  // output layer starts small so the first multipliers are near exp(0) = 1
  std::vector<float> h(n.po.n, 0.f);
  uint64_t s = 0x9E3779B97F4A7C15ull ^ ((uint64_t)seed << 1);
  auto uni = [&]() {
    s ^= s >> 12; s ^= s << 25; s ^= s >> 27;
    return (float)(((s * 0x2545F4914F6CDD1Dull) >> 40) * (1.0 / 16777216.0)) * 2.f - 1.f;
  };
  auto fill = [&](long off, long cnt, float a) { for (long i = 0; i < cnt; ++i) h[off + i] = a * uni(); };
  fill(n.po.W1, (long)MLP_H * n.F, std::sqrt(6.f / n.F));
  fill(n.po.W2, (long)MLP_H * MLP_H, std::sqrt(6.f / MLP_H));
  fill(n.po.W3, (long)MLP_H * MLP_H, std::sqrt(6.f / MLP_H));
  fill(n.po.W4, (long)n.G * MLP_H, 0.1f * std::sqrt(6.f / MLP_H));
  UMT_CUDA(cudaMemcpy(n.p, h.data(), n.po.n * sizeof(float), cudaMemcpyHostToDevice));
  UMT_CUDA(cudaMemset(n.m, 0, n.po.n * sizeof(float)));
  UMT_CUDA(cudaMemset(n.v, 0, n.po.n * sizeof(float)));
  LTRY(set_smem((const void *)k_mlp_forward<true>, forward_smem(n.K1, n.N4)));
  LTRY(set_smem((const void *)k_mlp_forward<false>, forward_smem(n.K1, n.N4)));
  LTRY(set_smem((const void *)k_mlp_backward, backward_smem(n.N4)));
  LTRY(set_smem((const void *)k_mlp_wgrad, wgrad_smem()));
  LTRY(mlp_pack(n));
  UMT_CUDA(cudaStreamSynchronize(n.stream));
  n.step = 0;
  n.ready = true;
  return 0;
}

void umt103_mlp_finalize(void) { mlp_free(g_mlp); }

int umt103_mlp_info(int *features, int *hidden, long long *nparams) {
  if (!g_mlp.ready) return set_error(UMT_ERR_STATE, "learned model: umt103_mlp_init not called");
  if (features) *features = g_mlp.F;
  if (hidden) *hidden = MLP_H;
  if (nparams) *nparams = g_mlp.po.n;
  return 0;
}

int umt103_mlp_get_params(float *params) {
  Mlp &n = g_mlp;
  if (!n.ready) return set_error(UMT_ERR_STATE, "learned model: umt103_mlp_init not called");
  if (!params) return set_error(UMT_ERR_ARG, "null params");
  UMT_CUDA(cudaMemcpy(params, n.p, n.po.n * sizeof(float), cudaMemcpyDeviceToHost));
  return 0;
}

int umt103_mlp_set_params(const float *params) {
  Mlp &n = g_mlp;
  if (!n.ready) return set_error(UMT_ERR_STATE, "learned model: umt103_mlp_init not called");
  if (!params) return set_error(UMT_ERR_ARG, "null params");
  UMT_CUDA(cudaMemcpy(n.p, params, n.po.n * sizeof(float), cudaMemcpyHostToDevice));
  UMT_CUDA(cudaMemset(n.m, 0, n.po.n * sizeof(float)));
  UMT_CUDA(cudaMemset(n.v, 0, n.po.n * sizeof(float)));
  n.step = 0;
  LTRY(mlp_pack(n));
  UMT_CUDA(cudaStreamSynchronize(n.stream));
  return 0;
}

int umt103_mlp_forward(const float *X, int rows, float *Y) {
  Mlp &n = g_mlp;
  if (!n.ready) return set_error(UMT_ERR_STATE, "learned model: umt103_mlp_init not called");
  if (!X || !Y || rows <= 0) return set_error(UMT_ERR_ARG, "bad forward arguments");
  LTRY(mlp_workspace(n, rows));
  UMT_CUDA(cudaMemcpyAsync(n.Xf, X, (size_t)rows * n.F * sizeof(float), cudaMemcpyHostToDevice, n.stream));
  k_mlp_x_from_float<<<152, 256, 0, n.stream>>>(rows, n.F, n.K1, n.Xf, n.X);
  UMT_CUDA(cudaGetLastError());
  LTRY(mlp_forward(n, rows, false, n.stream));
  std::vector<float> o((size_t)rows * n.N4);
  UMT_CUDA(cudaMemcpyAsync(o.data(), n.O, o.size() * sizeof(float), cudaMemcpyDeviceToHost, n.stream));
  LTRY(mlp_check_status(n));
  for (int r = 0; r < rows; ++r)
    std::memcpy(Y + (size_t)r * n.G, o.data() + (size_t)r * n.N4, n.G * sizeof(float));
  return 0;
}

int umt103_mlp_gradient(const float *X, const float *dY, int rows, float *grad) {
  Mlp &n = g_mlp;
  if (!n.ready) return set_error(UMT_ERR_STATE, "learned model: umt103_mlp_init not called");
  if (!X || !dY || !grad || rows <= 0 || rows % 128)
    return set_error(UMT_ERR_ARG, "gradient: rows must be a positive multiple of 128");
  LTRY(mlp_workspace(n, rows));
  UMT_CUDA(cudaMemcpyAsync(n.Xf, X, (size_t)rows * n.F * sizeof(float), cudaMemcpyHostToDevice, n.stream));
  UMT_CUDA(cudaMemcpyAsync(n.dYf, dY, (size_t)rows * n.G * sizeof(float), cudaMemcpyHostToDevice, n.stream));
  k_mlp_x_from_float<<<152, 256, 0, n.stream>>>(rows, n.F, n.K1, n.Xf, n.X);
  k_mlp_transpose_x<<<152, 256, 0, n.stream>>>(rows, n.K1, n.cap, n.X, n.XT);
  LTRY(mlp_forward(n, rows, true, n.stream));
  k_mlp_dy<<<152, 256, 0, n.stream>>>(rows, n.G, n.N4, n.cap, n.dYf, n.dO, n.dOT);
  UMT_CUDA(cudaGetLastError());
  LTRY(mlp_backward(n, rows));
  UMT_CUDA(cudaMemcpyAsync(grad, n.g, n.po.n * sizeof(float), cudaMemcpyDeviceToHost, n.stream));
  return mlp_check_status(n);
}

// Training set: snapshots of the current context's source iteration.
int umt103_mlp_collect(int *rows_added) {
  Mlp &n = g_mlp;
  Ctx &c = cur();
  if (!n.ready || n.G != c.G) return set_error(UMT_ERR_STATE, "learned model: none for this context's groups");
  if (!c.ready || !c.Phi || !c.siDelta || !c.siDeltaPrev)
    return set_error(UMT_ERR_STATE, "collect: run umt103_source_iterate (two iterations at least) first");
  if (n.pendingNz && n.pendingNz != c.nz) return set_error(UMT_ERR_STATE, "collect: targets of the previous problem not set");
  const long need = n.nrows + c.nz;
  if (need > n.rowCap) {
    const long cap = std::max(need, 2 * n.rowCap + 4096);
    __nv_bfloat16 *X = nullptr; float *D = nullptr, *P = nullptr, *T = nullptr, *W = nullptr;
    LTRY(malloc_n(&X, (size_t)cap * n.K1)); LTRY(malloc_n(&D, (size_t)cap * n.G)); LTRY(malloc_n(&P, (size_t)cap * n.G));
    LTRY(malloc_n(&T, (size_t)cap * n.G)); LTRY(malloc_n(&W, (size_t)cap));
    if (n.nrows) {
      UMT_CUDA(cudaMemcpy(X, n.Xd, (size_t)n.nrows * n.K1 * 2, cudaMemcpyDeviceToDevice));
      UMT_CUDA(cudaMemcpy(D, n.Dd, (size_t)n.nrows * n.G * 4, cudaMemcpyDeviceToDevice));
      UMT_CUDA(cudaMemcpy(P, n.Pd, (size_t)n.nrows * n.G * 4, cudaMemcpyDeviceToDevice));
      UMT_CUDA(cudaMemcpy(T, n.Td, (size_t)n.nrows * n.G * 4, cudaMemcpyDeviceToDevice));
      UMT_CUDA(cudaMemcpy(W, n.Wd, (size_t)n.nrows * 4, cudaMemcpyDeviceToDevice));
    }
    free_n(n.Xd); free_n(n.Dd); free_n(n.Pd); free_n(n.Td); free_n(n.Wd);
    n.Xd = X; n.Dd = D; n.Pd = P; n.Td = T; n.Wd = W; n.rowCap = cap;
  }
  if (!(c.hMean > 0.0)) {
    std::vector<double> vz(c.nz);
    UMT_CUDA(cudaMemcpy(vz.data(), c.VolumeZone, c.nz * sizeof(double), cudaMemcpyDeviceToHost));
    double vt = 0.0;
    for (double x : vz) vt += x;
    c.hMean = std::cbrt(vt / c.nz);
  }
  k_mlp_features<<<(c.nz + 127) / 128, 128, 0, c.stream>>>(c.nz, c.G, n.K1, c.hMean, c.numCorner, c.cOffSet, c.Volume,
                                                           c.Sigt, c.SigS, c.Phi, c.siDelta, c.siDeltaPrev,
                                                           n.Xd + (size_t)n.nrows * n.K1, n.Dd + (size_t)n.nrows * n.G,
                                                           n.Pd + (size_t)n.nrows * n.G);
  UMT_CUDA(cudaGetLastError());
  UMT_CUDA(cudaStreamSynchronize(c.stream));
  if (!n.pendingNz) n.pendingFrom = n.nrows;
  n.pendingNz = c.nz;
  n.nrows += c.nz;
  if (rows_added) *rows_added = c.nz;
  return 0;
}

// Targets for the snapshots collected from the current context since the
// last call: e = zone mean of PhiStar - zone mean of the snapshot's iterate;
// each snapshot's rows are weighted by 1 / sum e^2.
int umt103_mlp_set_targets(const double *PhiStar) {
  Mlp &n = g_mlp;
  Ctx &c = cur();
  if (!n.ready || !PhiStar) return set_error(UMT_ERR_ARG, "set_targets: no model or no PhiStar");
  if (!n.pendingNz) return 0;
  if (n.pendingNz != c.nz) return set_error(UMT_ERR_STATE, "set_targets: the pending snapshots are of another problem");
  double *dphi = nullptr;
  LTRY(malloc_n(&dphi, (size_t)c.nc * c.G));
  int rc = 0;
  cudaError_t e = cudaMemcpy(dphi, PhiStar, (size_t)c.nc * c.G * 8, cudaMemcpyHostToDevice);
  for (long r0 = n.pendingFrom; r0 < n.nrows && e == cudaSuccess; r0 += c.nz) {
    double s = 0.0;
    e = cudaMemsetAsync(n.red, 0, sizeof(double), c.stream);
    k_mlp_targets<<<(c.nz + 127) / 128, 128, 0, c.stream>>>(c.nz, c.G, c.numCorner, c.cOffSet, c.Volume, dphi,
                                                            n.Pd + (size_t)r0 * c.G, n.Td + (size_t)r0 * c.G, n.red);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&s, n.red, sizeof(double), cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    const float w = s > 0.0 ? (float)(1.0 / s) : 0.f;
    k_fill_f<<<64, 256, 0, c.stream>>>(c.nz, n.Wd + r0, w);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
  if (e != cudaSuccess) rc = set_error(UMT_ERR_CUDA, "set_targets: %s", cudaGetErrorString(e));
  cudaFree(dphi);
  n.pendingNz = 0;
  return rc;
}

int umt103_mlp_rows(long long *rows) {
  if (!rows) return set_error(UMT_ERR_ARG, "null rows");
  *rows = g_mlp.nrows;
  return 0;
}

int umt103_mlp_clear(void) {
  g_mlp.nrows = 0;
  g_mlp.pendingNz = 0;
  return 0;
}

// Adam steps on random batches of the training set.  loss[0], loss[1]: the
// fraction of the targets' squared error left after the correction, over the
// first and the last tenth of the steps (1 = no gain, 0 = exact).
int umt103_mlp_train(int steps, int batch, float lr, float *loss) {
  Mlp &n = g_mlp;
  if (!n.ready) return set_error(UMT_ERR_STATE, "learned model: umt103_mlp_init not called");
  if (steps <= 0 || batch <= 0 || batch % 128 || !(lr > 0.f)) return set_error(UMT_ERR_ARG, "train: bad arguments");
  if (n.pendingNz) return set_error(UMT_ERR_STATE, "train: targets of the last snapshots not set");
  if (n.nrows < 1) return set_error(UMT_ERR_STATE, "train: empty training set");
  LTRY(mlp_workspace(n, batch));
  const int tenth = std::max(1, steps / 10);
  double acc[2][2] = {{0, 0}, {0, 0}};
  std::vector<double> h((size_t)steps * 2);
  const long nparam = n.po.n;
  for (int it = 0; it < steps; ++it) {
    ++n.step;
    const uint32_t seed = mix32((uint32_t)n.step * 0x9E3779B9u + 0x632BE5ABu);
    k_mlp_gather<<<152 * 4, 256, 0, n.stream>>>(batch, n.K1, n.G, n.cap, n.nrows, seed, n.Xd, n.Dd, n.Td, n.Wd,
                                                n.X, n.XT, n.bD, n.bT, n.bW);
    LTRY(mlp_forward(n, batch, true, n.stream));
    UMT_CUDA(cudaMemsetAsync(n.red, 0, 2 * sizeof(double), n.stream));
    k_mlp_loss<<<152 * 2, 256, 0, n.stream>>>(batch, n.G, n.N4, n.cap, n.O, n.bD, n.bT, n.bW, n.dO, n.dOT, n.red);
    UMT_CUDA(cudaGetLastError());
    UMT_CUDA(cudaMemcpyAsync(h.data() + 2 * it, n.red, 2 * sizeof(double), cudaMemcpyDeviceToHost, n.stream));
    LTRY(mlp_backward(n, batch));
    const float b1 = 0.9f, b2 = 0.999f;
    const float bc1 = 1.f - std::pow(b1, (float)n.step), bc2 = 1.f - std::pow(b2, (float)n.step);
    k_mlp_adam<<<152, 256, 0, n.stream>>>(nparam, n.p, n.g, n.m, n.v, lr, b1, b2, 1e-8f, bc1, bc2, 1e3f);
    UMT_CUDA(cudaGetLastError());
    LTRY(mlp_pack(n));
  }
  LTRY(mlp_check_status(n));
  for (int it = 0; it < steps; ++it) {
    const int k = it < tenth ? 0 : (it >= steps - tenth ? 1 : -1);
    if (k < 0) continue;
    acc[k][0] += h[2 * it];
    acc[k][1] += h[2 * it + 1];
  }
  if (loss) {
    loss[0] = acc[0][1] > 0 ? (float)(acc[0][0] / acc[0][1]) : 0.f;
    loss[1] = acc[1][1] > 0 ? (float)(acc[1][0] / acc[1][1]) : 0.f;
  }
  return 0;
}

}  // extern "C"
