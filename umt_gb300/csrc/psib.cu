// psib.cu -- PsiB rows between the caller's FP64 array and the device's FP32
// copy, for FP32 sweeps called with host buffers.
//
// A row is (direction a, boundary element b): G values.  The FP32 sweep reads
// a row when the FP32 projection Omega_a.A_fp of b's corner face is < 0
// (incoming) and writes it when it is > 0 (exiting); every row it reads is
// read by exactly one work item, the one of direction a and b's zone, in the
// dependency stage level[a][zone].  The rows the sweep does not write are
// therefore ordered once by that stage (rows it never reads last) and copied
// in a few chunks on a side stream inside the sweep's graph; the first stage
// of each chunk waits for it, so the transfer overlaps the early stages
// instead of preceding them.
#include "umt_common.cuh"
#include "../../include/umt103.h"

#include <algorithm>

namespace umt {

// Boundary element b's corner face c*3 + f (cFP holds nc + b on boundary faces).
__global__ void k_bface(int nc, int nb, const int *nCFaces, const int *cFP, int *bFace) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  for (int f = 0; f < nCFaces[c]; ++f) {
    const int v = cFP[c * UMT_MAXCF + f];
    if (v >= nc && v - nc < nb) bFace[v - nc] = c * UMT_MAXCF + f;
  }
}

int ensure_bface(Ctx &c) {
  if (c.bFace) return 0;
  const size_t n = (size_t)std::max(c.nb, 1);
  if (cudaMalloc((void **)&c.bFace, n * sizeof(int)) != cudaSuccess) {
    c.bFace = nullptr;
    return set_error(UMT_ERR_NOMEM, "boundary face map: allocation failed");
  }
  UMT_CUDA(cudaMemset(c.bFace, 0xff, n * sizeof(int)));
  k_bface<<<(c.nc + 255) / 256, 256>>>(c.nc, c.nb, c.nCFaces, c.cFP, c.bFace);
  UMT_CUDA(cudaGetLastError());
  UMT_CUDA(cudaDeviceSynchronize());
  return 0;
}

// The stage that reads row r, nStages for a row no stage reads, -1 for an
// exiting row.
__device__ __forceinline__ int row_stage(size_t r, int nb, int nc, int nz, int nStages, const int *bFace,
                                         const float *afp32, const int *cToZone, const int *level) {
  const int a = (int)(r / (size_t)nb), b = (int)(r - (size_t)a * nb);
  const int bf = bFace[b];
  if (bf < 0) return nStages;
  const float v = afp32[(size_t)a * nc * UMT_MAXCF + bf];
  if (v > 0.f) return -1;
  if (v < 0.f) return level[(size_t)a * nz + cToZone[bf / UMT_MAXCF]];
  return nStages;
}

__global__ void k_row_count(int A, int nb, int nc, int nz, int nStages, const int *bFace, const float *afp32,
                            const int *cToZone, const int *level, int *count) {
  const size_t n = (size_t)A * nb;
  for (size_t r = blockIdx.x * (size_t)blockDim.x + threadIdx.x; r < n; r += (size_t)gridDim.x * blockDim.x) {
    const int s = row_stage(r, nb, nc, nz, nStages, bFace, afp32, cToZone, level);
    if (s >= 0) atomicAdd(&count[min(s, nStages)], 1);
  }
}

__global__ void k_row_scatter(int A, int nb, int nc, int nz, int nStages, const int *bFace, const float *afp32,
                              const int *cToZone, const int *level, int *cursor, int *rowOrder) {
  const size_t n = (size_t)A * nb;
  for (size_t r = blockIdx.x * (size_t)blockDim.x + threadIdx.x; r < n; r += (size_t)gridDim.x * blockDim.x) {
    const int s = row_stage(r, nb, nc, nz, nStages, bFace, afp32, cToZone, level);
    if (s >= 0) rowOrder[atomicAdd(&cursor[min(s, nStages)], 1)] = (int)r;
  }
}

// One chunk: rows[0..n) from the FP64 array *src (page-locked host memory or
// the staging copy, 16-byte aligned) into the FP32 copy, G even; nothing when
// *src is null.  It runs beside the latency-bound stage kernels, so it uses
// few blocks (PSIB_GATHER_BLOCKS) and keeps 8 pairs of values in flight per
// thread instead: 64 blocks hold ~2 MB in flight (24 blocks, ~0.8 MB, reached
// only ~110 GB/s of the link's ~210 under its loaded latency).
constexpr int PSIB_GATHER_BLOCKS = 64;

__global__ void __launch_bounds__(256) k_psib_gather(const int *rows, int n, int G, double *const *src,
                                                     float *psiB32) {
  const double *s = *src;
  if (!s) return;
  constexpr int U = 8;
  const int G2 = G / 2;
  const size_t m = (size_t)n * G2;                 // value pairs
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  for (; i + (U - 1) * stride < m; i += U * stride) {
    double2 v[U];
    size_t e[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const size_t j = i + u * stride;
      e[u] = (size_t)rows[j / G2] * G + 2 * (j % G2);
      v[u] = *reinterpret_cast<const double2 *>(s + e[u]);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) *reinterpret_cast<float2 *>(psiB32 + e[u]) = make_float2((float)v[u].x, (float)v[u].y);
  }
  for (; i < m; i += stride) {
    const size_t e = (size_t)rows[i / G2] * G + 2 * (i % G2);
    const double2 v = *reinterpret_cast<const double2 *>(s + e);
    *reinterpret_cast<float2 *>(psiB32 + e) = make_float2((float)v.x, (float)v.y);
  }
}

int ensure_psib_order(Ctx &c) {
  if (c.rowOrder) return 0;
  if (!c.afp32 || !c.psiB32) return set_error(UMT_ERR_STATE, "FP32 flux not allocated");
  if ((long long)c.A * c.nb >= (1LL << 31)) return set_error(UMT_ERR_ARG, "PsiB rows exceed 2^31");
  int rc = ensure_bface(c);
  if (rc) return rc;
  const int S = c.sch.nStages;
  int *count = nullptr;
  if (cudaMalloc((void **)&count, (size_t)(S + 1) * sizeof(int)) != cudaSuccess)
    return set_error(UMT_ERR_NOMEM, "PsiB row order: allocation failed");
  UMT_CUDA(cudaMemset(count, 0, (size_t)(S + 1) * sizeof(int)));
  k_row_count<<<1024, 256>>>(c.A, c.nb, c.nc, c.nz, S, c.bFace, c.afp32, c.cToZone, c.sch.level, count);
  std::vector<int> h(S + 1);
  UMT_CUDA(cudaMemcpy(h.data(), count, (size_t)(S + 1) * sizeof(int), cudaMemcpyDeviceToHost));
  std::vector<int> start(S + 2, 0);
  for (int s = 0; s <= S; ++s) start[s + 1] = start[s] + h[s];
  const int total = start[S + 1];
  if (cudaMalloc((void **)&c.rowOrder, (size_t)std::max(total, 1) * sizeof(int)) != cudaSuccess) {
    cudaFree(count);
    c.rowOrder = nullptr;
    return set_error(UMT_ERR_NOMEM, "PsiB row order: allocation failed");
  }
  UMT_CUDA(cudaMemcpy(count, start.data(), (size_t)(S + 1) * sizeof(int), cudaMemcpyHostToDevice));
  k_row_scatter<<<1024, 256>>>(c.A, c.nb, c.nc, c.nz, S, c.bFace, c.afp32, c.cToZone, c.sch.level, count,
                               c.rowOrder);
  UMT_CUDA(cudaGetLastError());
  UMT_CUDA(cudaDeviceSynchronize());
  cudaFree(count);
  // chunks: stages [0,2), [2,4), [4,8), ... doubling, then the rows no stage reads
  c.chunkOff.clear();
  c.chunkStage.clear();
  int lo = 0;
  for (int hi = 2; lo < S; hi *= 2) {
    const int e = std::min(hi, S);
    if (start[e] > start[lo]) {
      c.chunkOff.push_back(start[lo]);
      c.chunkStage.push_back(lo);
    }
    lo = e;
  }
  if (start[S + 1] > start[S]) {
    c.chunkOff.push_back(start[S]);
    c.chunkStage.push_back(S);
  }
  c.chunkOff.push_back(total);
  const size_t K = c.chunkStage.size();
  if (!c.stream2) UMT_CUDA(cudaStreamCreateWithFlags(&c.stream2, cudaStreamNonBlocking));
  if (!c.evFork) UMT_CUDA(cudaEventCreateWithFlags(&c.evFork, cudaEventDisableTiming));
  while (c.evChunk.size() < K) {
    cudaEvent_t e = nullptr;
    UMT_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    c.evChunk.push_back(e);
  }
  if (!c.psibIn) {
    if (cudaMalloc((void **)&c.psibIn, sizeof(double *)) != cudaSuccess) {
      c.psibIn = nullptr;
      return set_error(UMT_ERR_NOMEM, "PsiB source word: allocation failed");
    }
    UMT_CUDA(cudaMemset(c.psibIn, 0, sizeof(double *)));
  }
  return 0;
}

// Inside the host-facing graph: fork the chunk copies onto the side stream.
int enqueue_psib_chunks(Ctx &c) {
  if (!c.rowOrder) return 0;
  UMT_CUDA(cudaEventRecord(c.evFork, c.stream));
  UMT_CUDA(cudaStreamWaitEvent(c.stream2, c.evFork, 0));
  for (size_t k = 0; k < c.chunkStage.size(); ++k) {
    const int n = c.chunkOff[k + 1] - c.chunkOff[k];
    const size_t m = (size_t)n * (c.G / 2);
    const int blocks = (int)std::min<size_t>((m + 255) / 256, PSIB_GATHER_BLOCKS);
    k_psib_gather<<<std::max(blocks, 1), 256, 0, c.stream2>>>(c.rowOrder + c.chunkOff[k], n, c.G, c.psibIn,
                                                               c.psiB32);
    UMT_CUDA(cudaGetLastError());
    UMT_CUDA(cudaEventRecord(c.evChunk[k], c.stream2));
  }
  return 0;
}

// Before the launch of stage s (and with s == nStages at the end of the
// sweep, which joins the side stream): wait for the chunks that begin there.
int wait_psib_chunks(Ctx &c, int s) {
  if (!c.rowOrder) return 0;
  for (size_t k = 0; k < c.chunkStage.size(); ++k)
    if (c.chunkStage[k] == s) UMT_CUDA(cudaStreamWaitEvent(c.stream, c.evChunk[k], 0));
  return 0;
}

void free_psib(Ctx &c) {
  if (c.rowOrder) cudaFree(c.rowOrder);
  if (c.psibIn) cudaFree(c.psibIn);
  c.rowOrder = nullptr;
  c.psibIn = nullptr;
  for (cudaEvent_t e : c.evChunk) cudaEventDestroy(e);
  c.evChunk.clear();
  if (c.evFork) cudaEventDestroy(c.evFork);
  if (c.stream2) cudaStreamDestroy(c.stream2);
  c.evFork = nullptr;
  c.stream2 = nullptr;
  c.chunkOff.clear();
  c.chunkStage.clear();
}

}  // namespace umt
