// psib.cu -- PsiB rows between the caller's FP64 array and the device's FP32
// copy, for FP32 sweeps called with host buffers.
//
// A row is (direction a, boundary element b): G values.  The FP32 sweep reads
// a row when the FP32 projection Omega_a.A_fp of b's corner face is < 0
// (incoming) and writes it when it is > 0 (exiting); every row it reads is
// read by exactly one work item, the one of direction a and b's zone, in the
// dependency stage level[a][zone].  The rows the sweep does not write are
// therefore ordered once by that stage (rows it never reads last) and copied
// in chunks of a few MB on a side stream inside the sweep's graph; the first
// stage that reads a chunk's rows waits for it, so the transfer runs ahead of
// the stages instead of preceding them.
//
// The source STotal goes the same way when the caller's array is page-locked:
// corner c's row is first read by the first stage, over all directions, that
// sweeps c's zone, so the corners are ordered by that stage and converted to
// FP32 in chunks the same way, interleaved with the PsiB chunks on the
// side stream.  Otherwise the chunks convert the device's FP64 copy.
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
// exiting row; with EXIT, the stage that writes an exiting row, -1 for any
// other row.
template <bool EXIT>
__device__ __forceinline__ int row_stage(size_t r, int nb, int nc, int nz, int nStages, const int *bFace,
                                         const float *afp32, const int *cToZone, const int *level) {
  const int a = (int)(r / (size_t)nb), b = (int)(r - (size_t)a * nb);
  const int bf = bFace[b];
  if (bf < 0) return EXIT ? -1 : nStages;
  const float v = afp32[(size_t)a * nc * UMT_MAXCF + bf];
  const int lv = level[(size_t)a * nz + cToZone[bf / UMT_MAXCF]];
  if (EXIT) return v > 0.f ? lv : -1;
  if (v > 0.f) return -1;
  if (v < 0.f) return lv;
  return nStages;
}

template <bool EXIT>
__global__ void k_row_count(int A, int nb, int nc, int nz, int nStages, const int *bFace, const float *afp32,
                            const int *cToZone, const int *level, int *count) {
  const size_t n = (size_t)A * nb;
  for (size_t r = blockIdx.x * (size_t)blockDim.x + threadIdx.x; r < n; r += (size_t)gridDim.x * blockDim.x) {
    const int s = row_stage<EXIT>(r, nb, nc, nz, nStages, bFace, afp32, cToZone, level);
    if (s >= 0) atomicAdd(&count[min(s, nStages)], 1);
  }
}

template <bool EXIT>
__global__ void k_row_scatter(int A, int nb, int nc, int nz, int nStages, const int *bFace, const float *afp32,
                              const int *cToZone, const int *level, int *cursor, int *rowOrder) {
  const size_t n = (size_t)A * nb;
  for (size_t r = blockIdx.x * (size_t)blockDim.x + threadIdx.x; r < n; r += (size_t)gridDim.x * blockDim.x) {
    const int s = row_stage<EXIT>(r, nb, nc, nz, nStages, bFace, afp32, cToZone, level);
    if (s >= 0) rowOrder[atomicAdd(&cursor[min(s, nStages)], 1)] = (int)r;
  }
}

// One chunk of exiting rows: rows[0..n) of the device FP32 copy to the FP64
// array *dst (page-locked host memory or the staging copy, 16-byte aligned),
// G even; nothing when *dst is null.
__global__ void __launch_bounds__(256) k_rows_out(const int *rows, int n, int G, const float *psiB32,
                                                  double *const *dst) {
  double *d = *dst;
  if (!d) return;
  const int G2 = G / 2;
  const size_t m = (size_t)n * G2;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < m; i += (size_t)gridDim.x * blockDim.x) {
    const size_t e = (size_t)rows[i / G2] * G + 2 * (i % G2);
    const float2 v = *reinterpret_cast<const float2 *>(psiB32 + e);
    *reinterpret_cast<double2 *>(d + e) = make_double2((double)v.x, (double)v.y);
  }
}

// One chunk: rows[0..n) (row r = values [r*G, r*G + G)) from the FP64 array
// *src (page-locked host memory or a device staging copy, 16-byte aligned)
// into the FP32 copy dst32, G even.  With *src null: nothing (PsiB), or, with
// SRC, the rows of the device copy dev64.  With SRC and a host array the rows
// also go to dev64, so the device keeps the call's FP64 source as a copy of
// the whole array would.  It runs beside the latency-bound stage kernels, so it uses
// few blocks (PSIB_GATHER_BLOCKS) and keeps 8 pairs of values in flight per
// thread instead: 64 blocks hold ~2 MB in flight (24 blocks, ~0.8 MB, reached
// only ~110 GB/s of the link's ~210 under its loaded latency).
constexpr int PSIB_GATHER_BLOCKS = 64;
// The exit-row copies write to the link, posted, so fewer blocks keep up: a
// call took 15.8 ms with 32 blocks, 16.2 with 64 (more stage blocks
// displaced) and 17.9 with 16 (the copies fell behind the stages).
constexpr int EXIT_OUT_BLOCKS = 32;

template <bool SRC>
__global__ void __launch_bounds__(256) k_rows_gather(const int *rows, int n, int G, double *const *src,
                                                     double *dev64, float *dst32) {
  const double *h = *src;
  if (!SRC && !h) return;
  const double *s = h ? h : dev64;
  const bool keep = SRC && h;
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
    for (int u = 0; u < U; ++u) {
      *reinterpret_cast<float2 *>(dst32 + e[u]) = make_float2((float)v[u].x, (float)v[u].y);
      if (keep) *reinterpret_cast<double2 *>(dev64 + e[u]) = v[u];
    }
  }
  for (; i < m; i += stride) {
    const size_t e = (size_t)rows[i / G2] * G + 2 * (i % G2);
    const double2 v = *reinterpret_cast<const double2 *>(s + e);
    *reinterpret_cast<float2 *>(dst32 + e) = make_float2((float)v.x, (float)v.y);
    if (keep) *reinterpret_cast<double2 *>(dev64 + e) = v;
  }
}

// The first stage, over all directions, that sweeps each zone.
__global__ void k_zone_first(int A, int nz, const int *level, int *first) {
  for (int z = blockIdx.x * blockDim.x + threadIdx.x; z < nz; z += gridDim.x * blockDim.x) {
    int m = level[z];
    for (int a = 1; a < A; ++a) m = min(m, level[(size_t)a * nz + z]);
    first[z] = m;
  }
}

__global__ void k_corner_count(int nc, int nStages, const int *cToZone, const int *first, int *count) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x)
    atomicAdd(&count[min(max(first[cToZone[c]], 0), nStages - 1)], 1);
}

__global__ void k_corner_scatter(int nc, int nStages, const int *cToZone, const int *first, int *cursor,
                                 int *order) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x)
    order[atomicAdd(&cursor[min(max(first[cToZone[c]], 0), nStages - 1)], 1)] = c;
}

// Chunks of a list ordered by stage (start[s] = first entry of stage s),
// cut at stage boundaries into pieces of at least about 4 MB of FP64 rows
// and at least 1/CHUNK_MAX of the list, the empty ones left out.  stage[k]
// is the first stage with a row in chunk k, (*last)[k] the last one.  With
// tail, the entries past the last stage (rows no stage reads) are one more
// chunk, waited for at the end of the sweep.  Small chunks matter: with
// chunks of doubling stage span, stage 2^k would wait for every row read up
// to stage 2^(k+1), milliseconds of link time at 20^3 tiles.
constexpr int CHUNK_MAX = 96;
static void stage_chunks(const std::vector<int> &start, int S, bool tail, int G, std::vector<int> &off,
                         std::vector<int> &stage, std::vector<int> *last = nullptr) {
  off.clear();
  stage.clear();
  if (last) last->clear();
  const long long total = start[S] - start[0];
  const long long minRows = (4ll << 20) / (8ll * std::max(G, 1));      // about 4 MB of FP64 rows
  const long long target = std::max<long long>((total + CHUNK_MAX - 1) / CHUNK_MAX, std::max(minRows, 1ll));
  int lo = 0;
  for (int s = 0; s < S; ++s) {
    if (start[s + 1] - start[lo] >= target || s == S - 1) {
      if (start[s + 1] > start[lo]) {
        int first = lo, end = s;
        while (start[first + 1] == start[first]) ++first;             // the first stage with rows
        while (start[end + 1] == start[end]) --end;                   // the last
        off.push_back(start[lo]);
        stage.push_back(first);
        if (last) last->push_back(end);
      }
      lo = s + 1;
    }
  }
  if (tail && start[S + 1] > start[S]) {
    off.push_back(start[S]);
    stage.push_back(S);
  }
  off.push_back(tail ? start[S + 1] : start[S]);
}

static int ensure_side_stream(Ctx &c) {
  if (!c.stream2) UMT_CUDA(cudaStreamCreateWithFlags(&c.stream2, cudaStreamNonBlocking));
  if (!c.evFork) UMT_CUDA(cudaEventCreateWithFlags(&c.evFork, cudaEventDisableTiming));
  return 0;
}

static int ensure_events(std::vector<cudaEvent_t> &ev, size_t K) {
  while (ev.size() < K) {
    cudaEvent_t e = nullptr;
    UMT_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    ev.push_back(e);
  }
  return 0;
}

static int alloc_word(double ***w, const char *what) {
  if (*w) return 0;
  if (cudaMalloc((void **)w, sizeof(double *)) != cudaSuccess) {
    *w = nullptr;
    return set_error(UMT_ERR_NOMEM, "%s: allocation failed", what);
  }
  UMT_CUDA(cudaMemset(*w, 0, sizeof(double *)));
  return 0;
}

// The PsiB rows (a*nb + b) counting-sorted by stage: the rows the sweep
// reads by the stage that reads them, the rows it reads nowhere last (stage
// S); with EXIT, the exiting rows by the stage that writes them.  *order
// (device) and start[s] = the first entry of stage s, start[S + 1] = total.
template <bool EXIT>
static int row_order(Ctx &c, const char *what, int **orderOut, std::vector<int> &start) {
  const int S = c.sch.nStages;
  int *count = nullptr, *order = nullptr;
  auto fail = [&](int rc) { cudaFree(count); if (order) cudaFree(order); return rc; };
  if (cudaMalloc((void **)&count, (size_t)(S + 1) * sizeof(int)) != cudaSuccess) {
    count = nullptr;
    return fail(set_error(UMT_ERR_NOMEM, "%s: allocation failed", what));
  }
  cudaMemset(count, 0, (size_t)(S + 1) * sizeof(int));
  k_row_count<EXIT><<<1024, 256>>>(c.A, c.nb, c.nc, c.nz, S, c.bFace, c.afp32, c.cToZone, c.sch.level, count);
  std::vector<int> h(S + 1);
  if (cudaMemcpy(h.data(), count, (size_t)(S + 1) * sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    return fail(set_error(UMT_ERR_CUDA, "%s: %s", what, cudaGetErrorString(cudaGetLastError())));
  start.assign(S + 2, 0);
  for (int s = 0; s <= S; ++s) start[s + 1] = start[s] + h[s];
  if (EXIT && start[S + 1] != start[S]) return fail(set_error(UMT_ERR_STATE, "%s: a row past the last stage", what));
  if (cudaMalloc((void **)&order, (size_t)std::max(start[S + 1], 1) * sizeof(int)) != cudaSuccess) {
    order = nullptr;
    return fail(set_error(UMT_ERR_NOMEM, "%s: allocation failed", what));
  }
  cudaMemcpy(count, start.data(), (size_t)(S + 1) * sizeof(int), cudaMemcpyHostToDevice);
  k_row_scatter<EXIT><<<1024, 256>>>(c.A, c.nb, c.nc, c.nz, S, c.bFace, c.afp32, c.cToZone, c.sch.level, count,
                                     order);
  const cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return fail(set_error(UMT_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e)));
  cudaFree(count);
  *orderOut = order;
  return 0;
}

// The exiting rows by the stage that writes them, in chunks of ~4 MB or
// more, each copied out after the last stage that writes one of its rows.
// Kept (c.exitOrder) only once its chunks, stream and events exist.
static int ensure_exit_order(Ctx &c) {
  if (c.exitOrder) return 0;
  int *order = nullptr;
  std::vector<int> start, firstStage;
  int rc = row_order<true>(c, "exit row order", &order, start);
  if (rc) return rc;
  stage_chunks(start, c.sch.nStages, false, c.G, c.exitChunkOff, firstStage, &c.exitChunkLast);
  if (!c.stream3 && cudaStreamCreateWithFlags(&c.stream3, cudaStreamNonBlocking) != cudaSuccess) {
    c.stream3 = nullptr;
    rc = set_error(UMT_ERR_CUDA, "exit row order: stream creation failed");
  }
  if (!rc && !c.evExitJoin && cudaEventCreateWithFlags(&c.evExitJoin, cudaEventDisableTiming) != cudaSuccess) {
    c.evExitJoin = nullptr;
    rc = set_error(UMT_ERR_CUDA, "exit row order: event creation failed");
  }
  if (!rc) rc = ensure_events(c.evExit, c.exitChunkLast.size());
  if (rc) {
    cudaFree(order);
    return rc;
  }
  c.exitOrder = order;
  return 0;
}

// The rows the sweep reads, in chunks of ~4 MB or more in stage order, then
// the rows no stage reads; then the exit rows.  Kept (c.rowOrder) only once
// its chunks and their events exist.
int ensure_psib_order(Ctx &c) {
  if (c.rowOrder) return ensure_exit_order(c);
  if (!c.afp32 || !c.psiB32) return set_error(UMT_ERR_STATE, "FP32 flux not allocated");
  if ((long long)c.A * c.nb >= (1LL << 31)) return set_error(UMT_ERR_ARG, "PsiB rows exceed 2^31");
  int rc = ensure_bface(c);
  if (rc) return rc;
  int *order = nullptr;
  std::vector<int> start;
  rc = row_order<false>(c, "PsiB row order", &order, start);
  if (rc) return rc;
  stage_chunks(start, c.sch.nStages, true, c.G, c.chunkOff, c.chunkStage);
  rc = ensure_side_stream(c);
  if (!rc) rc = ensure_events(c.evChunk, c.chunkStage.size());
  if (!rc) rc = alloc_word(&c.psibIn, "PsiB source word");
  if (rc) {
    cudaFree(order);
    return rc;
  }
  c.rowOrder = order;
  return ensure_exit_order(c);
}

int ensure_src_order(Ctx &c) {
  if (c.srcOrder) return 0;
  if (!c.STotal32) return set_error(UMT_ERR_STATE, "FP32 source not allocated");
  const int S = c.sch.nStages;
  if (S <= 0) return set_error(UMT_ERR_STATE, "no schedule");
  int *first = nullptr, *count = nullptr;
  if (cudaMalloc((void **)&first, (size_t)std::max(c.nz, 1) * sizeof(int)) != cudaSuccess)
    return set_error(UMT_ERR_NOMEM, "source row order: allocation failed");
  if (cudaMalloc((void **)&count, (size_t)S * sizeof(int)) != cudaSuccess) {
    cudaFree(first);
    return set_error(UMT_ERR_NOMEM, "source row order: allocation failed");
  }
  int *order = nullptr;
  // the order is kept (c.srcOrder) only once it, its chunks and their events exist
  auto fail = [&](int rc) { cudaFree(first); cudaFree(count); if (order) cudaFree(order); return rc; };
  if (cudaMalloc((void **)&order, (size_t)std::max(c.nc, 1) * sizeof(int)) != cudaSuccess) {
    order = nullptr;
    return fail(set_error(UMT_ERR_NOMEM, "source row order: allocation failed"));
  }
  cudaMemset(count, 0, (size_t)S * sizeof(int));
  k_zone_first<<<std::max(1, std::min((c.nz + 255) / 256, 152 * 8)), 256>>>(c.A, c.nz, c.sch.level, first);
  k_corner_count<<<std::max(1, std::min((c.nc + 255) / 256, 152 * 8)), 256>>>(c.nc, S, c.cToZone, first, count);
  std::vector<int> h(S);
  if (cudaMemcpy(h.data(), count, (size_t)S * sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    return fail(set_error(UMT_ERR_CUDA, "source row order: %s", cudaGetErrorString(cudaGetLastError())));
  std::vector<int> start(S + 2, 0);
  for (int s = 0; s < S; ++s) start[s + 1] = start[s] + h[s];
  start[S + 1] = start[S];
  if (start[S] != c.nc) return fail(set_error(UMT_ERR_STATE, "source row order: %d of %d corners", start[S], c.nc));
  cudaMemcpy(count, start.data(), (size_t)S * sizeof(int), cudaMemcpyHostToDevice);
  k_corner_scatter<<<std::max(1, std::min((c.nc + 255) / 256, 152 * 8)), 256>>>(c.nc, S, c.cToZone, first, count,
                                                                                 order);
  const cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return fail(set_error(UMT_ERR_CUDA, "source row order: %s", cudaGetErrorString(e)));
  stage_chunks(start, S, false, c.G, c.srcChunkOff, c.srcChunkStage);
  int re = ensure_side_stream(c);
  if (!re) re = ensure_events(c.evSrc, c.srcChunkStage.size());
  if (!re) re = alloc_word(&c.srcIn, "source word");
  if (re) return fail(re);
  cudaFree(first);
  cudaFree(count);
  c.srcOrder = order;
  return 0;
}

// A row-copy kernel at the device's highest priority.  With equal
// priorities, a copy launched while a stage still has blocks waiting got SM
// slots only as that stage's last wave drained, and the link sat idle.
template <typename... KArgs, typename... Args>
static int launch_copy(void (*kern)(KArgs...), int blocks, cudaStream_t st, Args... args) {
  int least = 0, greatest = 0;
  UMT_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributePriority;
  at[0].val.priority = greatest;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(std::max(blocks, 1));
  cfg.blockDim = dim3(256);
  cfg.stream = st;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  UMT_CUDA(cudaLaunchKernelEx(&cfg, kern, args...));
  return 0;
}

// Inside the host-facing graph: fork the chunk copies onto the side stream,
// in stage order (a source chunk before the PsiB chunk that begins at the
// same stage), each followed by its event.
int enqueue_psib_chunks(Ctx &c) {
  const bool src = c.srcChunksNow && c.srcOrder;
  if (!c.rowOrder && !src) return 0;
  UMT_CUDA(cudaEventRecord(c.evFork, c.stream));
  UMT_CUDA(cudaStreamWaitEvent(c.stream2, c.evFork, 0));
  const size_t KP = c.rowOrder ? c.chunkStage.size() : 0, KS = src ? c.srcChunkStage.size() : 0;
  size_t kp = 0, ks = 0;
  while (kp < KP || ks < KS) {
    if (ks < KS && (kp >= KP || c.srcChunkStage[ks] <= c.chunkStage[kp])) {
      const int n = c.srcChunkOff[ks + 1] - c.srcChunkOff[ks];
      const size_t m = (size_t)n * (c.G / 2);
      const int blocks = (int)std::min<size_t>((m + 255) / 256, PSIB_GATHER_BLOCKS);
      const int rl = launch_copy(k_rows_gather<true>, blocks, c.stream2, (const int *)(c.srcOrder + c.srcChunkOff[ks]),
                                 n, c.G, (double *const *)c.srcIn, c.STotal, c.STotal32);
      if (rl) return rl;
      UMT_CUDA(cudaEventRecord(c.evSrc[ks], c.stream2));
      ++ks;
    } else {
      const int n = c.chunkOff[kp + 1] - c.chunkOff[kp];
      const size_t m = (size_t)n * (c.G / 2);
      const int blocks = (int)std::min<size_t>((m + 255) / 256, PSIB_GATHER_BLOCKS);
      const int rl = launch_copy(k_rows_gather<false>, blocks, c.stream2, (const int *)(c.rowOrder + c.chunkOff[kp]),
                                 n, c.G, (double *const *)c.psibIn, (double *)nullptr, c.psiB32);
      if (rl) return rl;
      UMT_CUDA(cudaEventRecord(c.evChunk[kp], c.stream2));
      ++kp;
    }
  }
  return 0;
}

// Before the launch of stage s (and with s == nStages at the end of the
// sweep, which joins the side stream): wait for the chunks that begin there.
int wait_psib_chunks(Ctx &c, int s) {
  if (c.rowOrder)
    for (size_t k = 0; k < c.chunkStage.size(); ++k)
      if (c.chunkStage[k] == s) UMT_CUDA(cudaStreamWaitEvent(c.stream, c.evChunk[k], 0));
  if (c.srcChunksNow && c.srcOrder)
    for (size_t k = 0; k < c.srcChunkStage.size(); ++k)
      if (c.srcChunkStage[k] == s) UMT_CUDA(cudaStreamWaitEvent(c.stream, c.evSrc[k], 0));
  return 0;
}

// After the launch of stage s (zone-program kernel, plain variant): the
// exit chunks whose last stage is s go to *psibOut on the third stream.
int enqueue_exit_chunks(Ctx &c, int s) {
  if (!c.exitOrder) return 0;
  for (size_t k = 0; k < c.exitChunkLast.size(); ++k) {
    if (c.exitChunkLast[k] != s) continue;
    UMT_CUDA(cudaEventRecord(c.evExit[k], c.stream));
    UMT_CUDA(cudaStreamWaitEvent(c.stream3, c.evExit[k], 0));
    const int n = c.exitChunkOff[k + 1] - c.exitChunkOff[k];
    const size_t m = (size_t)n * (c.G / 2);
    const int blocks = (int)std::min<size_t>((m + 255) / 256, EXIT_OUT_BLOCKS);
    const int rl = launch_copy(k_rows_out, blocks, c.stream3, (const int *)(c.exitOrder + c.exitChunkOff[k]), n,
                               c.G, (const float *)c.psiB32, (double *const *)c.psibOut);
    if (rl) return rl;
  }
  return 0;
}

int join_exit_chunks(Ctx &c) {
  if (!c.exitOrder || c.exitChunkLast.empty()) return 0;
  UMT_CUDA(cudaEventRecord(c.evExitJoin, c.stream3));
  UMT_CUDA(cudaStreamWaitEvent(c.stream, c.evExitJoin, 0));
  return 0;
}

void free_psib(Ctx &c) {
  if (c.rowOrder) cudaFree(c.rowOrder);
  if (c.psibIn) cudaFree(c.psibIn);
  if (c.srcOrder) cudaFree(c.srcOrder);
  if (c.srcIn) cudaFree(c.srcIn);
  c.rowOrder = nullptr;
  c.psibIn = nullptr;
  c.srcOrder = nullptr;
  c.srcIn = nullptr;
  for (cudaEvent_t e : c.evChunk) cudaEventDestroy(e);
  c.evChunk.clear();
  for (cudaEvent_t e : c.evSrc) cudaEventDestroy(e);
  c.evSrc.clear();
  if (c.exitOrder) cudaFree(c.exitOrder);
  c.exitOrder = nullptr;
  for (cudaEvent_t e : c.evExit) cudaEventDestroy(e);
  c.evExit.clear();
  c.exitChunkOff.clear();
  c.exitChunkLast.clear();
  if (c.evExitJoin) cudaEventDestroy(c.evExitJoin);
  if (c.stream3) cudaStreamDestroy(c.stream3);
  c.evExitJoin = nullptr;
  c.stream3 = nullptr;
  c.srcChunkOff.clear();
  c.srcChunkStage.clear();
  if (c.evFork) cudaEventDestroy(c.evFork);
  if (c.stream2) cudaStreamDestroy(c.stream2);
  c.evFork = nullptr;
  c.stream2 = nullptr;
  c.chunkOff.clear();
  c.chunkStage.clear();
}

}  // namespace umt
