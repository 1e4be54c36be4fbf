// noalloc.cu -- energy edits without any device allocation.
//
// umt103_tally (capi.cu) copies the absorption opacities to a buffer it
// allocates, and reduces into a context buffer.  Some callers cannot let a
// library allocate device memory during a call: a host code whose memory pool
// must account for every device byte (an Umpire-style pool that owns the
// device heap), or a run that reserved all free device memory up front and
// would see an allocation fail mid time step.  This file gives them
// umt103_tally_noalloc: the caller passes its absorption opacities already on
// the device (or NULL), and the reduction works in a fixed scratch array that
// lives in the library's image for as long as the library is loaded (one copy
// per GPU that loads it, never freed before exit).
//
// The scratch holds one 4-value partial per thread block, and each block
// reduces a fixed 4096-element slice, so the largest problem is bounded:
// max(ncornr*G, nangles*nbelem) <= UMT_NOALLOC_MAX_BLOCKS * 4096
// (= 134,217,728 elements, 1 MiB of scratch).  The blocks' partials are then
// summed in a fixed order by one block, so the result is deterministic.
// Nothing in the scratch has to start at zero: every partial slot the final
// sum reads, and the four result values, are written earlier in the same call.
#include "umt_common.cuh"
#include "../../include/umt103.h"

#include <mutex>

namespace umt {

constexpr int kNaThreads = 256;
constexpr int kNaPerThread = 16;
constexpr int kNaChunk = kNaThreads * kNaPerThread;     // elements per block

// File-scope scratch.  Host code must not pass `g_noalloc_scratch` itself to a
// kernel (on the host that symbol is only a stand-in, not a device address);
// the device address is looked up with cudaGetSymbolAddress on every call, for
// the device current at that call.  The lookup allocates nothing; repeating it
// means a primary context that another library reset and recreated (which
// reloads the module at a new address) is never served a stale pointer.
static __device__ __align__(256) double g_noalloc_scratch[4 * UMT_NOALLOC_MAX_BLOCKS + 8];

static std::mutex g_scratch_mutex;

static int scratch_for_current_device(double **out) {
  std::lock_guard<std::mutex> lk(g_scratch_mutex);
  void *p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p)
    return set_error(UMT_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
  *out = static_cast<double *>(p);
  return 0;
}

// Per block: the same four sums as k_energy (si.cu) over a fixed slice.
template <typename T>
__global__ void __launch_bounds__(kNaThreads) k_energy_partials(int nc, int nb, int A, int G, const int *cToZone,
                                                                const double *Volume, const double *siga,
                                                                const double *Phi, const double *A_bdy,
                                                                const int *bdyToC, const double *omega,
                                                                const double *weight, const T *psi, const T *psiB,
                                                                double *partials) {
  double v[4] = {0.0, 0.0, 0.0, 0.0};
  const size_t base = (size_t)blockIdx.x * kNaChunk;
  for (int k = 0; k < kNaPerThread; ++k) {
    const size_t i = base + (size_t)k * kNaThreads + threadIdx.x;
    if (i < (size_t)nc * G) {
      const int c = (int)(i / G), g = (int)(i - (size_t)c * G);
      const double vp = Volume[c] * Phi[i];
      v[0] += vp;
      if (siga) v[1] += vp * siga[(size_t)cToZone[c] * G + g];
    }
    if (i < (size_t)A * nb) {
      const int a = (int)(i / nb), b = (int)(i - (size_t)a * nb);
      const double *o = omega + 3 * a;
      const double d = o[0] * A_bdy[3 * b] + o[1] * A_bdy[3 * b + 1] + o[2] * A_bdy[3 * b + 2];
      double s = 0.0;
      if (d > 0.0) {
        const T *pp = psi + ((size_t)a * nc + bdyToC[b]) * G;
        for (int g = 0; g < G; ++g) s += (double)pp[g];
        v[2] += weight[a] * d * s;
      } else if (d < 0.0) {
        const T *pp = psiB + ((size_t)a * nb + b) * G;
        for (int g = 0; g < G; ++g) s += (double)pp[g];
        v[3] -= weight[a] * d * s;
      }
    }
  }
  __shared__ double sh[4][kNaThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    double x = v[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sh[k][w] = x;
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    double x = 0.0;
    for (int j = 0; j < kNaThreads / 32; ++j) x += sh[threadIdx.x][j];
    partials[4 * (size_t)blockIdx.x + threadIdx.x] = x;    // every block writes its slot
  }
}

// One block: sum the partials in a fixed order into out[0..3].
__global__ void k_energy_final(int nblocks, const double *partials, double *out) {
  __shared__ double sh[4][kNaThreads];
  for (int k = 0; k < 4; ++k) {
    double x = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += kNaThreads) x += partials[4 * (size_t)b + k];
    sh[k][threadIdx.x] = x;
  }
  __syncthreads();
  for (int s = kNaThreads / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s)
      for (int k = 0; k < 4; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x < 4) out[threadIdx.x] = sh[threadIdx.x][0];
}

}  // namespace umt

using namespace umt;

extern "C" int umt103_tally_noalloc(const double *siga_dev, double speed_light, int precision,
                                    UmtEnergyTally *tally) {
  Ctx &c = cur();
  if (!c.ready) return set_error(UMT_ERR_STATE, "umt103_init not called");
  if (c.rz) return set_error(UMT_ERR_STATE, "umt103_tally_noalloc: the context holds an RZ problem");
  if (!tally || !(speed_light > 0.0)) return set_error(UMT_ERR_ARG, "bad tally arguments");
  if (precision == UMT_FP64 && !c.psi64[0]) return set_error(UMT_ERR_STATE, "FP64 flux not allocated");
  if (precision == UMT_FP32 && !c.psi32[0]) return set_error(UMT_ERR_STATE, "FP32 flux not allocated");
  if (precision != UMT_FP64 && precision != UMT_FP32) return set_error(UMT_ERR_ARG, "precision");
  const size_t n = std::max((size_t)c.nc * c.G, (size_t)c.A * c.nb);
  const size_t nblocks = (n + kNaChunk - 1) / kNaChunk;
  if (nblocks > (size_t)UMT_NOALLOC_MAX_BLOCKS)
    return set_error(UMT_ERR_ARG,
                     "umt103_tally_noalloc: problem too large for the fixed scratch: max(ncornr*G, nangles*nbelem)"
                     " = %zu exceeds %lld elements; use umt103_tally",
                     n, (long long)UMT_NOALLOC_MAX_BLOCKS * kNaChunk);
  double *scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc) return rc;
  double *partials = scratch, *out = scratch + 4 * (size_t)UMT_NOALLOC_MAX_BLOCKS;
  if (precision == UMT_FP64)
    k_energy_partials<double><<<(unsigned)std::max<size_t>(nblocks, 1), kNaThreads, 0, c.stream>>>(
        c.nc, c.nb, c.A, c.G, c.cToZone, c.Volume, siga_dev, c.Phi, c.A_bdy, c.bdyToC, c.omega, c.weight,
        c.psi64[c.cur64], c.psiB64, partials);
  else
    k_energy_partials<float><<<(unsigned)std::max<size_t>(nblocks, 1), kNaThreads, 0, c.stream>>>(
        c.nc, c.nb, c.A, c.G, c.cToZone, c.Volume, siga_dev, c.Phi, c.A_bdy, c.bdyToC, c.omega, c.weight,
        c.psi32[c.cur32], c.psiB32, partials);
  k_energy_final<<<1, kNaThreads, 0, c.stream>>>((int)std::max<size_t>(nblocks, 1), partials, out);
  UMT_CUDA(cudaGetLastError());
  double h[4];
  UMT_CUDA(cudaMemcpyAsync(h, out, sizeof(h), cudaMemcpyDeviceToHost, c.stream));
  UMT_CUDA(cudaStreamSynchronize(c.stream));
  tally->EnergyRadiation = h[0] / speed_light;
  tally->PowerAbsorbed = h[1];
  tally->PowerEscape = h[2];
  tally->PowerIncident = h[3];
  tally->Balance = 0.0;
  return 0;
}
