// si.cu -- source iteration and energy tallies on the device.
//
// The outer loop restates rtmainsn/LinearSolver (rt/rtmainsn.F90:167-246,
// rt/LinearSolver.F90:10-124) for a problem with isotropic scattering: the
// sweep source is STotal = wtiso*(sigma_s*PhiTotal + q) (the role of
// GSet%STotal, mods/GroupSet_mod.F90:22, whose assembly lives in the
// material-coupling solver that the reference does not ship), the sweep is
// repeated until the relative L2 change of PhiTotal drops below the
// tolerance, and a final savePsi sweep stores the angular flux.  All
// reductions accumulate in FP64.
#include "umt_common.cuh"

namespace umt {

constexpr double WTISO = 0.079577471545947667884;   // 1/(4 pi), mods/Size_mod.F90:281

__global__ void k_build_source(int nc, int G, const int *cToZone, const double *sigs,
                               const double *q, const double *Phi, double *STotal) {
  const size_t n = (size_t)nc * G;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(i / G), g = (int)(i - (size_t)c * G);
    const size_t zg = (size_t)cToZone[c] * G + g;
    const double qq = q ? q[zg] : 0.0;
    STotal[i] = WTISO * (sigs[zg] * Phi[i] + qq);
  }
}

// block reduction of NV doubles into out[0..NV)
template <int NV>
__device__ void block_reduce_add(double (&v)[NV], double *out) {
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

// sum (phi - prev)^2, sum phi^2; then prev = phi
__global__ void k_change_norm(size_t n, const double *Phi, double *prev, double *out2) {
  double v[2] = {0.0, 0.0};
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double d = Phi[i] - prev[i];
    v[0] += d * d;
    v[1] += Phi[i] * Phi[i];
    prev[i] = Phi[i];
  }
  block_reduce_add<2>(v, out2);
}

// Energy edits (aux/rtedit.F90:139-160, control/BoundaryEdit.F90:83-122):
// out[0] = sum V*phi, out[1] = sum V*sigma_a*phi, out[2] = escape power
// sum_a w_a sum_{b: A_bdy.Omega>0} (A_bdy.Omega) sum_g psi_a(g, BdyToC(b)),
// out[3] = incident power from PsiB on faces with A_bdy.Omega<0.
template <typename T>
__global__ void k_energy(int nc, int nb, int A, int G, const int *cToZone, const double *Volume,
                         const double *siga, const double *Phi, const double *A_bdy, const int *bdyToC,
                         const double *omega, const double *weight, const T *psi, const T *psiB, double *out) {
  double v[4] = {0.0, 0.0, 0.0, 0.0};
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const size_t t0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  for (size_t i = t0; i < (size_t)nc * G; i += stride) {
    const int c = (int)(i / G), g = (int)(i - (size_t)c * G);
    const double vp = Volume[c] * Phi[i];
    v[0] += vp;
    if (siga) v[1] += vp * siga[(size_t)cToZone[c] * G + g];
  }
  for (size_t i = t0; i < (size_t)A * nb; i += stride) {
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
  block_reduce_add<4>(v, out);
}

int launch_build_source(Ctx &c, const double *q) {
  const size_t n = (size_t)c.nc * c.G;
  k_build_source<<<(int)std::min<size_t>((n + 255) / 256, 152 * 16), 256, 0, c.stream>>>(
      c.nc, c.G, c.cToZone, c.SigS, q, c.Phi, c.STotal);
  UMT_CUDA(cudaGetLastError());
  return 0;
}

int launch_change_norm(Ctx &c, double *prev, double *out2) {
  const size_t n = (size_t)c.nc * c.G;
  UMT_CUDA(cudaMemsetAsync(out2, 0, 2 * sizeof(double), c.stream));
  k_change_norm<<<152 * 4, 256, 0, c.stream>>>(n, c.Phi, prev, out2);
  UMT_CUDA(cudaGetLastError());
  return 0;
}

int launch_energy(Ctx &c, const double *siga_dev, int precision, double *out4) {
  UMT_CUDA(cudaMemsetAsync(out4, 0, 4 * sizeof(double), c.stream));
  if (precision == 0)
    k_energy<double><<<152 * 4, 256, 0, c.stream>>>(c.nc, c.nb, c.A, c.G, c.cToZone, c.Volume, siga_dev, c.Phi,
                                                   c.A_bdy, c.bdyToC, c.omega, c.weight, c.psi64[c.cur64],
                                                   c.psiB64, out4);
  else
    k_energy<float><<<152 * 4, 256, 0, c.stream>>>(c.nc, c.nb, c.A, c.G, c.cToZone, c.Volume, siga_dev, c.Phi,
                                                  c.A_bdy, c.bdyToC, c.omega, c.weight, c.psi32[c.cur32],
                                                  c.psiB32, out4);
  UMT_CUDA(cudaGetLastError());
  return 0;
}

}  // namespace umt
