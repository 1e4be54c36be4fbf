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

#include <algorithm>
#include <cmath>

namespace umt {

constexpr double WTISO = 0.079577471545947667884;   // 1/(4 pi), mods/Size_mod.F90:281
#define TRY_SI(x) do { int rc_ = (x); if (rc_) return rc_; } while (0)

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

// Amplification weight of a zone and group: the infinite-medium factor
// 1/(1 - c), c = sigma_s/sigma_t, by which source iteration's residual
// understates its error where scattering dominates (capped at 1e3).
__device__ __forceinline__ double amp_weight(const double *Sigt, const double *SigS, size_t zg) {
  return 1.0 / fmax(1.0 - SigS[zg] / Sigt[zg], 1.0e-3);
}

// sum (phi - prev)^2, sum phi^2, and (with weights) sum (w (phi - prev))^2
// into out[0], out[1], out[2]; then prev = phi.  With delta given, the change
// is kept too (deltaPrev, if given, receives the change before it).
__global__ void k_change_norm(size_t n, int G, const double *Phi, double *prev, double *out, double *delta,
                              double *deltaPrev, const int *cToZone, const double *Sigt, const double *SigS) {
  double v[3] = {0.0, 0.0, 0.0};
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double d = Phi[i] - prev[i];
    v[0] += d * d;
    v[1] += Phi[i] * Phi[i];
    if (cToZone) {
      const int c = (int)(i / G), g = (int)(i - (size_t)c * G);
      const double wd = amp_weight(Sigt, SigS, (size_t)cToZone[c] * G + g) * d;
      v[2] += wd * wd;
    }
    prev[i] = Phi[i];
    if (delta) {
      if (deltaPrev) deltaPrev[i] = delta[i];
      delta[i] = d;
    }
  }
  block_reduce_add<3>(v, out);
}

// STotal = wtiso (sigma_s vec + q)
__global__ void k_build_source_vec(int nc, int G, const int *cToZone, const double *sigs, const double *q,
                                   const double *vec, double *STotal) {
  const size_t n = (size_t)nc * G;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(i / G), g = (int)(i - (size_t)c * G);
    const size_t zg = (size_t)cToZone[c] * G + g;
    STotal[i] = WTISO * (sigs[zg] * vec[i] + (q ? q[zg] : 0.0));
  }
}

// R = Phi - X; out2 += {|R|^2, |Phi|^2}
__global__ void k_residual(size_t n, const double *Phi, const double *X, double *R, double *out2) {
  double v[2] = {0.0, 0.0};
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double r = Phi[i] - X[i];
    R[i] = r;
    v[0] += r * r;
    v[1] += Phi[i] * Phi[i];
  }
  block_reduce_add<2>(v, out2);
}

// One step of the correction iteration D <- K D + R (Phi = K D from the
// homogeneous sweep): d = (Phi + R) - D, D = Phi + R, the change history
// shifted; out += {|d|^2, |D|^2, |w d|^2} (w: amp_weight)
__global__ void k_inner_update(size_t n, int G, const double *Phi, const double *R, double *D, double *delta,
                               double *deltaPrev, const int *cToZone, const double *Sigt, const double *SigS,
                               double *out) {
  double v[3] = {0.0, 0.0, 0.0};
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double dn = Phi[i] + R[i];
    const double d = dn - D[i];
    D[i] = dn;
    deltaPrev[i] = delta[i];
    delta[i] = d;
    const int c = (int)(i / G), g = (int)(i - (size_t)c * G);
    const double wd = amp_weight(Sigt, SigS, (size_t)cToZone[c] * G + g) * d;
    v[0] += d * d;
    v[1] += dn * dn;
    v[2] += wd * wd;
  }
  block_reduce_add<3>(v, out);
}

// sum (phi - ref)^2, sum ref^2
__global__ void k_distance(size_t n, const double *Phi, const double *ref, double *out2) {
  double v[2] = {0.0, 0.0};
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double d = Phi[i] - ref[i];
    v[0] += d * d;
    v[1] += ref[i] * ref[i];
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

// ---------------------------------------------------------------------------
// Grey transport acceleration (GTA).  After a multigroup sweep the change of
// the scalar flux leaves a scattering residual R = sum_g sigma_s,g (phi_g -
// phi_g_prev) (getCollisionRate, rt/getCollisionRate.F90:64-87).  The error it
// drives is estimated by one grey S2 transport problem on the same mesh,
//   Omega.grad(psi) + sigma_t,grey psi = (sigma_s,grey phi + R) / (4 pi),
// solved by BiCGStab on (I - K) eps = K0 R with K = one grey sweep of the
// scattering source (rt/GTASolver.F90:219-402), and added back as
// phi_g += chi_g eps (rt/addGreyCorrections.F90:85).  Grey cross sections are
// spectrum-weighted harmonic means (setGTAOpacity, rt/setGTAOpacity.F90:
// 176-205, with no material coupling).  The spectrum chi that the
// reference takes from its (absent) material-coupling solver is defined here
// per zone as the shape of the current residual, |sigma_s,g dphi_g| summed
// over the zone's corners and normalised.
// ---------------------------------------------------------------------------
__global__ void k_gta_spectrum(int nz, int G, double tau, int mode, const int *numCorner, const int *cOffSet,
                               const double *Volume, const double *Sigt, const double *SigS, const double *Phi,
                               const double *Prev, double *chi, double *greySigt, double *greySigs) {
  for (int z = blockIdx.x * blockDim.x + threadIdx.x; z < nz; z += gridDim.x * blockDim.x) {
    const int c0 = cOffSet[z], nC = numCorner[z];
    double rsum = 0.0;
    for (int g = 0; g < G; ++g) {
      double r = 0.0;
      for (int k = 0; k < nC; ++k) {
        const size_t e = (size_t)(c0 + k) * G + g;
        r += Volume[c0 + k] * fabs(SigS[(size_t)z * G + g] * (Phi[e] - Prev[e]));
      }
      // mode 1: weight by the infinite-medium amplification 1/(1-c) of the
      // group's residual, which favours the slowly converging groups
      if (mode == 1) r /= fmax(1.0 - SigS[(size_t)z * G + g] / Sigt[(size_t)z * G + g], 1.0e-6);
      chi[(size_t)z * G + g] = r;
      rsum += r;
    }
    double inv = 0.0, inv2 = 0.0, aav = 0.0;
    for (int g = 0; g < G; ++g) {
      const double x = rsum > 0.0 ? chi[(size_t)z * G + g] / rsum : 1.0 / G;
      const double st = Sigt[(size_t)z * G + g];
      const double si = 1.0 / st;
      const double sa = st - SigS[(size_t)z * G + g] - tau;
      inv += x * si;
      inv2 += x * si * si;
      aav += x * sa * si;
      chi[(size_t)z * G + g] = x * si;
    }
    double gt, gs;
    if (inv > 0.0) {
      for (int g = 0; g < G; ++g) chi[(size_t)z * G + g] /= inv;
      gt = inv / inv2;
      const double ga = tau + aav / inv;
      gs = gt - ga;
      if (gs / gt <= 1.0e-10) { gs = 0.0; gt = ga; }
    } else {
      gt = tau > 0.0 ? tau : 1.0;
      gs = 0.0;
    }
    greySigt[z] = gt;
    greySigs[z] = gs;
  }
}

// R(c) = sum_g sigma_s,g (phi_g - prev_g)
__global__ void k_gta_residual(int nc, int G, const int *cToZone, const double *SigS, const double *Phi,
                               const double *Prev, double *R) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
    const int z = cToZone[c];
    double s = 0.0;
    for (int g = 0; g < G; ++g) {
      const size_t e = (size_t)c * G + g;
      s += SigS[(size_t)z * G + g] * (Phi[e] - Prev[e]);
    }
    R[c] = s;
  }
}

// grey source: STotal(c) = wtiso (sigma_s,grey x(c) + wR R(c))
__global__ void k_gta_source(int nc, const int *cToZone, const double *greySigs, const double *x, const double *R,
                             double wR, double *STotal) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
    const double sx = x ? greySigs[cToZone[c]] * x[c] : 0.0;
    STotal[c] = WTISO * (sx + wR * R[c]);
  }
}

// y = a*x + b*y + c*z (any pointer may alias y; z may be null)
__global__ void k_axpbypcz(int n, double a, const double *x, double b, double *y, double c, const double *z) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double v = a * x[i];
    if (b != 0.0) v += b * y[i];
    if (z) v += c * z[i];
    y[i] = v;
  }
}

__global__ void k_dot2(int n, const double *x, const double *y, const double *u, const double *w, double *out2) {
  double v[2] = {0.0, 0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    v[0] += x[i] * y[i];
    if (u) v[1] += u[i] * w[i];
  }
  block_reduce_add<2>(v, out2);
}

// phi_g(c) += chi_g(zone) eps(c)
__global__ void k_gta_correct(int nc, int G, const int *cToZone, const double *chi, const double *eps, double *Phi) {
  const size_t n = (size_t)nc * G;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(i / G), g = (int)(i - (size_t)c * G);
    Phi[i] += chi[(size_t)cToZone[c] * G + g] * eps[c];
  }
}

// Stretched-TSA opacities of each zone (rt/setGTAOpacity.F90:225-232):
// eps = 1/sqrt(1 - sigma_s/sigma_t) of the grey problem and the stretched
// total opacity sigma_t/eps, for which the stretched problem's scattering
// term vanishes.  sigt1 keeps sigma_t for the restore after a stretched sweep.
__global__ void k_gta_stretch(int nz, const double *greySigt, const double *greySigs, double *eps, double *sigt1,
                              double *sigt2) {
  for (int z = blockIdx.x * blockDim.x + threadIdx.x; z < nz; z += gridDim.x * blockDim.x) {
    const double gt = greySigt[z];
    const double e = 1.0 / sqrt(1.0 - greySigs[z] / gt);
    eps[z] = e;
    sigt1[z] = gt;
    sigt2[z] = gt / e;
  }
}

// Stretched-TSA sweep source (snac/GTASweep.F90, GTA%ID = 2):
// STotal = wtiso sigma_s eps (P - Pold)
__global__ void k_gta_source2(int nc, const int *cToZone, const double *greySigs, const double *eps, const double *P,
                              const double *Pold, double *STotal) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
    const int z = cToZone[c];
    STotal[c] = WTISO * greySigs[z] * eps[z] * (P[c] - (Pold ? Pold[c] : 0.0));
  }
}

// Zone radiation energy density sum_c V_c sum_g phi_c,g / V_z (rt/GTASolver.F90
// ZoneLoop) and pzOld = 0.
__global__ void k_gta_zone_energy(int nz, int G, const int *numCorner, const int *cOffSet, const double *Volume,
                                  const double *VolumeZone, const double *Phi, double *radE, double *pzOld) {
  for (int z = blockIdx.x * blockDim.x + threadIdx.x; z < nz; z += gridDim.x * blockDim.x) {
    const int c0 = cOffSet[z], nC = numCorner[z];
    double e = 0.0;
    for (int k = 0; k < nC; ++k) {
      double s = 0.0;
      for (int g = 0; g < G; ++g) s += Phi[(size_t)(c0 + k) * G + g];
      e += Volume[c0 + k] * s;
    }
    radE[z] = e / VolumeZone[z];
    pzOld[z] = 0.0;
  }
}

// Convergence of the zone-averaged grey correction (rt/GTASolver.F90
// CorrectionZoneLoop): out[0] += V_z (pz - pzOld)^2, out[1] += V_z (radE +
// pz)^2, out[2] = max |pz - pzOld| / |radE + pz| (bit pattern of a
// non-negative double, so an integer max orders it); pzOld = pz.
__global__ void k_gta_converge(int nz, const int *numCorner, const int *cOffSet, const double *Volume,
                               const double *VolumeZone, const double *x, const double *radE, double *pzOld,
                               double *out) {
  double v[2] = {0.0, 0.0};
  double mx = 0.0;
  for (int z = blockIdx.x * blockDim.x + threadIdx.x; z < nz; z += gridDim.x * blockDim.x) {
    const int c0 = cOffSet[z], nC = numCorner[z];
    double pz = 0.0;
    for (int k = 0; k < nC; ++k) pz += Volume[c0 + k] * x[c0 + k];
    pz /= VolumeZone[z];
    const double err = pz - pzOld[z];
    const double phiNew = radE[z] + pz;
    v[0] += VolumeZone[z] * err * err;
    v[1] += VolumeZone[z] * phiNew * phiNew;
    if (phiNew != 0.0) mx = fmax(mx, fabs(err / phiNew));
    pzOld[z] = pz;
  }
  block_reduce_add<2>(v, out);
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<unsigned long long *>(out + 2), (unsigned long long)__double_as_longlong(mx));
}

// Inner products weighted by sigma_s,grey V (rt/scat_prod.F90, scat_prod1.F90):
// out[0] += sum x y s, out[1] += sum u w s with s = sigma_s,grey(zone) V_c;
// a null y or w stands for 1 (scat_prod1), a null u skips the second sum.
__global__ void k_sdot2(int nc, const int *cToZone, const double *greySigs, const double *Volume, const double *x,
                        const double *y, const double *u, const double *w, double *out2) {
  double v[2] = {0.0, 0.0};
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
    const double s = greySigs[cToZone[c]] * Volume[c];
    v[0] += x[c] * (y ? y[c] : 1.0) * s;
    if (u) v[1] += u[c] * (w ? w[c] : 1.0) * s;
  }
  block_reduce_add<2>(v, out2);
}

// ---------------------------------------------------------------------------
// The newer grey solver (Size%useNewGTASolver; driver option gta_kernel = 2):
// the stretched-TSA sweep is replaced by a direct solve, per zone, of the
// zone-local scattering.
//
// k_gta_tt restates snac/InitSweepGreyUCBxyz.F90:10-253: for every grey
// direction, the matrix Pvv[c][cc] = d psi(c) / d TsaSource(cc) of the zone's
// corner solve (volume source, EZ closure, corner order by least need) is
// formed and TT = sum_a w_a Pvv is kept; then A = I - TT diag(wtiso sigma_s)
// is factored in place as snac/UpdateScalarIntensity.F90's
// ScalarIntensityDecompose does (unit lower L, upper U, the same loop order).
// Storage per corner row: tt[(c0+c)*8 + cc] = TT(cc, c0+c) of the reference,
// lu[(c0+row)*8 + col] = its factored TT(col, c0+row).
//
// The reference's sweep also accumulates PhiInc, the part of the scalar flux
// carried in by upwind flux (SweepGreyUCBxyzKernelNew's pInc).  The sweep is
// linear, so PhiInc = tPhi - TT TsaSource exactly: k_gta_zone_solve takes
// the library's ordinary grey sweep and subtracts the zone-local part.  With
// TsaSource = wtiso (sigma_s P + [R]), the right-hand side of either call of
// ScalarIntensityDecompose (PhiInc, plus TT wtiso R when the source is on)
// is tPhi - TT wtiso sigma_s P.
// ---------------------------------------------------------------------------
__global__ void k_gta_tt(int nz, int nc, int A, const int *numCorner, const int *cOffSet, const int *nCFaces,
                         const int *cEZ, const double *Volume, const double *afp, const double *aez,
                         const double *weight, const double *greySigt, const double *greySigs, double *tt,
                         double *lu) {
  for (int z = blockIdx.x * blockDim.x + threadIdx.x; z < nz; z += gridDim.x * blockDim.x) {
    const int c0 = cOffSet[z], nC = numCorner[z];
    const double sig = greySigt[z];
    double T[8][8];                                // T[cc][c] = TT(cc, c0+c)
    for (int a = 0; a < 8; ++a)
      for (int b = 0; b < 8; ++b) T[a][b] = 0.0;
    for (int ang = 0; ang < A; ++ang) {
      const double w = weight[ang];
      double P[8][8];                              // P[col][row] = Pvv(col, row)
      double denom[8], coefpsi[8][3];
      int need[8], nxez[8], ezx[8][3];
      for (int a = 0; a < 8; ++a) {
        need[a] = 0; nxez[a] = 0; denom[a] = 0.0;
        for (int b = 0; b < 8; ++b) P[a][b] = 0.0;
      }
      for (int c = 0; c < nC; ++c) P[c][c] = Volume[c0 + c];
      for (int c = 0; c < nC; ++c) {
        const size_t cc = (size_t)ang * nc + c0 + c;
        const double sigv = Volume[c0 + c] * sig;
        denom[c] = sigv;
        const int ncf = nCFaces[c0 + c];
        double af[3];
        for (int f = 0; f < ncf; ++f) {
          af[f] = afp[cc * UMT_MAXCF + f];
          if (af[f] > 0.0) denom[c] += af[f];
        }
        for (int f = 0; f < ncf; ++f) {
          const double ae = aez[cc * UMT_MAXCF + f];
          const int cez = cEZ[(size_t)(c0 + c) * UMT_MAXCF + f];
          if (cez > c) {
            if (ae > 0.0) {
              need[cez] += 1;
              ezx[c][nxez[c]] = cez; coefpsi[c][nxez[c]] = ae; nxez[c] += 1;
            } else if (ae < 0.0) {
              need[c] += 1;
              ezx[cez][nxez[cez]] = c; coefpsi[cez][nxez[cez]] = -ae; nxez[cez] += 1;
            }
          }
          if (ae > 0.0) {
            denom[c] += ae;
            double area_opp = 0.0;
            if (ncf == 3) {
              const int ifp = (f + 1) % ncf;
              if (af[ifp] < 0.0) area_opp = -af[ifp];
            } else {
              int ifp = f;
              for (int k = 0; k < ncf - 2; ++k) {
                ifp = (ifp + 1) % ncf;
                if (af[ifp] < 0.0) area_opp -= af[ifp];
              }
            }
            double B1, B2;
            if (area_opp > 0.0) {
              const double sigv2 = sigv * sigv;
              const double gnum = ae * ae * (1.82 * sigv2 + ae * (4.0 * sigv + 3.0 * ae));
              const double gtau = gnum / (gnum + 4.0 * sigv2 * sigv2 + ae * sigv * (6.0 * sigv2 + 2.0 * ae * (2.0 * sigv + ae)));
              const double B0 = 0.5 * ae * (1.0 - gtau);
              B1 = (B0 - gtau * sigv) / sig;
              B2 = B0 / sig;
            } else {
              B1 = 0.5 * ae / sig;
              B2 = 0.5 * ae / sig;
            }
            P[c][c] += B1;
            P[cez][c] -= B2;
            P[c][cez] -= B1;
            P[cez][cez] += B2;
          }
        }
      }
      for (int i = 0; i < nC; ++i) {
        int c = 0;                                 // minloc: first index of the least need
        for (int k = 1; k < nC; ++k) if (need[k] < need[c]) c = k;
        const double dInv = 1.0 / denom[c];
        for (int c1 = 0; c1 < nC; ++c1) P[c1][c] *= dInv;
        for (int f = 0; f < nxez[c]; ++f) {
          const int cez = ezx[c][f];
          const double coef = coefpsi[c][f];
          need[cez] -= 1;
          for (int c1 = 0; c1 < nC; ++c1) P[c1][cez] += coef * P[c1][c];
        }
        need[c] = 99;
      }
      for (int c1 = 0; c1 < nC; ++c1)
        for (int c = 0; c < nC; ++c) T[c][c1] += w * P[c][c1];
    }
    for (int c = 0; c < nC; ++c)
      for (int cc = 0; cc < 8; ++cc) tt[(size_t)(c0 + c) * 8 + cc] = cc < nC ? T[cc][c] : 0.0;
    // A = I - TT diag(wtiso sigma_s), factored in place
    const double ws = WTISO * greySigs[z];
    for (int cc = 0; cc < nC; ++cc)
      for (int c = 0; c < nC; ++c) T[cc][c] = -ws * T[cc][c];
    for (int c = 0; c < nC; ++c) T[c][c] = 1.0 + T[c][c];
    for (int i = 0; i < nC; ++i) {
      double t = 0.0;
      for (int k = 0; k < i; ++k) t += T[k][i] * T[i][k];
      T[i][i] -= t;
      const double diagInv = 1.0 / T[i][i];
      for (int j = i + 1; j < nC; ++j) {
        double t2 = 0.0, v = 0.0;
        for (int k = 0; k < i; ++k) {
          t2 += T[k][i] * T[j][k];
          v += T[k][j] * T[i][k];
        }
        T[j][i] -= t2;
        T[i][j] = diagInv * (T[i][j] - v);
      }
    }
    for (int row = 0; row < nC; ++row)
      for (int col = 0; col < 8; ++col) lu[(size_t)(c0 + row) * 8 + col] = col < nC ? T[col][row] : 0.0;
  }
}

// out = A^-1 (tPhi - TT wtiso sigma_s P) per zone (ScalarIntensitySolve:
// L y = S, then U x = y); P may be null (zero).
__global__ void k_gta_zone_solve(int nz, const int *numCorner, const int *cOffSet, const double *greySigs,
                                 const double *tt, const double *lu, const double *tPhi, const double *P,
                                 double *out) {
  for (int z = blockIdx.x * blockDim.x + threadIdx.x; z < nz; z += gridDim.x * blockDim.x) {
    const int c0 = cOffSet[z], nC = numCorner[z];
    const double ws = WTISO * greySigs[z];
    double x[8];
    for (int c = 0; c < nC; ++c) {
      double r = tPhi[c0 + c];
      if (P)
        for (int cc = 0; cc < nC; ++cc) r -= tt[(size_t)(c0 + c) * 8 + cc] * ws * P[c0 + cc];
      x[c] = r;
    }
    for (int j = 1; j < nC; ++j) {
      double t = 0.0;
      for (int i = 0; i < j; ++i) t -= lu[(size_t)(c0 + j) * 8 + i] * x[i];
      x[j] += t;
    }
    x[nC - 1] /= lu[(size_t)(c0 + nC - 1) * 8 + nC - 1];
    for (int k = nC - 2; k >= 0; --k) {
      double t = 0.0;
      for (int i = k + 1; i < nC; ++i) t += x[i] * lu[(size_t)(c0 + k) * 8 + i];
      x[k] = (x[k] - t) / lu[(size_t)(c0 + k) * 8 + k];
    }
    for (int c = 0; c < nC; ++c) out[c0 + c] = x[c];
  }
}

// Grey problem of this iterate: spectrum and grey opacities (k_gta_spectrum),
// the stretched-TSA opacities, the grey source R = sum_g sigma_s,g (phi_g -
// phi_g_prev) in slot 7 of the vectors, the zone radiation energy.
int gta_prepare(Ctx &c) {
  Ctx &q = *c.gta;
  const int B = 152 * 4;
  double *Z = c.gtaZ;                              // [5][nz]: eps, sigt1, sigt2, radE, pzOld
  k_gta_spectrum<<<(c.nz + 127) / 128, 128, 0, c.stream>>>(c.nz, c.G, c.tau, c.gtaSpectrum, c.numCorner, c.cOffSet, c.Volume,
                                                          c.Sigt, c.SigS, c.Phi, c.PhiPrev, c.gtaChi, q.Sigt,
                                                          c.gtaSigS);
  k_gta_stretch<<<(c.nz + 127) / 128, 128, 0, c.stream>>>(c.nz, q.Sigt, c.gtaSigS, Z, Z + c.nz, Z + 2 * (size_t)c.nz);
  UMT_CUDA(cudaMemcpyAsync(q.SigS, c.gtaSigS, c.nz * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
  k_gta_residual<<<B, 256, 0, c.stream>>>(c.nc, c.G, c.cToZone, c.SigS, c.Phi, c.PhiPrev, c.gtaVec + 7 * (size_t)c.nc);
  k_gta_zone_energy<<<(c.nz + 127) / 128, 128, 0, c.stream>>>(c.nz, c.G, c.numCorner, c.cOffSet, c.Volume,
                                                              c.VolumeZone, c.Phi, Z + 3 * (size_t)c.nz,
                                                              Z + 4 * (size_t)c.nz);
  UMT_CUDA(cudaGetLastError());
  return 0;
}

// out = M P: the grey operator of rt/GreySweep.F90 (GreySweep): one grey S2
// sweep of wtiso (sigma_s P + [R]) with sigma_t, then the stretched-TSA sweep
// of wtiso sigma_s eps (P1 - P) with sigma_t/eps, added to it.  P may be null
// (zero); out must not alias P.  Two grey sweeps.
int gta_op(Ctx &c, const double *P, double *out, bool withSource) {
  Ctx &q = *c.gta;
  double *Z = c.gtaZ;
  const size_t n = (size_t)c.nc;
  k_gta_source<<<152 * 4, 256, 0, c.stream>>>(c.nc, c.cToZone, c.gtaSigS, P, c.gtaVec + 7 * n,
                                              withSource ? 1.0 : 0.0, q.STotal);
  UMT_CUDA(cudaGetLastError());
  UMT_CUDA(cudaStreamSynchronize(c.stream));
  TRY_SI(launch_sweep_once(q, 0, true));
  UMT_CUDA(cudaMemcpyAsync(out, q.Phi, n * 8, cudaMemcpyDeviceToDevice, q.stream));
  k_gta_source2<<<152 * 4, 256, 0, q.stream>>>(c.nc, c.cToZone, c.gtaSigS, Z, out, P, q.STotal);
  UMT_CUDA(cudaMemcpyAsync(q.Sigt, Z + 2 * (size_t)c.nz, c.nz * 8, cudaMemcpyDeviceToDevice, q.stream));
  TRY_SI(launch_sweep_once(q, 0, true));
  UMT_CUDA(cudaMemcpyAsync(q.Sigt, Z + c.nz, c.nz * 8, cudaMemcpyDeviceToDevice, q.stream));
  k_axpbypcz<<<152 * 4, 256, 0, q.stream>>>(c.nc, 1.0, q.Phi, 1.0, out, 0.0, nullptr);
  UMT_CUDA(cudaGetLastError());
  UMT_CUDA(cudaStreamSynchronize(q.stream));
  return 0;
}

// The newer solver's transfer matrices and their factors for this iterate's
// grey opacities (after gta_prepare).
int gta_prepare_zone(Ctx &c) {
  Ctx &q = *c.gta;
  k_gta_tt<<<(c.nz + 63) / 64, 64, 0, c.stream>>>(c.nz, c.nc, q.A, c.numCorner, c.cOffSet, c.nCFaces, c.cEZ,
                                                  c.Volume, q.afp64, q.aez64, q.weight, q.Sigt, c.gtaSigS,
                                                  c.gtaTT, c.gtaLU);
  UMT_CUDA(cudaGetLastError());
  return 0;
}

// out = M P of the newer solver (rt/GreySweep.F90 GreySweepNEW): one grey S2
// sweep of wtiso (sigma_s P + [R]), then the per-zone solve.  One grey sweep.
int gta_op_zone(Ctx &c, const double *P, double *out, bool withSource) {
  Ctx &q = *c.gta;
  k_gta_source<<<152 * 4, 256, 0, c.stream>>>(c.nc, c.cToZone, c.gtaSigS, P, c.gtaVec + 7 * (size_t)c.nc,
                                              withSource ? 1.0 : 0.0, q.STotal);
  UMT_CUDA(cudaGetLastError());
  UMT_CUDA(cudaStreamSynchronize(c.stream));
  TRY_SI(launch_sweep_once(q, 0, true));
  k_gta_zone_solve<<<(c.nz + 127) / 128, 128, 0, q.stream>>>(c.nz, c.numCorner, c.cOffSet, c.gtaSigS, c.gtaTT,
                                                              c.gtaLU, q.Phi, P, out);
  UMT_CUDA(cudaGetLastError());
  UMT_CUDA(cudaStreamSynchronize(q.stream));
  return 0;
}

int gta_sdot2(Ctx &c, const double *x, const double *y, const double *u, const double *w, double *h2) {
  UMT_CUDA(cudaMemsetAsync(c.red + 4, 0, 2 * sizeof(double), c.stream));
  k_sdot2<<<152 * 4, 256, 0, c.stream>>>(c.nc, c.cToZone, c.gtaSigS, c.Volume, x, y, u, w, c.red + 4);
  UMT_CUDA(cudaMemcpyAsync(h2, c.red + 4, 2 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  UMT_CUDA(cudaStreamSynchronize(c.stream));
  return 0;
}

// relative change of the zone-averaged correction: max(pointwise, L2)
int gta_converge(Ctx &c, const double *x, double *rel) {
  double *Z = c.gtaZ;
  UMT_CUDA(cudaMemsetAsync(c.red + 10, 0, 3 * sizeof(double), c.stream));
  k_gta_converge<<<(c.nz + 255) / 256, 256, 0, c.stream>>>(c.nz, c.numCorner, c.cOffSet, c.Volume, c.VolumeZone, x,
                                                           Z + 3 * (size_t)c.nz, Z + 4 * (size_t)c.nz, c.red + 10);
  double h[3];
  UMT_CUDA(cudaMemcpyAsync(h, c.red + 10, 3 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  UMT_CUDA(cudaStreamSynchronize(c.stream));
  const double l2 = h[1] != 0.0 ? std::sqrt(std::fabs(h[0] / h[1])) : 0.0;
  *rel = std::max(h[2], l2);
  return 0;
}

int gta_axpbypcz(Ctx &c, int n, double a, const double *x, double b, double *y, double cc, const double *z) {
  k_axpbypcz<<<152 * 4, 256, 0, c.stream>>>(n, a, x, b, y, cc, z);
  UMT_CUDA(cudaGetLastError());
  return 0;
}

int gta_dot2(Ctx &c, int n, const double *x, const double *y, const double *u, const double *w, double *h2) {
  UMT_CUDA(cudaMemsetAsync(c.red + 4, 0, 2 * sizeof(double), c.stream));
  k_dot2<<<152 * 4, 256, 0, c.stream>>>(n, x, y, u, w, c.red + 4);
  UMT_CUDA(cudaMemcpyAsync(h2, c.red + 4, 2 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  UMT_CUDA(cudaStreamSynchronize(c.stream));
  return 0;
}

int gta_correct(Ctx &c, const double *eps) {
  const size_t n = (size_t)c.nc * c.G;
  k_gta_correct<<<(int)std::min<size_t>((n + 255) / 256, 152 * 16), 256, 0, c.stream>>>(c.nc, c.G, c.cToZone,
                                                                                       c.gtaChi, eps, c.Phi);
  UMT_CUDA(cudaGetLastError());
  return 0;
}

int launch_build_source(Ctx &c, const double *q) {
  const size_t n = (size_t)c.nc * c.G;
  k_build_source<<<(int)std::min<size_t>((n + 255) / 256, 152 * 16), 256, 0, c.stream>>>(
      c.nc, c.G, c.cToZone, c.SigS, q, c.Phi, c.STotal);
  UMT_CUDA(cudaGetLastError());
  return 0;
}

int launch_change_norm(Ctx &c, double *prev, double *out3, double *delta, double *deltaPrev, bool weighted) {
  const size_t n = (size_t)c.nc * c.G;
  UMT_CUDA(cudaMemsetAsync(out3, 0, 3 * sizeof(double), c.stream));
  k_change_norm<<<152 * 4, 256, 0, c.stream>>>(n, c.G, c.Phi, prev, out3, delta, deltaPrev,
                                               weighted ? c.cToZone : nullptr, c.Sigt, c.SigS);
  UMT_CUDA(cudaGetLastError());
  return 0;
}

int launch_distance(Ctx &c, const double *ref, double *out2, const double *x) {
  UMT_CUDA(cudaMemsetAsync(out2, 0, 2 * sizeof(double), c.stream));
  k_distance<<<152 * 4, 256, 0, c.stream>>>((size_t)c.nc * c.G, x ? x : c.Phi, ref, out2);
  UMT_CUDA(cudaGetLastError());
  return 0;
}

int launch_build_source_vec(Ctx &c, const double *vec, const double *q) {
  const size_t n = (size_t)c.nc * c.G;
  k_build_source_vec<<<(int)std::min<size_t>((n + 255) / 256, 152 * 16), 256, 0, c.stream>>>(
      c.nc, c.G, c.cToZone, c.SigS, q, vec, c.STotal);
  UMT_CUDA(cudaGetLastError());
  return 0;
}

int launch_residual(Ctx &c, const double *X, double *R, double *out2) {
  UMT_CUDA(cudaMemsetAsync(out2, 0, 2 * sizeof(double), c.stream));
  k_residual<<<152 * 4, 256, 0, c.stream>>>((size_t)c.nc * c.G, c.Phi, X, R, out2);
  UMT_CUDA(cudaGetLastError());
  return 0;
}

int launch_inner_update(Ctx &c, const double *R, double *D, double *delta, double *deltaPrev, double *out3) {
  UMT_CUDA(cudaMemsetAsync(out3, 0, 3 * sizeof(double), c.stream));
  k_inner_update<<<152 * 4, 256, 0, c.stream>>>((size_t)c.nc * c.G, c.G, c.Phi, R, D, delta, deltaPrev, c.cToZone,
                                                c.Sigt, c.SigS, out3);
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
