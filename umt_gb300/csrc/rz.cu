// rz.cu -- the 2-D cylindrical (RZ) UCB sweep, FP64.
//
// Arithmetic of snac/SweepUCBrz.F90:87-276 (R-weighted face terms, the
// angular-derivative term with the half-angle intensity PsiM) and the RZ part
// of snac/SetSweep.F90: the directions of one xi-level are swept in
// quadrature order, each starting from the PsiM the previous one left;
// finishing directions are not swept and receive PsiM.
//
// The corner-face vectors are 2-vectors; they are stored as 3-vectors with a
// zero third component, so the device schedule of the 3-D path (face-sign
// dependencies, corner order, hyperplane levels) orders every RZ direction
// unchanged.  Stages: item (direction a, zone z) waits for its upwind zones
// in direction a and for zone z in the level's previous swept direction (the
// only reader of the PsiM that one leaves), so a level's directions follow one
// another as wavefronts one stage apart and the levels run concurrently.  One
// kernel launch per stage; a team of GT lanes per item, lanes over groups, as
// in the FP64 kernel of sweep.cu.
#include "umt_common.cuh"
#include "sweep32_util.cuh"
#include "../../include/umt103.h"

#include <algorithm>
#include <cmath>

#define TRY_RC(x) do { int rc_ = (x); if (rc_) return rc_; } while (0)

namespace umt {

int init_context(Ctx &c, const UmtMesh *m, const UmtQuad *q, int ngr, int flags);
void release_current_context();

struct RZData {
  double *Area = nullptr, *RadiusFP = nullptr, *RadiusEZ = nullptr;   // [nc], [nc*2]
  double *angDerivFac = nullptr, *W1 = nullptr, *W2 = nullptr;        // [A]
  int *starting = nullptr, *nextFinishing = nullptr, *level = nullptr; // [A]
  int *cFP2 = nullptr, *cEZ2 = nullptr;                              // [nc*2], 0-based
  double *PsiM = nullptr;                                            // [nLevels][nc][G]
  uint32_t *items = nullptr;                                         // stage order, a*nz + z
  int nLevels = 0, nStages = 0, maxStageItems = 0, maxC = 0;
  std::vector<int> hCount, hOffset;
  std::vector<double> hArea, hVolume, hRfp, hRez;
  // FP32 path (init flag bit 1)
  float4 *recA = nullptr, *recB = nullptr;   // [A][nc] per (direction, corner), see k_rz_prep32
  float4 *corner32 = nullptr;                // [nc] {Volume, RadiusEZ0*Area, RadiusEZ1*Area, Area}
  int2 *link32 = nullptr;                    // [nc] {cFP0 << 3 | cEZ0, cFP1 << 3 | cEZ1}
  float *fac32 = nullptr, *W1_32 = nullptr, *W2_32 = nullptr;   // [A]
  float *PsiM32 = nullptr;                   // [nLevels][nc][G]
  int *bFace2 = nullptr;                     // [nb] corner face 2*c + f of each boundary element (-1: none)
  cudaGraphExec_t graph32[2] = {nullptr, nullptr};   // one FP32 sweep per buffer parity
  double graphTau = 0.0;
};

static void destroy_rz_graphs(RZData &r) {
  for (auto &g : r.graph32)
    if (g) { cudaGraphExecDestroy(g); g = nullptr; }
}

void free_rz(Ctx &c) {
  RZData *r = c.rz;
  if (!r) return;
  destroy_rz_graphs(*r);
  for (void *p : {(void *)r->Area, (void *)r->RadiusFP, (void *)r->RadiusEZ, (void *)r->angDerivFac, (void *)r->W1,
                  (void *)r->W2, (void *)r->starting, (void *)r->nextFinishing, (void *)r->level, (void *)r->cFP2,
                  (void *)r->cEZ2, (void *)r->PsiM, (void *)r->items, (void *)r->recA, (void *)r->recB,
                  (void *)r->corner32, (void *)r->link32, (void *)r->fac32, (void *)r->W1_32, (void *)r->W2_32,
                  (void *)r->PsiM32, (void *)r->bFace2})
    if (p) cudaFree(p);
  delete r;
  c.rz = nullptr;
}

template <typename T>
static int upload(T **d, const T *h, size_t n) {
  if (cudaMalloc((void **)d, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess)
    return set_error(UMT_ERR_NOMEM, "RZ: device allocation of %zu bytes failed", n * sizeof(T));
  if (n) UMT_CUDA(cudaMemcpy(*d, h, n * sizeof(T), cudaMemcpyHostToDevice));
  return 0;
}

// rt/geometryUCBrz.F90:48-150 per corner (zone centre = vertex average,
// mods/Geometry_mod.F90 getZoneCenter).  Each corner's face vectors are
// formed from its own vertices; the reference's writes of a neighbour's
// entries give the same values (exact negations of the same differences).
static void geometry_rz(int nz, const int *numCorner, const int *cOffSet, const int *cEZ, const double *px,
                        std::vector<double> &A_fp, std::vector<double> &A_ez, RZData &r) {
  const size_t nc = r.hArea.size();
  A_fp.assign(nc * 2 * 3, 0.0);
  A_ez.assign(nc * 2 * 3, 0.0);
  for (int zone = 0; zone < nz; ++zone) {
    const int nC = numCorner[zone], c0 = cOffSet[zone];
    double rz = 0.0, zz = 0.0;
    for (int c = 0; c < nC; ++c) { rz += px[2 * (c0 + c)]; zz += px[2 * (c0 + c) + 1]; }
    rz /= (double)nC;
    zz /= (double)nC;
    for (int c = 0; c < nC; ++c) {
      const size_t cc = (size_t)c0 + c;
      const int c1 = cEZ[2 * cc], c2 = cEZ[2 * cc + 1];
      const double r0 = px[2 * cc], z0 = px[2 * cc + 1];
      const double r1 = px[2 * (c0 + c1)], z1 = px[2 * (c0 + c1) + 1];
      const double r2 = px[2 * (c0 + c2)], z2 = px[2 * (c0 + c2) + 1];
      const double re1 = 0.5 * (r0 + r1), ze1 = 0.5 * (z0 + z1);
      const double re2 = 0.5 * (r0 + r2), ze2 = 0.5 * (z0 + z2);
      r.hRfp[2 * cc] = 0.5 * (r0 + re2);
      r.hRfp[2 * cc + 1] = 0.5 * (r0 + re1);
      r.hRez[2 * cc] = 0.5 * (rz + re1);
      r.hRez[2 * cc + 1] = 0.5 * (rz + re2);
      A_fp[(cc * 2 + 0) * 3 + 0] = 0.5 * (z2 - z0);
      A_fp[(cc * 2 + 0) * 3 + 1] = 0.5 * (r0 - r2);
      A_fp[(cc * 2 + 1) * 3 + 0] = 0.5 * (z0 - z1);
      A_fp[(cc * 2 + 1) * 3 + 1] = 0.5 * (r1 - r0);
      A_ez[(cc * 2 + 0) * 3 + 0] = ze1 - zz;
      A_ez[(cc * 2 + 0) * 3 + 1] = rz - re1;
      A_ez[(cc * 2 + 1) * 3 + 0] = zz - ze2;
      A_ez[(cc * 2 + 1) * 3 + 1] = re2 - rz;
      const double area1 = std::fabs((re2 - r0) * (zz - z0) - (ze2 - z0) * (rz - r0));
      const double area2 = std::fabs((rz - r0) * (ze1 - z0) - (zz - z0) * (re1 - r0));
      r.hArea[cc] = 0.5 * (area1 + area2);
      const double rbar1 = (r0 + re2 + rz) / 3.0, rbar2 = (r0 + re1 + rz) / 3.0;
      r.hVolume[cc] = 0.5 * (rbar1 * area1 + rbar2 * area2);
    }
  }
}

struct RZP {
  int nz, nc, nb, G;
  const uint32_t *items;
  int stageBegin, stageCount;
  const uint32_t *order;
  const int *numCorner, *cOffSet, *cFP2, *cEZ2;
  const double *afp, *aez;               // [A][nc][UMT_MAXCF] projections
  const double *Area, *Volume, *RadiusFP, *RadiusEZ;
  const double *Sigt, *STotal;
  double tau;
  const double *angDerivFac, *W1, *W2;
  const int *starting, *nextFinishing, *level;
  const double *psi_old;
  double *psi_new, *psiB, *PsiM;
};

constexpr int RZ_NT = 128;
constexpr int RZ_MAXC = UMT_MAXCORNER;

template <int GT>
__global__ void __launch_bounds__(RZ_NT) k_sweep_rz(RZP p) {
  constexpr int TEAMS = RZ_NT / GT;
  __shared__ double s_src[RZ_MAXC][RZ_NT];
  __shared__ double s_Q[RZ_MAXC][RZ_NT];
  __shared__ double s_afp[TEAMS][RZ_MAXC][2], s_aez[TEAMS][RZ_MAXC][2];
  __shared__ double s_rfp[TEAMS][RZ_MAXC][2], s_rez[TEAMS][RZ_MAXC][2];
  __shared__ double s_area[TEAMS][RZ_MAXC], s_vol[TEAMS][RZ_MAXC], s_sum[TEAMS][RZ_MAXC];
  __shared__ int s_cfp[TEAMS][RZ_MAXC][2];
  __shared__ int8_t s_cez[TEAMS][RZ_MAXC][2];
  const int tid = threadIdx.x, team = tid / GT, lane = tid % GT;
  const int k = blockIdx.x * TEAMS + team;
  if (k >= p.stageCount) return;                       // whole teams leave together
  const unsigned teammask = (GT == 32) ? 0xffffffffu : (((1u << GT) - 1u) << ((tid & 31) / GT * GT));
  const uint32_t it = p.items[p.stageBegin + k];
  const int a = (int)(it / (uint32_t)p.nz);
  const int z = (int)(it - (uint32_t)a * p.nz);
  const int nC = p.numCorner[z], c0 = p.cOffSet[z];
  const uint32_t ord = p.order[it];
  const size_t abase = (size_t)a * p.nc;
  const double fac = p.angDerivFac[a];
  for (int c = lane; c < nC; c += GT) {
    const size_t cc = (size_t)c0 + c;
    s_area[team][c] = p.Area[cc];
    s_vol[team][c] = p.Volume[cc];
#pragma unroll
    for (int f = 0; f < 2; ++f) {
      s_afp[team][c][f] = p.afp[(abase + cc) * UMT_MAXCF + f];
      s_aez[team][c][f] = p.aez[(abase + cc) * UMT_MAXCF + f];
      s_rfp[team][c][f] = p.RadiusFP[2 * cc + f];
      s_rez[team][c][f] = p.RadiusEZ[2 * cc + f];
      s_cfp[team][c][f] = p.cFP2[2 * cc + f];
      s_cez[team][c][f] = (int8_t)p.cEZ2[2 * cc + f];
    }
  }
  __syncwarp(teammask);
  // sumArea in the reference's order: fac*Area for every corner, then the
  // corner / corner-face loop (SweepUCBrz.F90:128-151)
  if (lane == 0) {
    for (int c = 0; c < nC; ++c) s_sum[team][c] = fac * s_area[team][c];
    for (int c = 0; c < nC; ++c)
      for (int f = 0; f < 2; ++f) {
        const double afp = s_afp[team][c][f], aez = s_aez[team][c][f];
        if (afp < 0.0) s_sum[team][c] = s_sum[team][c] - s_rfp[team][c][f] * afp;
        if (aez > 0.0) {
          const int cez = s_cez[team][c][f];
          s_sum[team][cez] = s_sum[team][cez] + s_rez[team][c][f] * aez;
        }
      }
  }
  __syncwarp(teammask);
  const double fouralpha = 1.82;
  const double *sigz = p.Sigt + (size_t)z * p.G;
  const bool start = p.starting[a] != 0, nextFin = p.nextFinishing[a] != 0;
  double *psiM = p.PsiM + (size_t)p.level[a] * p.nc * p.G;
  for (int g = lane; g < p.G; g += GT) {
    const double sig = sigz[g];
    for (int c = 0; c < nC; ++c) {
      const size_t e = ((size_t)c0 + c) * p.G + g;
      const double q = p.STotal[e] + p.tau * p.psi_old[abase * p.G + e];
      s_Q[c][tid] = q;
      s_src[c][tid] = s_vol[team][c] * q;
    }
    for (int c = 0; c < nC; ++c) {
      for (int f = 0; f < 2; ++f) {
        const double afp = s_afp[team][c][f], aez = s_aez[team][c][f];
        double pu = 0.0;
        if (afp < 0.0) {
          const int cfp = s_cfp[team][c][f];
          pu = (cfp < p.nc) ? p.psi_new[(abase + cfp) * p.G + g]
                            : p.psiB[((size_t)a * p.nb + (cfp - p.nc)) * p.G + g];
          const double R_afp = s_rfp[team][c][f] * afp;
          s_src[c][tid] = s_src[c][tid] - R_afp * pu;
        }
        if (aez > 0.0) {
          const double R = s_rez[team][c][f];
          const int cez = s_cez[team][c][f];
          const double area = s_area[team][c];
          const double Qc = s_Q[c][tid], Qz = s_Q[cez][tid];
          double sez;
          if (afp < 0.0) {
            const double sigA = sig * area, sigA2 = sigA * sigA;
            const double gnum = aez * aez * (fouralpha * sigA2 + aez * (4.0 * sigA + 3.0 * aez));
            const double gden = area * (4.0 * sigA * sigA2 + aez * (6.0 * sigA2 + 2.0 * aez * (2.0 * sigA + aez)));
            sez = R * (area * gnum * (sig * pu - Qc) + 0.5 * aez * gden * (Qc - Qz)) / (gnum + gden * sig);
          } else {
            sez = 0.5 * R * aez * (Qc - Qz) / sig;
          }
          s_src[c][tid] = s_src[c][tid] + sez;
          s_src[cez][tid] = s_src[cez][tid] - sez;
        }
      }
    }
    double *out = p.psi_new + abase * p.G;
    for (int i = 0; i < nC; ++i) {
      const int c = (int)((ord >> (4 * i)) & 15u);
      const size_t e = ((size_t)c0 + c) * p.G + g;
      const double v = (s_src[c][tid] + s_area[team][c] * fac * psiM[e]) / (s_sum[team][c] + sig * s_vol[team][c]);
      out[e] = v;
      s_Q[c][tid] = v;                       // Q is no longer needed: keep the solved flux
      for (int f = 0; f < 2; ++f) {
        const double aez = s_aez[team][c][f];
        if (aez > 0.0) {
          const int cez = s_cez[team][c][f];
          s_src[cez][tid] = s_src[cez][tid] + (s_rez[team][c][f] * aez) * v;
        }
      }
    }
    for (int c = 0; c < nC; ++c) {
      const size_t e = ((size_t)c0 + c) * p.G + g;
      const double v = s_Q[c][tid];
      const double m = start ? v : p.W1[a] * v - p.W2[a] * psiM[e];
      psiM[e] = m;
      if (nextFin) p.psi_new[((size_t)(a + 1) * p.nc) * p.G + e] = m;
      for (int f = 0; f < 2; ++f) {
        const int cfp = s_cfp[team][c][f];
        if (cfp >= p.nc && s_afp[team][c][f] > 0.0) {
          const size_t b = (size_t)(cfp - p.nc);
          p.psiB[((size_t)a * p.nb + b) * p.G + g] = v;
          if (nextFin) p.psiB[((size_t)(a + 1) * p.nb + b) * p.G + g] = m;
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// FP32 RZ sweep.
//
// Per (direction, corner) the FP32 kernel reads two records built once from
// the FP64 projections the schedule was decided with, so every face is
// classified exactly as the schedule classified it:
//   recA = {RadiusFP0*afp0, RadiusFP1*afp1, RadiusEZ0*aez0, RadiusEZ1*aez1}
//   recB = {sumArea, Area/aez0, Area/aez1, face bits}
// with sumArea = angDerivFac*Area + sum of RadiusFP*|afp| over incoming FP
// faces + RadiusEZ*aez over the EZ faces that feed the corner, and face bits
// 1<<f (afp_f < 0, incoming), 4<<f (afp_f > 0, exiting), 16<<f (aez_f > 0).
// One thread per (direction, zone); sums in FP64, rounded once.
__global__ void k_rz_prep32(int A, int nz, int nc, const int *numCorner, const int *cOffSet, const int *cEZ2,
                            const double *afp, const double *aez, const double *Area, const double *Rfp,
                            const double *Rez, const double *angDerivFac, float4 *recA, float4 *recB) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= (size_t)A * nz) return;
  const int a = (int)(t / (size_t)nz), z = (int)(t - (size_t)a * nz);
  const int nC = numCorner[z], c0 = cOffSet[z];
  const size_t abase = (size_t)a * nc;
  const double fac = angDerivFac[a];
  double sum[RZ_MAXC];
  for (int c = 0; c < nC; ++c) sum[c] = fac * Area[c0 + c];
  for (int c = 0; c < nC; ++c)
    for (int f = 0; f < 2; ++f) {
      const size_t cc = (size_t)c0 + c;
      const double fp = afp[(abase + cc) * UMT_MAXCF + f], ez = aez[(abase + cc) * UMT_MAXCF + f];
      if (fp < 0.0) sum[c] -= Rfp[2 * cc + f] * fp;
      if (ez > 0.0) sum[cEZ2[2 * cc + f]] += Rez[2 * cc + f] * ez;
    }
  for (int c = 0; c < nC; ++c) {
    const size_t cc = (size_t)c0 + c;
    double fp[2], ez[2];
    unsigned bits = 0;
    for (int f = 0; f < 2; ++f) {
      fp[f] = afp[(abase + cc) * UMT_MAXCF + f];
      ez[f] = aez[(abase + cc) * UMT_MAXCF + f];
      if (fp[f] < 0.0) bits |= 1u << f;
      if (fp[f] > 0.0) bits |= 4u << f;
      if (ez[f] > 0.0) bits |= 16u << f;
    }
    recA[abase + cc] = make_float4((float)(Rfp[2 * cc] * fp[0]), (float)(Rfp[2 * cc + 1] * fp[1]),
                                   (float)(Rez[2 * cc] * ez[0]), (float)(Rez[2 * cc + 1] * ez[1]));
    recB[abase + cc] = make_float4((float)sum[c], ez[0] > 0.0 ? (float)(Area[cc] / ez[0]) : 0.f,
                                   ez[1] > 0.0 ? (float)(Area[cc] / ez[1]) : 0.f, __uint_as_float(bits));
  }
}

__global__ void k_rz_to_float(size_t n, const double *x, float *y) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] = (float)x[i];
}

// Boundary element b's corner face 2*c + f (cFP2 holds nc + b on boundary faces).
__global__ void k_rz_bface(int nc, int nb, const int *cFP2, int *bFace2) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  for (int f = 0; f < 2; ++f) {
    const int v = cFP2[2 * c + f];
    if (v >= nc && v - nc < nb) bFace2[v - nc] = 2 * c + f;
  }
}

// The PsiB rows an RZ sweep writes, FP32 copy -> FP64 array: row (a, b) when
// b's corner face exits in direction a, or, for a finishing direction a (not
// swept), in direction a - 1, whose exits also hand it their PsiM.  Every
// other row of the FP64 array keeps the caller's value.
__global__ void k_rz_psib_out(int A, int nb, int nc, int G, const int *bFace2, const double *afp,
                              const int *nextFinishing, const float *psiB32, double *dst) {
  const size_t n = (size_t)A * nb * G;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const size_t row = i / (size_t)G;
    const int a = (int)(row / (size_t)nb), b = (int)(row - (size_t)a * nb);
    const int bf = bFace2[b];
    if (bf < 0) continue;
    const int as = (a > 0 && nextFinishing[a - 1]) ? a - 1 : a;
    if (afp[((size_t)as * nc + (bf >> 1)) * UMT_MAXCF + (bf & 1)] > 0.0) dst[i] = (double)psiB32[i];
  }
}

struct RZP32 {
  int nz, nc, nb, G;
  const uint32_t *items;
  int stageBegin, stageCount;
  const uint32_t *order;
  const int *numCorner, *cOffSet;
  const float4 *recA, *recB, *corner;
  const int2 *link;
  const float *Sigt, *STotal;
  float tau;
  const float *fac, *W1, *W2;
  const int *starting, *nextFinishing, *level;
  const float *psi_old;
  float *psi_new, *psiB, *PsiM;
};

// One dependency stage of the FP32 RZ sweep: a team of GT lanes per
// (direction, zone), lanes over groups; MAXC (4 or 8) bounds the corners of
// a zone, and the corner loops are unrolled to it.  The operations of
// k_sweep_rz, with three changes of rounding order:
// * the angular-derivative term Area*angDerivFac*PsiM enters the corner's
//   source before the solve instead of at it;
// * the EZ closure of a corner face whose FP face is incoming is divided
//   through by aez^4 (x = sigma*Area/aez):
//     sez = RadiusEZ*Area (N (sigma psi_fp - Q_c) + D (Q_c - Q_z)) / (N + 2 x D),
//     N = 1.82 x^2 + 4 x + 3,  D = 2 x^3 + 3 x^2 + 2 x + 1,
//   algebraically the reference's gnum/gden form (x is capped at 1e8 so every
//   term stays finite in FP32);
// * divisions are approximate reciprocals times a multiply.
// Offsets within one direction are 32-bit (ncornr*G, nbelem*G and nzones*G
// are below 2^31, checked at init).  Programmatic dependent launch: everything
// before pdl_wait() reads only data no stage writes.
template <int GT, int MAXC>
__global__ void __launch_bounds__(RZ_NT, MAXC == 4 ? 5 : 4) k_sweep_rz32(RZP32 p) {
  pdl_launch_dependents();
  constexpr int TEAMS = RZ_NT / GT;
  __shared__ float s_src[MAXC][RZ_NT], s_Q[MAXC][RZ_NT];
  __shared__ float4 s_A[TEAMS][MAXC], s_B[TEAMS][MAXC], s_C[TEAMS][MAXC];
  __shared__ int2 s_L[TEAMS][MAXC];
  const int tid = threadIdx.x, team = tid / GT, lane = tid % GT;
  const int k = blockIdx.x * TEAMS + team;
  if (k >= p.stageCount) return;                       // whole teams leave together
  const unsigned teammask = team_mask(GT, tid);
  const uint32_t it = p.items[p.stageBegin + k];
  const int a = (int)(it / (uint32_t)p.nz);
  const int z = (int)(it - (uint32_t)a * p.nz);
  const int nC = p.numCorner[z], c0 = p.cOffSet[z];
  const uint32_t ord = p.order[it];
  const int G = p.G, nc = p.nc;
  const size_t abase = (size_t)a * nc;
  for (int c = lane; c < nC; c += GT) {
    s_A[team][c] = p.recA[abase + c0 + c];
    s_B[team][c] = p.recB[abase + c0 + c];
    s_C[team][c] = p.corner[c0 + c];
    s_L[team][c] = p.link[c0 + c];
  }
  const float fac = p.fac[a], W1 = p.W1[a], W2 = p.W2[a];
  const bool start = p.starting[a] != 0, nextFin = p.nextFinishing[a] != 0;
  const float *pold = p.psi_old + abase * G;                      // direction a
  float *pnew = p.psi_new + abase * G;
  float *pnext = pnew + (size_t)nc * G;                           // direction a + 1
  float *pB = p.psiB + (size_t)a * p.nb * G;
  float *pBnext = pB + (size_t)p.nb * G;
  float *psiM = p.PsiM + (size_t)p.level[a] * nc * G;
  const int e0 = c0 * G;
  __syncwarp(teammask);
  for (int g = lane; g < G; g += GT) {
    const float sig = p.Sigt[z * G + g];
#pragma unroll
    for (int c = 0; c < MAXC; ++c)
      if (c < nC) {
        const float q = fmaf(p.tau, pold[e0 + c * G + g], p.STotal[e0 + c * G + g]);
        s_Q[c][tid] = q;
        s_src[c][tid] = s_C[team][c].x * q;
      }
    pdl_wait();                                          // the previous stage is complete from here on
    float pm[MAXC], pu[MAXC][2];
#pragma unroll
    for (int c = 0; c < MAXC; ++c) {
      pm[c] = pu[c][0] = pu[c][1] = 0.f;
      if (c < nC) {
        pm[c] = psiM[e0 + c * G + g];
        const unsigned bits = __float_as_uint(s_B[team][c].w);
        const int2 L = s_L[team][c];
#pragma unroll
        for (int f = 0; f < 2; ++f)
          if (bits & (1u << f)) {
            const int cfp = (f ? L.y : L.x) >> 3;
            pu[c][f] = cfp < nc ? pnew[cfp * G + g] : pB[(cfp - nc) * G + g];
          }
      }
    }
    const float rsig = rcp_approx(sig);
    // corner c's source, kept in a register while its faces are added; other
    // corners' EZ terms reach it through shared memory (cez != c)
#pragma unroll
    for (int c = 0; c < MAXC; ++c) {
      if (c >= nC) continue;
      const float4 A = s_A[team][c], B = s_B[team][c], C = s_C[team][c];
      const unsigned bits = __float_as_uint(B.w);
      const int2 L = s_L[team][c];
      const float Qc = s_Q[c][tid];
      float sc = fmaf(C.w * fac, pm[c], s_src[c][tid]);
#pragma unroll
      for (int f = 0; f < 2; ++f) {
        const float kfp = f ? A.y : A.x, rae = f ? A.w : A.z, xa = f ? B.z : B.y, rza = f ? C.z : C.y;
        if (bits & (1u << f)) sc = fmaf(-kfp, pu[c][f], sc);
        if (bits & (16u << f)) {
          const int cez = (f ? L.y : L.x) & (MAXC - 1);
          const float Qz = s_Q[cez][tid];
          float sez;
          if (bits & (1u << f)) {
            const float x = fminf(sig * xa, 1e8f);
            const float N = fmaf(fmaf(1.82f, x, 4.f), x, 3.f);
            const float D = fmaf(fmaf(fmaf(2.f, x, 3.f), x, 2.f), x, 1.f);
            sez = rza * fmaf(N, fmaf(sig, pu[c][f], -Qc), D * (Qc - Qz)) * rcp_approx(fmaf(2.f * x, D, N));
          } else {
            sez = 0.5f * rae * (Qc - Qz) * rsig;
          }
          sc += sez;
          s_src[cez][tid] -= sez;
        }
      }
      s_src[c][tid] = sc;
    }
#pragma unroll
    for (int i = 0; i < MAXC; ++i) {
      if (i >= nC) continue;
      const int c = (int)((ord >> (4 * i)) & (unsigned)(MAXC - 1));
      const float4 B = s_B[team][c], C = s_C[team][c], A = s_A[team][c];
      const int2 L = s_L[team][c];
      const float v = s_src[c][tid] * rcp_approx(fmaf(sig, C.x, B.x));
      pnew[e0 + c * G + g] = v;
      s_Q[c][tid] = v;                       // Q is no longer needed: keep the solved flux
      const unsigned bits = __float_as_uint(B.w);
      if (bits & 16u) s_src[L.x & (MAXC - 1)][tid] = fmaf(A.z, v, s_src[L.x & (MAXC - 1)][tid]);
      if (bits & 32u) s_src[L.y & (MAXC - 1)][tid] = fmaf(A.w, v, s_src[L.y & (MAXC - 1)][tid]);
    }
#pragma unroll
    for (int c = 0; c < MAXC; ++c) {
      if (c >= nC) continue;
      const int e = e0 + c * G + g;
      const float v = s_Q[c][tid];
      const float m = start ? v : fmaf(W1, v, -W2 * pm[c]);
      psiM[e] = m;
      if (nextFin) pnext[e] = m;
      const unsigned bits = __float_as_uint(s_B[team][c].w);
      const int2 L = s_L[team][c];
#pragma unroll
      for (int f = 0; f < 2; ++f) {
        const int cfp = (f ? L.y : L.x) >> 3;
        if ((bits & (4u << f)) && cfp >= nc) {
          const int b = (cfp - nc) * G + g;
          pB[b] = v;
          if (nextFin) pBnext[b] = m;
        }
      }
    }
  }
}

// Launch every stage of one FP32 RZ sweep (conversions, PsiM reset, stages,
// tally) on the context's stream; stages after the first carry the
// programmatic-serialization attribute.
static int enqueue_sweep_rz32(Ctx &c, RZData &r) {
  const size_t ncG = (size_t)c.nc * c.G, nzG = (size_t)c.nz * c.G;
  k_rz_to_float<<<(int)std::min<size_t>((nzG + 255) / 256, 4096), 256, 0, c.stream>>>(nzG, c.Sigt, c.Sigt32);
  k_rz_to_float<<<(int)std::min<size_t>((ncG + 255) / 256, 4096), 256, 0, c.stream>>>(ncG, c.STotal, c.STotal32);
  UMT_CUDA(cudaMemsetAsync(r.PsiM32, 0, (size_t)r.nLevels * ncG * sizeof(float), c.stream));
  RZP32 p;
  p.nz = c.nz; p.nc = c.nc; p.nb = c.nb; p.G = c.G;
  p.items = r.items; p.order = c.sch.order;
  p.numCorner = c.numCorner; p.cOffSet = c.cOffSet;
  p.recA = r.recA; p.recB = r.recB; p.corner = r.corner32; p.link = r.link32;
  p.Sigt = c.Sigt32; p.STotal = c.STotal32; p.tau = (float)c.tau;
  p.fac = r.fac32; p.W1 = r.W1_32; p.W2 = r.W2_32;
  p.starting = r.starting; p.nextFinishing = r.nextFinishing; p.level = r.level;
  p.psi_old = c.psi32[c.cur32]; p.psi_new = c.psi32[1 - c.cur32]; p.psiB = c.psiB32; p.PsiM = r.PsiM32;
  int GT = 1;
  while (GT < c.G && GT < 32) GT *= 2;
  const int TEAMS = RZ_NT / GT;
  void (*kern)(RZP32) = nullptr;
#define UMT_RZ32(gt)                                                    \
  case gt: kern = r.maxC <= 4 ? k_sweep_rz32<gt, 4> : k_sweep_rz32<gt, 8>; break;
  switch (GT) {
    UMT_RZ32(1) UMT_RZ32(2) UMT_RZ32(4) UMT_RZ32(8) UMT_RZ32(16)
    default: kern = r.maxC <= 4 ? k_sweep_rz32<32, 4> : k_sweep_rz32<32, 8>; break;
  }
#undef UMT_RZ32
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  bool first = true;
  for (int s = 0; s < r.nStages; ++s) {
    if (r.hCount[s] == 0) continue;
    p.stageBegin = r.hOffset[s];
    p.stageCount = r.hCount[s];
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)((r.hCount[s] + TEAMS - 1) / TEAMS));
    cfg.blockDim = dim3(RZ_NT);
    cfg.stream = c.stream;
    cfg.attrs = attr;
    cfg.numAttrs = first ? 0 : 1;            // the first stage follows the conversions in full
    first = false;
    UMT_CUDA(cudaLaunchKernelEx(&cfg, kern, p));
  }
  return launch_tally(c, UMT_FP32);
}

}  // namespace umt

using namespace umt;

extern "C" {

int umt103_init_rz(const UmtMeshRZ *m, const UmtQuadRZ *q, int ngr, int flags) {
  if (!m || !q || ngr < 1 || q->nangles < 2 || !q->omega || !q->weight || !q->angDerivFac || !q->quadTauW1 ||
      !q->quadTauW2 || !q->starting || !q->finishing || !m->px || !m->cEZ || !m->cFP || !m->numCorner ||
      !m->cOffSet)
    return set_error(UMT_ERR_ARG, "umt103_init_rz: null argument or bad sizes");
  if (m->index_base != 0 && m->index_base != 1) return set_error(UMT_ERR_ARG, "index_base must be 0 or 1");
  const int nz = m->nzones, nc = m->ncornr, nb = m->nbelem, A = q->nangles, base = m->index_base;
  if (nz <= 0 || nc <= 0 || nb < 0) return set_error(UMT_ERR_ARG, "bad RZ mesh sizes");
  for (int zn = 0; zn < nz; ++zn) {
    if (m->numCorner[zn] < 3 || m->numCorner[zn] > UMT_MAXCORNER)
      return set_error(UMT_ERR_ARG, "RZ zone %d has %d corners (3..%d supported)", zn, m->numCorner[zn], UMT_MAXCORNER);
    const int c0 = m->cOffSet[zn];                 // an offset (0-based) in both index conventions
    if (c0 < 0 || c0 + m->numCorner[zn] > nc) return set_error(UMT_ERR_ARG, "RZ zone %d corner range", zn);
  }
  // starting / finishing pattern: every level is start, weighted..., finish
  int nLevels = 0;
  std::vector<int> level(A, -1), nextFin(A, 0), start(A, 0);
  {
    bool open = false;
    for (int a = 0; a < A; ++a) {
      if (q->starting[a]) {
        if (open) return set_error(UMT_ERR_ARG, "RZ quadrature: level %d has no finishing direction", nLevels - 1);
        open = true;
        ++nLevels;
      }
      if (!open) return set_error(UMT_ERR_ARG, "RZ quadrature: direction %d outside a level", a);
      level[a] = nLevels - 1;
      start[a] = q->starting[a] ? 1 : 0;
      if (q->finishing[a]) {
        if (q->starting[a] || a == 0) return set_error(UMT_ERR_ARG, "RZ quadrature: bad finishing direction %d", a);
        nextFin[a - 1] = 1;
        open = false;
      }
    }
    if (open) return set_error(UMT_ERR_ARG, "RZ quadrature: last level has no finishing direction");
  }
  // 0-based connectivity and the geometry
  std::vector<int> cez((size_t)nc * 2), cfp((size_t)nc * 2), noff(nz);
  for (size_t i = 0; i < (size_t)nc * 2; ++i) { cez[i] = m->cEZ[i] - base; cfp[i] = m->cFP[i] - base; }
  for (int zn = 0; zn < nz; ++zn) noff[zn] = m->cOffSet[zn];
  for (int zn = 0; zn < nz; ++zn)
    for (int c = 0; c < m->numCorner[zn]; ++c)
      for (int f = 0; f < 2; ++f) {
        const int v = cez[2 * ((size_t)noff[zn] + c) + f];
        if (v < 0 || v >= m->numCorner[zn]) return set_error(UMT_ERR_ARG, "RZ cEZ out of range at zone %d", zn);
        const int w = cfp[2 * ((size_t)noff[zn] + c) + f];
        if (w < 0 || w >= nc + nb) return set_error(UMT_ERR_ARG, "RZ cFP out of range at zone %d", zn);
      }
  RZData *r = new RZData();
  r->hArea.assign(nc, 0.0); r->hVolume.assign(nc, 0.0);
  r->hRfp.assign((size_t)nc * 2, 0.0); r->hRez.assign((size_t)nc * 2, 0.0);
  std::vector<double> A_fp, A_ez;
  geometry_rz(nz, m->numCorner, noff.data(), cez.data(), m->px, A_fp, A_ez, *r);
  // the shared context: 3-vector geometry (third component 0), FP64 flux
  std::vector<int> ncf(nc, 2);
  UmtMesh m3 = {};
  m3.index_base = base; m3.nzones = nz; m3.ncornr = nc; m3.nbelem = nb; m3.maxcf = 2; m3.maxFaces = m->maxFaces;
  m3.numCorner = m->numCorner; m3.cOffSet = m->cOffSet; m3.zoneFaces = m->zoneFaces; m3.zoneOpp = m->zoneOpp;
  m3.faceOpp = m->faceOpp; m3.nCFaces = ncf.data(); m3.cFP = m->cFP; m3.cEZ = m->cEZ; m3.CToFace = m->CToFace;
  m3.bdyToC = m->bdyToC; m3.px = nullptr; m3.A_fp = A_fp.data(); m3.A_ez = A_ez.data();
  m3.Volume = r->hVolume.data();
  std::vector<double> om3((size_t)A * 3, 0.0);
  for (int a = 0; a < A; ++a) { om3[3 * a] = q->omega[2 * a]; om3[3 * a + 1] = q->omega[2 * a + 1]; }
  UmtQuad q3 = {A, om3.data(), q->weight};
  const int precFlags = (flags & 3) ? (flags & 3) : 3;     // bit 0: FP64 flux, bit 1: FP32 flux
  if ((precFlags & 2) && ((long long)nc + nb >= (1LL << 28) || (long long)(nc + nb) * ngr >= (1LL << 31) ||
                          (long long)nz * ngr >= (1LL << 31))) {
    delete r;
    return set_error(UMT_ERR_ARG, "RZ FP32 path: ncornr + nbelem must be below 2^28 and (ncornr + nbelem)*G, "
                                  "nzones*G below 2^31");
  }
  for (int zn = 0; zn < nz; ++zn) r->maxC = std::max(r->maxC, m->numCorner[zn]);
  release_current_context();
  Ctx &c = cur();
  int rc = init_context(c, &m3, &q3, ngr, precFlags);
  if (rc) { delete r; return rc; }
  c.rz = r;
  // the schedule must be cycle-free (convex RZ zones have no intra-zone
  // cycles; the RZ sweep carries no cycle list)
  if (c.sch.nCyc > 0) return set_error(UMT_ERR_CYCLE, "RZ: the mesh has a dependency cycle, not supported");
  {
    std::vector<uint8_t> bad((size_t)A * nz);
    UMT_CUDA(cudaMemcpy(bad.data(), c.sch.bad, bad.size(), cudaMemcpyDeviceToHost));
    for (uint8_t v : bad)
      if (v) return set_error(UMT_ERR_CYCLE, "RZ: the schedule has a lagged zone, not supported");
  }
  // Stages.  Item (a, z) needs its upwind zones in direction a, and PsiM of
  // zone z from the previous swept direction of its level:
  //   stage(a, z) = max(stage(prev(a), z) + 1, stage(a, u) + 1 over upwind u),
  // so a level's directions follow one another zone by zone (a wavefront
  // right behind the previous one), and the levels run concurrently.
  std::vector<int> lev((size_t)A * nz), nh(A), zopp((size_t)nz * UMT_MAXFACES), zfac(nz);
  std::vector<uint8_t> exm((size_t)A * nz);
  UMT_CUDA(cudaMemcpy(lev.data(), c.sch.level, lev.size() * sizeof(int), cudaMemcpyDeviceToHost));
  UMT_CUDA(cudaMemcpy(nh.data(), c.sch.nHyper, A * sizeof(int), cudaMemcpyDeviceToHost));
  UMT_CUDA(cudaMemcpy(exm.data(), c.sch.exitMask, exm.size(), cudaMemcpyDeviceToHost));
  UMT_CUDA(cudaMemcpy(zopp.data(), c.zoneOpp, zopp.size() * sizeof(int), cudaMemcpyDeviceToHost));
  UMT_CUDA(cudaMemcpy(zfac.data(), c.zoneFaces, nz * sizeof(int), cudaMemcpyDeviceToHost));
  std::vector<int> stg((size_t)A * nz, 0);
  int nStages = 0;
  {
    std::vector<int> prevOf(nLevels, -1), byLevel(nz), cnt;
    for (int a = 0; a < A; ++a) {
      if (q->finishing[a]) continue;
      const int p = prevOf[level[a]];
      int *sa = stg.data() + (size_t)a * nz;
      for (int zn = 0; zn < nz; ++zn) sa[zn] = p >= 0 ? stg[(size_t)p * nz + zn] + 1 : 0;
      // zones in hyperplane order (a topological order of direction a)
      cnt.assign(nh[a] + 1, 0);
      for (int zn = 0; zn < nz; ++zn) ++cnt[lev[(size_t)a * nz + zn] + 1];
      for (int h = 0; h < nh[a]; ++h) cnt[h + 1] += cnt[h];
      for (int zn = 0; zn < nz; ++zn) byLevel[cnt[lev[(size_t)a * nz + zn]]++] = zn;
      for (int i = 0; i < nz; ++i) {
        const int zn = byLevel[i];
        const uint8_t mask = exm[(size_t)a * nz + zn];
        for (int f = 0; f < zfac[zn]; ++f)
          if (mask & (1u << f)) {
            const int d = zopp[(size_t)zn * UMT_MAXFACES + f];
            if (d >= 0) sa[d] = std::max(sa[d], sa[zn] + 1);
          }
      }
      for (int zn = 0; zn < nz; ++zn) nStages = std::max(nStages, sa[zn] + 1);
      prevOf[level[a]] = a;
    }
  }
  r->nLevels = nLevels;
  r->nStages = nStages;
  r->hCount.assign(nStages, 0);
  for (int a = 0; a < A; ++a) {
    if (q->finishing[a]) continue;
    for (int zn = 0; zn < nz; ++zn) ++r->hCount[stg[(size_t)a * nz + zn]];
  }
  r->hOffset.assign(nStages, 0);
  for (int s = 1; s < nStages; ++s) r->hOffset[s] = r->hOffset[s - 1] + r->hCount[s - 1];
  std::vector<uint32_t> items((size_t)(nStages ? r->hOffset[nStages - 1] + r->hCount[nStages - 1] : 0));
  {
    std::vector<int> fill(r->hOffset);
    for (int a = 0; a < A; ++a) {
      if (q->finishing[a]) continue;
      for (int zn = 0; zn < nz; ++zn) items[fill[stg[(size_t)a * nz + zn]]++] = (uint32_t)a * (uint32_t)nz + (uint32_t)zn;
    }
  }
  for (int s = 0; s < nStages; ++s) r->maxStageItems = std::max(r->maxStageItems, r->hCount[s]);
  rc = upload(&r->items, items.data(), items.size());
  if (!rc) rc = upload(&r->Area, r->hArea.data(), (size_t)nc);
  if (!rc) rc = upload(&r->RadiusFP, r->hRfp.data(), (size_t)nc * 2);
  if (!rc) rc = upload(&r->RadiusEZ, r->hRez.data(), (size_t)nc * 2);
  if (!rc) rc = upload(&r->angDerivFac, q->angDerivFac, (size_t)A);
  if (!rc) rc = upload(&r->W1, q->quadTauW1, (size_t)A);
  if (!rc) rc = upload(&r->W2, q->quadTauW2, (size_t)A);
  if (!rc) rc = upload(&r->starting, start.data(), (size_t)A);
  if (!rc) rc = upload(&r->nextFinishing, nextFin.data(), (size_t)A);
  if (!rc) rc = upload(&r->level, level.data(), (size_t)A);
  if (!rc) rc = upload(&r->cFP2, cfp.data(), cfp.size());
  if (!rc) rc = upload(&r->cEZ2, cez.data(), cez.size());
  if (rc) return rc;
  if ((c.flags & 1) && cudaMalloc((void **)&r->PsiM, (size_t)nLevels * nc * ngr * sizeof(double)) != cudaSuccess)
    return set_error(UMT_ERR_NOMEM, "RZ: PsiM allocation failed");
  if (c.flags & 2) {
    std::vector<float4> corner(nc);
    std::vector<int2> link(nc);
    for (int cc = 0; cc < nc; ++cc) {
      const double ar = r->hArea[cc];
      corner[cc] = make_float4((float)r->hVolume[cc], (float)(r->hRez[2 * cc] * ar), (float)(r->hRez[2 * cc + 1] * ar),
                               (float)ar);
      link[cc] = make_int2(cfp[2 * (size_t)cc] << 3 | cez[2 * (size_t)cc], cfp[2 * (size_t)cc + 1] << 3 | cez[2 * (size_t)cc + 1]);
    }
    std::vector<float> fac(A), w1(A), w2(A);
    for (int a = 0; a < A; ++a) {
      fac[a] = (float)q->angDerivFac[a]; w1[a] = (float)q->quadTauW1[a]; w2[a] = (float)q->quadTauW2[a];
    }
    rc = upload(&r->corner32, corner.data(), (size_t)nc);
    if (!rc) rc = upload(&r->link32, link.data(), (size_t)nc);
    if (!rc) rc = upload(&r->fac32, fac.data(), (size_t)A);
    if (!rc) rc = upload(&r->W1_32, w1.data(), (size_t)A);
    if (!rc) rc = upload(&r->W2_32, w2.data(), (size_t)A);
    if (rc) return rc;
    const size_t nAC = (size_t)A * nc;
    if (cudaMalloc((void **)&r->recA, nAC * sizeof(float4)) != cudaSuccess ||
        cudaMalloc((void **)&r->recB, nAC * sizeof(float4)) != cudaSuccess ||
        cudaMalloc((void **)&r->PsiM32, (size_t)nLevels * nc * ngr * sizeof(float)) != cudaSuccess)
      return set_error(UMT_ERR_NOMEM, "RZ: FP32 record allocation failed");
    const size_t nAZ = (size_t)A * nz;
    k_rz_prep32<<<(unsigned)((nAZ + 255) / 256), 256>>>(A, nz, nc, c.numCorner, c.cOffSet, r->cEZ2, c.afp64, c.aez64,
                                                         r->Area, r->RadiusFP, r->RadiusEZ, r->angDerivFac, r->recA,
                                                         r->recB);
    UMT_CUDA(cudaGetLastError());
    UMT_CUDA(cudaDeviceSynchronize());
  }
  return 0;
}

// FP32: conversions, stages and tally replayed from one CUDA graph per
// buffer parity (captured again when tau, a kernel argument, changes);
// PsiB crosses the host link in FP64 through the context's staging buffer.
static int sweep_rz32(Ctx &c, RZData &r, int savePsi, double *PhiTotal, double *PsiB_inout) {
  const size_t ncG = (size_t)c.nc * c.G, psiBN = (size_t)c.A * c.nb * c.G;
  if (PsiB_inout) {
    double *tmp = nullptr;
    TRY_RC(staging_buffer64(c, psiBN, &tmp));
    UMT_CUDA(cudaMemcpyAsync(tmp, PsiB_inout, psiBN * 8, cudaMemcpyHostToDevice, c.stream));
    k_rz_to_float<<<4096, 256, 0, c.stream>>>(psiBN, tmp, c.psiB32);
  }
  if (r.graphTau != c.tau) {
    destroy_rz_graphs(r);
    r.graphTau = c.tau;
  }
  cudaGraphExec_t &ex = r.graph32[c.cur32];
  if (!ex) {
    cudaGraph_t gr = nullptr;
    UMT_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
    const int rc = enqueue_sweep_rz32(c, r);
    const cudaError_t e = cudaStreamEndCapture(c.stream, &gr);
    if (rc) { if (gr) cudaGraphDestroy(gr); return rc; }
    if (e != cudaSuccess) return set_error(UMT_ERR_CUDA, "RZ graph capture: %s", cudaGetErrorString(e));
    const cudaError_t ei = cudaGraphInstantiate(&ex, gr, 0);
    cudaGraphDestroy(gr);
    if (ei != cudaSuccess) { ex = nullptr; return set_error(UMT_ERR_CUDA, "RZ graph instantiate: %s", cudaGetErrorString(ei)); }
  }
  UMT_CUDA(cudaEventRecord(c.ev0, c.stream));
  UMT_CUDA(cudaGraphLaunch(ex, c.stream));
  UMT_CUDA(cudaEventRecord(c.ev1, c.stream));
  if (PhiTotal) UMT_CUDA(cudaMemcpyAsync(PhiTotal, c.Phi, ncG * 8, cudaMemcpyDeviceToHost, c.stream));
  if (PsiB_inout) {
    // the staging copy still holds the caller's rows: only the written ones change
    double *tmp = nullptr;
    TRY_RC(staging_buffer64(c, psiBN, &tmp));
    if (!r.bFace2) {
      if (cudaMalloc((void **)&r.bFace2, (size_t)std::max(c.nb, 1) * sizeof(int)) != cudaSuccess) {
        r.bFace2 = nullptr;
        return set_error(UMT_ERR_NOMEM, "RZ boundary face map: allocation failed");
      }
      UMT_CUDA(cudaMemsetAsync(r.bFace2, 0xff, (size_t)std::max(c.nb, 1) * sizeof(int), c.stream));
      k_rz_bface<<<(c.nc + 255) / 256, 256, 0, c.stream>>>(c.nc, c.nb, r.cFP2, r.bFace2);
    }
    k_rz_psib_out<<<4096, 256, 0, c.stream>>>(c.A, c.nb, c.nc, c.G, r.bFace2, c.afp64, r.nextFinishing, c.psiB32,
                                              tmp);
    UMT_CUDA(cudaGetLastError());
    UMT_CUDA(cudaMemcpyAsync(PsiB_inout, tmp, psiBN * 8, cudaMemcpyDeviceToHost, c.stream));
  }
  UMT_CUDA(cudaStreamSynchronize(c.stream));
  cudaEventElapsedTime(&c.lastMs, c.ev0, c.ev1);
  if (savePsi) c.cur32 = 1 - c.cur32;
  return 0;
}

int umt103_sweep_rz(const double *STotal, int savePsi, double *PhiTotal, double *PsiB_inout, int precision) {
  Ctx &c = cur();
  if (!c.ready || !c.rz) return set_error(UMT_ERR_STATE, "umt103_init_rz not called");
  if (precision != UMT_FP64 && precision != UMT_FP32) return set_error(UMT_ERR_ARG, "precision must be UMT_FP64 or UMT_FP32");
  if (precision == UMT_FP64 && !c.psi64[0]) return set_error(UMT_ERR_STATE, "FP64 flux not allocated (init flags)");
  if (precision == UMT_FP32 && (!c.psi32[0] || !c.rz->recA)) return set_error(UMT_ERR_STATE, "FP32 flux not allocated (init flags)");
  RZData &r = *c.rz;
  const size_t ncG = (size_t)c.nc * c.G, psiBN = (size_t)c.A * c.nb * c.G;
  if (STotal) UMT_CUDA(cudaMemcpyAsync(c.STotal, STotal, ncG * 8, cudaMemcpyHostToDevice, c.stream));
  else UMT_CUDA(cudaMemsetAsync(c.STotal, 0, ncG * 8, c.stream));
  if (precision == UMT_FP32) return sweep_rz32(c, r, savePsi, PhiTotal, PsiB_inout);
  if (PsiB_inout) UMT_CUDA(cudaMemcpyAsync(c.psiB64, PsiB_inout, psiBN * 8, cudaMemcpyHostToDevice, c.stream));
  UMT_CUDA(cudaMemsetAsync(r.PsiM, 0, (size_t)r.nLevels * ncG * 8, c.stream));
  RZP p;
  p.nz = c.nz; p.nc = c.nc; p.nb = c.nb; p.G = c.G;
  p.items = r.items; p.order = c.sch.order;
  p.numCorner = c.numCorner; p.cOffSet = c.cOffSet; p.cFP2 = r.cFP2; p.cEZ2 = r.cEZ2;
  p.afp = c.afp64; p.aez = c.aez64;
  p.Area = r.Area; p.Volume = c.Volume; p.RadiusFP = r.RadiusFP; p.RadiusEZ = r.RadiusEZ;
  p.Sigt = c.Sigt; p.STotal = c.STotal; p.tau = c.tau;
  p.angDerivFac = r.angDerivFac; p.W1 = r.W1; p.W2 = r.W2;
  p.starting = r.starting; p.nextFinishing = r.nextFinishing; p.level = r.level;
  p.psi_old = c.psi64[c.cur64]; p.psi_new = c.psi64[1 - c.cur64]; p.psiB = c.psiB64; p.PsiM = r.PsiM;
  int GT = 1;
  while (GT < c.G && GT < 32) GT *= 2;
  const int TEAMS = RZ_NT / GT;
  UMT_CUDA(cudaEventRecord(c.ev0, c.stream));
  for (int s = 0; s < r.nStages; ++s) {
    if (r.hCount[s] == 0) continue;
    p.stageBegin = r.hOffset[s];
    p.stageCount = r.hCount[s];
    const int blocks = (r.hCount[s] + TEAMS - 1) / TEAMS;
    switch (GT) {
      case 1: k_sweep_rz<1><<<blocks, RZ_NT, 0, c.stream>>>(p); break;
      case 2: k_sweep_rz<2><<<blocks, RZ_NT, 0, c.stream>>>(p); break;
      case 4: k_sweep_rz<4><<<blocks, RZ_NT, 0, c.stream>>>(p); break;
      case 8: k_sweep_rz<8><<<blocks, RZ_NT, 0, c.stream>>>(p); break;
      case 16: k_sweep_rz<16><<<blocks, RZ_NT, 0, c.stream>>>(p); break;
      default: k_sweep_rz<32><<<blocks, RZ_NT, 0, c.stream>>>(p); break;
    }
  }
  UMT_CUDA(cudaGetLastError());
  // PhiTotal = sum_a w_a psi_a (starting and finishing directions weigh 0)
  int rc = launch_tally(c, UMT_FP64);
  if (rc) return rc;
  UMT_CUDA(cudaEventRecord(c.ev1, c.stream));
  UMT_CUDA(cudaStreamSynchronize(c.stream));
  cudaEventElapsedTime(&c.lastMs, c.ev0, c.ev1);
  if (PhiTotal) UMT_CUDA(cudaMemcpy(PhiTotal, c.Phi, ncG * 8, cudaMemcpyDeviceToHost));
  if (PsiB_inout) UMT_CUDA(cudaMemcpy(PsiB_inout, c.psiB64, psiBN * 8, cudaMemcpyDeviceToHost));
  if (savePsi) c.cur64 = 1 - c.cur64;
  return 0;
}

int umt103_get_geometry_rz(double *Area, double *Volume, double *RadiusFP, double *RadiusEZ) {
  Ctx &c = cur();
  if (!c.ready || !c.rz) return set_error(UMT_ERR_STATE, "umt103_init_rz not called");
  const RZData &r = *c.rz;
  if (Area) std::copy(r.hArea.begin(), r.hArea.end(), Area);
  if (Volume) std::copy(r.hVolume.begin(), r.hVolume.end(), Volume);
  if (RadiusFP) std::copy(r.hRfp.begin(), r.hRfp.end(), RadiusFP);
  if (RadiusEZ) std::copy(r.hRez.begin(), r.hRez.end(), RadiusEZ);
  return 0;
}

}  // extern "C"
