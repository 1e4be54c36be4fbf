// sweep.cu -- the upstream-corner-balance sweep, the psi->phi tally and the
// source/energy helpers.
//
// Work decomposition: the schedule orders every (direction, zone) pair into
// dependency stages; one kernel per stage processes all pairs of the stage,
// for every direction at once.  A team of GT consecutive lanes owns one
// (direction, zone) pair and walks its groups g = lane, lane+GT, ...; the
// zone's corner-face data (Omega.A, neighbour corners, volumes) is staged
// once per team in shared memory and read by all lanes.  Psi is stored
// group-innermost, [direction][corner][group], so a team's loads and stores
// of one corner are one contiguous segment.  The per-stage launches of a
// whole sweep, plus the tally, are captured once into a CUDA graph.
//
// Arithmetic per (corner, group) restates snac/SweepUCBxyz.F90:103-312 in the
// same operation order (FP64 instantiation is the parity path; the FP32
// instantiation is the production path).
#include "umt_common.cuh"

namespace umt {

#define TRY_RC(x) do { int rc_ = (x); if (rc_) return rc_; } while (0)

template <typename T>
struct SweepP {
  int nz, nc, nb, A, G;
  const uint32_t *items;
  const int *stageOffset, *stageCount;
  const uint32_t *order;
  const int *numCorner, *cOffSet, *nCFaces, *cFP, *cEZ;
  const T *afp, *aez;
  const double *Volume;
  const T *Sigt, *STotal;
  T tau;
  const T *psi_old;
  T *psi_new, *psiB;
};

constexpr int SWEEP_NT = 128;

// Per (direction, zone) the team first classifies the zone's corner faces
// once, into integer masks (incoming FP faces, exiting boundary faces, EZ
// faces that carry flux, and of those the ones whose opposite FP face is
// incoming), so that the per-group loop runs no floating-point comparison of
// geometry.  With PRE (four or more lanes per zone) it also forms, per EZ
// face that carries flux, the coefficients of the closure as polynomials in
// the group's total opacity s = sigma_t:
//   gnum   = aez^2 (1.82 s^2 V^2 + 4 aez s V + 3 aez^2) = (k0 s + k1) s + k2
//   gden   = V (4 s^3 V^3 + 6 aez s^2 V^2 + 4 aez^2 s V + 2 aez^3)
//          = ((k3 s + k4) s + k5) s + k6,                       k7 = aez/2
//   sez    = (V gnum (s psi_opp - Qc) + k7 gden (Qc - Qz)) / (gnum + gden s)
// (SweepUCBxyz.F90:219-243 with the products over the corner and face
// gathered), so a group pays 5 FMAs for both polynomials instead of forming
// them from the products again.  GB300's FP64 pipe executes two lanes per
// clock per SM, and this kernel's time is its FP64 instruction count.
template <typename T, int GT>
__global__ void __launch_bounds__(SWEEP_NT) k_sweep(SweepP<T> p, int stage) {
  constexpr int TEAMS = SWEEP_NT / GT;
  constexpr bool PRE = GT >= 4;
  constexpr int KT = PRE ? TEAMS : 1;
  __shared__ T s_src[UMT_MAXCORNER][SWEEP_NT];
  __shared__ T s_Q[UMT_MAXCORNER][SWEEP_NT];
  __shared__ T s_psi[UMT_MAXCORNER][SWEEP_NT];
  __shared__ T s_afp[TEAMS][UMT_MAXCORNER][UMT_MAXCF];
  __shared__ T s_aez[TEAMS][UMT_MAXCORNER][UMT_MAXCF];
  __shared__ T s_sum[TEAMS][UMT_MAXCORNER];
  __shared__ T s_vol[TEAMS][UMT_MAXCORNER];
  __shared__ T s_k[KT][UMT_MAXCORNER][UMT_MAXCF][8];
  __shared__ int s_cfp[TEAMS][UMT_MAXCORNER][UMT_MAXCF];
  __shared__ int8_t s_cez[TEAMS][UMT_MAXCORNER][UMT_MAXCF];
  __shared__ uint8_t s_in[TEAMS][UMT_MAXCORNER], s_ex[TEAMS][UMT_MAXCORNER];
  __shared__ uint8_t s_ez[TEAMS][UMT_MAXCORNER], s_opp[TEAMS][UMT_MAXCORNER];
  __shared__ int s_anyNoOpp[TEAMS];

  const int tid = threadIdx.x, team = tid / GT, lane = tid % GT;
  const int k = blockIdx.x * TEAMS + team;
  const int cnt = p.stageCount[stage];
  if (k >= cnt) return;                       // whole teams leave together
  const unsigned teammask = (GT == 32) ? 0xffffffffu : (((1u << GT) - 1u) << ((tid & 31) / GT * GT));
  uint32_t it = p.items[p.stageOffset[stage] + k];
  const bool bad = (it >> 31) != 0;
  it &= 0x7fffffffu;
  const int a = (int)(it / (uint32_t)p.nz);
  const int z = (int)(it - (uint32_t)a * p.nz);
  const int nCorner = p.numCorner[z], c0 = p.cOffSet[z];
  const uint32_t ord = p.order[it];
  const size_t abase = (size_t)a * p.nc;

  if (lane == 0) s_anyNoOpp[team] = 0;
  __syncwarp(teammask);
  for (int c = lane; c < nCorner; c += GT) {
    const int cc = c0 + c;
    const int ncf = p.nCFaces[cc];
    const T vol = (T)p.Volume[cc];
    s_vol[team][c] = vol;
    T sum = T(0), af[UMT_MAXCF];
    uint32_t in = 0, ex = 0, ez = 0, opp = 0;
#pragma unroll
    for (int cf = 0; cf < UMT_MAXCF; ++cf) {
      const T v = p.afp[(abase + cc) * UMT_MAXCF + cf];
      const int cfp = p.cFP[cc * UMT_MAXCF + cf];
      af[cf] = v;
      s_afp[team][c][cf] = v;
      s_cfp[team][c][cf] = cfp;
      if (cf < ncf && v > T(0)) {
        sum = sum + v;
        if (cfp >= p.nc) ex |= 1u << cf;
      }
      if (cf < ncf && v < T(0)) in |= 1u << cf;
    }
#pragma unroll
    for (int cf = 0; cf < UMT_MAXCF; ++cf) {
      const T v = p.aez[(abase + cc) * UMT_MAXCF + cf];
      s_aez[team][c][cf] = v;
      s_cez[team][c][cf] = (int8_t)p.cEZ[cc * UMT_MAXCF + cf];
      if (cf < ncf && v > T(0)) {
        sum = sum + v;
        ez |= 1u << cf;
        const bool o = ncf == 3 && af[(cf + 1) % 3] < T(0);
        if (o) opp |= 1u << cf;
        else s_anyNoOpp[team] = 1;
        if constexpr (PRE) {
          if (o) {
            const T aez2 = v * v, V2 = vol * vol;
            T *kc = s_k[team][c][cf];
            kc[0] = T(1.82) * aez2 * V2;
            kc[1] = T(4) * aez2 * v * vol;
            kc[2] = T(3) * aez2 * aez2;
            kc[3] = T(4) * V2 * V2;
            kc[4] = T(6) * v * V2 * vol;
            kc[5] = T(4) * aez2 * V2;
            kc[6] = T(2) * aez2 * v * vol;
            kc[7] = T(0.5) * v;
          }
        }
      }
    }
    s_sum[team][c] = sum;
    s_in[team][c] = (uint8_t)in;
    s_ex[team][c] = (uint8_t)ex;
    s_ez[team][c] = (uint8_t)ez;
    s_opp[team][c] = (uint8_t)opp;
  }
  __syncwarp(teammask);

  const T fouralpha = T(1.82);
  const T *sigz = p.Sigt + (size_t)z * p.G;
  const bool anyNoOpp = s_anyNoOpp[team] != 0;
  for (int g = lane; g < p.G; g += GT) {
    const T sig = sigz[g];
    const T sigInv = anyNoOpp ? T(1) / sig : T(0);
    for (int c = 0; c < nCorner; ++c) {
      const size_t e = (size_t)(c0 + c) * p.G + g;
      const T st = p.STotal ? p.STotal[e] : T(0);
      const T q = st + p.tau * p.psi_old[abase * p.G + e];
      s_Q[c][tid] = q;
      s_src[c][tid] = s_vol[team][c] * q;
    }
    for (int c = 0; c < nCorner; ++c) {
      const uint32_t in = s_in[team][c], ezm = s_ez[team][c], opp = s_opp[team][c];
      T psifp[UMT_MAXCF];
      T srcc = s_src[c][tid];
#pragma unroll
      for (int cf = 0; cf < UMT_MAXCF; ++cf) {
        psifp[cf] = T(0);
        if ((in >> cf) & 1u) {
          const int cfp = s_cfp[team][c][cf];
          const T pu = (cfp < p.nc) ? p.psi_new[(abase + cfp) * p.G + g]
                                    : p.psiB[((size_t)a * p.nb + (cfp - p.nc)) * p.G + g];
          psifp[cf] = pu;
          srcc = srcc - s_afp[team][c][cf] * pu;
        }
      }
      s_src[c][tid] = srcc;
      const T Qc = s_Q[c][tid];
#pragma unroll
      for (int cf = 0; cf < UMT_MAXCF; ++cf) {
        if ((ezm >> cf) & 1u) {
          const int cez = s_cez[team][c][cf];
          const T Qz = s_Q[cez][tid];
          T sez;
          if ((opp >> cf) & 1u) {
            const T psi_opp = psifp[(cf + 1) % 3];
            const T vol = s_vol[team][c];
            T gnum, gden, half_aez;
            if constexpr (PRE) {
              const T *kc = s_k[team][c][cf];
              gnum = (kc[0] * sig + kc[1]) * sig + kc[2];
              gden = ((kc[3] * sig + kc[4]) * sig + kc[5]) * sig + kc[6];
              half_aez = kc[7];
            } else {
              const T aez = s_aez[team][c][cf];
              const T aez2 = aez * aez;
              const T sigv = sig * vol;
              const T sigv2 = sigv * sigv;
              gnum = aez2 * (fouralpha * sigv2 + aez * (T(4) * sigv + T(3) * aez));
              gden = vol * (T(4) * sigv * sigv2 + aez * (T(6) * sigv2 + T(2) * aez * (T(2) * sigv + aez)));
              half_aez = T(0.5) * aez;
            }
            sez = (vol * gnum * (sig * psi_opp - Qc) + half_aez * gden * (Qc - Qz)) / (gnum + gden * sig);
          } else {
            sez = T(0.5) * s_aez[team][c][cf] * sigInv * (Qc - Qz);
          }
          s_src[c][tid] = s_src[c][tid] + sez;
          s_src[cez][tid] = s_src[cez][tid] - sez;
        }
      }
    }
    T *out = p.psi_new + abase * p.G;
    if (!bad) {
      for (int i = 0; i < nCorner; ++i) {
        const int c = (int)((ord >> (4 * i)) & 15u);
        const T v = s_src[c][tid] / (s_sum[team][c] + sig * s_vol[team][c]);
        out[(size_t)(c0 + c) * p.G + g] = v;
        s_psi[c][tid] = v;
        const uint32_t ezm = s_ez[team][c];
#pragma unroll
        for (int cf = 0; cf < UMT_MAXCF; ++cf) {
          if ((ezm >> cf) & 1u) {
            const int cez = s_cez[team][c][cf];
            s_src[cez][tid] = s_src[cez][tid] + s_aez[team][c][cf] * v;
          }
        }
      }
    } else {
      // direct solve with the previous iterate of this zone (SweepUCBxyz.F90:283-297)
      for (int c = 0; c < nCorner; ++c) {
        const T old = out[(size_t)(c0 + c) * p.G + g];
        const uint32_t ezm = s_ez[team][c];
        for (int cf = 0; cf < UMT_MAXCF; ++cf) {
          if ((ezm >> cf) & 1u) {
            const int cez = s_cez[team][c][cf];
            s_src[cez][tid] = s_src[cez][tid] + s_aez[team][c][cf] * old;
          }
        }
      }
      for (int c = 0; c < nCorner; ++c) {
        const T v = s_src[c][tid] / (s_sum[team][c] + sig * s_vol[team][c]);
        out[(size_t)(c0 + c) * p.G + g] = v;
        s_psi[c][tid] = v;
      }
    }
    // exiting boundary fluxes
    for (int c = 0; c < nCorner; ++c) {
      const uint32_t ex = s_ex[team][c];
      for (int cf = 0; cf < UMT_MAXCF; ++cf)
        if ((ex >> cf) & 1u) {
          const int cfp = s_cfp[team][c][cf];
          p.psiB[((size_t)a * p.nb + (cfp - p.nc)) * p.G + g] = s_psi[c][tid];
        }
    }
  }
}

// The grey problem's sweep (one group, FP64: the GTA grey and zone-solve
// sweeps).  With one group a (direction, zone) pair has no group loop to
// spread over lanes, and one lane per pair made every stage as long as one
// zone's serial chain of corner work.  Here a team of 8 lanes owns a pair,
// lane c the zone's corner c: each lane stages its corner's faces, forms its
// source and inflow, and computes the EZ closure of the faces its corner owns
// (aez > 0) into shared memory.  Each corner then gathers the closures of
// its own faces (+) and of its neighbours' faces toward it (-) in face order;
// only the corner solve, in the schedule's corner order, runs one corner at a
// time.  Arithmetic per face and corner is SweepUCBxyz.F90's (IEEE
// division); the sums over a corner's faces are taken in face order rather
// than in the reference's corner order.
constexpr int GREY_NT = 128, GREY_GT = UMT_MAXCORNER;

__global__ void __launch_bounds__(GREY_NT) k_sweep_grey(SweepP<double> p, int stage) {
  constexpr int TEAMS = GREY_NT / GREY_GT;
  __shared__ double s_Q[TEAMS][UMT_MAXCORNER], s_src[TEAMS][UMT_MAXCORNER], s_psi[TEAMS][UMT_MAXCORNER];
  __shared__ double s_sez[TEAMS][UMT_MAXCORNER][UMT_MAXCF];
  __shared__ int8_t s_cez[TEAMS][UMT_MAXCORNER][UMT_MAXCF];
  const int tid = threadIdx.x, team = tid / GREY_GT, c = tid % GREY_GT;
  const int k = blockIdx.x * TEAMS + team;
  if (k >= p.stageCount[stage]) return;            // whole teams leave together
  const unsigned tm = 0xffu << ((tid & 31) / GREY_GT * GREY_GT);
  uint32_t it = p.items[p.stageOffset[stage] + k];
  const bool bad = (it >> 31) != 0;
  it &= 0x7fffffffu;
  const int a = (int)(it / (uint32_t)p.nz);
  const int z = (int)(it - (uint32_t)a * p.nz);
  const int nCorner = p.numCorner[z], c0 = p.cOffSet[z];
  const uint32_t ord = p.order[it];
  const size_t abase = (size_t)a * p.nc;
  const bool own = c < nCorner;
  const int cc = c0 + c;
  double af[UMT_MAXCF] = {0.0, 0.0, 0.0}, ae[UMT_MAXCF] = {0.0, 0.0, 0.0}, psifp[UMT_MAXCF] = {0.0, 0.0, 0.0};
  int cfp[UMT_MAXCF] = {0, 0, 0}, cez[UMT_MAXCF] = {0, 0, 0};
  uint32_t in = 0, ex = 0, ezm = 0, opp = 0;
  int ncf = 0;
  double vol = 0.0, sum = 0.0, src = 0.0, Q = 0.0;
  const double sig = p.Sigt[z];
  if (own) {
    ncf = p.nCFaces[cc];
    vol = p.Volume[cc];
#pragma unroll
    for (int f = 0; f < UMT_MAXCF; ++f) {
      af[f] = p.afp[(abase + cc) * UMT_MAXCF + f];
      cfp[f] = p.cFP[cc * UMT_MAXCF + f];
      if (f < ncf && af[f] > 0.0) { sum += af[f]; if (cfp[f] >= p.nc) ex |= 1u << f; }
      if (f < ncf && af[f] < 0.0) in |= 1u << f;
    }
#pragma unroll
    for (int f = 0; f < UMT_MAXCF; ++f) {
      ae[f] = p.aez[(abase + cc) * UMT_MAXCF + f];
      cez[f] = p.cEZ[cc * UMT_MAXCF + f];
      s_cez[team][c][f] = (int8_t)(f < ncf ? cez[f] : -1);
      if (f < ncf && ae[f] > 0.0) {
        sum += ae[f];
        ezm |= 1u << f;
        if (ncf == 3 && af[(f + 1) % 3] < 0.0) opp |= 1u << f;
      }
    }
    const double st = p.STotal ? p.STotal[cc] : 0.0;
    Q = st + p.tau * p.psi_old[abase + cc];
    src = vol * Q;
    s_Q[team][c] = Q;
#pragma unroll
    for (int f = 0; f < UMT_MAXCF; ++f)
      if ((in >> f) & 1u) {
        const double pu = (cfp[f] < p.nc) ? p.psi_new[abase + cfp[f]]
                                          : p.psiB[(size_t)a * p.nb + (cfp[f] - p.nc)];
        psifp[f] = pu;
        src = src - af[f] * pu;
      }
  }
  __syncwarp(tm);
  if (own) {
#pragma unroll
    for (int f = 0; f < UMT_MAXCF; ++f) {
      s_sez[team][c][f] = 0.0;                     // faces this corner does not own
      if (!((ezm >> f) & 1u)) continue;
      const double aez = ae[f];
      const double Qz = s_Q[team][cez[f]];
      double sez;
      if ((opp >> f) & 1u) {
        const double psi_opp = psifp[(f + 1) % 3];
        const double aez2 = aez * aez;
        const double sigv = sig * vol;
        const double sigv2 = sigv * sigv;
        const double gnum = aez2 * (1.82 * sigv2 + aez * (4.0 * sigv + 3.0 * aez));
        const double gden = vol * (4.0 * sigv * sigv2 + aez * (6.0 * sigv2 + 2.0 * aez * (2.0 * sigv + aez)));
        sez = (vol * gnum * (sig * psi_opp - Q) + 0.5 * aez * gden * (Q - Qz)) / (gnum + gden * sig);
      } else {
        sez = 0.5 * aez * (1.0 / sig) * (Q - Qz);
      }
      s_sez[team][c][f] = sez;
    }
  }
  __syncwarp(tm);
  if (own) {
#pragma unroll
    for (int f = 0; f < UMT_MAXCF; ++f) {
      if (f >= ncf) continue;
      if ((ezm >> f) & 1u) {
        src = src + s_sez[team][c][f];
      } else if (ae[f] < 0.0) {
        const int o = cez[f];                      // the neighbour corner owns this face
        for (int g = 0; g < UMT_MAXCF; ++g)
          if (s_cez[team][o][g] == c) { src = src - s_sez[team][o][g]; break; }
      }
    }
    s_src[team][c] = src;
  }
  __syncwarp(tm);
  double *out = p.psi_new + abase;
  const double den = sum + sig * vol;
  if (!bad) {
    for (int i = 0; i < nCorner; ++i) {
      if (c == (int)((ord >> (4 * i)) & 15u)) {
        const double v = s_src[team][c] / den;
        out[cc] = v;
        s_psi[team][c] = v;
#pragma unroll
        for (int f = 0; f < UMT_MAXCF; ++f)
          if ((ezm >> f) & 1u) s_src[team][cez[f]] += ae[f] * v;
      }
      __syncwarp(tm);
    }
  } else {
    // direct solve with the previous iterate of this zone (SweepUCBxyz.F90:283-297)
    for (int i = 0; i < nCorner; ++i) {
      if (c == i) {
        const double old = out[cc];
#pragma unroll
        for (int f = 0; f < UMT_MAXCF; ++f)
          if ((ezm >> f) & 1u) s_src[team][cez[f]] += ae[f] * old;
      }
      __syncwarp(tm);
    }
    if (own) {
      const double v = s_src[team][c] / den;
      out[cc] = v;
      s_psi[team][c] = v;
    }
  }
  __syncwarp(tm);
  if (own) {
#pragma unroll
    for (int f = 0; f < UMT_MAXCF; ++f)
      if ((ex >> f) & 1u) p.psiB[(size_t)a * p.nb + (cfp[f] - p.nc)] = s_psi[team][c];
  }
}

// psi -> phi tally: PhiTotal(g,c) = sum_a w_a psi_a(g,c), accumulated in FP64
// (control/getPhiTotal_OMPOL.F90:63-131 does the same per direction).
// FP32 angular flux: each thread owns 4 consecutive (corner, group) entries
// and sums w_a*psi_a over the directions with compensated (Kahan) FP32
// summation, the product entering each step unrounded; the sum and its
// compensation are combined in FP64 at the end.  The error is a few FP32 ulps
// of the sum whatever the number of directions, and the loop holds no FP64
// operation: GB300's FP64 rate is 1/64 of FP32, and FP64 accumulation kept
// the FP64 pipe ~60% busy and this pass below the read bandwidth.  Each
// thread has 16 float4 loads in flight.
__device__ __forceinline__ void kahan_add(float &s, float &c, float w, float x) {
  const float y = fmaf(w, x, -c);           // the product enters unrounded
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

// WT: PhiTotal also goes to *phiOut (the caller's page-locked array) when set.
template <bool WT>
__global__ void __launch_bounds__(256) k_tally32(int A, size_t ncG, const float *__restrict__ w32,
                                                 const float *__restrict__ psi, double *__restrict__ Phi,
                                                 double *const *phiOut) {
  constexpr int U = 16;                       // float4 loads per thread per step
  const size_t n4 = ncG / 4;
  double *host = nullptr;
  if constexpr (WT) host = *phiOut;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n4; q += (size_t)gridDim.x * blockDim.x) {
    float s[4] = {0.f, 0.f, 0.f, 0.f}, c[4] = {0.f, 0.f, 0.f, 0.f};
    const float *p = psi + 4 * q;
    int a = 0;
    for (; a + U <= A; a += U) {
      float4 v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) v[u] = *reinterpret_cast<const float4 *>(p + (size_t)(a + u) * ncG);
      asm volatile("" ::: "memory");          // compiler barrier between the loads and the sums
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const float w = w32[a + u];
        kahan_add(s[0], c[0], w, v[u].x); kahan_add(s[1], c[1], w, v[u].y);
        kahan_add(s[2], c[2], w, v[u].z); kahan_add(s[3], c[3], w, v[u].w);
      }
    }
    for (; a < A; ++a) {
      const float w = w32[a];
      const float4 v = *reinterpret_cast<const float4 *>(p + (size_t)a * ncG);
      kahan_add(s[0], c[0], w, v.x); kahan_add(s[1], c[1], w, v.y);
      kahan_add(s[2], c[2], w, v.z); kahan_add(s[3], c[3], w, v.w);
    }
    const double2 lo = make_double2((double)s[0] - (double)c[0], (double)s[1] - (double)c[1]);
    const double2 hi = make_double2((double)s[2] - (double)c[2], (double)s[3] - (double)c[3]);
    *reinterpret_cast<double2 *>(Phi + 4 * q) = lo;
    *reinterpret_cast<double2 *>(Phi + 4 * q + 2) = hi;
    if constexpr (WT) {
      if (host) {
        *reinterpret_cast<double2 *>(host + 4 * q) = lo;
        *reinterpret_cast<double2 *>(host + 4 * q + 2) = hi;
      }
    }
  }
  for (size_t e = 4 * n4 + blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < ncG; e += (size_t)gridDim.x * blockDim.x) {
    double t = 0.0;
    for (int a = 0; a < A; ++a) t += (double)(w32[a] * psi[(size_t)a * ncG + e]);
    Phi[e] = t;
    if constexpr (WT) {
      if (host) host[e] = t;
    }
  }
}

// FP64 angular flux (parity path): FP64 products and sums; each thread owns 4
// consecutive entries and walks the directions with 4 independent partial sums.
template <typename T>
__global__ void __launch_bounds__(256) k_tally(int A, size_t ncG, const double *weight, const T *psi, double *Phi) {
  const size_t n4 = ncG / 4;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n4; q += (size_t)gridDim.x * blockDim.x) {
    double s[4][4] = {};
    int a = 0;
    for (; a + 4 <= A; a += 4) {
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const double w = weight[a + u];
        const T *p = psi + (size_t)(a + u) * ncG + 4 * q;
        if constexpr (sizeof(T) == 4) {
          const float4 v = *reinterpret_cast<const float4 *>(p);
          s[u][0] += w * v.x; s[u][1] += w * v.y; s[u][2] += w * v.z; s[u][3] += w * v.w;
        } else {
          const double2 v0 = *reinterpret_cast<const double2 *>(p);
          const double2 v1 = *reinterpret_cast<const double2 *>(p + 2);
          s[u][0] += w * v0.x; s[u][1] += w * v0.y; s[u][2] += w * v1.x; s[u][3] += w * v1.y;
        }
      }
    }
    for (; a < A; ++a) {
      const double w = weight[a];
      const T *p = psi + (size_t)a * ncG + 4 * q;
      for (int j = 0; j < 4; ++j) s[0][j] += w * (double)p[j];
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) Phi[4 * q + j] = (s[0][j] + s[1][j]) + (s[2][j] + s[3][j]);
  }
  // remainder entries (ncG not a multiple of 4)
  for (size_t e = 4 * n4 + blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < ncG; e += (size_t)gridDim.x * blockDim.x) {
    double t = 0.0;
    for (int a = 0; a < A; ++a) t += weight[a] * (double)psi[(size_t)a * ncG + e];
    Phi[e] = t;
  }
}

__global__ void k_to_float(size_t n, const double *x, float *y) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] = (float)x[i];
}

template <typename T>
static int enqueue_sweep(Ctx &c, int cur) {
  SweepP<T> p;
  p.nz = c.nz; p.nc = c.nc; p.nb = c.nb; p.A = c.A; p.G = c.G;
  p.items = c.sch.items; p.stageOffset = c.sch.stageOffset; p.stageCount = c.sch.stageCount;
  p.order = c.sch.order;
  p.numCorner = c.numCorner; p.cOffSet = c.cOffSet; p.nCFaces = c.nCFaces; p.cFP = c.cFP; p.cEZ = c.cEZ;
  p.Volume = c.Volume;
  p.tau = (T)c.tau;
  if constexpr (sizeof(T) == 8) {
    p.afp = (const T *)c.afp64; p.aez = (const T *)c.aez64;
    p.Sigt = (const T *)c.Sigt; p.STotal = (const T *)c.STotal;
    p.psi_old = (const T *)c.psi64[cur]; p.psi_new = (T *)c.psi64[1 - cur]; p.psiB = (T *)c.psiB64;
  } else {
    p.afp = (const T *)c.afp32; p.aez = (const T *)c.aez32;
    p.Sigt = (const T *)c.Sigt32; p.STotal = (const T *)c.STotal32;
    p.psi_old = (const T *)c.psi32[cur]; p.psi_new = (T *)c.psi32[1 - cur]; p.psiB = (T *)c.psiB32;
  }
  const int prec = sizeof(T) == 8 ? 0 : 1;
  int GT = c.sweepGT[prec];
  if (GT <= 0) {
    GT = 1;
    while (GT < c.G && GT < 32) GT *= 2;
    c.sweepGT[prec] = GT;
  }
  const int TEAMS = SWEEP_NT / GT;
  c.launchesPerSweep[prec] = c.sch.nStages + 1 + (sizeof(T) == 4 ? 2 : 0) + (c.sch.nCyc ? 2 : 0);
  bool done = false;
  if constexpr (sizeof(T) == 4) {
    c.exitsThrough = false;                   // set again by the zone-program path below
    const size_t n = (size_t)c.nz * c.G;
    k_to_float<<<(int)std::min<size_t>((n + 255) / 256, 4096), 256, 0, c.stream>>>(n, c.Sigt, c.Sigt32);
    if (c.tileGT == 0) default_tile(c.G, &c.tileGT, &c.tileGPL);
    // the host-facing zone-program sweep converts the source in stage-ordered
    // chunks beside its stages (enqueue_psib_chunks); every other sweep here
    const bool srcChunks = c.wantExitsThrough && c.wantSrcChunks && c.srcOrder && c.rec32Ready &&
                           c.sweepMode == 0 && c.progState == 1 && c.tileGT > 0 &&
                           sweep32_supported(c.G, c.tileGT, c.tileGPL) &&
                           sweep32p_supported(c.G, c.tileGT, c.tileGPL);
    if (!srcChunks) {
      const size_t m = (size_t)c.nc * c.G;
      k_to_float<<<(int)std::min<size_t>((m + 255) / 256, 4096), 256, 0, c.stream>>>(m, c.STotal, c.STotal32);
    }
    c.srcChunksNow = srcChunks;
    TRY_RC(enqueue_cycle_init(c, prec, cur));
    if (c.tileGT > 0 && sweep32_supported(c.G, c.tileGT, c.tileGPL)) {
      if (!c.rec32Ready) {
        int rc = prepare_sweep32(c);
        if (rc) return rc;
        c.rec32Ready = true;
      }
      int rc = enqueue_sweep32(c, cur, c.tileGT, c.tileGPL);
      if (rc) return rc;
      done = true;
    }
  }
  if constexpr (sizeof(T) == 8) TRY_RC(enqueue_cycle_init(c, prec, cur));
  if constexpr (sizeof(T) == 8) {
    if (c.G == 1 && !done) {                      // the grey problem: a team of lanes per pair, one per corner
      for (int s = 0; s < c.sch.nStages; ++s) {
        const int blocks = (c.sch.hCount[s] + GREY_NT / GREY_GT - 1) / (GREY_NT / GREY_GT);
        k_sweep_grey<<<blocks, GREY_NT, 0, c.stream>>>(p, s);
      }
      done = true;
    }
  }
  for (int s = 0; s < c.sch.nStages && !done; ++s) {
    const int blocks = (c.sch.hCount[s] + TEAMS - 1) / TEAMS;
    switch (GT) {
      case 1: k_sweep<T, 1><<<blocks, SWEEP_NT, 0, c.stream>>>(p, s); break;
      case 2: k_sweep<T, 2><<<blocks, SWEEP_NT, 0, c.stream>>>(p, s); break;
      case 4: k_sweep<T, 4><<<blocks, SWEEP_NT, 0, c.stream>>>(p, s); break;
      case 8: k_sweep<T, 8><<<blocks, SWEEP_NT, 0, c.stream>>>(p, s); break;
      case 16: k_sweep<T, 16><<<blocks, SWEEP_NT, 0, c.stream>>>(p, s); break;
      default: k_sweep<T, 32><<<blocks, SWEEP_NT, 0, c.stream>>>(p, s); break;
    }
  }
  TRY_RC(enqueue_cycle_update(c, prec, cur));
  if (!c.inSIGraph) TRY_RC(record_mid(c));       // no event nodes inside a conditional body
  const size_t ncG = (size_t)c.nc * c.G;
  const int tb = (int)std::min<size_t>((ncG / 4 + 255) / 256 + 1, 152 * 16);
  if constexpr (sizeof(T) == 4) {
    if (c.wantExitsThrough) {
      k_tally32<true><<<tb, 256, 0, c.stream>>>(c.A, ncG, c.weight32, c.psi32[1 - cur], c.Phi, c.phiOut);
      // the last exit chunks are copied out beside the tally
      if (c.exitsThrough) TRY_RC(join_exit_chunks(c));
    } else
      k_tally32<false><<<tb, 256, 0, c.stream>>>(c.A, ncG, c.weight32, c.psi32[1 - cur], c.Phi, nullptr);
  } else {
    k_tally<double><<<tb, 256, 0, c.stream>>>(c.A, ncG, c.weight, c.psi64[1 - cur], c.Phi);
  }
  UMT_CUDA(cudaGetLastError());
  return 0;
}

static int prepare_precision(Ctx &c, int precision);

// The parts of a resident FP32 zone-program sweep around its stages, for a
// batch whose stages are launched together (enqueue_batch_stages): before,
// the FP32 copies of the cross sections and the source and the cycle list's
// lagged rows; after, the cycle list's update and the tally.  On c.stream.
int enqueue_sweep32_pre(Ctx &c, int cur) {
  const size_t n = (size_t)c.nz * c.G;
  k_to_float<<<(int)std::min<size_t>((n + 255) / 256, 4096), 256, 0, c.stream>>>(n, c.Sigt, c.Sigt32);
  const size_t m = (size_t)c.nc * c.G;
  k_to_float<<<(int)std::min<size_t>((m + 255) / 256, 4096), 256, 0, c.stream>>>(m, c.STotal, c.STotal32);
  UMT_CUDA(cudaGetLastError());
  return enqueue_cycle_init(c, 1, cur);
}

int enqueue_sweep32_post(Ctx &c, int cur) {
  TRY_RC(enqueue_cycle_update(c, 1, cur));
  const size_t ncG = (size_t)c.nc * c.G;
  const int tb = (int)std::min<size_t>((ncG / 4 + 255) / 256 + 1, 152 * 16);
  k_tally32<false><<<tb, 256, 0, c.stream>>>(c.A, ncG, c.weight32, c.psi32[1 - cur], c.Phi, nullptr);
  UMT_CUDA(cudaGetLastError());
  return 0;
}

// Whether an FP32 sweep of this context runs the zone-program kernel (the
// path of the chunked host-facing graph); prepares the FP32 records first.
int fp32_program_path(Ctx &c, bool *yes) {
  TRY_RC(prepare_precision(c, 1));
  *yes = c.sweepMode == 0 && c.progState == 1 && c.tileGT > 0 && sweep32_supported(c.G, c.tileGT, c.tileGPL) &&
         sweep32p_supported(c.G, c.tileGT, c.tileGPL);
  return 0;
}

// PhiTotal = sum_a w_a psi_a over the new angular flux (psi[1 - cur]) of the
// given precision, on the context's stream.
int launch_tally(Ctx &c, int precision) {
  const size_t ncG = (size_t)c.nc * c.G;
  const int tb = (int)std::min<size_t>((ncG / 4 + 255) / 256 + 1, 152 * 16);
  if (precision == 1)
    k_tally32<false><<<tb, 256, 0, c.stream>>>(c.A, ncG, c.weight32, c.psi32[1 - c.cur32], c.Phi, nullptr);
  else
    k_tally<double><<<tb, 256, 0, c.stream>>>(c.A, ncG, c.weight, c.psi64[1 - c.cur64], c.Phi);
  UMT_CUDA(cudaGetLastError());
  return 0;
}

int record_mid(Ctx &c) {
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  UMT_CUDA(cudaStreamIsCapturing(c.stream, &st));
  if (st == cudaStreamCaptureStatusActive)
    UMT_CUDA(cudaEventRecordWithFlags(c.evMid, c.stream, cudaEventRecordExternal));
  else
    UMT_CUDA(cudaEventRecord(c.evMid, c.stream));
  return 0;
}

// A process-wide counter: every invalidation gives the context a fresh
// generation, so graphs built from its earlier captures (the batch graphs of
// umt103_batch_sweep) are recognised as stale.
static unsigned long long g_graph_gen = 0;

void invalidate_graphs(Ctx &c) {
  c.graphGen = ++g_graph_gen;
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j)
      if (c.graphs[i][j]) { cudaGraphExecDestroy(c.graphs[i][j]); c.graphs[i][j] = nullptr; }
  for (auto &g : c.graphsWT)
    if (g) { cudaGraphExecDestroy(g); g = nullptr; }
  for (auto &g : c.graphsH)
    if (g) { cudaGraphExecDestroy(g); g = nullptr; }
  for (auto &a : c.siGraph)
    for (auto &b : a)
      for (auto &g : b)
        if (g) { cudaGraphExecDestroy(g); g = nullptr; }
}

// Capture one sweep (source conversion, every dependency stage, tally) for
// the current precision and buffer parity into a CUDA graph, once; later
// sweeps replay it with a single launch.
static int sweep_via_graph(Ctx &c, int precision) {
  const int cur = precision == 0 ? c.cur64 : c.cur32;
  cudaGraphExec_t &ex = (precision == 1 && c.homog32) ? c.graphsH[cur]
                        : (precision == 1 && c.wantExitsThrough) ? c.graphsWT[cur] : c.graphs[precision][cur];
  if (!ex) {
    cudaGraph_t gr = nullptr;
    UMT_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
    int rc = precision == 0 ? enqueue_sweep<double>(c, cur) : enqueue_sweep<float>(c, cur);
    cudaError_t e = cudaStreamEndCapture(c.stream, &gr);
    if (rc) { if (gr) cudaGraphDestroy(gr); return rc; }
    if (e != cudaSuccess) return set_error(-3, "graph capture: %s", cudaGetErrorString(e));
    // the host-facing graph runs its nodes at their own priorities (the row
    // copies above the stages)
    e = cudaGraphInstantiate(&ex, gr, precision == 1 && c.wantExitsThrough && !c.homog32
                                          ? cudaGraphInstantiateFlagUseNodePriority : 0);
    cudaGraphDestroy(gr);
    if (e != cudaSuccess) { ex = nullptr; return set_error(-3, "graph instantiate: %s", cudaGetErrorString(e)); }
  }
  UMT_CUDA(cudaGraphLaunch(ex, c.stream));
  return 0;
}

static int prepare_precision(Ctx &c, int precision) {
  // one-time preparation; must not run inside a capture
  if (precision == 1) {
    if (c.tileGT == 0) default_tile(c.G, &c.tileGT, &c.tileGPL);
    if (!c.rec32Ready && c.tileGT > 0) {
      int rc = prepare_sweep32(c);
      if (rc) return rc;
      c.rec32Ready = true;
    }
  }
  return 0;
}

// A fresh, uninstantiated graph of one sweep of this context (the caller owns
// it); used to combine several contexts into one launch.
int capture_sweep_graph(Ctx &c, int precision, cudaGraph_t *out) {
  TRY_RC(prepare_precision(c, precision));
  const int cur = precision == 0 ? c.cur64 : c.cur32;
  UMT_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
  int rc = precision == 0 ? enqueue_sweep<double>(c, cur) : enqueue_sweep<float>(c, cur);
  cudaGraph_t gr = nullptr;
  cudaError_t e = cudaStreamEndCapture(c.stream, &gr);
  if (rc) { if (gr) cudaGraphDestroy(gr); return rc; }
  if (e != cudaSuccess) return set_error(-3, "graph capture: %s", cudaGetErrorString(e));
  *out = gr;
  return 0;
}

int launch_sweep_once(Ctx &c, int precision, bool /*tally*/) {
  if (c.useGraphs) {
    TRY_RC(prepare_precision(c, precision));
    return sweep_via_graph(c, precision);
  }
  if (precision == 0) return enqueue_sweep<double>(c, c.cur64);
  return enqueue_sweep<float>(c, c.cur32);
}


}  // namespace umt
