// sweep32.cu -- production FP32 UCB sweep kernel.
//
// Same arithmetic as snac/SweepUCBxyz.F90:103-312, reorganised for latency and
// SIMT throughput:
//   * a team of GT lanes owns one (direction, zone) pair and each lane owns
//     GPL consecutive groups, so every global and shared access of a corner is
//     one GPL-wide vector per lane;
//   * a zone costs three dependent memory round trips: (1) the packed work
//     item {direction, zone, corner offset, corner count}; (2) at once, the
//     zone's corner records staged cooperatively into shared memory, and every
//     corner's previous-cycle flux and source (loops over the 8 corner slots
//     are unrolled and predicated); (3) at once, every upwind flux of the zone;
//   * per (direction, corner) the FP and EZ projections, the outflow area sum
//     and the corner volume are prepacked (two float4), per corner the
//     connectivity is one int4;
//   * corner-face slots are walked with fixed trip counts (3 FP + 3 EZ) and
//     predicates, so lanes of different zones in one warp stay converged;
//   * the EZ coupling uses the reference's gnum/gden closure with fast
//     reciprocals (the FP64 parity path in sweep.cu keeps IEEE division).
// Corner sources and running sums live in shared memory, [team][corner][group],
// padded so that the teams of one warp fall in different banks.  Each lane
// touches only its own groups there; the staged corner records are shared by
// the team and published with one __syncwarp over the team's lanes.
#include "umt_common.cuh"
#include "sweep32_util.cuh"

namespace umt {

struct Sweep32P {
  int nz, nc, nb, A, G, stride;   // stride: floats per team per array
  const uint2 *items2;
  const int *stageOffset, *stageCount;
  const uint32_t *order;
  const float4 *rec;     // [A][nc][2]
  const int4 *conn;      // [nc]
  const float *Sigt;     // [nz][G]
  const float *STotal;   // [nc][G]
  float tau;
  const float *psi_old;
  float *psi_new, *psiB;
};

template <int N> struct VecT;
template <> struct VecT<1> { using T = float; };
template <> struct VecT<2> { using T = float2; };
template <> struct VecT<4> { using T = float4; };

template <int N>
__device__ __forceinline__ void vload(const float *p, float (&v)[N]) {
  using V = typename VecT<N>::T;
  V t = *reinterpret_cast<const V *>(p);
  const float *f = reinterpret_cast<const float *>(&t);
#pragma unroll
  for (int j = 0; j < N; ++j) v[j] = f[j];
}
template <int N>
__device__ __forceinline__ void vstore(float *p, const float (&v)[N]) {
  using V = typename VecT<N>::T;
  V t;
  float *f = reinterpret_cast<float *>(&t);
#pragma unroll
  for (int j = 0; j < N; ++j) f[j] = v[j];
  *reinterpret_cast<V *>(p) = t;
}

constexpr int SW32_NT = 128;

// Upwind fluxes written by other teams of the same launch (persistent mode)
// are read through L2 only (ld.global.cg), never from a possibly stale L1 line.
template <int N, bool COHERENT>
__device__ __forceinline__ void vload_up(const float *p, float (&v)[N]) {
  if constexpr (!COHERENT) {
    vload<N>(p, v);
  } else if constexpr (N == 1) {
    v[0] = __ldcg(p);
  } else if constexpr (N == 2) {
    const float2 t = __ldcg(reinterpret_cast<const float2 *>(p));
    v[0] = t.x; v[1] = t.y;
  } else {
    const float4 t = __ldcg(reinterpret_cast<const float4 *>(p));
    v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
  }
}

// One (direction, zone) pair for the GT lanes of a team.  sRec/sConn are this
// team's staging slots; sQ/sS its [8][G] source and running-source arrays.
template <int GT, int GPL, bool COHERENT>
__device__ __forceinline__ void sweep_zone(const Sweep32P &p, const uint2 w, const int lane, const unsigned teammask,
                                           float *sQ, float *sS, float4 (*sRec)[2], int4 *sConn) {
  const int G = GT * GPL;
  const bool bad = (w.x >> 31) != 0;
  const uint32_t it = w.x & 0x7fffffffu;
  const int a = (int)(it / (uint32_t)p.nz);
  const int z = (int)(it - (uint32_t)a * p.nz);
  const int c0 = (int)(w.y & 0x0fffffffu), nC = (int)(w.y >> 28);
  const int g0 = lane * GPL;
  const size_t abase = (size_t)a * p.nc;
  // ---- round trip 2: structure (cooperative), sources, cross sections ----
  for (int e = lane; e < 3 * nC; e += GT) {
    if (e < 2 * nC) sRec[e >> 1][e & 1] = p.rec[(abase + c0) * 2 + e];
    else sConn[e - 2 * nC] = p.conn[c0 + e - 2 * nC];
  }
  float po[UMT_MAXCORNER][GPL], st[UMT_MAXCORNER][GPL];
#pragma unroll
  for (int c = 0; c < UMT_MAXCORNER; ++c) {
    if (c < nC) {
      const size_t e = (size_t)(c0 + c) * G + g0;
      vload<GPL>(p.psi_old + abase * G + e, po[c]);
      vload<GPL>(p.STotal + e, st[c]);
    }
  }
  float sig[GPL], rsig[GPL];
  vload<GPL>(p.Sigt + (size_t)z * G + g0, sig);
  const uint32_t ord = p.order[it];
  __syncwarp(teammask);
#pragma unroll
  for (int j = 0; j < GPL; ++j) rsig[j] = __frcp_rn(sig[j]);
#pragma unroll
  for (int c = 0; c < UMT_MAXCORNER; ++c) {
    if (c < nC) {
      const float v = sRec[c][1].w;
      float q[GPL], s[GPL];
#pragma unroll
      for (int j = 0; j < GPL; ++j) { q[j] = fmaf(p.tau, po[c][j], st[c][j]); s[j] = v * q[j]; }
      vstore<GPL>(sQ + c * G + g0, q);
      vstore<GPL>(sS + c * G + g0, s);
    }
  }
  // ---- round trip 3: every upwind flux of the zone ----
  float pf[UMT_MAXCORNER][3][GPL];
#pragma unroll
  for (int c = 0; c < UMT_MAXCORNER; ++c) {
    const float4 r0 = sRec[c][0];
    const int4 cn = sConn[c];
    const float afp[3] = {r0.x, r0.y, r0.z};
    const int cfp[3] = {cn.x, cn.y, cn.z};
    const int ncf = cn.w >> 9;
#pragma unroll
    for (int cf = 0; cf < 3; ++cf) {
#pragma unroll
      for (int j = 0; j < GPL; ++j) pf[c][cf][j] = 0.f;
      if (c < nC && cf < ncf && afp[cf] < 0.f) {
        const int up = cfp[cf];
        const float *src_p = up >= 0 ? p.psi_new + (abase + up) * G + g0
                                     : p.psiB + ((size_t)a * p.nb + (size_t)(-up - 1)) * G + g0;
        vload_up<GPL, COHERENT>(src_p, pf[c][cf]);
      }
    }
  }
  // ---- incoming FP faces and EZ couplings, corner by corner ----
#pragma unroll
  for (int c = 0; c < UMT_MAXCORNER; ++c) {
    if (c < nC) {
      const float4 r0 = sRec[c][0];
      const float4 r1 = sRec[c][1];
      const int4 cn = sConn[c];
      const float afp[3] = {r0.x, r0.y, r0.z};
      const float aez[3] = {r1.x, r1.y, r1.z};
      const int meta = cn.w;
      const int ncf = meta >> 9;
      const float vol = r1.w;
      float src[GPL], Qc[GPL];
      vload<GPL>(sS + c * G + g0, src);
      vload<GPL>(sQ + c * G + g0, Qc);
#pragma unroll
      for (int cf = 0; cf < 3; ++cf)
        if (cf < ncf && afp[cf] < 0.f)
#pragma unroll
          for (int j = 0; j < GPL; ++j) src[j] = fmaf(-afp[cf], pf[c][cf][j], src[j]);
#pragma unroll
      for (int cf = 0; cf < 3; ++cf) {
        const float ae = aez[cf];
        if (cf < ncf && ae > 0.f) {
          const int cez = (meta >> (3 * cf)) & 7;
          float Qz[GPL], sz[GPL], sez[GPL];
          vload<GPL>(sQ + cez * G + g0, Qz);
          vload<GPL>(sS + cez * G + g0, sz);
          const int ifp = (cf + 1) % 3;
          if (ncf == 3 && afp[ifp] < 0.f) {
            // The reference's closure (SweepUCBxyz.F90:230-243) divided through by
            // aez^4: with x = sigma*V/aez, gnum = aez^4*N(x), gden*sigma = aez^4*2x*Dh(x),
            // N = 1.82x^2+4x+3, Dh = 2x^3+3x^2+2x+1, so
            //   sez = V*(N*(sigma*psi_opp - Qc) + Dh*(Qc - Qz)) / (N + 2x*Dh).
            // x is capped at 1e8 (sez ~ V*(Qc-Qz)/(2x) there) to stay finite in FP32.
            const float rae = __frcp_rn(ae);
#pragma unroll
            for (int j = 0; j < GPL; ++j) {
              const float x = fminf(sig[j] * vol * rae, 1.0e8f);
              const float N = fmaf(fmaf(1.82f, x, 4.f), x, 3.f);
              const float Dh = fmaf(fmaf(fmaf(2.f, x, 3.f), x, 2.f), x, 1.f);
              const float den = fmaf(2.f * x, Dh, N);
              const float num = fmaf(N, fmaf(sig[j], pf[c][ifp][j], -Qc[j]), Dh * (Qc[j] - Qz[j]));
              sez[j] = vol * __fdividef(num, den);
            }
          } else {
#pragma unroll
            for (int j = 0; j < GPL; ++j) sez[j] = 0.5f * ae * rsig[j] * (Qc[j] - Qz[j]);
          }
#pragma unroll
          for (int j = 0; j < GPL; ++j) { src[j] += sez[j]; sz[j] -= sez[j]; }
          vstore<GPL>(sS + cez * G + g0, sz);
        }
      }
      vstore<GPL>(sS + c * G + g0, src);
    }
  }
  // ---- corner solve in the schedule's order, exits ----
  float *out = p.psi_new + abase * G + g0;
  float *outB = p.psiB + (size_t)a * p.nb * G + g0;
  if (!bad) {
    for (int i = 0; i < nC; ++i) {
      const int c = (int)((ord >> (4 * i)) & 15u);
      const float4 r0 = sRec[c][0];
      const float4 r1 = sRec[c][1];
      const int4 cn = sConn[c];
      const int ncf = cn.w >> 9;
      float s[GPL], v[GPL];
      vload<GPL>(sS + c * G + g0, s);
#pragma unroll
      for (int j = 0; j < GPL; ++j) v[j] = __fdividef(s[j], fmaf(sig[j], r1.w, r0.w));
      vstore<GPL>(out + (size_t)(c0 + c) * G, v);
      const float aez[3] = {r1.x, r1.y, r1.z};
      const float afp[3] = {r0.x, r0.y, r0.z};
      const int cfp[3] = {cn.x, cn.y, cn.z};
#pragma unroll
      for (int cf = 0; cf < 3; ++cf) {
        if (cf < ncf && aez[cf] > 0.f) {
          const int cez = (cn.w >> (3 * cf)) & 7;
          float t[GPL];
          vload<GPL>(sS + cez * G + g0, t);
#pragma unroll
          for (int j = 0; j < GPL; ++j) t[j] = fmaf(aez[cf], v[j], t[j]);
          vstore<GPL>(sS + cez * G + g0, t);
        }
        if (cf < ncf && cfp[cf] < 0 && afp[cf] > 0.f) vstore<GPL>(outB + (size_t)(-cfp[cf] - 1) * G, v);
      }
    }
  } else {
    // direct solve with the previous iterate of the zone's corners
    for (int c = 0; c < nC; ++c) {
      const float4 r1 = sRec[c][1];
      const int4 cn = sConn[c];
      const int ncf = cn.w >> 9;
      float old[GPL];
      vload<GPL>(out + (size_t)(c0 + c) * G, old);
      const float aez[3] = {r1.x, r1.y, r1.z};
      for (int cf = 0; cf < 3; ++cf)
        if (cf < ncf && aez[cf] > 0.f) {
          const int cez = (cn.w >> (3 * cf)) & 7;
          float t[GPL];
          vload<GPL>(sS + cez * G + g0, t);
#pragma unroll
          for (int j = 0; j < GPL; ++j) t[j] = fmaf(aez[cf], old[j], t[j]);
          vstore<GPL>(sS + cez * G + g0, t);
        }
    }
    for (int c = 0; c < nC; ++c) {
      const float4 r0 = sRec[c][0];
      const float4 r1 = sRec[c][1];
      const int4 cn = sConn[c];
      const int ncf = cn.w >> 9;
      float s[GPL], v[GPL];
      vload<GPL>(sS + c * G + g0, s);
#pragma unroll
      for (int j = 0; j < GPL; ++j) v[j] = __fdividef(s[j], fmaf(sig[j], r1.w, r0.w));
      vstore<GPL>(out + (size_t)(c0 + c) * G, v);
      const float afp[3] = {r0.x, r0.y, r0.z};
      const int cfp[3] = {cn.x, cn.y, cn.z};
      for (int cf = 0; cf < 3; ++cf)
        if (cf < ncf && cfp[cf] < 0 && afp[cf] > 0.f) vstore<GPL>(outB + (size_t)(-cfp[cf] - 1) * G, v);
    }
  }
}

// Level-synchronous form: one launch per dependency stage; the stage's
// (direction, zone) pairs are independent.
template <int GT, int GPL>
__global__ void __launch_bounds__(SW32_NT) k_sweep32(Sweep32P p, int stage) {
  constexpr int TEAMS = SW32_NT / GT;
  extern __shared__ float4 smem4[];
  __shared__ float4 sRec[TEAMS][UMT_MAXCORNER][2];
  __shared__ int4 sConn[TEAMS][UMT_MAXCORNER];
  const int tid = threadIdx.x, team = tid / GT, lane = tid % GT;
  const int k = blockIdx.x * TEAMS + team;
  if (k >= p.stageCount[stage]) return;            // whole teams leave together
  float *sQ = reinterpret_cast<float *>(smem4) + (size_t)team * p.stride;
  float *sS = sQ + (size_t)TEAMS * p.stride;
  const uint2 w = p.items2[p.stageOffset[stage] + k];
  sweep_zone<GT, GPL, false>(p, w, lane, team_mask(GT, tid), sQ, sS, sRec[team], sConn[team]);
}

// Persistent form: every team takes work items in dependency-stage order from
// a global ticket, waits until all its upwind zones have signalled, sweeps the
// zone and signals its downwind zones.  Items are taken in stage order, so the
// earliest unfinished item never waits on anything unfinished: no deadlock, and
// no block needs to be co-resident.  Waits are bounded: after kWaitLimit polls
// the team records UMT_DEV_TIMEOUT in the status word and proceeds, so the
// launch always ends and the host reports the error.
constexpr long long kWaitLimit = 1ll << 22;   // ~0.5 s of polling

// umt103_hold_item: one more upwind zone than the item has, so its wait can
// only end by the bounded-wait rule (a host-side injection; nothing faults).
__global__ void k_hold_item(int *dep) { *dep += 1; }

struct PersistP {
  int total;                      // A * nz items
  int *ticket;                    // reset to 0 before the launch
  int *dep;                       // per item: upwind zones not yet done
  const uint8_t *exitMask;        // per item: exit faces
  const int *zoneOpp, *zoneFaces;
  unsigned int *status;
};

template <int GT, int GPL>
__global__ void __launch_bounds__(SW32_NT) k_sweep32_persistent(Sweep32P p, PersistP q) {
  constexpr int TEAMS = SW32_NT / GT;
  extern __shared__ float4 smem4[];
  __shared__ float4 sRec[TEAMS][UMT_MAXCORNER][2];
  __shared__ int4 sConn[TEAMS][UMT_MAXCORNER];
  const int tid = threadIdx.x, team = tid / GT, lane = tid % GT;
  const unsigned tm = team_mask(GT, tid);
  const int leader = (tid & 31) / GT * GT;       // lane id (in warp) of the team's first lane
  float *sQ = reinterpret_cast<float *>(smem4) + (size_t)team * p.stride;
  float *sS = sQ + (size_t)TEAMS * p.stride;
  while (true) {
    int t = 0;
    if (lane == 0) t = atomicAdd(q.ticket, 1);
    t = __shfl_sync(tm, t, leader);
    if (t >= q.total) break;
    const uint2 w = p.items2[t];
    const uint32_t it = w.x & 0x7fffffffu;
    if (lane == 0) {
      long long n = 0;
      while (*((volatile int *)(q.dep + it)) > 0) {
        if (++n > kWaitLimit) { atomicOr(q.status, UMT_DEV_TIMEOUT); break; }
        // once any team has given up, nobody waits any more: the launch drains
        if ((n & 1023) == 0 && (*((volatile unsigned *)q.status) & UMT_DEV_TIMEOUT)) break;
        __nanosleep(32);
      }
      __threadfence();
    }
    __syncwarp(tm);
    sweep_zone<GT, GPL, true>(p, w, lane, tm, sQ, sS, sRec[team], sConn[team]);
    __threadfence();
    __syncwarp(tm);
    if (lane == 0) {
      const int a = (int)(it / (uint32_t)p.nz);
      const int z = (int)(it - (uint32_t)a * p.nz);
      const uint8_t m = q.exitMask[it];
      for (int f = 0; f < q.zoneFaces[z]; ++f)
        if (m & (1u << f)) {
          const int zo = q.zoneOpp[z * UMT_MAXFACES + f];
          if (zo >= 0) atomicSub(q.dep + (size_t)a * p.nz + zo, 1);
        }
    }
    __syncwarp(tm);
  }
}

// Per (direction, corner) record: FP projections, outflow area sum
// (sumArea of SweepUCBxyz.F90:135-176, summed FP then EZ in face order),
// EZ projections and the corner volume.
__global__ void k_corner_rec(int A, int nc, const int *nCFaces, const double *afp64,
                             const double *aez64, const double *Volume, float4 *rec) {
  const size_t n = (size_t)A * nc;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % nc);
    const int ncf = nCFaces[c];
    float f[3], e[3];
    float sum = 0.f;
    for (int cf = 0; cf < 3; ++cf) {
      f[cf] = cf < ncf ? (float)afp64[i * 3 + cf] : 0.f;
      if (f[cf] > 0.f) sum += f[cf];
    }
    for (int cf = 0; cf < 3; ++cf) {
      e[cf] = cf < ncf ? (float)aez64[i * 3 + cf] : 0.f;
      if (e[cf] > 0.f) sum += e[cf];
    }
    rec[2 * i] = make_float4(f[0], f[1], f[2], sum);
    rec[2 * i + 1] = make_float4(e[0], e[1], e[2], (float)Volume[c]);
  }
}

__global__ void k_conn(int nc, const int *nCFaces, const int *cFP, const int *cEZ, int4 *conn, float *vol32,
                       const double *Volume) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
    const int ncf = nCFaces[c];
    int v[3];
    int meta = ncf << 9;
    for (int cf = 0; cf < 3; ++cf) {
      const int x = cf < ncf ? cFP[c * 3 + cf] : 0;
      v[cf] = x >= nc ? -(x - nc) - 1 : x;
      if (cf < ncf) meta |= (cEZ[c * 3 + cf] & 7) << (3 * cf);
    }
    conn[c] = make_int4(v[0], v[1], v[2], meta);
    vol32[c] = (float)Volume[c];
  }
}

// Let a kernel use all the shared memory its static arrays leave free.
int allow_dynamic_smem(const void *fn) {
  int dev = 0, optin = 0;
  UMT_CUDA(cudaGetDevice(&dev));
  UMT_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  cudaFuncAttributes fa;
  UMT_CUDA(cudaFuncGetAttributes(&fa, fn));
  const int dyn = optin - (int)fa.sharedSizeBytes;
  UMT_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn > 0 ? dyn : 0));
  return 0;
}
#define TRY_ATTR(x) do { int rc_ = (x); if (rc_) return rc_; } while (0)

int prepare_sweep32(Ctx &c) {
  if (!c.rec32) {
    cudaError_t e1 = cudaMalloc((void **)&c.rec32, (size_t)c.A * c.nc * 2 * sizeof(float4));
    cudaError_t e2 = cudaMalloc((void **)&c.conn32, (size_t)c.nc * sizeof(int4));
    cudaError_t e3 = cudaMalloc((void **)&c.vol32, (size_t)c.nc * sizeof(float));
    if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess)
      return set_error(-7, "allocation of the FP32 corner records failed");
  }
#define UMT_ATTR32(gt, gpl) \
  TRY_ATTR(allow_dynamic_smem((const void *)k_sweep32<gt, gpl>)); \
  TRY_ATTR(allow_dynamic_smem((const void *)k_sweep32_persistent<gt, gpl>));
  UMT_ATTR32(1, 1) UMT_ATTR32(1, 2) UMT_ATTR32(1, 4) UMT_ATTR32(2, 1) UMT_ATTR32(2, 2) UMT_ATTR32(2, 4)
  UMT_ATTR32(4, 1) UMT_ATTR32(4, 2) UMT_ATTR32(4, 4) UMT_ATTR32(8, 1) UMT_ATTR32(8, 2) UMT_ATTR32(8, 4)
  UMT_ATTR32(16, 1) UMT_ATTR32(16, 2) UMT_ATTR32(16, 4) UMT_ATTR32(32, 1) UMT_ATTR32(32, 2) UMT_ATTR32(32, 4)
#undef UMT_ATTR32
  const size_t n = (size_t)c.A * c.nc;
  k_corner_rec<<<(int)std::min<size_t>((n + 255) / 256, 152 * 16), 256, 0, c.stream>>>(
      c.A, c.nc, c.nCFaces, c.afp64, c.aez64, c.Volume, (float4 *)c.rec32);
  k_conn<<<(c.nc + 255) / 256, 256, 0, c.stream>>>(c.nc, c.nCFaces, c.cFP, c.cEZ, (int4 *)c.conn32, c.vol32,
                                                   c.Volume);
  UMT_CUDA(cudaGetLastError());
  return prepare_prog32(c);
}

// Group tile: GT lanes per (direction, zone), GPL groups per lane, G = GT*GPL.
bool sweep32_supported(int G, int GT, int GPL) {
  return GT * GPL == G && (GT == 1 || GT == 2 || GT == 4 || GT == 8 || GT == 16 || GT == 32) &&
         (GPL == 1 || GPL == 2 || GPL == 4);
}

void default_tile(int G, int *GT, int *GPL) {
  *GT = 0; *GPL = 0;
  const int pref[3] = {2, 1, 4};        // register use: GPL=2 ~124, GPL=1 ~96, GPL=4 ~200 per thread
  for (int gpl : pref)
    if (G % gpl == 0 && sweep32_supported(G, G / gpl, gpl)) { *GT = G / gpl; *GPL = gpl; return; }
}

static int team_stride(int G) {
  const int base = 8 * G;
  return base + (((G - (base % 32)) % 32) + 32) % 32;
}

int enqueue_sweep32(Ctx &c, int cur, int GT, int GPL) {
  Sweep32P p;
  p.nz = c.nz; p.nc = c.nc; p.nb = c.nb; p.A = c.A; p.G = c.G; p.stride = team_stride(c.G);
  p.items2 = c.sch.items2; p.stageOffset = c.sch.stageOffset; p.stageCount = c.sch.stageCount;
  p.order = c.sch.order;
  p.rec = (const float4 *)c.rec32; p.conn = (const int4 *)c.conn32;
  p.Sigt = c.Sigt32; p.STotal = c.STotal32; p.tau = c.homog32 ? 0.f : (float)c.tau;
  p.psi_old = c.psi32[cur]; p.psi_new = c.psi32[1 - cur]; p.psiB = c.homog32 ? c.psiB32h : c.psiB32;
  const int TEAMS = 128 / GT;
  const size_t smem = (size_t)2 * TEAMS * p.stride * sizeof(float);
  PersistP q;
  q.total = c.A * c.nz; q.ticket = c.ticket; q.dep = c.dep; q.exitMask = c.sch.exitMask;
  q.zoneOpp = c.zoneOpp; q.zoneFaces = c.zoneFaces; q.status = c.status;
  if (c.sweepMode == 1) {
    UMT_CUDA(cudaMemcpyAsync(c.dep, c.sch.needInit, (size_t)q.total * sizeof(int), cudaMemcpyDeviceToDevice, c.stream));
    UMT_CUDA(cudaMemsetAsync(c.ticket, 0, sizeof(int), c.stream));
    if (c.holdItem >= 0 && c.holdItem < q.total) k_hold_item<<<1, 1, 0, c.stream>>>(c.dep + c.holdItem);
  }
  int dev = 0, nsm = 0;
  UMT_CUDA(cudaGetDevice(&dev));
  UMT_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  c.exitsThrough = false;
  if (c.sweepMode == 0) {
    const int rc = enqueue_sweep32p(c, cur, GT, GPL);
    if (rc == 0) c.exitsThrough = true;            // the exit chunks write *psibOut's rows
    if (rc <= 0) return rc;                        // 1: no program kernel for this tile
  }
#define UMT_LAUNCH32(gt, gpl)                                                                      \
  if (GT == gt && GPL == gpl) {                                                                    \
    if (c.sweepMode == 1) {                                                                        \
      int per = 0;                                                                                 \
      UMT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sweep32_persistent<gt, gpl>, 128, smem)); \
      const int blocks = std::max(1, std::min(per * nsm, (q.total + TEAMS - 1) / TEAMS));         \
      k_sweep32_persistent<gt, gpl><<<blocks, 128, smem, c.stream>>>(p, q);                        \
    } else {                                                                                       \
      for (int s = 0; s < c.sch.nStages; ++s) {                                                    \
        const int blocks = (c.sch.hCount[s] + TEAMS - 1) / TEAMS;                                  \
        k_sweep32<gt, gpl><<<blocks, 128, smem, c.stream>>>(p, s);                                 \
      }                                                                                            \
    }                                                                                              \
    UMT_CUDA(cudaGetLastError());                                                                  \
    return 0;                                                                                      \
  }
  UMT_LAUNCH32(1, 1) UMT_LAUNCH32(1, 2) UMT_LAUNCH32(1, 4)
  UMT_LAUNCH32(2, 1) UMT_LAUNCH32(2, 2) UMT_LAUNCH32(2, 4)
  UMT_LAUNCH32(4, 1) UMT_LAUNCH32(4, 2) UMT_LAUNCH32(4, 4)
  UMT_LAUNCH32(8, 1) UMT_LAUNCH32(8, 2) UMT_LAUNCH32(8, 4)
  UMT_LAUNCH32(16, 1) UMT_LAUNCH32(16, 2) UMT_LAUNCH32(16, 4)
  UMT_LAUNCH32(32, 1) UMT_LAUNCH32(32, 2) UMT_LAUNCH32(32, 4)
#undef UMT_LAUNCH32
  return set_error(-1, "unsupported group tile GT=%d GPL=%d", GT, GPL);
}

}  // namespace umt
