// geom_sched.cu -- corner geometry and the device-built sweep schedule.
//
// Compiled with -fmad=false: the geometry and the signs of Omega.A that
// decide upwind/downwind are computed with the same operation order as
// Teton's Fortran (no contraction), so every dependency decision matches the
// CPU schedule bit for bit and the sweep never reads a flux that its
// schedule did not produce.
#include "umt_common.cuh"

#include <algorithm>
#include <vector>

namespace umt {

#define TRY_RC(x) do { int rc_ = (x); if (rc_) return rc_; } while (0)

// ---------------------------------------------------------------------------
// Geometry: rt/geometryUCBxyz.F90:9-185 (area vectors of FP and EZ corner
// faces, corner volumes) with the zone volume and boundary area vectors of
// rt/volumeUCBxyz.F90.  One thread per zone.  Pass 1 computes each zone's own
// FP area vectors and its EZ areas; pass 2 makes the FP vectors of shared
// faces equal and opposite (the lower zone's vector wins, as in the
// reference) and accumulates the volumes.
// ---------------------------------------------------------------------------
struct GeoArgs {
  int nz, nc;
  const int *numCorner, *cOffSet, *zoneFaces, *zoneOpp, *nCFaces, *cFP, *cEZ, *CToFace;
  const double *px;
  double *Afp_raw, *A_fp, *A_ez, *Volume, *VolumeZone, *A_bdy;
};

__device__ inline void zone_centres(const GeoArgs &p, int zone, double zc[3], double fc[UMT_MAXFACES][3]) {
  const int nCorner = p.numCorner[zone], c0 = p.cOffSet[zone];
  zc[0] = zc[1] = zc[2] = 0.0;
  for (int c = 0; c < nCorner; ++c)
    for (int d = 0; d < 3; ++d) zc[d] += p.px[3 * (c0 + c) + d];
  for (int d = 0; d < 3; ++d) zc[d] /= (double)nCorner;
  int ncf[UMT_MAXFACES];
  for (int f = 0; f < UMT_MAXFACES; ++f) { ncf[f] = 0; fc[f][0] = fc[f][1] = fc[f][2] = 0.0; }
  for (int c = 0; c < nCorner; ++c)
    for (int cf = 0; cf < p.nCFaces[c0 + c]; ++cf) {
      const int f = p.CToFace[(c0 + c) * UMT_MAXCF + cf];
      ncf[f] += 1;
      for (int d = 0; d < 3; ++d) fc[f][d] += p.px[3 * (c0 + c) + d];
    }
  for (int f = 0; f < UMT_MAXFACES; ++f)
    for (int d = 0; d < 3; ++d) fc[f][d] = ncf[f] ? fc[f][d] / (double)ncf[f] : 0.0;
}

__global__ void k_geometry_pass1(GeoArgs p) {
  const int zone = blockIdx.x * blockDim.x + threadIdx.x;
  if (zone >= p.nz) return;
  double zc[3], fc[UMT_MAXFACES][3];
  zone_centres(p, zone, zc, fc);
  const int nCorner = p.numCorner[zone], c0 = p.cOffSet[zone];
  for (int c = 0; c < nCorner; ++c)
    for (int k = 0; k < UMT_MAXCF * 3; ++k) p.A_ez[(size_t)(c0 + c) * UMT_MAXCF * 3 + k] = 0.0;
  for (int c = 0; c < nCorner; ++c) {
    const int cc = c0 + c, nCF = p.nCFaces[cc];
    for (int cf1 = 0; cf1 < nCF; ++cf1) {
      const int cf2 = (cf1 + 1) % nCF;
      const int cez1 = p.cEZ[cc * UMT_MAXCF + cf1], cez2 = p.cEZ[cc * UMT_MAXCF + cf2];
      const int face = p.CToFace[cc * UMT_MAXCF + cf1];
      const double *p0 = p.px + 3 * cc, *p1 = p.px + 3 * (c0 + cez1), *p2 = p.px + 3 * (c0 + cez2);
      double tdl[3], tfl[3], tfz[3], tfe1[3], tfe2[3];
      for (int d = 0; d < 3; ++d) {
        tdl[d] = 0.5 * (p1[d] - p2[d]);
        tfl[d] = fc[face][d] - p0[d];
        tfz[d] = fc[face][d] - zc[d];
        tfe1[d] = fc[face][d] - 0.5 * (p1[d] + p0[d]);
        tfe2[d] = fc[face][d] - 0.5 * (p2[d] + p0[d]);
      }
      double *raw = p.Afp_raw + ((size_t)cc * UMT_MAXCF + cf1) * 3;
      raw[0] = 0.5 * (tfl[2] * tdl[1] - tfl[1] * tdl[2]);
      raw[1] = 0.5 * (tfl[0] * tdl[2] - tfl[2] * tdl[0]);
      raw[2] = 0.5 * (tfl[1] * tdl[0] - tfl[0] * tdl[1]);
      double A1[3], A2[3];
      A1[0] = 0.5 * (tfz[2] * tfe1[1] - tfz[1] * tfe1[2]);
      A1[1] = 0.5 * (tfz[0] * tfe1[2] - tfz[2] * tfe1[0]);
      A1[2] = 0.5 * (tfz[1] * tfe1[0] - tfz[0] * tfe1[1]);
      A2[0] = 0.5 * (tfz[1] * tfe2[2] - tfz[2] * tfe2[1]);
      A2[1] = 0.5 * (tfz[2] * tfe2[0] - tfz[0] * tfe2[2]);
      A2[2] = 0.5 * (tfz[0] * tfe2[1] - tfz[1] * tfe2[0]);
      for (int d = 0; d < 3; ++d) {
        p.A_ez[((size_t)cc * UMT_MAXCF + cf1) * 3 + d] += A1[d];
        p.A_ez[((size_t)cc * UMT_MAXCF + cf2) * 3 + d] += A2[d];
      }
    }
  }
  for (int c = 0; c < nCorner; ++c) {
    const int cc = c0 + c;
    for (int cf1 = 0; cf1 < p.nCFaces[cc]; ++cf1) {
      const int cez = p.cEZ[cc * UMT_MAXCF + cf1];
      if (cez > c)
        for (int cf2 = 0; cf2 < p.nCFaces[c0 + cez]; ++cf2)
          if (p.cEZ[(c0 + cez) * UMT_MAXCF + cf2] == c)
            for (int d = 0; d < 3; ++d)
              p.A_ez[((size_t)(c0 + cez) * UMT_MAXCF + cf2) * 3 + d] =
                  -p.A_ez[((size_t)cc * UMT_MAXCF + cf1) * 3 + d];
    }
  }
}

__global__ void k_geometry_pass2(GeoArgs p) {
  const int zone = blockIdx.x * blockDim.x + threadIdx.x;
  if (zone >= p.nz) return;
  double zc[3], fc[UMT_MAXFACES][3];
  zone_centres(p, zone, zc, fc);
  const int nCorner = p.numCorner[zone], c0 = p.cOffSet[zone];
  double vz = 0.0;
  for (int c = 0; c < nCorner; ++c) {
    const int cc = c0 + c, nCF = p.nCFaces[cc];
    double vol = 0.0;
    for (int cf1 = 0; cf1 < nCF; ++cf1) {
      const int face = p.CToFace[cc * UMT_MAXCF + cf1];
      const int zOpp = p.zoneOpp[zone * UMT_MAXFACES + face];
      const int cfp = p.cFP[cc * UMT_MAXCF + cf1];
      double A[3];
      const double *raw = p.Afp_raw + ((size_t)cc * UMT_MAXCF + cf1) * 3;
      if (zOpp >= 0 && zOpp < zone) {
        int cfo = -1;
        for (int cf = 0; cf < p.nCFaces[cfp]; ++cf)
          if (p.cFP[cfp * UMT_MAXCF + cf] == cc) cfo = cf;
        const double *o = p.Afp_raw + ((size_t)cfp * UMT_MAXCF + (cfo < 0 ? 0 : cfo)) * 3;
        for (int d = 0; d < 3; ++d) A[d] = -o[d];
      } else {
        for (int d = 0; d < 3; ++d) A[d] = raw[d];
        if (zOpp < 0)
          for (int d = 0; d < 3; ++d) p.A_bdy[3 * (size_t)(cfp - p.nc) + d] = raw[d];
      }
      for (int d = 0; d < 3; ++d) p.A_fp[((size_t)cc * UMT_MAXCF + cf1) * 3 + d] = A[d];
      double tzl[3];
      for (int d = 0; d < 3; ++d) tzl[d] = zc[d] - p.px[3 * cc + d];
      vol += (1.0 / 3.0) * fabs(tzl[0] * A[0] + tzl[1] * A[1] + tzl[2] * A[2]);
    }
    p.Volume[cc] = vol;
    vz += vol;
  }
  p.VolumeZone[zone] = vz;
}

int launch_geometry(Ctx &c) {
  GeoArgs p{c.nz, c.nc, c.numCorner, c.cOffSet, c.zoneFaces, c.zoneOpp, c.nCFaces, c.cFP,
            c.cEZ, c.CToFace, c.px, c.Afp_raw, c.A_fp, c.A_ez, c.Volume, c.VolumeZone, c.A_bdy};
  const int T = 128, B = (c.nz + T - 1) / T;
  k_geometry_pass1<<<B, T, 0, c.stream>>>(p);
  k_geometry_pass2<<<B, T, 0, c.stream>>>(p);
  UMT_CUDA(cudaGetLastError());
  return 0;
}

// ---------------------------------------------------------------------------
// Per-direction corner-face projections Omega.A_fp and Omega.A_ez (the
// reference precomputes the same products as AfpNorm/AezNorm in
// gpu/SweepUCBxyz_OMPOL.F90:141-252 and d_afp/d_aez in compAfpKernel,
// gpu/GPU_SweepUCBxyz.cu:141-160).  FP64, summed in DOT_PRODUCT order.
// ---------------------------------------------------------------------------
__device__ inline double dot3(const double *o, const double *a) {
  double s = 0.0;
  s = s + o[0] * a[0];
  s = s + o[1] * a[1];
  s = s + o[2] * a[2];
  return s;
}

__global__ void k_projections(int A, int nc, const double *omega, const int *nCFaces,
                              const double *A_fp, const double *A_ez, double *afp64,
                              double *aez64, float *afp32, float *aez32) {
  const size_t n = (size_t)A * nc * UMT_MAXCF;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int cf = (int)(i % UMT_MAXCF);
    const size_t ac = i / UMT_MAXCF;
    const int c = (int)(ac % nc);
    const int a = (int)(ac / nc);
    double vf = 0.0, ve = 0.0;
    if (cf < nCFaces[c]) {
      const double *o = omega + 3 * a;
      const double *af = A_fp + ((size_t)c * UMT_MAXCF + cf) * 3;
      const double *ae = A_ez + ((size_t)c * UMT_MAXCF + cf) * 3;
      vf = dot3(o, af);
      ve = dot3(o, ae);
      // A face parallel to the direction (Omega.A = 0 in exact arithmetic, e.g.
      // a 45-degree face and an S2 direction) would otherwise get a rounding-
      // noise sign per corner face; such projections are set to exactly zero,
      // so the face carries no flux and creates no dependency.
      const double nf = fabs(af[0]) + fabs(af[1]) + fabs(af[2]);
      const double ne = fabs(ae[0]) + fabs(ae[1]) + fabs(ae[2]);
      if (fabs(vf) <= 1.0e-12 * nf) vf = 0.0;
      if (fabs(ve) <= 1.0e-12 * ne) ve = 0.0;
    }
    if (afp64) { afp64[i] = vf; aez64[i] = ve; }
    if (afp32) { afp32[i] = (float)vf; aez32[i] = (float)ve; }
  }
}

int launch_projections(Ctx &c) {
  const size_t n = (size_t)c.A * c.nc * UMT_MAXCF;
  int B = (int)std::min<size_t>((n + 255) / 256, 152 * 16);
  k_projections<<<B, 256, 0, c.stream>>>(c.A, c.nc, c.omega, c.nCFaces, c.A_fp, c.A_ez,
                                         c.afp64, c.aez64, c.afp32, c.aez32);
  UMT_CUDA(cudaGetLastError());
  return 0;
}

// ---------------------------------------------------------------------------
// Schedule.  k_need restates snneed (snac/snneed.F90:104-187): per zone face
// the sum of Omega.A_fp over its corner faces decides the flow direction;
// the downstream zone's need count is incremented and the upstream side's
// face is marked as an exit.  A face whose corner faces disagree in sign
// makes the upstream zone read some corners of the downstream zone before
// they are computed: those corners go on the direction's cycle list (the
// downstream zone is flagged in cycZ), as snneed.F90 does.
// k_corner_order restates getDownStreamData (snac/getDownStreamData.F90:
// 59-150): the corner solve order within a zone by repeated minloc of the
// remaining EZ need; a zone whose corners cannot be ordered is "bad".
// ---------------------------------------------------------------------------
struct SchedArgs {
  int nz, nc, A;
  const int *numCorner, *cOffSet, *zoneFaces, *zoneOpp, *faceOpp, *nCFaces, *cEZ, *CToFace;
  const double *afp64, *aez64;
  int *need;
  uint8_t *exitMask, *bad;
  uint32_t *order;
  unsigned int *status;
  uint8_t *cycZ;
};

__global__ void k_need(SchedArgs p) {
  const size_t n = (size_t)p.A * p.nz;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int zone = (int)(i % p.nz), a = (int)(i / p.nz);
    const int nCorner = p.numCorner[zone], c0 = p.cOffSet[zone];
    double afpm_Face[UMT_MAXFACES];
    int nInc[UMT_MAXFACES], nExit[UMT_MAXFACES];
    for (int f = 0; f < UMT_MAXFACES; ++f) { afpm_Face[f] = 0.0; nInc[f] = 0; nExit[f] = 0; }
    for (int c = 0; c < nCorner; ++c) {
      const int cc = c0 + c;
      for (int cf = 0; cf < p.nCFaces[cc]; ++cf) {
        const int face = p.CToFace[cc * UMT_MAXCF + cf];
        if (p.zoneOpp[zone * UMT_MAXFACES + face] > zone) {
          const double afpm = p.afp64[((size_t)a * p.nc + cc) * UMT_MAXCF + cf];
          afpm_Face[face] = afpm_Face[face] + afpm;
          if (afpm < 0.0) nInc[face] += 1;
          else if (afpm > 0.0) nExit[face] += 1;
        }
      }
    }
    for (int face = 0; face < p.zoneFaces[zone]; ++face) {
      const int zOpp = p.zoneOpp[zone * UMT_MAXFACES + face];
      if (zOpp > zone) {
        const int fOpp = p.faceOpp[zone * UMT_MAXFACES + face];
        if (afpm_Face[face] < 0.0) {
          atomicAdd(&p.need[(size_t)a * p.nz + zone], 1);
          atomicOr((unsigned int *)(p.exitMask + (((size_t)a * p.nz + zOpp) & ~(size_t)3)),
                   (1u << fOpp) << (8 * (((size_t)a * p.nz + zOpp) & 3)));
          if (nExit[face] > 0) p.cycZ[i] = 1;
        } else if (afpm_Face[face] > 0.0) {
          atomicAdd(&p.need[(size_t)a * p.nz + zOpp], 1);
          atomicOr((unsigned int *)(p.exitMask + (i & ~(size_t)3)), (1u << face) << (8 * (i & 3)));
          if (nInc[face] > 0) p.cycZ[(size_t)a * p.nz + zOpp] = 1;
        }
      }
    }
  }
}

__global__ void k_corner_order(SchedArgs p) {
  const size_t n = (size_t)p.A * p.nz;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int zone = (int)(i % p.nz), a = (int)(i / p.nz);
    const int nCorner = p.numCorner[zone], c0 = p.cOffSet[zone];
    int need[UMT_MAXCORNER], nDSC[UMT_MAXCORNER];
    int DSC[UMT_MAXCORNER][UMT_MAXCORNER];
    for (int c = 0; c < UMT_MAXCORNER; ++c) { need[c] = 0; nDSC[c] = 0; }
    for (int c = 0; c < nCorner; ++c) {
      const int cc = c0 + c;
      for (int cf = 0; cf < p.nCFaces[cc]; ++cf) {
        const int cez = p.cEZ[cc * UMT_MAXCF + cf];
        if (cez > c) {
          const double aez = p.aez64[((size_t)a * p.nc + cc) * UMT_MAXCF + cf];
          if (aez < 0.0) { need[c] += 1; DSC[cez][nDSC[cez]++] = c; }
          else if (aez > 0.0) { need[cez] += 1; DSC[c][nDSC[c]++] = cez; }
        }
      }
    }
    bool isbad = false;
    uint32_t ord = 0;
    for (int k = 0; k < nCorner; ++k) {
      int c = 0;
      for (int m = 1; m < nCorner; ++m) if (need[m] < need[c]) c = m;
      ord |= (uint32_t)c << (4 * k);
      if (need[c] != 0) isbad = true;
      for (int m = 0; m < nDSC[c]; ++m) need[DSC[c][m]] -= 1;
      need[c] = 99;
    }
    if (isbad) {                      // fixZone: the zone is swept from its corners' previous values
      ord = 0;
      for (int k = 0; k < nCorner; ++k) ord |= (uint32_t)k << (4 * k);
      p.cycZ[i] = 1;
    }
    p.order[i] = ord;
    p.bad[i] = isbad ? 1 : 0;
  }
}

// Stage 0: every (direction, zone) that needs no upwind zone (findseeds,
// snac/findseeds.F90:58-65).
__global__ void k_seed(int nz, int A, const int *need, const uint8_t *bad, uint32_t *items,
                       int *stageCount, int *level, unsigned long long *processed) {
  const size_t n = (size_t)A * nz;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    if (need[i] == 0) {
      const int pos = atomicAdd(&stageCount[0], 1);
      items[pos] = (uint32_t)i | (bad[i] ? 0x80000000u : 0u);
      level[i] = 0;
    }
  }
}

// zones with no upwind need, per direction
__global__ void k_seed_count(int nz, int A, const int *need, int *count) {
  const size_t n = (size_t)A * nz;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    if (need[i] == 0) atomicAdd(&count[i / nz], 1);
}

// Stage h -> h+1 (the hyperplane loop of snac/snnext.F90:109-163): every item
// of stage h decrements the need of its downstream zones; a zone whose need
// reaches zero joins stage h+1.  Items of one stage are independent.
__global__ void k_stage(int h, int nz, int A, const int *zoneFaces, const int *zoneOpp,
                        const uint8_t *exitMask, const uint8_t *bad, int *need, uint32_t *items,
                        int *stageCount, int *stageOffset, int *level, int *nHyper,
                        unsigned long long *processed) {
  const int off = stageOffset[h], cnt = stageCount[h];
  const int offn = off + cnt;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    stageOffset[h + 1] = offn;
    if (cnt) atomicAdd(processed, (unsigned long long)cnt);
  }
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += gridDim.x * blockDim.x) {
    const uint32_t it = items[off + k] & 0x7fffffffu;
    const int a = (int)(it / (uint32_t)nz), z = (int)(it - (uint32_t)a * nz);
    atomicMax(&nHyper[a], h + 1);
    const uint8_t m = exitMask[it];
    for (int f = 0; f < zoneFaces[z]; ++f) {
      if (m & (1u << f)) {
        const int zo = zoneOpp[z * UMT_MAXFACES + f];
        if (zo >= 0) {
          const size_t j = (size_t)a * nz + zo;
          if (atomicSub(&need[j], 1) == 1) {
            const int pos = atomicAdd(&stageCount[h + 1], 1);
            items[offn + pos] = (uint32_t)j | (bad[j] ? 0x80000000u : 0u);
            level[j] = h + 1;
          }
        }
      }
    }
  }
}

// Items with the zone's corner offset and count packed alongside, so a sweep
// team learns everything it needs to address its zone from one 64-bit load.
__global__ void k_items2(size_t n, int nz, const uint32_t *items, const int *cOffSet, const int *numCorner,
                         uint2 *items2) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const uint32_t it = items[i];
    const int z = (int)((it & 0x7fffffffu) % (uint32_t)nz);
    items2[i] = make_uint2(it, (uint32_t)cOffSet[z] | ((uint32_t)numCorner[z] << 28));
  }
}

// ---------------------------------------------------------------------------
// Cycle breaking on the host, for the directions whose wavefront stalls.
// Restates the decisions of snac/findseeds.F90:58-112 (no seed at all: the
// boundary zone of least need starts, the zones across its non-exit faces go
// on the cycle list) and snac/cyclebreaker.F90:88-143 with
// snac/sccsearch.F90:8-187 (Tarjan's strongly connected components over the
// zones not yet placed; in each component of more than one zone, the root's
// incoming faces from zones still on the search stack are cut and those
// zones' corners go on the cycle list; a root left with no need starts the
// next hyperplane).  The search visits zones in increasing order and faces in
// face order, depth first, as the recursive reference does; it keeps an
// explicit stack so that deep meshes cannot overflow the host stack.  Every
// cut is recorded, so that order_direction can give it the reference's
// outcome.
// ---------------------------------------------------------------------------
struct DirGraph {
  int nz;
  const int *zoneFaces, *zoneOpp, *faceOpp;     // host copies [nz], [nz*UMT_MAXFACES]
  int *need;                                    // [nz] this direction's slice
  uint8_t *exitMask, *cyc;                      // [nz]
  bool exit(int z, int f) const { return (exitMask[z] >> f) & 1u; }
  void clear_exit(int z, int f) { exitMask[z] &= (uint8_t)~(1u << f); }
  void set_exit(int z, int f) { exitMask[z] |= (uint8_t)(1u << f); }
};

struct Cut { int from, face, root; };            // the edge from -> root across face `face` of `from`

static int seed_fallback(DirGraph &g, std::vector<int> &freed, std::vector<Cut> &cuts) {
  int minNeed = g.nz, zoneID = -1;
  for (int z = 0; z < g.nz; ++z) {
    bool bdy = false;
    for (int f = 0; f < g.zoneFaces[z]; ++f) bdy |= g.zoneOpp[z * UMT_MAXFACES + f] < 0;
    if (bdy && g.need[z] < minNeed) { zoneID = z; minNeed = g.need[z]; }
  }
  if (zoneID < 0) return -1;
  g.need[zoneID] = 0;
  for (int f = 0; f < g.zoneFaces[zoneID]; ++f) {
    if (g.exit(zoneID, f)) continue;
    const int zo = g.zoneOpp[zoneID * UMT_MAXFACES + f], fo = g.faceOpp[zoneID * UMT_MAXFACES + f];
    if (zo >= 0) {
      g.cyc[zo] = 1;
      if (g.exit(zo, fo)) cuts.push_back({zo, fo, zoneID});
      g.clear_exit(zo, fo);
    }
  }
  freed.push_back(zoneID);
  return 0;
}

static int break_cycles(DirGraph &g, std::vector<int> &freed, std::vector<Cut> &cuts) {
  const int nz = g.nz;
  std::vector<int> dfnum(nz, 0), lowlink(nz, 0), stk, breakList, tmp;
  std::vector<char> isnew(nz, 0), onstack(nz, 0);
  struct Frame { int zone, face; };
  std::vector<Frame> frames;
  for (int z = 0; z < nz; ++z) isnew[z] = g.need[z] != 0;
  int ncount = 0;
  auto enter = [&](int z) {
    ++ncount;
    dfnum[z] = lowlink[z] = ncount;
    isnew[z] = 0;
    stk.push_back(z);
    onstack[z] = 1;
    frames.push_back({z, 0});
  };
  auto finish = [&](int zone) {
    if (lowlink[zone] != dfnum[zone]) return;
    int z2 = stk.back();
    stk.pop_back();
    onstack[z2] = 0;
    if (z2 == zone) return;
    tmp.clear();
    while (z2 != zone) {
      tmp.push_back(z2);
      z2 = stk.back();
      stk.pop_back();
    }
    tmp.push_back(z2);
    onstack[tmp[0]] = 1;
    const int root = tmp.back();
    for (int f = 0; f < g.zoneFaces[root]; ++f) {
      const int zb = g.zoneOpp[root * UMT_MAXFACES + f], fb = g.faceOpp[root * UMT_MAXFACES + f];
      if (zb >= 0 && onstack[zb] && g.exit(zb, fb)) {
        g.cyc[zb] = 1;
        g.need[root] -= 1;
        g.clear_exit(zb, fb);
        cuts.push_back({zb, fb, root});
        if (g.need[root] == 0) breakList.push_back(root);
      }
    }
    for (int v : tmp) onstack[v] = 0;
  };
  for (int z0 = 0; z0 < nz; ++z0) {
    if (!isnew[z0]) continue;
    enter(z0);
    while (!frames.empty()) {
      Frame &fr = frames.back();
      const int zone = fr.zone;
      if (fr.face < g.zoneFaces[zone]) {
        const int f = fr.face++;
        if (!g.exit(zone, f)) continue;
        const int z2 = g.zoneOpp[zone * UMT_MAXFACES + f];
        if (z2 < 0) continue;
        if (isnew[z2]) {
          enter(z2);                              // invalidates fr
        } else if (dfnum[z2] < dfnum[zone] && onstack[z2] && lowlink[z2] < lowlink[zone]) {
          lowlink[zone] = lowlink[z2];
        }
      } else {
        finish(zone);
        frames.pop_back();
        if (!frames.empty()) {
          const int parent = frames.back().zone;
          if (lowlink[zone] < lowlink[parent]) lowlink[parent] = lowlink[zone];
        }
      }
    }
  }
  for (int z : breakList) {
    if (g.need[z] == 0) freed.push_back(z);
    else if (g.need[z] < 0) return -1;
  }
  return freed.empty() ? -1 : 0;
}

// One direction whose graph holds a cycle (or has no seed), ordered the way
// the reference's sequential hyperplane loop orders it (snac/snnext.F90:
// 109-195: the zones of a hyperplane one after another, each releasing the
// zones across its exit faces in face order; findseeds when nothing starts;
// cyclebreaker when the loop stalls, its freed zones in the order found).
// That order decides what every zone reads across an edge the reference
// cuts: the upstream zone's new flux when the upstream zone comes first, its
// previous flux (the cycle list's) otherwise.  The schedule takes the same
// decisions as dependency edges: a cut edge whose upstream zone comes first
// stays an edge, any other is reversed.  Every edge then points forward in
// the reference's order, so the direction's graph is acyclic, the wavefront
// places it without a stall, and no two zones that read one another share a
// stage.  The cycle flags (g.cyc) become the reference's cycle list.
static int order_direction(DirGraph &g) {
  const int nz = g.nz;
  std::vector<int> need(g.need, g.need + nz);
  std::vector<uint8_t> ex(g.exitMask, g.exitMask + nz);
  DirGraph w{nz, g.zoneFaces, g.zoneOpp, g.faceOpp, need.data(), ex.data(), g.cyc};
  std::vector<int> list, seq(nz, -1);
  std::vector<Cut> cuts;
  list.reserve(nz);
  for (int z = 0; z < nz; ++z)
    if (need[z] == 0) list.push_back(z);
  if (list.empty() && seed_fallback(w, list, cuts)) return -1;
  size_t head = 0;
  while (list.size() < (size_t)nz) {
    if (head == list.size()) {                    // stalled: break the cycles that hold it up
      std::vector<int> freed;
      if (break_cycles(w, freed, cuts)) return -1;
      list.insert(list.end(), freed.begin(), freed.end());
      continue;
    }
    const size_t end = list.size();
    for (; head < end; ++head) {
      const int z = list[head];
      seq[z] = (int)head;
      for (int f = 0; f < g.zoneFaces[z]; ++f) {
        if (!w.exit(z, f)) continue;
        const int zo = g.zoneOpp[z * UMT_MAXFACES + f];
        if (zo < 0 || seq[zo] >= 0) continue;
        if (--need[zo] == 0) list.push_back(zo);
        else if (need[zo] < 0) return -1;
      }
    }
  }
  for (; head < list.size(); ++head) seq[list[head]] = (int)head;
  for (const Cut &e : cuts) {
    if (!g.exit(e.from, e.face) || seq[e.from] < seq[e.root]) continue;
    g.clear_exit(e.from, e.face);                 // the root comes first: it reads the previous flux
    g.need[e.root] -= 1;
    g.set_exit(e.root, g.faceOpp[e.from * UMT_MAXFACES + e.face]);
    g.need[e.from] += 1;
  }
  return 0;
}

// Host copies of the mesh connectivity the breaker needs.
struct HostConn {
  std::vector<int> zoneFaces, zoneOpp, faceOpp, numCorner, cOffSet;
};
static int host_conn(Ctx &c, HostConn &h) {
  h.zoneFaces.resize(c.nz); h.zoneOpp.resize((size_t)c.nz * UMT_MAXFACES); h.faceOpp.resize((size_t)c.nz * UMT_MAXFACES);
  h.numCorner.resize(c.nz); h.cOffSet.resize(c.nz);
  UMT_CUDA(cudaMemcpy(h.zoneFaces.data(), c.zoneFaces, c.nz * sizeof(int), cudaMemcpyDeviceToHost));
  UMT_CUDA(cudaMemcpy(h.zoneOpp.data(), c.zoneOpp, h.zoneOpp.size() * sizeof(int), cudaMemcpyDeviceToHost));
  UMT_CUDA(cudaMemcpy(h.faceOpp.data(), c.faceOpp, h.faceOpp.size() * sizeof(int), cudaMemcpyDeviceToHost));
  UMT_CUDA(cudaMemcpy(h.numCorner.data(), c.numCorner, c.nz * sizeof(int), cudaMemcpyDeviceToHost));
  UMT_CUDA(cudaMemcpy(h.cOffSet.data(), c.cOffSet, c.nz * sizeof(int), cudaMemcpyDeviceToHost));
  return 0;
}

// The per-direction dependency graphs (snneed) and corner orders, from scratch.
static int build_graphs(Ctx &c, const SchedArgs &p, int B) {
  Schedule &s = c.sch;
  const size_t n = (size_t)c.A * c.nz;
  UMT_CUDA(cudaMemsetAsync(s.need, 0, n * sizeof(int), c.stream));
  UMT_CUDA(cudaMemsetAsync(s.exitMask, 0, ((n + 3) & ~(size_t)3), c.stream));
  UMT_CUDA(cudaMemsetAsync(s.cycZ, 0, n, c.stream));
  k_need<<<B, 256, 0, c.stream>>>(p);
  k_corner_order<<<B, 256, 0, c.stream>>>(p);
  UMT_CUDA(cudaGetLastError());
  return 0;
}

// The wavefront over every direction at once.  Returns 0 when every item was
// placed, 1 when it stalled (a direction with a cycle, or without a seed).
static int run_wavefront(Ctx &c, int B, int *stalledAt) {
  Schedule &s = c.sch;
  const size_t n = (size_t)c.A * c.nz;
  UMT_CUDA(cudaMemsetAsync(s.level, 0xff, n * sizeof(int), c.stream));
  UMT_CUDA(cudaMemsetAsync(s.stageCount, 0, (c.nz + 2) * sizeof(int), c.stream));
  UMT_CUDA(cudaMemsetAsync(s.stageOffset, 0, (c.nz + 2) * sizeof(int), c.stream));
  UMT_CUDA(cudaMemsetAsync(s.nHyper, 0, c.A * sizeof(int), c.stream));
  UMT_CUDA(cudaMemsetAsync(s.processed, 0, sizeof(unsigned long long), c.stream));
  UMT_CUDA(cudaMemcpyAsync(s.needInit, s.need, n * sizeof(int), cudaMemcpyDeviceToDevice, c.stream));
  k_seed<<<B, 256, 0, c.stream>>>(c.nz, c.A, s.need, s.bad, s.items, s.stageCount, s.level, s.processed);
  UMT_CUDA(cudaGetLastError());
  const int batch = 32, SB = 152 * 8;
  unsigned long long placed = 0;
  int h = 0;
  while (true) {
    for (int k = 0; k < batch && h < c.nz; ++k, ++h)
      k_stage<<<SB, 256, 0, c.stream>>>(h, c.nz, c.A, c.zoneFaces, c.zoneOpp, s.exitMask, s.bad, s.need,
                                        s.items, s.stageCount, s.stageOffset, s.level, s.nHyper, s.processed);
    UMT_CUDA(cudaGetLastError());
    UMT_CUDA(cudaMemcpyAsync(&placed, s.processed, sizeof(placed), cudaMemcpyDeviceToHost, c.stream));
    UMT_CUDA(cudaStreamSynchronize(c.stream));
    if (placed == n) return 0;
    std::vector<int> cnt(h + 1);
    UMT_CUDA(cudaMemcpy(cnt.data(), s.stageCount, (h + 1) * sizeof(int), cudaMemcpyDeviceToHost));
    int h0 = cnt[0] == 0 ? 0 : -1;
    for (int k = 1; k <= h && h0 < 0; ++k)
      if (cnt[k] == 0) h0 = k;
    if (h0 >= 0) { *stalledAt = h0; return 1; }
    if (h >= c.nz) return set_error(-4, "schedule: %llu of %zu items placed after %d stages", placed, n, h);
  }
}

int build_schedule(Ctx &c) {
  Schedule &s = c.sch;
  const size_t n = (size_t)c.A * c.nz;
  SchedArgs p{c.nz, c.nc, c.A, c.numCorner, c.cOffSet, c.zoneFaces, c.zoneOpp, c.faceOpp,
              c.nCFaces, c.cEZ, c.CToFace, c.afp64, c.aez64, s.need, s.exitMask, s.bad, s.order, c.status, s.cycZ};
  const int B = (int)std::min<size_t>((n + 255) / 256, 152 * 32);
  TRY_RC(build_graphs(c, p, B));
  HostConn hc;
  bool haveConn = false;
  s.breaks = 0;
  int h0 = 0;
  int rc = run_wavefront(c, B, &h0);
  if (rc < 0) return rc;
  if (rc == 1) {
    // The directions left unplaced hold a cycle (or have no seed).  Their
    // graphs are rebuilt and put in the reference's sequential order on the
    // host; the wavefront then runs again over every direction.
    std::vector<int> lev(n);
    UMT_CUDA(cudaMemcpy(lev.data(), s.level, n * sizeof(int), cudaMemcpyDeviceToHost));
    std::vector<int> cyclic;
    for (int a = 0; a < c.A; ++a) {
      const size_t o = (size_t)a * c.nz;
      for (int z = 0; z < c.nz; ++z)
        if (lev[o + z] < 0) { cyclic.push_back(a); break; }
    }
    lev.clear();
    lev.shrink_to_fit();
    TRY_RC(build_graphs(c, p, B));
    TRY_RC(host_conn(c, hc));
    haveConn = true;
    std::vector<int> need(c.nz);
    std::vector<uint8_t> ex(c.nz), cy(c.nz);
    for (int a : cyclic) {
      const size_t o = (size_t)a * c.nz;
      UMT_CUDA(cudaMemcpy(need.data(), s.need + o, c.nz * sizeof(int), cudaMemcpyDeviceToHost));
      UMT_CUDA(cudaMemcpy(ex.data(), s.exitMask + o, c.nz, cudaMemcpyDeviceToHost));
      UMT_CUDA(cudaMemcpy(cy.data(), s.cycZ + o, c.nz, cudaMemcpyDeviceToHost));
      DirGraph g{c.nz, hc.zoneFaces.data(), hc.zoneOpp.data(), hc.faceOpp.data(), need.data(), ex.data(), cy.data()};
      if (order_direction(g)) return set_error(-4, "direction %d: a dependency cycle could not be broken", a);
      UMT_CUDA(cudaMemcpy(s.need + o, need.data(), c.nz * sizeof(int), cudaMemcpyHostToDevice));
      UMT_CUDA(cudaMemcpy(s.exitMask + o, ex.data(), c.nz, cudaMemcpyHostToDevice));
      UMT_CUDA(cudaMemcpy(s.cycZ + o, cy.data(), c.nz, cudaMemcpyHostToDevice));
    }
    s.breaks = (int)cyclic.size();
    rc = run_wavefront(c, B, &h0);
    if (rc < 0) return rc;
    if (rc == 1) return set_error(-4, "schedule stalled at stage %d after the cycles were ordered", h0);
  }
  {
    const int B2 = (int)std::min<size_t>((n + 255) / 256, 152 * 32);
    k_items2<<<B2, 256, 0, c.stream>>>(n, c.nz, s.items, c.cOffSet, c.numCorner, s.items2);
    UMT_CUDA(cudaGetLastError());
  }
  s.hCount.assign(c.nz + 2, 0);
  s.hOffset.assign(c.nz + 2, 0);
  UMT_CUDA(cudaMemcpy(s.hCount.data(), s.stageCount, (c.nz + 2) * sizeof(int), cudaMemcpyDeviceToHost));
  UMT_CUDA(cudaMemcpy(s.hOffset.data(), s.stageOffset, (c.nz + 2) * sizeof(int), cudaMemcpyDeviceToHost));
  s.nStages = 0;
  s.maxStageItems = 0;
  for (int k = 0; k < c.nz + 1; ++k) {
    if (s.hCount[k] == 0) break;
    s.nStages = k + 1;
    s.maxStageItems = std::max(s.maxStageItems, s.hCount[k]);
  }
  // the cycle list of every direction: the corners of its flagged zones
  {
    std::vector<uint8_t> cy(n);
    UMT_CUDA(cudaMemcpy(cy.data(), s.cycZ, n, cudaMemcpyDeviceToHost));
    if (!haveConn) { TRY_RC(host_conn(c, hc)); haveConn = true; }
    std::vector<long long> rows;
    s.hCycOff.assign(c.A + 1, 0);
    for (int a = 0; a < c.A; ++a) {
      s.hCycOff[a] = (long long)rows.size();
      for (int z = 0; z < c.nz; ++z)
        if (cy[(size_t)a * c.nz + z])
          for (int k = 0; k < hc.numCorner[z]; ++k) rows.push_back((long long)a * c.nc + hc.cOffSet[z] + k);
    }
    s.hCycOff[c.A] = (long long)rows.size();
    s.nCyc = (long long)rows.size();
    if (s.cycRow) { cudaFree(s.cycRow); s.cycRow = nullptr; }
    if (s.nCyc) {
      UMT_CUDA(cudaMalloc((void **)&s.cycRow, s.nCyc * sizeof(long long)));
      UMT_CUDA(cudaMemcpy(s.cycRow, rows.data(), s.nCyc * sizeof(long long), cudaMemcpyHostToDevice));
    }
  }
  return 0;
}

// psi_new rows of the cycle list <- the stored previous values (initFromCycleList,
// control/constructDynMemory.F90:111-161), before a sweep's first stage
template <typename T>
__global__ void k_cycle_init(long long nCyc, int G, const long long *row, const T *store, T *psi) {
  const long long m = nCyc * G;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m; i += (long long)gridDim.x * blockDim.x) {
    const long long k = i / G;
    psi[row[k] * G + (i - k * G)] = store[i];
  }
}

// the stored values <- psi_new rows (updateCycleList, :166-214), after the last stage
template <typename T>
__global__ void k_cycle_update(long long nCyc, int G, const long long *row, T *store, const T *psi) {
  const long long m = nCyc * G;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m; i += (long long)gridDim.x * blockDim.x) {
    const long long k = i / G;
    store[i] = psi[row[k] * G + (i - k * G)];
  }
}

int enqueue_cycle_init(Ctx &c, int precision, int cur) {
  const Schedule &s = c.sch;
  if (!s.nCyc) return 0;
  const int blocks = (int)std::min<long long>((s.nCyc * c.G + 255) / 256, 152 * 8);
  if (precision == 0) k_cycle_init<double><<<blocks, 256, 0, c.stream>>>(s.nCyc, c.G, s.cycRow, c.cycPsi64, c.psi64[1 - cur]);
  else k_cycle_init<float><<<blocks, 256, 0, c.stream>>>(s.nCyc, c.G, s.cycRow, c.cycPsi32, c.psi32[1 - cur]);
  UMT_CUDA(cudaGetLastError());
  return 0;
}

int enqueue_cycle_update(Ctx &c, int precision, int cur) {
  const Schedule &s = c.sch;
  if (!s.nCyc) return 0;
  const int blocks = (int)std::min<long long>((s.nCyc * c.G + 255) / 256, 152 * 8);
  if (precision == 0) k_cycle_update<double><<<blocks, 256, 0, c.stream>>>(s.nCyc, c.G, s.cycRow, c.cycPsi64, c.psi64[1 - cur]);
  else k_cycle_update<float><<<blocks, 256, 0, c.stream>>>(s.nCyc, c.G, s.cycRow, c.cycPsi32, c.psi32[1 - cur]);
  UMT_CUDA(cudaGetLastError());
  return 0;
}

// The stored cycle values <- the saved angular flux (Psi) at those corners,
// as the reference sets cyclePsi at the start of a cycle
// (control/initializeRadiationField_OMPOL.F90:105); allocates the stores.
int cycle_from_psi(Ctx &c) {
  const Schedule &s = c.sch;
  if (!s.nCyc) return 0;
  const size_t m = (size_t)s.nCyc * c.G;
  if (c.psi64[0] && !c.cycPsi64) UMT_CUDA(cudaMalloc((void **)&c.cycPsi64, m * sizeof(double)));
  if (c.psi32[0] && !c.cycPsi32) UMT_CUDA(cudaMalloc((void **)&c.cycPsi32, m * sizeof(float)));
  const int blocks = (int)std::min<long long>((s.nCyc * c.G + 255) / 256, 152 * 8);
  if (c.cycPsi64) k_cycle_update<double><<<blocks, 256, 0, c.stream>>>(s.nCyc, c.G, s.cycRow, c.cycPsi64, c.psi64[c.cur64]);
  if (c.cycPsi32) k_cycle_update<float><<<blocks, 256, 0, c.stream>>>(s.nCyc, c.G, s.cycRow, c.cycPsi32, c.psi32[c.cur32]);
  UMT_CUDA(cudaGetLastError());
  UMT_CUDA(cudaStreamSynchronize(c.stream));
  return 0;
}

}  // namespace umt
