// sweep32p.cu -- FP32 UCB sweep driven by precompiled zone programs.
//
// The arithmetic is that of snac/SweepUCBxyz.F90:103-312 (and of the kernels
// in sweep32.cu); what changes is how a (direction, zone) pair finds its work.
// The corner-face geometry of a zone, seen from one direction, does not change
// between sweeps, so the classification the sweep would otherwise redo every
// time -- which FP faces are incoming, which EZ faces carry flux and which of
// those use the opposite FP face's flux, which corners feed which inside the
// zone, which faces leave the mesh -- is done once, on the device, and written
// as a compact program per (direction, zone), stored in dependency-stage order:
//
//   header (uint4, one per work item, same order as the stage items)
//     x  a*nz + z | lagged << 31        y  cOffSet | numCorner << 28
//     z  program offset, 16-byte units  w  solve order (3 bits x 8) | length << 24
//   program (16-byte aligned 32-bit words)
//     w0  nA | nB << 5 | nE << 10 | nX << 15 | nD << 20
//     w1  pulls per solve step (2 bits x 8)
//     corner records  [nC]     {sumArea, Volume}
//     FP-in entries   [nB+nA]  {upwind | c << 28 | boundary << 31, -Omega.A_fp}
//     EZ-opp entries  [nB]     {c | cez << 3, Volume/Omega.A_ez}  (pairs FP-in entry i < nB)
//     EZ entries      [nE]     {c | cez << 3, 0.5 Omega.A_ez}
//     pulls           [nD]     {n, Omega.A_ez}  solve order; n feeds the step's corner
//     exits           [nX]     b | c << 28
//
// A team of GT lanes runs one program; each lane carries GPL consecutive
// groups (paired FP32 instructions on group pairs).  Every loop of the program
// is uniform across the team, so the lanes of one team never diverge, and the
// teams of one warp differ only in trip counts.  Each lane reads and writes
// only its own groups of the team's shared arrays, so after the program has
// been staged no further synchronisation is needed.
//
// Memory round trips per zone: (1) header; (2) program, previous flux and
// source of every corner (three bulk copies by one lane onto an mbarrier),
// cross sections; (3) every upwind flux.  The intra-zone solve pulls from upstream corners in the order
// the reference pushes to downstream ones, so every FMA chain of the solve is
// the reference's.
#include "umt_common.cuh"
#include "sweep32_util.cuh"
#include "../../include/umt103.h"

#include <algorithm>

namespace umt {

constexpr int P32_NT = 64;             // two warps: a block's slot frees when its 8 items are done
constexpr int P32_MAXCHUNK = 48;        // 16-byte units: 8 + 8*(8+24+24+24) + 4*24 bytes

struct ProgP {
  int nz, nc, nb, tstride, bstride;     // tstride: floats per team (Q and S arrays); bstride: program bytes per team
  uint32_t nzMagic;                     // a = (it * nzMagic) >> nzShift equals it / nz for it < 2^31
  int nzShift;
  const uint4 *hdr;
  const uint4 *prog;
  const float *Sigt, *STotal;
  float tau;
  const float *psi_old;
  float *psi_new, *psiB;
  unsigned *status;                     // device status word (a copy that never completed)
};

template <int NP>
__device__ __forceinline__ void ldg2(const float *p, float2 (&v)[NP]) {
  if constexpr (NP == 2) {
    const float4 t = *reinterpret_cast<const float4 *>(p);
    v[0] = make_float2(t.x, t.y); v[1] = make_float2(t.z, t.w);
  } else {
    v[0] = *reinterpret_cast<const float2 *>(p);
  }
}

__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }

// a / b for positive, normal b: the hardware reciprocal approximation
// (rcp_approx) times a, one paired multiply per group pair.
__device__ __forceinline__ float2 div2(float2 a, float2 b) {
  return __fmul2_rn(a, make_float2(rcp_approx(b.x), rcp_approx(b.y)));
}

// Floats between rows c and c+1 of one array: Q and S rows interleaved, the
// pair padded to a whole number of 32-bank spans.
__host__ __device__ constexpr int pair_stride(int G) { return (2 * G + 31) / 32 * 32; }

// One work item per team: the body of the stage kernels below.  blk is the
// block's index among the blocks of this problem's stage.  Calls that return
// PsiB to the host run the same kernel; their exiting rows are copied out of
// the device rows in chunks beside the stages (psib.cu), so no stage waits
// for stores to host memory to complete.
template <int GT, int GPL>
__device__ __forceinline__ void sweep_items(const ProgP &p, int off, int nItems, int blk) {
  static_assert(GPL == 2 || GPL == 4, "group pairs");
  constexpr int TEAMS = P32_NT / GT, NP = GPL / 2, NFC = GPL == 2 ? 12 : 8;
  constexpr int G = GT * GPL;
  extern __shared__ float4 smem4[];
  const int tid = threadIdx.x, team = tid / GT, lane = tid % GT;
  // The next stage's launch may start now: its blocks fill SMs as this
  // stage's finish and run their independent first two round trips.
  pdl_launch_dependents();
  const int k = blk * TEAMS + team;
  if (k >= nItems) return;                         // whole teams leave together
  const unsigned tm = team_mask(GT, tid);
  const int g0 = lane * GPL;
  // The team's Q rows (later the solved psi) [8][G], then its S rows (running
  // source) [8][G], each block a contiguous image of the HBM rows it is copied
  // from.  Consecutive teams are G banks apart (team stride), so the teams
  // sharing a shared-memory wavefront read disjoint banks.
  constexpr int RP = G;
  __shared__ __align__(8) uint64_t sBar[TEAMS];
  float *sQ = reinterpret_cast<float *>(smem4) + (size_t)team * p.tstride;
  float *sS = sQ + 8 * G;
  unsigned char *sB = reinterpret_cast<unsigned char *>(smem4) + (size_t)TEAMS * p.tstride * 4 +
                      (size_t)team * p.bstride;
  const uint4 h = p.hdr[off + k];
  const bool bad = (h.x >> 31) != 0;
  const uint32_t it = h.x & 0x7fffffffu;
  const int a = (int)(((unsigned long long)it * p.nzMagic) >> p.nzShift);
  const int z = (int)(it - (uint32_t)a * p.nz);
  const int c0 = (int)(h.y & 0x0fffffffu), nC = (int)(h.y >> 28);
  const uint32_t ord = h.w & 0xffffffu;
  const int nch = (int)(h.w >> 24);
  const size_t abase = (size_t)a * p.nc;
  float *psiNew = p.psi_new + abase * G + g0;
  float *psiBA = p.psiB + (size_t)a * p.nb * G + g0;
  // ---- round trip 2: program, previous flux, source, cross sections ----
  // One lane moves the program and the corners' previous flux and source
  // rows, each contiguous in HBM, with bulk copies on the team's mbarrier.
  // The program and the previous flux are read once per sweep: evict-first.
  // Rows narrower than 16 bytes (G < 4) go lane by lane.
  constexpr bool BULK_ROWS = (G * 4) % 16 == 0;
  if (lane == 0) {
    const unsigned long long once = l2_evict_first_policy();
    const uint32_t rows = (uint32_t)(nC * G * 4);
    mbar_init_one(&sBar[team]);
    mbar_expect_tx(&sBar[team], (uint32_t)nch * 16u + (BULK_ROWS ? 2u * rows : 0u));
    bulk_copy_pol(sB, p.prog + h.z, (uint32_t)nch * 16u, &sBar[team], once);
    if constexpr (BULK_ROWS) {
      bulk_copy_pol(sQ, p.psi_old + (abase + c0) * G, rows, &sBar[team], once);
      bulk_copy(sS, p.STotal + (size_t)c0 * G, rows, &sBar[team]);
    }
  }
  if constexpr (!BULK_ROWS) {
    const float *po = p.psi_old + (abase + c0) * G + g0;
    const float *st = p.STotal + (size_t)c0 * G + g0;
    for (int c = 0; c < nC; ++c) {
      cp_async(sQ + c * RP + g0, po + (size_t)c * G, GPL * 4);
      cp_async(sS + c * RP + g0, st + (size_t)c * G, GPL * 4);
    }
  }
  float2 sg[NP];
  ldg2<NP>(p.Sigt + (size_t)z * G + g0, sg);
  if constexpr (!BULK_ROWS) cp_async_wait_all();
  __syncwarp(tm);                                  // the barrier is initialised before anyone waits on it
  if (!mbar_wait_phase0(&sBar[team])) {            // a copy that never completed: report, give the
    atomicOr(p.status, UMT_DEV_TIMEOUT);           // copies in flight one more bounded wait, leave
    mbar_wait_phase0(&sBar[team]);
    return;
  }
  const uint32_t *W = reinterpret_cast<const uint32_t *>(sB);
  const uint32_t cnt = W[0], pcnt = W[1];
  const int nA = cnt & 31, nB = (cnt >> 5) & 31, nE = (cnt >> 10) & 31, nX = (cnt >> 15) & 31,
            nD = (cnt >> 20) & 31;
  const float2 *crec = reinterpret_cast<const float2 *>(sB + 8);
  const uint2 *fin = reinterpret_cast<const uint2 *>(sB + 8 + 8 * nC);
  const uint2 *ezo = fin + nB + nA;
  const uint2 *eze = ezo + nB;
  const uint2 *pul = eze + nE;
  const uint32_t *ex = reinterpret_cast<const uint32_t *>(pul + nD);
  // ---- corner sources: Q = tau*psi_old + STotal, S = V*Q ----
  const float2 tau2 = f2(p.tau);
#pragma unroll
  for (int c = 0; c < UMT_MAXCORNER; ++c)
    if (c < nC) {
      float2 q[NP], s[NP];
      ld2<NP>(sQ + c * RP + g0, q);
      ld2<NP>(sS + c * RP + g0, s);
      const float2 v2 = f2(crec[c].y);
#pragma unroll
      for (int j = 0; j < NP; ++j) {
        q[j] = __ffma2_rn(tau2, q[j], s[j]);
        s[j] = __fmul2_rn(v2, q[j]);
      }
      st2<NP>(sQ + c * RP + g0, q);
      st2<NP>(sS + c * RP + g0, s);
    }
  // ---- round trip 3: upwind fluxes; FP inflow and the EZ closure that uses them ----
  // Upwind fluxes were written by earlier stages: wait for the previous
  // stage's launch to complete (everything above reads only data that no
  // stage of this sweep writes).
  pdl_wait();
  const int nF = nA + nB;
  for (int base = 0; base < nF; base += NFC) {
    float2 pf[NFC][NP];
    uint32_t cd[NFC];
#pragma unroll
    for (int j = 0; j < NFC; ++j) {
      cd[j] = 0u;
      if (base + j < nF) {
        cd[j] = fin[base + j].x;
        const size_t idx = cd[j] & 0x0fffffffu;
        ldg2<NP>(((cd[j] >> 31) ? psiBA : psiNew) + idx * G, pf[j]);
      }
    }
#pragma unroll
    for (int j = 0; j < NFC; ++j) {
      const int i = base + j;
      if (i < nF) {
        const int c = (cd[j] >> 28) & 7;
        const float2 w2 = f2(__uint_as_float(fin[i].y));
        float2 sc[NP];
        ld2<NP>(sS + c * RP + g0, sc);
#pragma unroll
        for (int q = 0; q < NP; ++q) sc[q] = __ffma2_rn(w2, pf[j][q], sc[q]);
        if (i < nB) {
          // closure of SweepUCBxyz.F90:219-243 divided through by aez^4: with
          // x = sigma*V/aez, N = 1.82x^2+4x+3, Dh = 2x^3+3x^2+2x+1,
          //   sez = V*(N*(sigma*psi_opp - Qc) + Dh*(Qc - Qz)) / (N + 2x*Dh),
          // x capped at 1e8 so the polynomials stay finite in FP32
          const uint2 o = ezo[i];
          const int cez = (o.x >> 3) & 7;
          const float2 r2 = f2(__uint_as_float(o.y));
          const float2 V2 = f2(crec[c].y);
          float2 Qc[NP], Qz[NP], sz[NP];
          ld2<NP>(sQ + c * RP + g0, Qc);
          ld2<NP>(sQ + cez * RP + g0, Qz);
          ld2<NP>(sS + cez * RP + g0, sz);
#pragma unroll
          for (int q = 0; q < NP; ++q) {
            float2 x = __fmul2_rn(sg[q], r2);
            x.x = fminf(x.x, 1.0e8f); x.y = fminf(x.y, 1.0e8f);
            const float2 N = __ffma2_rn(__ffma2_rn(f2(1.82f), x, f2(4.f)), x, f2(3.f));
            const float2 Dh = __ffma2_rn(__ffma2_rn(__ffma2_rn(f2(2.f), x, f2(3.f)), x, f2(2.f)), x, f2(1.f));
            const float2 den = __ffma2_rn(__fadd2_rn(x, x), Dh, N);
            const float2 Aq = __ffma2_rn(sg[q], pf[j][q], neg2(Qc[q]));
            const float2 Bq = __fadd2_rn(Qc[q], neg2(Qz[q]));
            const float2 num = __ffma2_rn(N, Aq, __fmul2_rn(Dh, Bq));
            const float2 sez = __fmul2_rn(V2, div2(num, den));
            sc[q] = __fadd2_rn(sc[q], sez);
            sz[q] = __fadd2_rn(sz[q], neg2(sez));
          }
          st2<NP>(sS + cez * RP + g0, sz);
        }
        st2<NP>(sS + c * RP + g0, sc);
      }
    }
  }
  // ---- EZ faces without an incoming opposite FP face: sez = 0.5*aez/sigma*(Qc - Qz) ----
  if (nE > 0) {
    float2 rs[NP];
#pragma unroll
    for (int q = 0; q < NP; ++q) rs[q] = make_float2(__frcp_rn(sg[q].x), __frcp_rn(sg[q].y));
    for (int i = 0; i < nE; ++i) {
      const uint2 o = eze[i];
      const int c = o.x & 7, cez = (o.x >> 3) & 7;
      const float2 h2 = f2(__uint_as_float(o.y));
      float2 Qc[NP], Qz[NP], sc[NP], sz[NP];
      ld2<NP>(sQ + c * RP + g0, Qc);
      ld2<NP>(sQ + cez * RP + g0, Qz);
      ld2<NP>(sS + c * RP + g0, sc);
      ld2<NP>(sS + cez * RP + g0, sz);
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        const float2 sez = __fmul2_rn(__fmul2_rn(h2, rs[q]), __fadd2_rn(Qc[q], neg2(Qz[q])));
        sc[q] = __fadd2_rn(sc[q], sez);
        sz[q] = __fadd2_rn(sz[q], neg2(sez));
      }
      st2<NP>(sS + c * RP + g0, sc);
      st2<NP>(sS + cez * RP + g0, sz);
    }
  }
  // ---- corner solve; a lagged zone (SweepUCBxyz.F90:283-297) takes its
  //      upstream terms from the previous values of its corners ----
  if (bad) {
    for (int c = 0; c < nC; ++c) {
      float2 old[NP];
      ldg2<NP>(psiNew + (size_t)(c0 + c) * G, old);
      st2<NP>(sQ + c * RP + g0, old);
    }
  }
  float *res = bad ? sS : sQ;                      // where solved corners are kept
  int dp = 0;
  for (int i = 0; i < nC; ++i) {
    const int c = (int)((ord >> (3 * i)) & 7u);
    const int np = (int)((pcnt >> (2 * i)) & 3u);
    float2 acc[NP];
    ld2<NP>(sS + c * RP + g0, acc);
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      if (j < np) {
        const uint2 d = pul[dp + j];
        const float2 ae = f2(__uint_as_float(d.y));
        float2 pn[NP];
        ld2<NP>(sQ + (int)(d.x & 7u) * RP + g0, pn);
#pragma unroll
        for (int q = 0; q < NP; ++q) acc[q] = __ffma2_rn(ae, pn[q], acc[q]);
      }
    }
    dp += np;
    const float2 cr = crec[c];
    float2 v[NP];
#pragma unroll
    for (int q = 0; q < NP; ++q) {
      const float2 dn = __ffma2_rn(sg[q], f2(cr.y), f2(cr.x));
      v[q] = div2(acc[q], dn);
    }
    st2<NP>(res + c * RP + g0, v);
    st2<NP>(psiNew + (size_t)(c0 + c) * G, v);
  }
  // exiting boundary fluxes
  for (int x = 0; x < nX; ++x) {
    const uint32_t e = ex[x];
    float2 v[NP];
    ld2<NP>(res + (int)((e >> 28) & 7u) * RP + g0, v);
    st2<NP>(psiBA + (size_t)(e & 0x0fffffffu) * G, v);
  }
}

template <int GT, int GPL>
__global__ void __launch_bounds__(P32_NT, GPL == 2 ? 14 : 12) k_sweep32p(ProgP p, int off, int nItems) {
  sweep_items<GT, GPL>(p, off, nItems, blockIdx.x);
}

// One dependency stage of several problems of the same group tile in one
// launch: the blocks of problem j are [blockStart[j], blockStart[j+1]); each
// problem brings its own parameters, stage offset and size.
constexpr int PB_MAX = 64;
struct ProgBatchP {
  int n;
  int blockStart[PB_MAX + 1];
  int off[PB_MAX], cnt[PB_MAX];
  ProgP p[PB_MAX];
};

template <int GT, int GPL>
__global__ void __launch_bounds__(P32_NT, GPL == 2 ? 14 : 12) k_sweep32pm(const __grid_constant__ ProgBatchP b) {
  int lo = 0, hi = b.n - 1;
  const int bx = (int)blockIdx.x;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (b.blockStart[mid] <= bx) lo = mid; else hi = mid - 1;
  }
  sweep_items<GT, GPL>(b.p[lo], b.off[lo], b.cnt[lo], bx - b.blockStart[lo]);
}

// ---------------------------------------------------------------------------
// Program builder: one thread per work item, run twice (sizes, then contents).
// ---------------------------------------------------------------------------
constexpr unsigned PROG_ERR_RANGE = 1u;       // an index does not fit its field
constexpr unsigned PROG_ERR_PULLS = 2u;       // more than 3 upstream corners feed one corner
constexpr unsigned PROG_ERR_ORDER = 4u;       // solve order is not a permutation
constexpr unsigned PROG_ERR_TOTAL = 8u;       // programs exceed 2^32 16-byte units

__device__ __forceinline__ float pick3(const float4 &v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
__device__ __forceinline__ int pick3i(const int4 &v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }

// Returns the program length in 16-byte units and the program's shape (every
// count and trip count the kernel's loops depend on); writes the program
// when `out` is set.
__device__ int prog_item(uint2 w, uint32_t ordNib, int nz, int nc, const float4 *rec, const int4 *conn,
                         uint32_t *out, uint32_t *ord3, unsigned long long *shape, unsigned *err) {
  const bool bad = (w.x >> 31) != 0;
  const uint32_t it = w.x & 0x7fffffffu;
  const int a = (int)(it / (uint32_t)nz);
  const int c0 = (int)(w.y & 0x0fffffffu), nC = (int)(w.y >> 28);
  float4 r0[UMT_MAXCORNER], r1[UMT_MAXCORNER];
  int4 cn[UMT_MAXCORNER];
  int ncf[UMT_MAXCORNER];
  for (int c = 0; c < nC; ++c) {
    const size_t i = ((size_t)a * nc + c0 + c) * 2;
    r0[c] = rec[i];
    r1[c] = rec[i + 1];
    cn[c] = conn[c0 + c];
    ncf[c] = cn[c].w >> 9;
  }
  int ordc[UMT_MAXCORNER];
  unsigned seen = 0;
  for (int i = 0; i < nC; ++i) {
    ordc[i] = bad ? i : (int)((ordNib >> (4 * i)) & 15u);
    if (ordc[i] >= nC || ((seen >> ordc[i]) & 1u)) { atomicOr(err, PROG_ERR_ORDER); ordc[i] = i; }
    seen |= 1u << ordc[i];
  }
  auto cezOf = [&](int c, int e) { return (cn[c].w >> (3 * e)) & 7; };
  auto isB = [&](int c, int f) {          // incoming FP face f whose partner EZ face carries flux
    const int e = f == 0 ? 2 : f - 1;
    return ncf[c] == 3 && pick3(r1[c], e) > 0.f;
  };
  int nA = 0, nB = 0, nE = 0, nX = 0, nD = 0;
  uint32_t pc = 0;
  for (int c = 0; c < nC; ++c)
    for (int f = 0; f < ncf[c]; ++f) {
      const float af = pick3(r0[c], f);
      if (af < 0.f) { if (isB(c, f)) ++nB; else ++nA; }
      if (pick3i(cn[c], f) < 0 && af > 0.f) ++nX;
      const float ae = pick3(r1[c], f);
      const int fo = f == 2 ? 0 : f + 1;
      if (ae > 0.f && !(ncf[c] == 3 && pick3(r0[c], fo) < 0.f)) ++nE;
    }
  for (int i = 0; i < nC; ++i) {
    const int t = ordc[i];
    int k = 0;
    for (int j = 0; j < nC; ++j) {
      if (!bad && j >= i) break;
      const int n = ordc[j];
      if (n == t) continue;
      for (int e = 0; e < ncf[n]; ++e)
        if (pick3(r1[n], e) > 0.f && cezOf(n, e) == t) ++k;
    }
    if (k > 3) { atomicOr(err, PROG_ERR_PULLS); k = 3; }
    pc |= (uint32_t)k << (2 * i);
    nD += k;
  }
  const int words = 2 + 2 * nC + 2 * (nA + nB) + 2 * nB + 2 * nE + 2 * nD + nX;
  const int chunks = (words * 4 + 15) / 16;
  const uint32_t counts =
      (uint32_t)nA | (uint32_t)nB << 5 | (uint32_t)nE << 10 | (uint32_t)nX << 15 | (uint32_t)nD << 20;
  *shape = (unsigned long long)counts | (unsigned long long)pc << 25 | (unsigned long long)nC << 41 |
           (unsigned long long)bad << 45;
  if (!out) return chunks;
  uint32_t o = 0;
  out[o++] = counts;
  out[o++] = pc;
  for (int c = 0; c < nC; ++c) { out[o++] = __float_as_uint(r0[c].w); out[o++] = __float_as_uint(r1[c].w); }
  auto upcode = [&](int c, int f) -> uint32_t {
    const int up = pick3i(cn[c], f);
    const uint32_t idx = up >= 0 ? (uint32_t)up : (uint32_t)(-up - 1);
    if (idx > 0x0fffffffu) atomicOr(err, PROG_ERR_RANGE);
    return (idx & 0x0fffffffu) | (uint32_t)c << 28 | (up < 0 ? 0x80000000u : 0u);
  };
  const uint32_t oB = o, oA = o + 2 * nB, oEo = o + 2 * (nA + nB);
  uint32_t ib = 0, ia = 0;
  for (int c = 0; c < nC; ++c)
    for (int f = 0; f < ncf[c]; ++f) {
      const float af = pick3(r0[c], f);
      if (!(af < 0.f)) continue;
      if (isB(c, f)) {
        const int e = f == 0 ? 2 : f - 1;
        out[oB + 2 * ib] = upcode(c, f);
        out[oB + 2 * ib + 1] = __float_as_uint(-af);
        out[oEo + 2 * ib] = (uint32_t)c | (uint32_t)cezOf(c, e) << 3;
        out[oEo + 2 * ib + 1] = __float_as_uint(r1[c].w * __frcp_rn(pick3(r1[c], e)));
        ++ib;
      } else {
        out[oA + 2 * ia] = upcode(c, f);
        out[oA + 2 * ia + 1] = __float_as_uint(-af);
        ++ia;
      }
    }
  o = oEo + 2 * nB;
  for (int c = 0; c < nC; ++c)
    for (int e = 0; e < ncf[c]; ++e) {
      const float ae = pick3(r1[c], e);
      const int fo = e == 2 ? 0 : e + 1;
      if (ae > 0.f && !(ncf[c] == 3 && pick3(r0[c], fo) < 0.f)) {
        out[o++] = (uint32_t)c | (uint32_t)cezOf(c, e) << 3;
        out[o++] = __float_as_uint(0.5f * ae);
      }
    }
  for (int i = 0; i < nC; ++i) {
    const int t = ordc[i];
    int k = 0;
    for (int j = 0; j < nC && k < 3; ++j) {
      if (!bad && j >= i) break;
      const int n = ordc[j];
      if (n == t) continue;
      for (int e = 0; e < ncf[n] && k < 3; ++e)
        if (pick3(r1[n], e) > 0.f && cezOf(n, e) == t) {
          out[o++] = (uint32_t)n;
          out[o++] = __float_as_uint(pick3(r1[n], e));
          ++k;
        }
    }
  }
  for (int c = 0; c < nC; ++c)
    for (int f = 0; f < ncf[c]; ++f) {
      const int up = pick3i(cn[c], f);
      if (up < 0 && pick3(r0[c], f) > 0.f) {
        const uint32_t b = (uint32_t)(-up - 1);
        if (b > 0x0fffffffu) atomicOr(err, PROG_ERR_RANGE);
        out[o++] = (b & 0x0fffffffu) | (uint32_t)c << 28;
      }
    }
  while (o < (uint32_t)chunks * 4) out[o++] = 0u;
  uint32_t o3 = 0;
  for (int i = 0; i < nC; ++i) o3 |= (uint32_t)ordc[i] << (3 * i);
  *ord3 = o3;
  return chunks;
}

// Items of one stage are independent, so their headers may be stored in any
// order within the stage.  They are grouped by program shape (hashed into
// PROG_BINS bins per stage), so that the teams of one warp mostly run programs
// with identical trip counts and take the same branches.
constexpr int PROG_BINS = 64;

__device__ __forceinline__ int shape_bin(unsigned long long shape) {
  return (int)((shape * 0x9E3779B97F4A7C15ull) >> 58);
}

__device__ __forceinline__ int stage_of(long long t, const int *stageOffset, int nStages) {
  int lo = 0, hi = nStages - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (stageOffset[mid] <= t) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__global__ void k_prog_sizes(long long n, const uint2 *items2, const uint32_t *order, int nz, int nc,
                             const float4 *rec, const int4 *conn, const int *stageOffset, int nStages,
                             uint32_t *sizes, int *binCount, unsigned *err, unsigned *maxch) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const uint2 w = items2[t];
    uint32_t o3 = 0;
    unsigned long long shape = 0;
    const int ch = prog_item(w, order[w.x & 0x7fffffffu], nz, nc, rec, conn, nullptr, &o3, &shape, err);
    sizes[t] = (uint32_t)ch;
    atomicMax(maxch, (unsigned)ch);
    atomicAdd(binCount + (size_t)stage_of(t, stageOffset, nStages) * PROG_BINS + shape_bin(shape), 1);
  }
}

__global__ void k_prog_write(long long n, const uint2 *items2, const uint32_t *order, int nz, int nc,
                             const float4 *rec, const int4 *conn, const int *stageOffset, int nStages,
                             const uint32_t *offs, const int *binStart, int *binFill, uint4 *prog, uint4 *hdr,
                             unsigned *err) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const uint2 w = items2[t];
    uint32_t o3 = 0;
    unsigned long long shape = 0;
    const uint32_t off = offs[t];
    const int ch = prog_item(w, order[w.x & 0x7fffffffu], nz, nc, rec, conn,
                             reinterpret_cast<uint32_t *>(prog + off), &o3, &shape, err);
    const size_t bin = (size_t)stage_of(t, stageOffset, nStages) * PROG_BINS + shape_bin(shape);
    const int dst = binStart[bin] + atomicAdd(binFill + bin, 1);
    hdr[dst] = make_uint4(w.x, w.y, off, o3 | (uint32_t)ch << 24);
  }
}

// Exclusive scan of 32-bit program lengths into 32-bit offsets, in place:
// per-block scans, a single-block scan of the block totals, then the add.
constexpr int SCAN_NT = 1024;

__device__ unsigned long long block_exclusive_scan(unsigned long long v, unsigned long long *total) {
  __shared__ unsigned long long ws[SCAN_NT / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned long long x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[w] = x;
  __syncthreads();
  if (w == 0) {
    unsigned long long s = lane < SCAN_NT / 32 ? ws[lane] : 0ull;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < SCAN_NT / 32) ws[lane] = s;
  }
  __syncthreads();
  const unsigned long long incl = x + (w > 0 ? ws[w - 1] : 0ull);
  *total = ws[SCAN_NT / 32 - 1];
  __syncthreads();
  return incl - v;
}

__global__ void __launch_bounds__(SCAN_NT) k_scan_local(long long n, uint32_t *v, unsigned long long *bsum) {
  const long long i = blockIdx.x * (long long)SCAN_NT + threadIdx.x;
  const unsigned long long x = i < n ? v[i] : 0u;
  unsigned long long tot = 0;
  const unsigned long long ex = block_exclusive_scan(x, &tot);
  if (i < n) v[i] = (uint32_t)ex;
  if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(SCAN_NT) k_scan_totals(long long nb, unsigned long long *bsum) {
  unsigned long long carry = 0;
  for (long long base = 0; base < nb; base += SCAN_NT) {
    const long long i = base + threadIdx.x;
    const unsigned long long x = i < nb ? bsum[i] : 0ull;
    unsigned long long tot = 0;
    const unsigned long long ex = block_exclusive_scan(x, &tot);
    if (i < nb) bsum[i] = ex + carry;
    carry += tot;
  }
  if (threadIdx.x == 0) bsum[nb] = carry;
}

__global__ void k_scan_add(long long n, uint32_t *v, const unsigned long long *bsum, unsigned *err) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const unsigned long long o = bsum[i / SCAN_NT] + v[i];
    if (o > 0xffffffffull) atomicOr(err, PROG_ERR_TOTAL);
    v[i] = (uint32_t)o;
  }
}

bool sweep32p_supported(int G, int GT, int GPL) {
  return GT * GPL == G && (GPL == 2 || GPL == 4) &&
         (GT == 1 || GT == 2 || GT == 4 || GT == 8 || GT == 16 || GT == 32);
}

// Floats per team: 8 row pairs, plus G so that consecutive teams start G
// banks apart (a team's row window is G words wide).
static int team_stride_p(int G) { return 8 * pair_stride(G) + G; }

// Program bytes staged per team: the longest program, rounded so that the
// teams' copies start 4 banks apart (entry reads of the teams of one warp are
// 4 different addresses).
static int blob_stride_p(int maxChunks) {
  int ch = maxChunks;
  while ((4 * ch) % 32 != 4) ++ch;
  return ch * 16;
}

// Build the zone programs of every work item (once per context, outside any
// stream capture).  On a geometry the program format cannot hold, the context
// keeps no programs and the FP32 sweep uses the corner-slot kernel.
int prepare_prog32(Ctx &c) {
  if (c.progState != 0) return 0;
  c.progState = -1;
  const long long n = (long long)c.A * c.nz;
  if (n <= 0 || n > 0x7fffffffll || c.nc > 0x0fffffff || c.nb > 0x0fffffff) return 0;
  const int nS = c.sch.nStages;
  if (nS <= 0 || (int)c.sch.hOffset.size() < nS || (int)c.sch.hCount.size() < nS) return 0;
  uint32_t *offs = nullptr;
  unsigned long long *bsum = nullptr;
  unsigned *flags = nullptr;                       // [0] error bits, [1] longest program
  int *bins = nullptr;                             // [2][nS][PROG_BINS] start, fill
  const long long nb = (n + SCAN_NT - 1) / SCAN_NT;
  const size_t nbin = (size_t)nS * PROG_BINS;
  auto cleanup = [&]() {
    if (offs) cudaFree(offs);
    if (bsum) cudaFree(bsum);
    if (flags) cudaFree(flags);
    if (bins) cudaFree(bins);
    offs = nullptr; bsum = nullptr; flags = nullptr; bins = nullptr;
  };
  if (cudaMalloc((void **)&offs, (size_t)n * 4) != cudaSuccess ||
      cudaMalloc((void **)&bsum, (size_t)(nb + 1) * 8) != cudaSuccess ||
      cudaMalloc((void **)&flags, 8) != cudaSuccess ||
      cudaMalloc((void **)&bins, 2 * nbin * sizeof(int)) != cudaSuccess) {
    cleanup();
    cudaGetLastError();
    return 0;                                      // no room for programs: corner-slot kernel
  }
  unsigned long long total = 0;
  unsigned hf[2] = {0, 0};
  std::vector<int> hb(nbin);
  const int grid = 152 * 8;
  auto fail = [&](cudaError_t e, const char *what) {
    cleanup();
    return set_error(UMT_ERR_CUDA, "zone programs: %s: %s", what, cudaGetErrorString(e));
  };
  cudaError_t e = cudaMemsetAsync(flags, 0, 8, c.stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(bins, 0, 2 * nbin * sizeof(int), c.stream);
  if (e != cudaSuccess) return fail(e, "memset");
  k_prog_sizes<<<grid, 256, 0, c.stream>>>(n, c.sch.items2, c.sch.order, c.nz, c.nc, (const float4 *)c.rec32,
                                           (const int4 *)c.conn32, c.sch.stageOffset, nS, offs, bins, flags,
                                           flags + 1);
  k_scan_local<<<(unsigned)nb, SCAN_NT, 0, c.stream>>>(n, offs, bsum);
  k_scan_totals<<<1, SCAN_NT, 0, c.stream>>>(nb, bsum);
  k_scan_add<<<grid, 256, 0, c.stream>>>(n, offs, bsum, flags);
  e = cudaMemcpyAsync(&total, bsum + nb, 8, cudaMemcpyDeviceToHost, c.stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hf, flags, 8, cudaMemcpyDeviceToHost, c.stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hb.data(), bins, nbin * sizeof(int), cudaMemcpyDeviceToHost, c.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return fail(e, "size pass");
  if (hf[0] != 0 || hf[1] > (unsigned)P32_MAXCHUNK || total == 0) { cleanup(); return 0; }
  // bin starts: stage offset + items of the stage's earlier bins
  for (int s = 0; s < nS; ++s) {
    int acc = c.sch.hOffset[s];
    for (int b = 0; b < PROG_BINS; ++b) {
      const int k = hb[(size_t)s * PROG_BINS + b];
      hb[(size_t)s * PROG_BINS + b] = acc;
      acc += k;
    }
    if (acc != c.sch.hOffset[s] + c.sch.hCount[s]) { cleanup(); return 0; }
  }
  if (cudaMalloc((void **)&c.prog32, (size_t)total * 16) != cudaSuccess ||
      cudaMalloc((void **)&c.hdr32, (size_t)n * 16) != cudaSuccess) {
    if (c.prog32) cudaFree(c.prog32);
    if (c.hdr32) cudaFree(c.hdr32);
    c.prog32 = nullptr; c.hdr32 = nullptr;
    cleanup();
    cudaGetLastError();
    return 0;
  }
  e = cudaMemcpyAsync(bins, hb.data(), nbin * sizeof(int), cudaMemcpyHostToDevice, c.stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(bins + nbin, 0, nbin * sizeof(int), c.stream);
  if (e != cudaSuccess) return fail(e, "bins");
  k_prog_write<<<grid, 256, 0, c.stream>>>(n, c.sch.items2, c.sch.order, c.nz, c.nc, (const float4 *)c.rec32,
                                           (const int4 *)c.conn32, c.sch.stageOffset, nS, offs, bins, bins + nbin,
                                           (uint4 *)c.prog32, (uint4 *)c.hdr32, flags);
  e = cudaMemcpyAsync(hf, flags, 8, cudaMemcpyDeviceToHost, c.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return fail(e, "write pass");
  cleanup();
  if (hf[0] != 0) {
    cudaFree(c.prog32); cudaFree(c.hdr32);
    c.prog32 = nullptr; c.hdr32 = nullptr;
    return 0;
  }
  c.progBytes = (size_t)total * 16;
  c.progMaxChunks = (int)hf[1];
#define UMT_ATTRP(gt, gpl)                                                    \
  TRY_RC_P(allow_dynamic_smem((const void *)k_sweep32p<gt, gpl>));            \
  TRY_RC_P(allow_dynamic_smem((const void *)k_sweep32pm<gt, gpl>));
#define TRY_RC_P(x) do { int rc_ = (x); if (rc_) return rc_; } while (0)
  UMT_ATTRP(1, 2) UMT_ATTRP(2, 2) UMT_ATTRP(4, 2) UMT_ATTRP(8, 2) UMT_ATTRP(16, 2) UMT_ATTRP(32, 2)
  UMT_ATTRP(1, 4) UMT_ATTRP(2, 4) UMT_ATTRP(4, 4) UMT_ATTRP(8, 4) UMT_ATTRP(16, 4) UMT_ATTRP(32, 4)
#undef UMT_ATTRP
#undef TRY_RC_P
  c.progState = 1;
  return 0;
}

// One launch per dependency stage.  Returns 1 when the tile or the context
// has no program kernel (the caller then uses the corner-slot kernel).
// The zone-program kernel's parameters for a context and buffer parity.
static ProgP make_progp(const Ctx &c, int cur) {
  ProgP p;
  p.nz = c.nz; p.nc = c.nc; p.nb = c.nb;
  {
    // division by the invariant nz as a multiply-high (round-up method):
    // s = ceil(log2 nz), m = ceil(2^(31+s) / nz) < 2^32; exact for it < 2^31
    int s = 0;
    while ((1ll << s) < (long long)c.nz) ++s;
    const unsigned long long m = ((1ull << (31 + s)) + (unsigned long long)c.nz - 1) / (unsigned long long)c.nz;
    p.nzMagic = (uint32_t)m;
    p.nzShift = 31 + s;
  }
  p.tstride = team_stride_p(c.G);
  p.bstride = blob_stride_p(c.progMaxChunks);
  p.hdr = (const uint4 *)c.hdr32; p.prog = (const uint4 *)c.prog32;
  p.Sigt = c.Sigt32; p.STotal = c.STotal32; p.tau = c.homog32 ? 0.f : (float)c.tau;
  p.psi_old = c.psi32[cur]; p.psi_new = c.psi32[1 - cur]; p.psiB = c.homog32 ? c.psiB32h : c.psiB32;
  p.status = c.status;
  return p;
}

int enqueue_sweep32p(Ctx &c, int cur, int GT, int GPL) {
  if (c.progState != 1 || !sweep32p_supported(c.G, GT, GPL)) return 1;
  const ProgP p = make_progp(c, cur);
  const int TEAMS = P32_NT / GT;
  const size_t smem = (size_t)TEAMS * ((size_t)p.tstride * 4 + p.bstride);
  // Stage 0 follows the source conversion with ordinary stream order; every
  // later stage is launched as a programmatic dependent of the one before.
  cudaLaunchAttribute pdl[1];
  pdl[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  pdl[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.blockDim = dim3(P32_NT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = c.stream;
#define UMT_LAUNCHP(gt, gpl)                                                                   \
  if (GT == gt && GPL == gpl) {                                                                \
    void (*kern)(ProgP, int, int) = k_sweep32p<gt, gpl>;                                       \
    if (c.wantExitsThrough) {                                                                  \
      const int rq = enqueue_psib_chunks(c);                                                   \
      if (rq) return rq;                                                                       \
    }                                                                                          \
    for (int s = 0; s < c.sch.nStages; ++s) {                                                  \
      if (c.wantExitsThrough) {                                                                \
        const int rq = wait_psib_chunks(c, s);                                                 \
        if (rq) return rq;                                                                     \
      }                                                                                        \
      cfg.gridDim = dim3((c.sch.hCount[s] + TEAMS - 1) / TEAMS);                               \
      cfg.attrs = s > 0 && c.usePDL ? pdl : nullptr;                                           \
      cfg.numAttrs = s > 0 && c.usePDL ? 1 : 0;                                                \
      UMT_CUDA(cudaLaunchKernelEx(&cfg, kern, p, c.sch.hOffset[s], c.sch.hCount[s]));          \
      if (c.wantExitsThrough) {                                                                \
        const int rq = enqueue_exit_chunks(c, s);                                              \
        if (rq) return rq;                                                                     \
      }                                                                                        \
    }                                                                                          \
    if (c.wantExitsThrough) {                                                                  \
      const int rq = wait_psib_chunks(c, c.sch.nStages);                                       \
      if (rq) return rq;                                                                       \
    }                                                                                          \
    return 0;                                                                                  \
  }
  UMT_LAUNCHP(1, 2) UMT_LAUNCHP(2, 2) UMT_LAUNCHP(4, 2) UMT_LAUNCHP(8, 2) UMT_LAUNCHP(16, 2) UMT_LAUNCHP(32, 2)
  UMT_LAUNCHP(1, 4) UMT_LAUNCHP(2, 4) UMT_LAUNCHP(4, 4) UMT_LAUNCHP(8, 4) UMT_LAUNCHP(16, 4) UMT_LAUNCHP(32, 4)
#undef UMT_LAUNCHP
  return 1;
}

// The stages of several resident FP32 sweeps that share one group tile
// (GT, GPL), on stream st: stage s of every problem that has one goes into
// one launch of k_sweep32pm (split every PB_MAX problems), each launch after
// the first a programmatic dependent of the one before, as in a single
// sweep.  Every context must be on the zone-program path (progState 1).
int enqueue_batch_stages(const std::vector<Ctx *> &cs, const std::vector<int> &curs, int GT, int GPL,
                         cudaStream_t st) {
  if (cs.empty()) return 0;
  const int G = GT * GPL, TEAMS = P32_NT / GT;
  int maxStages = 0, bstride = 0;
  for (const Ctx *c : cs) {
    if (c->progState != 1 || c->G != G || !sweep32p_supported(c->G, GT, GPL))
      return set_error(UMT_ERR_STATE, "batch stages: a context is not on the zone-program path of this tile");
    maxStages = std::max(maxStages, c->sch.nStages);
    bstride = std::max(bstride, blob_stride_p(c->progMaxChunks));
  }
  std::vector<ProgP> ps(cs.size());
  for (size_t j = 0; j < cs.size(); ++j) {
    ps[j] = make_progp(*cs[j], curs[j]);
    ps[j].bstride = bstride;                       // one shared-memory layout for the launch
  }
  const size_t smem = (size_t)TEAMS * ((size_t)team_stride_p(G) * 4 + bstride);
  cudaLaunchAttribute pdl[1];
  pdl[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  pdl[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.blockDim = dim3(P32_NT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  void (*kern)(ProgBatchP) = nullptr;
#define UMT_PICKM(gt, gpl) if (GT == gt && GPL == gpl) kern = k_sweep32pm<gt, gpl>;
  UMT_PICKM(1, 2) UMT_PICKM(2, 2) UMT_PICKM(4, 2) UMT_PICKM(8, 2) UMT_PICKM(16, 2) UMT_PICKM(32, 2)
  UMT_PICKM(1, 4) UMT_PICKM(2, 4) UMT_PICKM(4, 4) UMT_PICKM(8, 4) UMT_PICKM(16, 4) UMT_PICKM(32, 4)
#undef UMT_PICKM
  if (!kern) return set_error(UMT_ERR_ARG, "batch stages: no kernel for tile %d x %d", GT, GPL);
  std::vector<ProgBatchP> b(1);
  bool first = true;
  auto flush = [&](ProgBatchP &pb) -> int {
    if (pb.n == 0) return 0;
    cfg.gridDim = dim3(pb.blockStart[pb.n]);
    cfg.attrs = first ? nullptr : pdl;
    cfg.numAttrs = first ? 0 : 1;
    first = false;
    UMT_CUDA(cudaLaunchKernelEx(&cfg, kern, pb));
    pb.n = 0;
    pb.blockStart[0] = 0;
    return 0;
  };
  ProgBatchP &pb = b[0];
  pb.n = 0;
  pb.blockStart[0] = 0;
  for (int s = 0; s < maxStages; ++s) {
    for (size_t j = 0; j < cs.size(); ++j) {
      const Ctx &c = *cs[j];
      if (s >= c.sch.nStages || c.sch.hCount[s] <= 0) continue;
      if (pb.n == PB_MAX) {
        const int rf = flush(pb);
        if (rf) return rf;
      }
      const int k = pb.n++;
      pb.p[k] = ps[j];
      pb.off[k] = c.sch.hOffset[s];
      pb.cnt[k] = c.sch.hCount[s];
      pb.blockStart[k + 1] = pb.blockStart[k] + (c.sch.hCount[s] + TEAMS - 1) / TEAMS;
    }
    const int rf = flush(pb);
    if (rf) return rf;
  }
  return 0;
}

}  // namespace umt
