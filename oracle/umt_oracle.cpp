// umt_oracle.cpp -- CPU FP64 restatement of Teton's UCB sweep path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA product in
// umt_gb300/csrc: only tests/, __graft_entry__.smoke() and bench.py's
// cpu_baseline / --impl reference legs may load it.  Nothing in the product
// links or calls it.
//
// Every function restates one reference routine (paths relative to the UMT
// source tree, src/teton/...).  All indices are 0-based; where Teton stores a
// sign in a 1-based index (nextZ < 0 marks a zone with an intra-zone corner
// cycle) the oracle stores -(zone+1).
//
// Array layouts (C order, identical memory order to the Fortran arrays):
//   A_fp, A_ez   [c][cf][3]          Geometry%A_fp(3,maxcf,ncornr)
//   cFP, cEZ     [c][cf]             cFP: global corner, >= nc => boundary nc+b
//   CToFace      [c][cf]             zone-local face
//   zoneOpp/faceOpp [z][maxFaces]    -1 on the problem boundary
//   Psi          [a][c][g]           Set%Psi(G,ncornr,A)
//   Psi1         [c][g], c < nc+nbelem
//   PsiB         [a][b][g]           Set%PsiB(G,nbelem,A)
//   Phi, STotal  [c][g];  Sigt [z][g]
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <stdexcept>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct MeshView {
  int nz, nc, nbelem, maxcf, maxFaces;
  const int *numCorner, *cOffSet, *zoneFaces, *zoneOpp, *faceOpp;
  const int *nCFaces, *cFP, *cEZ, *CToFace;
};

inline double dot3(const double *o, const double *a) {
  // DOT_PRODUCT(omega, A): ((0 + o1*a1) + o2*a2) + o3*a3, no contraction
  double s = 0.0;
  s = s + o[0] * a[0];
  s = s + o[1] * a[1];
  s = s + o[2] * a[2];
  return s;
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------------------
// geometryUCBxyz (rt/geometryUCBxyz.F90:9-185) + the zone volume and boundary
// area vectors of volumeUCBxyz (rt/volumeUCBxyz.F90:9-200).  Zone and face
// centres are vertex averages (mods/Geometry_mod.F90:344-441).
// ---------------------------------------------------------------------------
int orc_geometry(int nz, int nc, int nbelem, int maxcf, int maxFaces,
                 const int *numCorner, const int *cOffSet, const int *zoneFaces,
                 const int *zoneOpp, const int *nCFaces, const int *cFP,
                 const int *cEZ, const int *CToFace, const double *px,
                 double *A_fp, double *A_ez, double *Volume, double *VolumeZone,
                 double *A_bdy) {
  std::vector<double> fc(3 * maxFaces);
  std::vector<int> ncf(maxFaces);
  std::fill(A_fp, A_fp + (size_t)nc * maxcf * 3, 0.0);
  for (int zone = 0; zone < nz; ++zone) {
    const int nCorner = numCorner[zone], c0 = cOffSet[zone], nF = zoneFaces[zone];
    double zc[3] = {0, 0, 0};
    for (int c = 0; c < nCorner; ++c)
      for (int d = 0; d < 3; ++d) zc[d] += px[3 * (c0 + c) + d];
    for (int d = 0; d < 3; ++d) zc[d] /= (double)nCorner;
    std::fill(fc.begin(), fc.end(), 0.0);
    std::fill(ncf.begin(), ncf.end(), 0);
    for (int c = 0; c < nCorner; ++c)
      for (int cf = 0; cf < nCFaces[c0 + c]; ++cf) {
        int f = CToFace[(c0 + c) * maxcf + cf];
        ncf[f] += 1;
        for (int d = 0; d < 3; ++d) fc[3 * f + d] += px[3 * (c0 + c) + d];
      }
    for (int f = 0; f < nF; ++f)
      for (int d = 0; d < 3; ++d) fc[3 * f + d] = ncf[f] ? fc[3 * f + d] / (double)ncf[f] : 0.0;

    for (int c = 0; c < nCorner; ++c) {
      Volume[c0 + c] = 0.0;
      for (int k = 0; k < maxcf * 3; ++k) A_ez[(size_t)(c0 + c) * maxcf * 3 + k] = 0.0;
    }
    VolumeZone[zone] = 0.0;
    for (int c = 0; c < nCorner; ++c) {
      const int cc = c0 + c, nCF = nCFaces[cc];
      for (int cf1 = 0; cf1 < nCF; ++cf1) {
        const int cf2 = (cf1 + 1) % nCF;
        const int cfp = cFP[cc * maxcf + cf1];
        const int cez1 = cEZ[cc * maxcf + cf1], cez2 = cEZ[cc * maxcf + cf2];
        const int face = CToFace[cc * maxcf + cf1];
        const double *p0 = px + 3 * cc, *p1 = px + 3 * (c0 + cez1), *p2 = px + 3 * (c0 + cez2);
        double tdl[3], tfl[3], tzl[3], tfz[3], tfe1[3], tfe2[3];
        for (int d = 0; d < 3; ++d) {
          tdl[d] = 0.5 * (p1[d] - p2[d]);
          tfl[d] = fc[3 * face + d] - p0[d];
          tzl[d] = zc[d] - p0[d];
          tfz[d] = fc[3 * face + d] - zc[d];
          tfe1[d] = fc[3 * face + d] - 0.5 * (p1[d] + p0[d]);
          tfe2[d] = fc[3 * face + d] - 0.5 * (p2[d] + p0[d]);
        }
        double A_fep[3];
        A_fep[0] = 0.5 * (tfl[2] * tdl[1] - tfl[1] * tdl[2]);
        A_fep[1] = 0.5 * (tfl[0] * tdl[2] - tfl[2] * tdl[0]);
        A_fep[2] = 0.5 * (tfl[1] * tdl[0] - tfl[0] * tdl[1]);
        const int zOpp = zoneOpp[zone * maxFaces + face];
        double *afp = A_fp + ((size_t)cc * maxcf + cf1) * 3;
        if (zOpp >= 0) {
          if (zOpp > zone) {
            for (int d = 0; d < 3; ++d) afp[d] = A_fep[d];
            for (int cf = 0; cf < nCFaces[cfp]; ++cf)
              if (cFP[cfp * maxcf + cf] == cc)
                for (int d = 0; d < 3; ++d) A_fp[((size_t)cfp * maxcf + cf) * 3 + d] = -A_fep[d];
          } else {
            for (int d = 0; d < 3; ++d) A_fep[d] = afp[d];
          }
        } else {
          for (int d = 0; d < 3; ++d) afp[d] = A_fep[d];
          if (A_bdy) {
            const int b = cfp - nc;
            for (int d = 0; d < 3; ++d) A_bdy[3 * b + d] = A_fep[d];
          }
        }
        double A_fez1[3], A_fez2[3];
        A_fez1[0] = 0.5 * (tfz[2] * tfe1[1] - tfz[1] * tfe1[2]);
        A_fez1[1] = 0.5 * (tfz[0] * tfe1[2] - tfz[2] * tfe1[0]);
        A_fez1[2] = 0.5 * (tfz[1] * tfe1[0] - tfz[0] * tfe1[1]);
        A_fez2[0] = 0.5 * (tfz[1] * tfe2[2] - tfz[2] * tfe2[1]);
        A_fez2[1] = 0.5 * (tfz[2] * tfe2[0] - tfz[0] * tfe2[2]);
        A_fez2[2] = 0.5 * (tfz[0] * tfe2[1] - tfz[1] * tfe2[0]);
        for (int d = 0; d < 3; ++d) {
          A_ez[((size_t)cc * maxcf + cf1) * 3 + d] += A_fez1[d];
          A_ez[((size_t)cc * maxcf + cf2) * 3 + d] += A_fez2[d];
        }
        Volume[cc] += (1.0 / 3.0) * std::fabs(tzl[0] * A_fep[0] + tzl[1] * A_fep[1] + tzl[2] * A_fep[2]);
      }
      VolumeZone[zone] += Volume[cc];
    }
    // equal and opposite EZ areas (geometryUCBxyz.F90:166-178)
    for (int c = 0; c < nCorner; ++c) {
      const int cc = c0 + c;
      for (int cf1 = 0; cf1 < nCFaces[cc]; ++cf1) {
        const int cez = cEZ[cc * maxcf + cf1];
        if (cez > c)
          for (int cf2 = 0; cf2 < nCFaces[c0 + cez]; ++cf2)
            if (cEZ[(c0 + cez) * maxcf + cf2] == c)
              for (int d = 0; d < 3; ++d)
                A_ez[((size_t)(c0 + cez) * maxcf + cf2) * 3 + d] = -A_ez[((size_t)cc * maxcf + cf1) * 3 + d];
      }
    }
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Sweep schedule for one direction: snnext (snac/snnext.F90:12-234) with
// snneed (snac/snneed.F90:17-197), findseeds (snac/findseeds.F90:18-119),
// getDownStreamData (snac/getDownStreamData.F90:9-155), fixZone,
// cyclebreaker (snac/cyclebreaker.F90:13-160) and sccsearch
// (snac/sccsearch.F90:8-187).
//
// Outputs: nextZ[nz] (signed, see header), nextC[nc] (zone-local corner order),
// zonesInPlane[<=nz], cycleList[<=nc] (global corners); returns nHyperPlanes
// (>0) or a negative error code.  *numCycles receives the cycle-list length.
// ---------------------------------------------------------------------------
namespace {

struct SccState {
  const MeshView *m;
  std::vector<int> dfnum, lowlink, stack, tempList, zoneBreakList;
  std::vector<char> isnew, onstack;
  int ncount = 0, stackindex = 0, nBreaks = 0;
};

void sccsearch(SccState &S, int zone, int &meshCycles, std::vector<int> &needZ,
               std::vector<char> &exitFace, std::vector<int> &cycleList,
               std::vector<char> &onCycleList) {
  const MeshView &m = *S.m;
  S.ncount += 1;
  S.dfnum[zone] = S.ncount;
  S.lowlink[zone] = S.ncount;
  S.isnew[zone] = 0;
  S.stack[S.stackindex++] = zone;
  S.onstack[zone] = 1;
  for (int face = 0; face < m.zoneFaces[zone]; ++face) {
    if (exitFace[zone * m.maxFaces + face]) {
      int zone2 = m.zoneOpp[zone * m.maxFaces + face];
      if (zone2 >= 0) {
        if (S.isnew[zone2]) {
          sccsearch(S, zone2, meshCycles, needZ, exitFace, cycleList, onCycleList);
          if (S.lowlink[zone2] < S.lowlink[zone]) S.lowlink[zone] = S.lowlink[zone2];
        } else if (S.dfnum[zone2] < S.dfnum[zone] && S.onstack[zone2] &&
                   S.lowlink[zone2] < S.lowlink[zone]) {
          S.lowlink[zone] = S.lowlink[zone2];
        }
      }
    }
  }
  if (S.lowlink[zone] == S.dfnum[zone]) {
    int zone2 = S.stack[--S.stackindex];
    S.onstack[zone2] = 0;
    if (zone2 != zone) {
      int cyclesize = 0;
      while (zone2 != zone) {
        S.tempList[cyclesize++] = zone2;
        zone2 = S.stack[--S.stackindex];
      }
      S.tempList[cyclesize++] = zone2;
      S.onstack[S.tempList[0]] = 1;
      const int lowlinkZ = S.tempList[cyclesize - 1];
      for (int face = 0; face < m.zoneFaces[lowlinkZ]; ++face) {
        const int zoneBreak = m.zoneOpp[lowlinkZ * m.maxFaces + face];
        const int faceBreak = m.faceOpp[lowlinkZ * m.maxFaces + face];
        if (zoneBreak >= 0) {
          if (S.onstack[zoneBreak] && exitFace[zoneBreak * m.maxFaces + faceBreak]) {
            if (!onCycleList[zoneBreak]) {
              for (int c = 0; c < m.numCorner[zoneBreak]; ++c)
                cycleList[meshCycles++] = m.cOffSet[zoneBreak] + c;
              onCycleList[zoneBreak] = 1;
            }
            needZ[lowlinkZ] -= 1;
            exitFace[zoneBreak * m.maxFaces + faceBreak] = 0;
            if (needZ[lowlinkZ] == 0) S.zoneBreakList[S.nBreaks++] = lowlinkZ;
          }
        }
      }
      for (int i = 0; i < cyclesize; ++i) S.onstack[S.tempList[i]] = 0;
    }
  }
}

}  // namespace

int orc_schedule(int nz, int nc, int maxcf, int maxFaces,
                 const int *numCorner, const int *cOffSet, const int *zoneFaces,
                 const int *zoneOpp, const int *faceOpp, const int *nCFaces,
                 const int *CToFace, const int *cEZ, const double *A_fp,
                 const double *A_ez, const double *omega,
                 int *nextZ, int *nextC, int *zonesInPlane, int *cycleList_out,
                 int *numCycles_out) {
  MeshView m{nz, nc, 0, maxcf, maxFaces, numCorner, cOffSet, zoneFaces, zoneOpp,
             faceOpp, nCFaces, nullptr, cEZ, CToFace};
  std::vector<int> needZ(nz, 0), listZone(nz), cycleList(nc + 1);
  std::vector<char> exitFace((size_t)nz * maxFaces, 0), onCycleList(nz, 0), doneZ(nz, 0), badZone(nz, 0);
  int meshCycles = 0;

  // ---- snneed (3-D branch, snneed.F90:104-187) ----
  std::vector<double> afpm_Face(maxFaces);
  std::vector<int> nInc(maxFaces), nExit(maxFaces);
  for (int zone = 0; zone < nz; ++zone) {
    const int nCorner = numCorner[zone], c0 = cOffSet[zone], nF = zoneFaces[zone];
    std::fill(afpm_Face.begin(), afpm_Face.end(), 0.0);
    std::fill(nInc.begin(), nInc.end(), 0);
    std::fill(nExit.begin(), nExit.end(), 0);
    for (int c = 0; c < nCorner; ++c) {
      const int cc = c0 + c;
      for (int cf = 0; cf < nCFaces[cc]; ++cf) {
        const int face = CToFace[cc * maxcf + cf];
        const int zOpp = zoneOpp[zone * maxFaces + face];
        if (zOpp > zone) {
          const double afpm = dot3(omega, A_fp + ((size_t)cc * maxcf + cf) * 3);
          afpm_Face[face] += afpm;
          if (afpm < 0.0) nInc[face] += 1;
          else if (afpm > 0.0) nExit[face] += 1;
        }
      }
    }
    for (int face = 0; face < nF; ++face) {
      const int zOpp = zoneOpp[zone * maxFaces + face];
      if (zOpp > zone) {
        const int fOpp = faceOpp[zone * maxFaces + face];
        if (afpm_Face[face] < 0.0) {
          needZ[zone] += 1;
          exitFace[zOpp * maxFaces + fOpp] = 1;
          if (nExit[face] > 0 && !onCycleList[zone]) {
            for (int c = 0; c < nCorner; ++c) cycleList[meshCycles++] = c0 + c;
            onCycleList[zone] = 1;
          }
        } else if (afpm_Face[face] > 0.0) {
          needZ[zOpp] += 1;
          exitFace[zone * maxFaces + face] = 1;
          if (nInc[face] > 0 && !onCycleList[zOpp]) {
            for (int c = 0; c < numCorner[zOpp]; ++c) cycleList[meshCycles++] = cOffSet[zOpp] + c;
            onCycleList[zOpp] = 1;
          }
        }
      }
    }
  }

  // ---- findseeds (findseeds.F90:58-112) ----
  int newZones = 0;
  for (int zone = 0; zone < nz; ++zone)
    if (needZ[zone] == 0) listZone[newZones++] = zone;
  if (newZones == 0) {
    int minNeed = nz, zoneID = -1;
    for (int zone = 0; zone < nz; ++zone) {
      bool bdy = false;
      for (int f = 0; f < zoneFaces[zone]; ++f) bdy |= zoneOpp[zone * maxFaces + f] < 0;
      if (bdy && needZ[zone] < minNeed) { zoneID = zone; minNeed = needZ[zone]; }
    }
    if (zoneID < 0) return -2;
    newZones = 1;
    listZone[0] = zoneID;
    needZ[zoneID] = 0;
    for (int face = 0; face < zoneFaces[zoneID]; ++face) {
      if (!exitFace[zoneID * maxFaces + face]) {
        const int zOpp = zoneOpp[zoneID * maxFaces + face];
        const int fOpp = faceOpp[zoneID * maxFaces + face];
        if (zOpp >= 0) {
          for (int c = 0; c < numCorner[zOpp]; ++c) cycleList[meshCycles++] = cOffSet[zOpp] + c;
          exitFace[zOpp * maxFaces + fOpp] = 0;
          onCycleList[zOpp] = 1;
        }
      }
    }
  }

  // ---- getDownStreamData (getDownStreamData.F90:59-150) ----
  {
    int need[64], nDSC[64], DSC[64][8];
    for (int zone = 0; zone < nz; ++zone) {
      const int nCorner = numCorner[zone], c0 = cOffSet[zone];
      for (int c = 0; c < nCorner; ++c) { need[c] = 0; nDSC[c] = 0; }
      for (int c = 0; c < nCorner; ++c) {
        const int cc = c0 + c;
        for (int cf = 0; cf < nCFaces[cc]; ++cf) {
          const int cez = cEZ[cc * maxcf + cf];
          if (cez > c) {
            const double aez = dot3(omega, A_ez + ((size_t)cc * maxcf + cf) * 3);
            if (aez < 0.0) { need[c] += 1; DSC[cez][nDSC[cez]++] = c; }
            else if (aez > 0.0) { need[cez] += 1; DSC[c][nDSC[c]++] = cez; }
          }
        }
      }
      bool bad = false;
      for (int i = 0; i < nCorner; ++i) {
        int c = 0;  // minloc: first index of the minimum
        for (int k = 1; k < nCorner; ++k) if (need[k] < need[c]) c = k;
        nextC[c0 + i] = c;
        if (need[c] != 0) bad = true;
        for (int k = 0; k < nDSC[c]; ++k) need[DSC[c][k]] -= 1;
        need[c] = 99;
      }
      badZone[zone] = bad;
      if (bad) {
        for (int i = 0; i < nCorner; ++i) nextC[c0 + i] = i;
        for (int c = 0; c < nCorner; ++c) cycleList[meshCycles++] = c0 + c;   // fixZone
      }
    }
  }

  // ---- hyperplane construction (snnext.F90:109-195) ----
  int ndoneZ = 0, nextZone = 0, lastZone = 0, nHyperPlanes = 0;
  while (true) {
    zonesInPlane[nHyperPlanes++] = newZones;
    nextZone = lastZone + newZones;
    int addedZones = 0;
    for (int zID = 0; zID < newZones; ++zID) {
      const int zone = listZone[lastZone + zID];
      ndoneZ += 1;
      doneZ[zone] = 1;
      for (int face = 0; face < zoneFaces[zone]; ++face) {
        if (exitFace[zone * maxFaces + face]) {
          const int Zexit = zoneOpp[zone * maxFaces + face];
          if (Zexit >= 0 && !doneZ[Zexit]) {
            needZ[Zexit] -= 1;
            if (needZ[Zexit] == 0) { listZone[nextZone++] = Zexit; addedZones += 1; }
            else if (needZ[Zexit] < 0) return -3;
          }
        }
      }
      nextZ[ndoneZ - 1] = badZone[zone] ? -(zone + 1) : zone;
    }
    lastZone += newZones;
    if (lastZone == nz) break;
    if (addedZones > 0) {
      newZones = addedZones;
    } else {
      // cyclebreaker (cyclebreaker.F90:88-143)
      SccState S;
      S.m = &m;
      const int ngraph = nz - ndoneZ;
      S.dfnum.assign(nz, 0); S.lowlink.assign(nz, 0);
      S.stack.assign(ngraph + 1, 0); S.tempList.assign(ngraph + 1, 0); S.zoneBreakList.assign(ngraph + 1, 0);
      S.isnew.assign(nz, 1); S.onstack.assign(nz, 0);
      std::vector<int> listZ;
      for (int zone = 0; zone < nz; ++zone) {
        if (needZ[zone] == 0) S.isnew[zone] = 0;
        else listZ.push_back(zone);
      }
      if ((int)listZ.size() != ngraph) return -4;
      for (int zone : listZ)
        if (S.isnew[zone]) sccsearch(S, zone, meshCycles, needZ, exitFace, cycleList, onCycleList);
      if (S.nBreaks == 0) return -5;
      addedZones = 0;
      for (int i = 0; i < S.nBreaks; ++i) {
        const int zone = S.zoneBreakList[i];
        if (needZ[zone] == 0) { listZone[nextZone++] = zone; addedZones += 1; }
        else if (needZ[zone] < 0) return -6;
      }
      if (addedZones == 0) return -7;
      newZones = addedZones;
    }
  }
  if (meshCycles > nc) return -8;
  if (ndoneZ != nz) return -9;
  for (int i = 0; i < meshCycles; ++i) cycleList_out[i] = cycleList[i];
  *numCycles_out = meshCycles;
  return nHyperPlanes;
}

// ---------------------------------------------------------------------------
// SweepUCBxyz (snac/SweepUCBxyz.F90:11-322): one direction, all groups.
// Psi1 [nc+nbelem][G] in/out, Phi [nc][G] accumulated, PsiB [nbelem][G] of
// this angle in/out, Psi [nc][G] of this angle (read; written if savePsi).
// ---------------------------------------------------------------------------
int orc_sweep_angle(int nz, int nc, int nbelem, int maxcf, int G,
                    const int *numCorner, const int *cOffSet, const int *nCFaces,
                    const int *cFP, const int *cEZ, const double *A_fp,
                    const double *A_ez, const double *Volume, const double *Sigt,
                    const double *STotal, double tau, const double *omega,
                    double quadwt, int nHyperPlanes, const int *zonesInPlane,
                    const int *nextZ, const int *nextC, double *Psi1, double *Phi,
                    double *PsiB, double *Psi, int savePsi) {
  const double fouralpha = 1.82;
  const int MC = 8, MCF = 3;
  if (maxcf > MCF) return -1;
  std::vector<double> psi_opp(G), SigtVol(G * MC), src(G * MC), Q(G * MC), psifp(G * MCF, 0.0);
  int nxez[MC], ez_exit[MC][MCF];
  double coefpsi[MC][MCF], sumArea[MC], afp[MCF];
  int bdy_exit[2][MCF * MC];

  for (int ib = 0; ib < nbelem; ++ib)
    for (int g = 0; g < G; ++g) Psi1[(size_t)(nc + ib) * G + g] = PsiB[(size_t)ib * G + g];

  int ndoneZ = 0;
  for (int hp = 0; hp < nHyperPlanes; ++hp) {
    const int nzones = zonesInPlane[hp];
    for (int ii = 0; ii < nzones; ++ii) {
      const int zone0 = nextZ[ndoneZ + ii];
      const int zone = zone0 >= 0 ? zone0 : -zone0 - 1;
      const int nCorner = numCorner[zone], c0 = cOffSet[zone];
      if (nCorner > MC) return -1;
      int nxBdy = 0;
      for (int c = 0; c < nCorner; ++c)
        for (int g = 0; g < G; ++g) {
          const double source = STotal[(size_t)(c0 + c) * G + g] + tau * Psi[(size_t)(c0 + c) * G + g];
          Q[c * G + g] = source;
          src[c * G + g] = Volume[c0 + c] * source;
          SigtVol[c * G + g] = Sigt[(size_t)zone * G + g] * Volume[c0 + c];
        }
      for (int c = 0; c < MC; ++c) nxez[c] = 0;
      for (int c = 0; c < nCorner; ++c) {
        sumArea[c] = 0.0;
        const int nCF = nCFaces[c0 + c];
        for (int cf = 0; cf < nCF; ++cf) {
          afp[cf] = dot3(omega, A_fp + ((size_t)(c0 + c) * maxcf + cf) * 3);
          const int cfp = cFP[(c0 + c) * maxcf + cf];
          if (afp[cf] > 0.0) {
            sumArea[c] += afp[cf];
            if (cfp >= nc) { bdy_exit[0][nxBdy] = c; bdy_exit[1][nxBdy] = cfp - nc; nxBdy++; }
          } else if (afp[cf] < 0.0) {
            for (int g = 0; g < G; ++g) {
              psifp[cf * G + g] = Psi1[(size_t)cfp * G + g];
              src[c * G + g] = src[c * G + g] - afp[cf] * Psi1[(size_t)cfp * G + g];
            }
          }
        }
        for (int cf = 0; cf < nCF; ++cf) {
          const double aez = dot3(omega, A_ez + ((size_t)(c0 + c) * maxcf + cf) * 3);
          const int cez = cEZ[(c0 + c) * maxcf + cf];
          if (cez > c) {
            if (aez > 0.0) {
              ez_exit[c][nxez[c]] = cez; coefpsi[c][nxez[c]] = aez; nxez[c]++;
            } else if (aez < 0.0) {
              ez_exit[cez][nxez[cez]] = c; coefpsi[cez][nxez[cez]] = -aez; nxez[cez]++;
            }
          }
          if (aez > 0.0) {
            sumArea[c] += aez;
            double area_opp = 0.0;
            if (nCF == 3) {
              const int ifp = (cf + 1) % nCF;
              if (afp[ifp] < 0.0) {
                for (int g = 0; g < G; ++g) psi_opp[g] = psifp[ifp * G + g];
                area_opp = -afp[ifp];
              }
            } else {
              int ifp = cf;
              area_opp = 0.0;
              for (int g = 0; g < G; ++g) psi_opp[g] = 0.0;
              for (int k = 0; k < nCF - 2; ++k) {
                ifp = (ifp + 1) % nCF;
                if (afp[ifp] < 0.0) {
                  area_opp = area_opp - afp[ifp];
                  for (int g = 0; g < G; ++g) psi_opp[g] = psi_opp[g] - afp[ifp] * psifp[ifp * G + g];
                }
              }
              if (area_opp > 0.0) {
                const double area_inv = 1.0 / area_opp;
                for (int g = 0; g < G; ++g) psi_opp[g] = psi_opp[g] * area_inv;
              }
            }
            if (area_opp > 0.0) {
              const double aez2 = aez * aez;
              const double vol = Volume[c0 + c];
              for (int g = 0; g < G; ++g) {
                const double sig = Sigt[(size_t)zone * G + g];
                const double sigv = sig * vol;
                const double sigv2 = sigv * sigv;
                const double gnum = aez2 * (fouralpha * sigv2 + aez * (4.0 * sigv + 3.0 * aez));
                const double gden = vol * (4.0 * sigv * sigv2 + aez * (6.0 * sigv2 + 2.0 * aez * (2.0 * sigv + aez)));
                const double sez = (vol * gnum * (sig * psi_opp[g] - Q[c * G + g]) +
                                    0.5 * aez * gden * (Q[c * G + g] - Q[cez * G + g])) /
                                   (gnum + gden * sig);
                src[c * G + g] = src[c * G + g] + sez;
                src[cez * G + g] = src[cez * G + g] - sez;
              }
            } else {
              for (int g = 0; g < G; ++g) {
                const double sigInv = 1.0 / Sigt[(size_t)zone * G + g];
                const double sez = 0.5 * aez * sigInv * (Q[c * G + g] - Q[cez * G + g]);
                src[c * G + g] = src[c * G + g] + sez;
                src[cez * G + g] = src[cez * G + g] - sez;
              }
            }
          }
        }
      }
      if (zone0 >= 0) {
        for (int i = 0; i < nCorner; ++i) {
          const int c = nextC[c0 + i];
          for (int g = 0; g < G; ++g) {
            const double v = src[c * G + g] / (sumArea[c] + SigtVol[c * G + g]);
            Psi1[(size_t)(c0 + c) * G + g] = v;
            Phi[(size_t)(c0 + c) * G + g] = Phi[(size_t)(c0 + c) * G + g] + quadwt * v;
          }
          for (int k = 0; k < nxez[c]; ++k) {
            const int cez = ez_exit[c][k];
            for (int g = 0; g < G; ++g)
              src[cez * G + g] = src[cez * G + g] + coefpsi[c][k] * Psi1[(size_t)(c0 + c) * G + g];
          }
        }
      } else {
        for (int c = 0; c < nCorner; ++c)
          for (int k = 0; k < nxez[c]; ++k) {
            const int cez = ez_exit[c][k];
            for (int g = 0; g < G; ++g)
              src[cez * G + g] = src[cez * G + g] + coefpsi[c][k] * Psi1[(size_t)(c0 + c) * G + g];
          }
        for (int c = 0; c < nCorner; ++c)
          for (int g = 0; g < G; ++g) {
            const double v = src[c * G + g] / (sumArea[c] + SigtVol[c * G + g]);
            Psi1[(size_t)(c0 + c) * G + g] = v;
            Phi[(size_t)(c0 + c) * G + g] = Phi[(size_t)(c0 + c) * G + g] + quadwt * v;
          }
      }
      for (int ib = 0; ib < nxBdy; ++ib) {
        const int c = bdy_exit[0][ib], b = bdy_exit[1][ib];
        for (int g = 0; g < G; ++g) PsiB[(size_t)b * G + g] = Psi1[(size_t)(c0 + c) * G + g];
      }
    }
    ndoneZ += nzones;
  }
  if (savePsi)
    for (size_t k = 0; k < (size_t)nc * G; ++k) Psi[k] = Psi1[k];
  return 0;
}

// ---------------------------------------------------------------------------
// SetSweep (snac/SetSweep.F90:10-214) for one angle set / one group set on
// one rank: Phi = 0, then per angle initFromCycleList, SweepUCBxyz and
// updateCycleList (control/constructDynMemory.F90:111-214).  With one set,
// getPhiTotal (control/getPhiTotal_OMPOL.F90:140-160) is PhiTotal = Phi.
//
// Schedules are packed per angle: nextZ[a*nz + i], nextC[a*nc + c],
// zonesInPlane[a*nz + h], nHyperPlanes[a], cycleList at cycleOffSet[a].
// nthreads > 1 sweeps angles concurrently, each thread with its own Psi1 and
// Phi (exact when no zone is lagged); nthreads == 1 is the reference order.
// ---------------------------------------------------------------------------
int orc_set_sweep(int nz, int nc, int nbelem, int maxcf, int G, int A,
                  const int *numCorner, const int *cOffSet, const int *nCFaces,
                  const int *cFP, const int *cEZ, const double *A_fp,
                  const double *A_ez, const double *Volume, const double *Sigt,
                  const double *STotal, double tau, const double *omega,
                  const double *weight, const int *nHyperPlanes,
                  const int *zonesInPlane, const int *nextZ, const int *nextC,
                  const int *numCycles, const int *cycleOffSet, const int *cycleList,
                  double *cyclePsi, double *Psi1, double *Phi, double *PsiB,
                  double *Psi, int savePsi, int nthreads) {
  const size_t ncG = (size_t)nc * G;
  std::fill(Phi, Phi + ncG, 0.0);
  int status = 0;
  auto one_angle = [&](int a, double *P1, double *Ph) {
    const int off = cycleOffSet[a];
    for (int m = 0; m < numCycles[a]; ++m) {
      const int c = cycleList[off + m];
      for (int g = 0; g < G; ++g) P1[(size_t)c * G + g] = cyclePsi[(size_t)(off + m) * G + g];
    }
    int rc = orc_sweep_angle(nz, nc, nbelem, maxcf, G, numCorner, cOffSet, nCFaces, cFP, cEZ,
                             A_fp, A_ez, Volume, Sigt, STotal, tau, omega + 3 * a, weight[a],
                             nHyperPlanes[a], zonesInPlane + (size_t)a * nz, nextZ + (size_t)a * nz,
                             nextC + (size_t)a * nc, P1, Ph, PsiB + (size_t)a * nbelem * G,
                             Psi + (size_t)a * ncG, savePsi);
    for (int m = 0; m < numCycles[a]; ++m) {
      const int c = cycleList[off + m];
      for (int g = 0; g < G; ++g) cyclePsi[(size_t)(off + m) * G + g] = P1[(size_t)c * G + g];
    }
    return rc;
  };
  if (nthreads <= 1) {
    for (int a = 0; a < A; ++a) {
      int rc = one_angle(a, Psi1, Phi);
      if (rc) return rc;
    }
    return 0;
  }
#ifdef _OPENMP
  const size_t p1n = (size_t)(nc + nbelem) * G;
#pragma omp parallel num_threads(nthreads)
  {
    std::vector<double> P1(Psi1, Psi1 + p1n), Ph(ncG, 0.0);
#pragma omp for schedule(dynamic, 1)
    for (int a = 0; a < A; ++a) {
      int rc = one_angle(a, P1.data(), Ph.data());
      if (rc) status = rc;
    }
#pragma omp critical
    for (size_t k = 0; k < ncG; ++k) Phi[k] += Ph[k];
  }
#endif
  return status;
}

// ---------------------------------------------------------------------------
// Black-body group integrals: the published rational approximation of Clark
// (J. Comput. Phys. 70 (1987) 311, eqs. 32 and 48) that
// misc/NormalizedBlackBody.cc:29-60,151-186 evaluates.
// ---------------------------------------------------------------------------
static double clark_cumulative(double e) {
  if (e < 0.01) {
    const double c3 = 0.05132991127342032, c4 = 0.01924871672753262;
    return e * e * e * (c3 - c4 * e);
  }
  const double p1 = 1.2807339766120354, p2 = 0.8578722513311724, p3 = 0.33288908614428098,
               p4 = 0.079984931563508915, p5 = 0.011878558806454416;
  const double q1 = 0.2807339758744, q2 = 0.07713864107538;
  const double tail = std::exp(-e) * (1.0 + e * (p1 + e * (p2 + e * (p3 + e * (p4 + e * p5))))) /
                      (1.0 + e * (q1 + e * q2));
  return 1.0 - tail;
}

void orc_planck_groups(double T, double k, double Bnorm, int ngr, const double *gnu, double *B) {
  const double kT = k * T;
  if (!(kT > 0.0)) { for (int g = 0; g < ngr; ++g) B[g] = 0.0; return; }
  const double full = Bnorm * (T * T) * (T * T);
  double lo = 0.0;
  for (int g = 0; g < ngr - 1; ++g) {
    const double hi = clark_cumulative(gnu[g + 1] / kT);
    B[g] = full * (hi - lo);
    lo = hi;
  }
  B[ngr - 1] = full * (1.0 - lo);
}

// ---------------------------------------------------------------------------
// 2-D RZ geometry: rt/geometryUCBrz.F90:36-150 (zone centre = vertex average,
// mods/Geometry_mod.F90 getZoneCenter).  Two corner faces per corner; cEZ is
// zone-local, cFP global (>= nc for a boundary element).  Face vectors are
// written as 3-vectors with a zero third component, so the 3-D schedule
// routines above order the RZ sweep.  The reference's `c < cfp` test compares
// a zone-local with a global 1-based index; it is kept as written.
// ---------------------------------------------------------------------------
int orc_geometry_rz(int nz, int nc, const int *numCorner, const int *cOffSet, const int *cEZ, const int *cFP,
                    const double *px, double *A_fp, double *A_ez, double *Area, double *Volume,
                    double *RadiusFP, double *RadiusEZ) {
  std::fill(A_fp, A_fp + (size_t)nc * 2 * 3, 0.0);
  std::fill(A_ez, A_ez + (size_t)nc * 2 * 3, 0.0);
  auto AF = [&](int cc, int f, int d) -> double & { return A_fp[((size_t)cc * 2 + f) * 3 + d]; };
  auto AE = [&](int cc, int f, int d) -> double & { return A_ez[((size_t)cc * 2 + f) * 3 + d]; };
  for (int zone = 0; zone < nz; ++zone) {
    const int nC = numCorner[zone], c0 = cOffSet[zone];
    double rz = 0.0, zz = 0.0;
    for (int c = 0; c < nC; ++c) { rz += px[2 * (c0 + c)]; zz += px[2 * (c0 + c) + 1]; }
    rz /= (double)nC;
    zz /= (double)nC;
    for (int c = 0; c < nC; ++c) {
      const int cc = c0 + c;
      const int c1 = cEZ[2 * cc], c2 = cEZ[2 * cc + 1];
      const int cfp1 = cFP[2 * cc], cfp2 = cFP[2 * cc + 1];
      const double r = px[2 * cc], z = px[2 * cc + 1];
      const double r1 = px[2 * (c0 + c1)], z1 = px[2 * (c0 + c1) + 1];
      const double r2 = px[2 * (c0 + c2)], z2 = px[2 * (c0 + c2) + 1];
      const double re1 = 0.5 * (r + r1), ze1 = 0.5 * (z + z1);
      const double re2 = 0.5 * (r + r2), ze2 = 0.5 * (z + z2);
      RadiusFP[2 * cc] = 0.5 * (r + re2);
      RadiusFP[2 * cc + 1] = 0.5 * (r + re1);
      RadiusEZ[2 * cc] = 0.5 * (rz + re1);
      RadiusEZ[2 * cc + 1] = 0.5 * (rz + re2);
      if (c < cfp1) {                        // (c+1) < (cfp1+1) in the 1-based original
        AF(cc, 0, 0) = 0.5 * (z2 - z);
        AF(cc, 0, 1) = 0.5 * (r - r2);
        if (cfp1 < nc) { AF(cfp1, 1, 0) = -AF(cc, 0, 0); AF(cfp1, 1, 1) = -AF(cc, 0, 1); }
      }
      if (c < cfp2) {
        AF(cc, 1, 0) = 0.5 * (z - z1);
        AF(cc, 1, 1) = 0.5 * (r1 - r);
        if (cfp2 < nc) { AF(cfp2, 0, 0) = -AF(cc, 1, 0); AF(cfp2, 0, 1) = -AF(cc, 1, 1); }
      }
      if (c < c1) {
        AE(cc, 0, 0) = ze1 - zz;
        AE(cc, 0, 1) = rz - re1;
        AE(c0 + c1, 1, 0) = -AE(cc, 0, 0);
        AE(c0 + c1, 1, 1) = -AE(cc, 0, 1);
      }
      if (c < c2) {
        AE(cc, 1, 0) = zz - ze2;
        AE(cc, 1, 1) = re2 - rz;
        AE(c0 + c2, 0, 0) = -AE(cc, 1, 0);
        AE(c0 + c2, 0, 1) = -AE(cc, 1, 1);
      }
      const double area1 = std::fabs((re2 - r) * (zz - z) - (ze2 - z) * (rz - r));
      const double area2 = std::fabs((rz - r) * (ze1 - z) - (zz - z) * (re1 - r));
      Area[cc] = 0.5 * (area1 + area2);
      const double rbar1 = (r + re2 + rz) / 3.0, rbar2 = (r + re1 + rz) / 3.0;
      Volume[cc] = 0.5 * (rbar1 * area1 + rbar2 * area2);
    }
  }
  return 0;
}

// One RZ direction: snac/SweepUCBrz.F90:87-276.  Psi1 [(nc+nb)][G] carries
// the previous direction's values; PsiM [nc][G] is the half-angle intensity.
static void sweep_rz_angle(int nz, int nc, int nb, int G, const int *numCorner, const int *cOffSet, const int *cFP,
                           const int *cEZ, const double *A_fp, const double *A_ez, const double *Area,
                           const double *Volume, const double *RadiusFP, const double *RadiusEZ, const double *Sigt,
                           const double *STotal, double tau, const double *om, double quadwt, double fac,
                           double W1, double W2, bool starting, int nHyper, const int *zonesInPlane,
                           const int *nextZ, const int *nextC, const double *psiA, double *Psi1, double *PsiM,
                           double *Phi) {
  const double fouralpha = 1.82;
  int maxC = 1;
  for (int z = 0; z < nz; ++z) maxC = std::max(maxC, numCorner[z]);
  std::vector<double> Q((size_t)maxC * G), src((size_t)maxC * G), coefpsi(2 * maxC);
  std::vector<double> sumArea(maxC);
  std::vector<int> nxez(maxC), ez_exit(2 * maxC);
  int ndoneZ = 0;
  for (int h = 0; h < nHyper; ++h) {
    const int nzones = zonesInPlane[h];
    for (int ii = 0; ii < nzones; ++ii) {
      const int zone0 = nextZ[ndoneZ + ii];
      const int zone = zone0 < 0 ? -zone0 - 1 : zone0;
      const int nC = numCorner[zone], c0 = cOffSet[zone];
      for (int c = 0; c < nC; ++c) {
        nxez[c] = 0;
        for (int g = 0; g < G; ++g) {
          const double source = STotal[(size_t)(c0 + c) * G + g] + tau * psiA[(size_t)(c0 + c) * G + g];
          Q[(size_t)c * G + g] = source;
          src[(size_t)c * G + g] = Volume[c0 + c] * source;
        }
        sumArea[c] = fac * Area[c0 + c];
      }
      for (int c = 0; c < nC; ++c) {
        const int cc = c0 + c;
        for (int cface = 0; cface < 2; ++cface) {
          const double afp = dot3(om, A_fp + ((size_t)cc * 2 + cface) * 3);
          const double aez = dot3(om, A_ez + ((size_t)cc * 2 + cface) * 3);
          int cfp = -1;
          if (afp < 0.0) {
            cfp = cFP[2 * cc + cface];
            const double R_afp = RadiusFP[2 * cc + cface] * afp;
            sumArea[c] = sumArea[c] - R_afp;
            for (int g = 0; g < G; ++g)
              src[(size_t)c * G + g] = src[(size_t)c * G + g] - R_afp * Psi1[(size_t)cfp * G + g];
          }
          if (aez > 0.0) {
            const double R = RadiusEZ[2 * cc + cface];
            const int cez = cEZ[2 * cc + cface];
            const double area = Area[cc];
            ez_exit[2 * c + nxez[c]] = cez;
            coefpsi[2 * c + nxez[c]] = R * aez;
            nxez[c] += 1;
            sumArea[cez] = sumArea[cez] + R * aez;
            if (afp < 0.0) {
              for (int g = 0; g < G; ++g) {
                const double sig = Sigt[(size_t)zone * G + g];
                const double sigA = sig * area, sigA2 = sigA * sigA;
                const double gnum = aez * aez * (fouralpha * sigA2 + aez * (4.0 * sigA + 3.0 * aez));
                const double gden = area * (4.0 * sigA * sigA2 + aez * (6.0 * sigA2 + 2.0 * aez * (2.0 * sigA + aez)));
                const double Qc = Q[(size_t)c * G + g], Qz = Q[(size_t)cez * G + g];
                const double sez = R * (area * gnum * (sig * Psi1[(size_t)cfp * G + g] - Qc) +
                                        0.5 * aez * gden * (Qc - Qz)) / (gnum + gden * sig);
                src[(size_t)c * G + g] = src[(size_t)c * G + g] + sez;
                src[(size_t)cez * G + g] = src[(size_t)cez * G + g] - sez;
              }
            } else {
              for (int g = 0; g < G; ++g) {
                const double Qc = Q[(size_t)c * G + g], Qz = Q[(size_t)cez * G + g];
                const double sez = 0.5 * R * aez * (Qc - Qz) / Sigt[(size_t)zone * G + g];
                src[(size_t)c * G + g] = src[(size_t)c * G + g] + sez;
                src[(size_t)cez * G + g] = src[(size_t)cez * G + g] - sez;
              }
            }
          }
        }
      }
      for (int i = 0; i < nC; ++i) {
        const int c = nextC[c0 + i];
        for (int g = 0; g < G; ++g)
          Psi1[(size_t)(c0 + c) * G + g] =
              (src[(size_t)c * G + g] + Area[c0 + c] * fac * PsiM[(size_t)(c0 + c) * G + g]) /
              (sumArea[c] + Sigt[(size_t)zone * G + g] * Volume[c0 + c]);
        for (int f = 0; f < nxez[c]; ++f) {
          const int cez = ez_exit[2 * c + f];
          for (int g = 0; g < G; ++g)
            src[(size_t)cez * G + g] = src[(size_t)cez * G + g] + coefpsi[2 * c + f] * Psi1[(size_t)(c0 + c) * G + g];
        }
      }
      for (int c = 0; c < nC; ++c)
        for (int g = 0; g < G; ++g) {
          const size_t e = (size_t)(c0 + c) * G + g;
          if (starting) {
            PsiM[e] = Psi1[e];
          } else {
            PsiM[e] = W1 * Psi1[e] - W2 * PsiM[e];
            Phi[e] = Phi[e] + quadwt * Psi1[e];
          }
        }
    }
    ndoneZ += nzones;
  }
}

// The RZ part of SetSweep (snac/SetSweep.F90:56-111): PsiM zeroed, the
// directions swept in quadrature order (finishing directions are not swept;
// they receive PsiM), Psi1 carried from direction to direction.  Schedules are
// packed per direction as for orc_set_sweep.
int orc_set_sweep_rz(int nz, int nc, int nb, int G, int A, const int *numCorner, const int *cOffSet,
                     const int *cFP, const int *cEZ, const double *A_fp, const double *A_ez, const double *Area,
                     const double *Volume, const double *RadiusFP, const double *RadiusEZ, const double *Sigt,
                     const double *STotal, double tau, const double *omega, const double *weight,
                     const double *angDerivFac, const double *quadTauW1, const double *quadTauW2,
                     const int *starting, const int *finishing, const int *nHyperPlanes, const int *zonesInPlane,
                     const int *nextZ, const int *nextC, const double *A_bdy, const int *bdyToC, double *Phi,
                     double *PsiB, double *Psi, int savePsi) {
  std::vector<double> Psi1((size_t)(nc + nb) * G, 0.0), PsiM((size_t)nc * G, 0.0);
  std::fill(Phi, Phi + (size_t)nc * G, 0.0);
  for (int a = 0; a < A; ++a) {
    if (finishing[a]) continue;
    for (int b = 0; b < nb; ++b)
      for (int g = 0; g < G; ++g) Psi1[(size_t)(nc + b) * G + g] = PsiB[((size_t)a * nb + b) * G + g];
    sweep_rz_angle(nz, nc, nb, G, numCorner, cOffSet, cFP, cEZ, A_fp, A_ez, Area, Volume, RadiusFP, RadiusEZ, Sigt,
                   STotal, tau, omega + 3 * a, weight[a], angDerivFac[a], quadTauW1[a], quadTauW2[a],
                   starting[a] != 0, nHyperPlanes[a], zonesInPlane + (size_t)a * nz, nextZ + (size_t)a * nz,
                   nextC + (size_t)a * nc, Psi + (size_t)a * nc * G, Psi1.data(), PsiM.data(), Phi);
    const bool nextFinishing = a + 1 < A && finishing[a + 1];
    for (int b = 0; b < nb; ++b) {
      if (!(dot3(omega + 3 * a, A_bdy + 3 * b) > 0.0)) continue;        // exit list (rt/findexit.F90:305-317)
      const int c = bdyToC[b];
      for (int g = 0; g < G; ++g) {
        PsiB[((size_t)a * nb + b) * G + g] = Psi1[(size_t)c * G + g];
        if (nextFinishing) PsiB[((size_t)(a + 1) * nb + b) * G + g] = PsiM[(size_t)c * G + g];
      }
    }
    if (savePsi) {
      std::copy(Psi1.begin(), Psi1.begin() + (size_t)nc * G, Psi + (size_t)a * nc * G);
      if (nextFinishing) std::copy(PsiM.begin(), PsiM.end(), Psi + (size_t)(a + 1) * nc * G);
    }
  }
  return 0;
}

}  // extern "C"
