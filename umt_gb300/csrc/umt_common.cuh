// umt_common.cuh -- device context shared by the translation units of
// libumt103.so.  One process-wide context (Teton keeps its mesh, quadrature
// and angular flux in module state the same way, mods/Geometry_mod.F90,
// mods/QuadratureList_mod.F90).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#define UMT_MAXCF 3
#define UMT_MAXCORNER 8
#define UMT_MAXFACES 6

// device status word bits (sticky until umt103_init / read)
#define UMT_DEV_CYCLE 1u
#define UMT_DEV_BOUNDS 2u
#define UMT_DEV_TIMEOUT 4u

namespace umt {

// Schedule of all directions of the angle set: work items (one per
// direction x zone) ordered by dependency stage; stage h holds every
// (direction, zone) whose longest upstream chain has h zones.
struct Schedule {
  uint32_t *items = nullptr;      // [A*nz] bit31 = lagged (bad) zone, low bits a*nz+z
  uint2 *items2 = nullptr;        // [A*nz] {items, cOffSet | numCorner << 28}
  int *stageCount = nullptr;      // [nz+2]
  int *stageOffset = nullptr;     // [nz+2]
  int *need = nullptr;            // [A*nz]
  int *needInit = nullptr;        // [A*nz] upwind-zone counts before the stage build
  uint8_t *exitMask = nullptr;    // [A*nz] bit f: zone face f is an exit face
  uint8_t *bad = nullptr;         // [A*nz] intra-zone corner cycle
  uint32_t *order = nullptr;      // [A*nz] corner solve order, 8 nibbles
  int *level = nullptr;           // [A*nz]
  int *nHyper = nullptr;          // [A]
  unsigned long long *processed = nullptr;  // items placed
  int nStages = 0;
  std::vector<int> hCount, hOffset;         // host copies
  int maxStageItems = 0;
  uint8_t *cycZ = nullptr;        // [A*nz] 1: the zone's corners are on the direction's cycle list
  // cycle list (constructDynMemory.F90:56-214): corner rows of psi read
  // before this sweep computes them, taken from the previous sweep
  long long *cycRow = nullptr;    // [nCyc] a*nc + c
  long long nCyc = 0;
  std::vector<long long> hCycOff; // [A+1] per-direction offsets into cycRow
  int breaks = 0;                 // directions the build ordered on the host (a cycle or no seed)
};

struct Ctx {
  bool ready = false;
  int nz = 0, nc = 0, nb = 0, A = 0, G = 0;
  int flags = 0;
  cudaStream_t stream = nullptr;
  // mesh (device, 0-based)
  int *numCorner = nullptr, *cOffSet = nullptr, *zoneFaces = nullptr;
  int *zoneOpp = nullptr, *faceOpp = nullptr;   // [nz*6]
  int *nCFaces = nullptr, *cFP = nullptr, *cEZ = nullptr, *CToFace = nullptr; // [nc*3]
  int *bdyToC = nullptr, *cToZone = nullptr;
  double *px = nullptr, *A_fp = nullptr, *A_ez = nullptr, *Volume = nullptr;
  double *VolumeZone = nullptr, *A_bdy = nullptr, *Afp_raw = nullptr;
  double *omega = nullptr, *weight = nullptr;
  float *weight32 = nullptr;
  std::vector<double> h_omega, h_weight;
  // per-direction corner-face projections Omega.A  [A][nc][3]
  double *afp64 = nullptr, *aez64 = nullptr;
  float *afp32 = nullptr, *aez32 = nullptr;
  // packed records of the production FP32 kernel (sweep32.cu)
  void *rec32 = nullptr;                        // [A][nc] 2 x float4
  void *conn32 = nullptr;                       // [nc] int4
  float *vol32 = nullptr;                       // [nc]
  bool rec32Ready = false;
  int tileGT = 0, tileGPL = 0;                  // FP32 group tile (0: choose)
  int sweepMode = 0;                            // FP32 kernel choice (umt103_set_sweep_mode)
  bool useCompact = true;                       // FP32: compact-list kernel where the tile allows
  // zone programs of the FP32 program kernel (sweep32p.cu)
  void *prog32 = nullptr;                       // programs, 16-byte units
  void *hdr32 = nullptr;                        // [A*nz] uint4 headers in stage order
  size_t progBytes = 0;
  int progMaxChunks = 0;                        // longest program, 16-byte units
  int progState = 0;                            // 0 not built, 1 built, -1 unavailable
  struct RZData *rz = nullptr;                  // 2-D RZ problem data (rz.cu), or none
  bool usePDL = true;                           // stage launches as programmatic dependents
  int *dep = nullptr;                           // [A*nz] persistent-mode dependency counters
  int *ticket = nullptr;                        // persistent-mode work ticket
  int holdItem = -1;                            // umt103_hold_item: item given an unsatisfiable dependency
  unsigned long long graphGen = 0;              // changes whenever this context's captured sweeps go stale
  Schedule sch;
  // materials and sources
  double *Sigt = nullptr, *SigS = nullptr;      // [nz][G]
  float *Sigt32 = nullptr;
  double tau = 0.0;
  double *STotal = nullptr;                     // [nc][G]
  float *STotal32 = nullptr;
  double *Phi = nullptr;                        // [nc][G]
  double *PhiPrev = nullptr;                    // [nc][G] previous iterate
  double *qExt = nullptr;                       // [nz][G] isotropic source
  double *siDelta = nullptr;                    // [nc][G] last change of PhiTotal in source iteration
  double *siDeltaPrev = nullptr;                // [nc][G] the change before it
  double *siKeep = nullptr;                     // [nc][G] iterate before a learned correction (kept for rollback)
  double hMean = 0.0;                           // mean zone size, (total volume / nz)^(1/3)
  // source iteration as one graph: a conditional while node around
  // build-source, sweep, change norm and a device-side convergence decision
  void *siState = nullptr;                      // device SIState (capi.cu)
  double *siRef = nullptr;                      // [nc][G] device copy of UmtSIParams.phi_ref
  cudaGraphExec_t siGraph[2][2][2] = {};        // [precision][cur][with phi_ref]
  bool inSIGraph = false;                       // enqueueing into that graph's body (no event records)
  int siGraphState = 0;                         // 0 untried, 1 works, -1 unavailable (host loop)
  // homogeneous FP32 sweeps (no tau*psi_old term, no boundary inflow): the
  // inner solves of mixed-precision source iteration
  bool homog32 = false;
  float *psiB32h = nullptr;                     // boundary rows of those sweeps (incoming rows stay zero)
  cudaGraphExec_t graphsH[2] = {nullptr, nullptr};
  double *mixX = nullptr, *mixR = nullptr, *mixD = nullptr;   // [nc][G] outer iterate, residual, correction
  double *cycPsi64 = nullptr;                   // [nCyc][G] previous-sweep flux of the cycle-list corners
  float *cycPsi32 = nullptr;
  double *red = nullptr;                        // [8] reduction slots
  // angular flux, double buffered: psi[cur] = saved Psi, psi[1-cur] = new
  double *psi64[2] = {nullptr, nullptr};
  float *psi32[2] = {nullptr, nullptr};
  int cur64 = 0, cur32 = 0;
  double *psiB64 = nullptr;                     // [A][nb][G]
  float *psiB32 = nullptr;
  unsigned int *status = nullptr;               // device status word
  double *scratch = nullptr;                    // reductions
  size_t scratchBytes = 0;
  int *bFace = nullptr;                         // [nb] corner face c*3 + f of each boundary element (-1: none)
  double **psibOut = nullptr;                   // device word read by the exit-row copies of the host-facing
                                                // graph: FP64 destination of the exiting PsiB rows, or null
  double **phiOut = nullptr;                    // device word: FP64 PhiTotal destination of the tally, or null
  bool exitsThrough = false;                    // the FP32 sweep as enqueued runs the zone-program kernel
  bool wantExitsThrough = false;                // enqueue the host-facing graph (row chunks, host-writing tally)
  cudaGraphExec_t graphsWT[2] = {nullptr, nullptr};   // FP32 sweeps of those variants, [cur]
  // PsiB rows the sweep does not write, ordered by the stage that reads them
  // (psib.cu), copied in chunks on a side stream inside the host-facing graph
  int *rowOrder = nullptr;                      // row indices a*nb + b
  std::vector<int> chunkOff, chunkStage;        // chunk k: rowOrder[chunkOff[k], chunkOff[k+1]), read from stage chunkStage[k]
  double **psibIn = nullptr;                    // device word: the FP64 rows to copy (host or staging), or null
  // The source rows (corners) in the same stage-ordered chunks, by the first
  // stage over all directions that sweeps the corner's zone; the host-facing
  // graph converts STotal chunk by chunk instead of all before stage 0
  int *srcOrder = nullptr;                      // corner indices
  std::vector<int> srcChunkOff, srcChunkStage;
  double **srcIn = nullptr;                     // device word: page-locked FP64 STotal, or null (convert the device copy)
  bool wantSrcChunks = false;                   // enqueue the chunked source conversion (host-facing zone-program graph)
  bool srcChunksNow = false;                    // the sweep being enqueued converts the source that way
  // The exiting PsiB rows ordered by the stage that writes them; the
  // host-facing graph copies them to *psibOut in chunks on a third stream,
  // each after the last stage that writes one of its rows
  int *exitOrder = nullptr;                     // row indices a*nb + b
  std::vector<int> exitChunkOff, exitChunkLast; // chunk k: exitOrder[off[k], off[k+1]), complete after stage last[k]
  cudaStream_t stream2 = nullptr, stream3 = nullptr;
  cudaEvent_t evFork = nullptr, evExitJoin = nullptr;
  std::vector<cudaEvent_t> evChunk, evSrc, evExit;
  double *stage64 = nullptr;                    // FP64 staging of PsiB for FP32 sweeps (kept)
  size_t stage64N = 0;
  // captured sweep graphs per precision
  cudaGraphExec_t graphs[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // [precision][cur]
  bool useGraphs = true;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, evMid = nullptr;
  float lastMs = -1.f, lastKernMs = -1.f, lastTallyMs = -1.f;
  int launchesPerSweep[2] = {0, 0};
  int sweepGT[2] = {0, 0};                      // group tile per precision
  Ctx *gta = nullptr;                           // grey S2 problem on the same mesh (GTA)
  // GTA work arrays (on the main context)
  double *gtaChi = nullptr;                     // [nz][G] correction spectrum
  double *gtaVec = nullptr;                     // [8][nc] BiCGStab vectors
  double *gtaSigS = nullptr;                    // [nz] grey scattering (for inner products)
  double *gtaZ = nullptr;                       // [5][nz] stretched-TSA eps, sigma_t, sigma_t/eps; zone energy; last zone correction
  int gtaMaxKrylov = 10;                        // BiCGStab iterations per correction (2 grey sweeps each)
  double gtaTol = 1.0e-4;                       // BiCGStab relative residual
  int gtaSpectrum = 0;                          // correction spectrum (see k_gta_spectrum)
  int gtaSolver = 1;                            // 1 UMT_GTA_TSA, 2 UMT_GTA_ZONE (umt103_set_gta_solver)
  double *gtaTT = nullptr, *gtaLU = nullptr;    // [nc][8] zone transfer matrices, factored A (UMT_GTA_ZONE)
};

extern Ctx *g_cur;
inline Ctx &cur() { return *g_cur; }
extern std::string g_err;

int set_error(int code, const char *fmt, ...);

#define UMT_CUDA(call)                                                       \
  do {                                                                       \
    cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess)                                                   \
      return set_error(-3, "%s:%d %s: %s", __FILE__, __LINE__, #call,         \
                       cudaGetErrorString(e_));                              \
  } while (0)

// launchers (geometry / schedule TU, compiled without FMA contraction)
int launch_geometry(Ctx &c);
int launch_projections(Ctx &c);
int build_schedule(Ctx &c);
// cycle list: psi_new rows <- stored previous values before a sweep, and the
// stored values <- psi_new rows after it (geom_sched.cu)
int enqueue_cycle_init(Ctx &c, int precision, int cur);
int enqueue_cycle_update(Ctx &c, int precision, int cur);
int cycle_from_psi(Ctx &c);
// launchers (sweep TU)
int capture_sweep_graph(Ctx &c, int precision, cudaGraph_t *out);
int launch_sweep_once(Ctx &c, int precision, bool tally);
int launch_tally(Ctx &c, int precision);
void invalidate_graphs(Ctx &c);
int record_mid(Ctx &c);
int launch_convert_source(Ctx &c);
// source iteration and edits (si.cu)
int launch_build_source(Ctx &c, const double *q);
// out3[0..2] = |change|^2, |phi|^2, |amplification-weighted change|^2 (the
// last only with weighted); out3 needs three slots
int launch_change_norm(Ctx &c, double *prev, double *out3, double *delta = nullptr, double *deltaPrev = nullptr,
                       bool weighted = false);
// learned correction (learn.cu)
bool mlp_ready_for(int G);
int mlp_correct(Ctx &c, double *Target, const double *Delta, const double *DeltaPrev);
int mlp_status();
int launch_energy(Ctx &c, const double *siga_dev, int precision, double *out4);
int launch_distance(Ctx &c, const double *ref, double *out2, const double *x = nullptr);
int launch_build_source_vec(Ctx &c, const double *vec, const double *q);
int launch_residual(Ctx &c, const double *X, double *R, double *out2);
int launch_inner_update(Ctx &c, const double *R, double *D, double *delta, double *deltaPrev, double *out3);
// grey transport acceleration (si.cu)
int gta_prepare(Ctx &c);
int gta_op(Ctx &c, const double *P, double *out, bool withSource);
int gta_prepare_zone(Ctx &c);
int gta_op_zone(Ctx &c, const double *P, double *out, bool withSource);
int gta_sdot2(Ctx &c, const double *x, const double *y, const double *u, const double *w, double *h2);
int gta_converge(Ctx &c, const double *x, double *rel);
int gta_axpbypcz(Ctx &c, int n, double a, const double *x, double b, double *y, double cc, const double *z);
int gta_dot2(Ctx &c, int n, const double *x, const double *y, const double *u, const double *w, double *h2);
int gta_correct(Ctx &c, const double *eps);
// production FP32 kernel (sweep32.cu)
int prepare_sweep32(Ctx &c);
bool sweep32_supported(int G, int GT, int GPL);
int enqueue_sweep32(Ctx &c, int cur, int GT, int GPL);
void default_tile(int G, int *GT, int *GPL);
// 2-D RZ sweep (rz.cu)
void free_rz(Ctx &c);
// persistent FP64 staging buffer of at least n elements (capi.cu)
int staging_buffer64(Ctx &c, size_t n, double **out);
// whether an FP32 sweep runs the zone-program kernel (sweep.cu)
int fp32_program_path(Ctx &c, bool *yes);
// PsiB rows between host arrays and the device copy (psib.cu)
int ensure_bface(Ctx &c);
int ensure_psib_order(Ctx &c);
int ensure_src_order(Ctx &c);
// the host-facing graph's side-stream chunks (PsiB rows, and the source rows
// when c.srcChunksNow), and the waits of stage s on those that begin there
int enqueue_psib_chunks(Ctx &c);
int wait_psib_chunks(Ctx &c, int stage);
// after the launch of stage s: copy out the exit chunks complete there; after
// the tally: join those copies
int enqueue_exit_chunks(Ctx &c, int stage);
int join_exit_chunks(Ctx &c);
void free_psib(Ctx &c);
// zone-program FP32 kernel (sweep32p.cu)
int prepare_prog32(Ctx &c);
bool sweep32p_supported(int G, int GT, int GPL);
int enqueue_sweep32p(Ctx &c, int cur, int GT, int GPL);
int enqueue_batch_stages(const std::vector<Ctx *> &cs, const std::vector<int> &curs, int GT, int GPL,
                         cudaStream_t st);
int enqueue_sweep32_pre(Ctx &c, int cur);
int enqueue_sweep32_post(Ctx &c, int cur);

}  // namespace umt
