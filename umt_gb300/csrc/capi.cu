// capi.cu -- the extern "C" entry points declared in include/umt103.h.
#include "umt_common.cuh"
#include "../../include/umt103.h"

#include <cstdarg>
#include <cstring>
#include <algorithm>
#include <map>

namespace umt {

// Contexts: slot 0 always exists; umt103_context_create adds more (independent
// problems resident together, e.g. for a batched launch).  Every entry point
// works on the current context.
static Ctx g_default;
Ctx *g_cur = &g_default;
static std::vector<Ctx *> g_ctx{&g_default};
std::string g_err;

int set_error(int code, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

template <typename T>
static int dalloc(T **p, size_t n) {
  *p = nullptr;
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
  if (e != cudaSuccess) {
    *p = nullptr;
    return set_error(UMT_ERR_NOMEM, "cudaMalloc of %zu bytes failed: %s", n * sizeof(T), cudaGetErrorString(e));
  }
  return 0;
}

template <typename T>
static void dfree(T *&p) {
  if (p) cudaFree((void *)p);
  p = nullptr;
}

static void free_ctx(Ctx &c);

static void free_all() {
  if (cur().gta) {
    free_ctx(*cur().gta);
    delete cur().gta;
    cur().gta = nullptr;
  }
  free_ctx(cur());
}

static void free_ctx(Ctx &c) {
  invalidate_graphs(c);
  dfree(c.numCorner); dfree(c.cOffSet); dfree(c.zoneFaces); dfree(c.zoneOpp); dfree(c.faceOpp);
  dfree(c.nCFaces); dfree(c.cFP); dfree(c.cEZ); dfree(c.CToFace); dfree(c.bdyToC); dfree(c.cToZone);
  dfree(c.px); dfree(c.A_fp); dfree(c.A_ez); dfree(c.Volume); dfree(c.VolumeZone); dfree(c.A_bdy);
  dfree(c.Afp_raw); dfree(c.omega); dfree(c.weight); dfree(c.weight32);
  dfree(c.afp64); dfree(c.aez64); dfree(c.afp32); dfree(c.aez32);
  dfree(c.rec32); dfree(c.conn32); dfree(c.vol32); dfree(c.prog32); dfree(c.hdr32);
  Schedule &s = c.sch;
  dfree(s.items); dfree(s.items2); dfree(s.stageCount); dfree(s.stageOffset); dfree(s.need); dfree(s.exitMask);
  dfree(s.needInit); dfree(c.dep); dfree(c.ticket);
  dfree(s.bad); dfree(s.order); dfree(s.level); dfree(s.nHyper); dfree(s.processed);
  dfree(s.cycZ); dfree(s.cycRow); dfree(c.cycPsi64); dfree(c.cycPsi32);
  dfree(c.Sigt); dfree(c.SigS); dfree(c.Sigt32); dfree(c.STotal); dfree(c.STotal32); dfree(c.Phi);
  dfree(c.PhiPrev); dfree(c.qExt); dfree(c.red); dfree(c.siDelta); dfree(c.siDeltaPrev); dfree(c.siKeep);
  dfree(c.siState); dfree(c.siRef); dfree(c.psiB32h); dfree(c.mixX); dfree(c.mixR); dfree(c.mixD);
  dfree(c.gtaChi); dfree(c.gtaVec); dfree(c.gtaSigS); dfree(c.gtaZ); dfree(c.gtaTT); dfree(c.gtaLU);
  for (int i = 0; i < 2; ++i) { dfree(c.psi64[i]); dfree(c.psi32[i]); }
  dfree(c.psiB64); dfree(c.psiB32); dfree(c.status); dfree(c.scratch); dfree(c.stage64); dfree(c.bFace);
  dfree(c.psibOut); dfree(c.phiOut);
  free_psib(c);
  c.stage64N = 0;
  if (c.ev0) cudaEventDestroy(c.ev0);
  if (c.ev1) cudaEventDestroy(c.ev1);
  if (c.evMid) cudaEventDestroy(c.evMid);
  free_rz(c);
  if (c.stream) cudaStreamDestroy(c.stream);
  c = Ctx();
}

static int upload_ints(int **dst, const int *src, size_t n, int shift) {
  int rc = dalloc(dst, n);
  if (rc) return rc;
  std::vector<int> tmp(src, src + n);
  if (shift)
    for (auto &v : tmp) v -= shift;
  UMT_CUDA(cudaMemcpy(*dst, tmp.data(), n * sizeof(int), cudaMemcpyHostToDevice));
  return 0;
}

}  // namespace umt

using namespace umt;

#define TRY(x) do { int rc_ = (x); if (rc_) { return rc_; } } while (0)

extern "C" {

const char *umt103_error_string(void) { return g_err.c_str(); }

void umt103_finalize(void) { free_all(); }

int umt103_context_create(int *id) {
  if (!id) return set_error(UMT_ERR_ARG, "null id");
  for (size_t k = 1; k < g_ctx.size(); ++k)
    if (!g_ctx[k]) { g_ctx[k] = new Ctx(); *id = (int)k; return 0; }
  g_ctx.push_back(new Ctx());
  *id = (int)g_ctx.size() - 1;
  return 0;
}

int umt103_context_select(int id) {
  if (id < 0 || id >= (int)g_ctx.size() || !g_ctx[id]) return set_error(UMT_ERR_ARG, "no context %d", id);
  g_cur = g_ctx[id];
  return 0;
}

int umt103_context_current(void) {
  for (size_t k = 0; k < g_ctx.size(); ++k)
    if (g_ctx[k] == g_cur) return (int)k;
  return -1;
}

int umt103_context_destroy(int id) {
  if (id <= 0 || id >= (int)g_ctx.size() || !g_ctx[id]) return set_error(UMT_ERR_ARG, "cannot destroy context %d", id);
  Ctx *victim = g_ctx[id], *keep = g_cur;
  g_cur = victim;
  free_all();
  delete victim;
  g_ctx[id] = nullptr;
  g_cur = (keep == victim) ? &g_default : keep;
  return 0;
}

// One CUDA graph that sweeps several contexts at once: each context's captured
// sweep graph (source conversion, every dependency stage, tally) becomes an
// independent child node, so problems of different sizes, group counts and
// direction counts run concurrently from a single launch.  The instantiated
// graph is kept for the same context list, precision, buffer parities and
// context generations, so a repeated batch costs one launch.
struct BatchGraph {
  std::vector<int> ids, curs;
  std::vector<unsigned long long> gens;
  int precision = -1, mode = -1;
  cudaGraphExec_t exec = nullptr;
};
static std::vector<BatchGraph> g_batch;          // most recently used last
constexpr size_t kBatchGraphsKept = 8;

static void drop_batch_graph(size_t k) {
  if (g_batch[k].exec) cudaGraphExecDestroy(g_batch[k].exec);
  g_batch.erase(g_batch.begin() + (long)k);
}

// ---------------------------------------------------------------------------
// Autotuner: the FP32 sweep's group tile (lanes per (direction, zone) pair x
// groups per lane) timed on the loaded problem, the fastest kept, and cached
// per problem shape (groups, directions, zones, corners, sweep mode) for
// every context of the process.
// ---------------------------------------------------------------------------
struct TileKey {
  int G, A, nz, nc, mode;
  bool operator<(const TileKey &o) const {
    if (G != o.G) return G < o.G;
    if (A != o.A) return A < o.A;
    if (nz != o.nz) return nz < o.nz;
    if (nc != o.nc) return nc < o.nc;
    return mode < o.mode;
  }
};
static std::map<TileKey, std::pair<int, int>> g_tiles;

static TileKey tile_key(const Ctx &c) { return TileKey{c.G, c.A, c.nz, c.nc, c.sweepMode}; }

// A context with no tile of its own takes the tuned tile of its shape.
static void apply_cached_tile(Ctx &c) {
  if (c.tileGT != 0) return;
  auto it = g_tiles.find(tile_key(c));
  if (it == g_tiles.end()) return;
  invalidate_graphs(c);
  c.tileGT = it->second.first;
  c.tileGPL = it->second.second;
}

static int autotune_ctx(Ctx &c, int reps, double *times, int maxTimes, int *ntimes) {
  if (!c.psi32[0]) return set_error(UMT_ERR_STATE, "autotune: the context has no FP32 flux");
  if (c.rz) return set_error(UMT_ERR_STATE, "autotune: RZ contexts are not tuned");
  reps = std::max(reps, 1);
  double best = 1e300;
  int bGT = 0, bGPL = 0, k = 0;
  for (int gpl : {1, 2, 4}) {
    if (c.G % gpl) continue;
    const int gt = c.G / gpl;
    if (!sweep32_supported(c.G, gt, gpl)) continue;
    invalidate_graphs(c);
    c.tileGT = gt; c.tileGPL = gpl;
    double t = 1e300;
    for (int r = 0; r <= reps; ++r) {                  // the first sweep captures the graph
      UMT_CUDA(cudaEventRecord(c.ev0, c.stream));
      TRY(launch_sweep_once(c, UMT_FP32, true));
      UMT_CUDA(cudaEventRecord(c.ev1, c.stream));
      UMT_CUDA(cudaStreamSynchronize(c.stream));
      float ms = 0.f;
      UMT_CUDA(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
      if (r > 0) t = std::min(t, (double)ms);
    }
    if (times && k < maxTimes) { times[3 * k] = gt; times[3 * k + 1] = gpl; times[3 * k + 2] = t; }
    ++k;
    if (t < best) { best = t; bGT = gt; bGPL = gpl; }
  }
  if (ntimes) *ntimes = k;
  if (!bGT) return set_error(UMT_ERR_ARG, "autotune: no group tile covers G=%d", c.G);
  invalidate_graphs(c);
  c.tileGT = bGT; c.tileGPL = bGPL;
  g_tiles[tile_key(c)] = {bGT, bGPL};
  return 0;
}

int umt103_autotune(int reps, int *lanes_per_zone, int *groups_per_lane, double *times, int max_times,
                    int *ntimes) {
  Ctx &c = cur();
  if (!c.ready) return set_error(UMT_ERR_STATE, "umt103_init not called");
  TRY(autotune_ctx(c, reps, times, max_times, ntimes));
  if (lanes_per_zone) *lanes_per_zone = c.tileGT;
  if (groups_per_lane) *groups_per_lane = c.tileGPL;
  return 0;
}

int umt103_autotune_contexts(const int *ids, int n, int reps) {
  if (!ids || n <= 0) return set_error(UMT_ERR_ARG, "no contexts");
  Ctx *keep = g_cur;
  int rc = 0;
  for (int k = 0; k < n && !rc; ++k) {
    const int id = ids[k];
    if (id < 0 || id >= (int)g_ctx.size() || !g_ctx[id] || !g_ctx[id]->ready) {
      rc = set_error(UMT_ERR_ARG, "autotune: context %d not initialised", id);
      break;
    }
    Ctx &c = *g_ctx[id];
    g_cur = &c;
    c.tileGT = 0;
    c.tileGPL = 0;
    if (g_tiles.count(tile_key(c))) apply_cached_tile(c);
    else rc = autotune_ctx(c, reps, nullptr, 0, nullptr);
  }
  g_cur = keep;
  return rc;
}

// Batch mode: UMT_BATCH_GRAPHS (default) nests each context's own sweep
// graph, so every problem's chain of stages advances at its own pace;
// UMT_BATCH_MERGED launches each dependency stage of all FP32 zone-program
// problems that share a group tile as one kernel (k_sweep32pm), one stream
// per tile, which holds those problems in lockstep, stage by stage (measured
// 5-22% slower on the config-4 draws).  Contexts the merged form cannot take
// (FP64, another FP32 kernel) make the batch use the nested graphs.
static int g_batchMode = UMT_BATCH_GRAPHS;

int umt103_set_batch_mode(int mode) {
  if (mode != UMT_BATCH_MERGED && mode != UMT_BATCH_GRAPHS) return set_error(UMT_ERR_ARG, "batch mode must be 0 or 1");
  g_batchMode = mode;
  return 0;
}

static cudaStream_t g_bStream[9];
static cudaEvent_t g_bEvent[9];

// The merged batch graph: every context's FP32 conversions and cycle rows,
// then per group tile a forked stream with one launch per dependency stage
// over the tile's problems, then every context's cycle update and tally.
// Returns 1 when a context cannot take part.
static int capture_batch_merged(const std::vector<int> &ids, cudaGraph_t *out) {
  std::map<std::pair<int, int>, std::vector<int>> cls;
  for (int id : ids) {
    const Ctx &c = *g_ctx[id];
    if (c.sweepMode != 0 || c.progState != 1 || c.homog32 || c.wantExitsThrough || c.tileGT <= 0 ||
        !sweep32p_supported(c.G, c.tileGT, c.tileGPL))
      return 1;
    cls[{c.tileGT, c.tileGPL}].push_back(id);
  }
  if (cls.size() > 8) return 1;
  for (int k = 0; k < 9; ++k) {
    if (!g_bStream[k]) UMT_CUDA(cudaStreamCreateWithFlags(&g_bStream[k], cudaStreamNonBlocking));
    if (!g_bEvent[k]) UMT_CUDA(cudaEventCreateWithFlags(&g_bEvent[k], cudaEventDisableTiming));
  }
  cudaStream_t s0 = g_bStream[0];
  std::vector<cudaStream_t> saved;
  for (int id : ids) saved.push_back(g_ctx[id]->stream);
  UMT_CUDA(cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal));
  for (int id : ids) g_ctx[id]->stream = s0;
  int rc = 0;
  cudaError_t e = cudaSuccess;
  for (size_t j = 0; j < ids.size() && !rc; ++j) rc = enqueue_sweep32_pre(*g_ctx[ids[j]], g_ctx[ids[j]]->cur32);
  if (!rc) e = cudaEventRecord(g_bEvent[0], s0);
  int k = 1;
  for (auto &kv : cls) {
    if (rc || e != cudaSuccess) break;
    cudaStream_t sk = g_bStream[k];
    std::vector<Ctx *> cs;
    std::vector<int> curs;
    for (int id : kv.second) { cs.push_back(g_ctx[id]); curs.push_back(g_ctx[id]->cur32); }
    e = cudaStreamWaitEvent(sk, g_bEvent[0], 0);
    if (e == cudaSuccess) rc = enqueue_batch_stages(cs, curs, kv.first.first, kv.first.second, sk);
    if (!rc && e == cudaSuccess) e = cudaEventRecord(g_bEvent[k], sk);
    if (!rc && e == cudaSuccess) e = cudaStreamWaitEvent(s0, g_bEvent[k], 0);
    ++k;
  }
  for (size_t j = 0; j < ids.size() && !rc && e == cudaSuccess; ++j)
    rc = enqueue_sweep32_post(*g_ctx[ids[j]], g_ctx[ids[j]]->cur32);
  for (size_t j = 0; j < ids.size(); ++j) g_ctx[ids[j]]->stream = saved[j];
  cudaGraph_t gr = nullptr;
  const cudaError_t e2 = cudaStreamEndCapture(s0, &gr);
  if (rc || e != cudaSuccess || e2 != cudaSuccess) {
    if (gr) cudaGraphDestroy(gr);
    if (rc) return rc;
    return set_error(UMT_ERR_CUDA, "batch capture: %s", cudaGetErrorString(e != cudaSuccess ? e : e2));
  }
  *out = gr;
  return 0;
}

int umt103_batch_sweep(const int *ids, int n, int precision, double *ms) {
  if (!ids || n <= 0) return set_error(UMT_ERR_ARG, "empty batch");
  if (precision != UMT_FP64 && precision != UMT_FP32) return set_error(UMT_ERR_ARG, "precision");
  BatchGraph key;
  key.precision = precision;
  key.mode = g_batchMode;
  for (int k = 0; k < n; ++k) {
    const int id = ids[k];
    if (id < 0 || id >= (int)g_ctx.size() || !g_ctx[id] || !g_ctx[id]->ready)
      return set_error(UMT_ERR_ARG, "batch: context %d not initialised", id);
    for (int j = 0; j < k; ++j)
      if (ids[j] == id) return set_error(UMT_ERR_ARG, "batch: context %d listed twice", id);
    Ctx &c = *g_ctx[id];
    if (c.rz) return set_error(UMT_ERR_STATE, "batch: context %d holds an RZ problem (umt103_sweep_rz)", id);
    if (c.holdItem >= 0)
      return set_error(UMT_ERR_STATE, "batch: context %d has a held work item (umt103_hold_item); sweep it alone", id);
    if (precision == UMT_FP64 && !c.psi64[0]) return set_error(UMT_ERR_STATE, "batch: context %d has no FP64 flux", id);
    if (precision == UMT_FP32 && !c.psi32[0]) return set_error(UMT_ERR_STATE, "batch: context %d has no FP32 flux", id);
    key.ids.push_back(id);
  }
  Ctx *keep = g_cur;
  int rc = 0;
  // tuned tiles of each context's shape, one-time preparation of each
  // context (outside any capture), then the key
  for (int k = 0; k < n && !rc; ++k) {
    g_cur = g_ctx[ids[k]];
    if (precision == UMT_FP32) apply_cached_tile(*g_cur);
    bool prog = false;
    if (precision == UMT_FP32) rc = fp32_program_path(*g_cur, &prog);
  }
  g_cur = keep;
  if (rc) return rc;
  for (int k = 0; k < n; ++k) {
    const Ctx &c = *g_ctx[ids[k]];
    key.curs.push_back(precision == UMT_FP64 ? c.cur64 : c.cur32);
    key.gens.push_back(c.graphGen);
  }
  cudaGraphExec_t exec = nullptr;
  for (size_t k = 0; k < g_batch.size(); ++k) {
    const BatchGraph &b = g_batch[k];
    if (b.precision == key.precision && b.mode == key.mode && b.ids == key.ids && b.curs == key.curs &&
        b.gens == key.gens) {
      key.exec = b.exec;
      g_batch.erase(g_batch.begin() + (long)k);
      exec = key.exec;
      break;
    }
  }
  if (!exec && precision == UMT_FP32 && g_batchMode == UMT_BATCH_MERGED) {
    cudaGraph_t merged = nullptr;
    const int mrc = capture_batch_merged(key.ids, &merged);
    if (mrc < 0) return mrc;
    if (mrc == 0) {
      const cudaError_t e = cudaGraphInstantiate(&exec, merged, 0);
      cudaGraphDestroy(merged);
      if (e != cudaSuccess) return set_error(UMT_ERR_CUDA, "batch graph: %s", cudaGetErrorString(e));
      key.exec = exec;
    }
  }
  if (!exec) {
    std::vector<cudaGraph_t> children;
    for (int k = 0; k < n && !rc; ++k) {
      g_cur = g_ctx[ids[k]];
      cudaGraph_t gr = nullptr;
      rc = capture_sweep_graph(*g_cur, precision, &gr);
      if (!rc) children.push_back(gr);
    }
    g_cur = keep;
    cudaGraph_t parent = nullptr;
    cudaError_t e = cudaSuccess;
    if (!rc) {
      e = cudaGraphCreate(&parent, 0);
      for (size_t k = 0; k < children.size() && e == cudaSuccess; ++k) {
        cudaGraphNode_t node;
        e = cudaGraphAddChildGraphNode(&node, parent, nullptr, 0, children[k]);
      }
      if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, parent, 0);
      if (e != cudaSuccess) {
        exec = nullptr;
        rc = set_error(UMT_ERR_CUDA, "batch graph: %s", cudaGetErrorString(e));
      }
    }
    if (parent) cudaGraphDestroy(parent);
    for (auto gr : children) cudaGraphDestroy(gr);
    if (rc) return rc;
    key.exec = exec;
  }
  // keep the graph (most recent last); entries of stale generations are dropped
  for (size_t k = 0; k < g_batch.size();) {
    bool stale = false;
    for (size_t j = 0; j < g_batch[k].ids.size() && !stale; ++j) {
      const int id = g_batch[k].ids[j];
      stale = id >= (int)g_ctx.size() || !g_ctx[id] || g_ctx[id]->graphGen != g_batch[k].gens[j];
    }
    if (stale) drop_batch_graph(k); else ++k;
  }
  while (g_batch.size() >= kBatchGraphsKept) drop_batch_graph(0);
  g_batch.push_back(key);

  cudaStream_t st = g_ctx[ids[0]]->stream;
  cudaEvent_t e0 = g_ctx[ids[0]]->ev0, e1 = g_ctx[ids[0]]->ev1;
  cudaError_t e = cudaEventRecord(e0, st);
  if (e == cudaSuccess) e = cudaGraphLaunch(exec, st);
  if (e == cudaSuccess) e = cudaEventRecord(e1, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess && ms) {
    float f = 0.f;
    e = cudaEventElapsedTime(&f, e0, e1);
    *ms = f;
  }
  if (e != cudaSuccess) return set_error(UMT_ERR_CUDA, "batch sweep: %s", cudaGetErrorString(e));
  // every context's device status word: read, cleared once reported
  int bad = 0;
  for (int k = 0; k < n; ++k) {
    Ctx &c = *g_ctx[ids[k]];
    unsigned w = 0;
    UMT_CUDA(cudaMemcpy(&w, c.status, sizeof(w), cudaMemcpyDeviceToHost));
    if (!w) continue;
    UMT_CUDA(cudaMemset(c.status, 0, sizeof(unsigned)));
    if (!bad) {
      if (w & UMT_DEV_BOUNDS) bad = set_error(UMT_ERR_BOUNDS, "batch: device bounds check in context %d", ids[k]);
      else if (w & UMT_DEV_TIMEOUT) bad = set_error(UMT_ERR_TIMEOUT, "batch: device wait timed out in context %d", ids[k]);
    }
  }
  return bad;
}

static int init_ctx(Ctx &c, const UmtMesh *m, const UmtQuad *q, int ngr, int flags);

int umt103_init(const UmtMesh *m, const UmtQuad *q, int ngr, int flags) {
  free_all();
  int rc = init_ctx(cur(), m, q, ngr, flags);
  if (rc) return rc;
  // The grey (GTA) problem: same mesh, level-symmetric S2 (8 directions,
  // |mu| = |eta| = |xi| = 1/sqrt(3), equal weights summing to 4 pi), one group,
  // FP64 (the reference's gtaorder = 2, test_driver.cc:1206).
  if (!(flags & 8)) {
    const double s = 0.57735026918962576451, w = 4.0 * 3.14159265358979323846 / 8.0;
    const double sg[8][3] = {{1, 1, 1}, {-1, 1, 1}, {-1, -1, 1}, {1, -1, 1},
                             {1, 1, -1}, {-1, 1, -1}, {-1, -1, -1}, {1, -1, -1}};
    double om[24], wt[8];
    for (int a = 0; a < 8; ++a) {
      for (int d = 0; d < 3; ++d) om[3 * a + d] = sg[a][d] * s;
      wt[a] = w;
    }
    UmtQuad q2{8, om, wt};
    cur().gta = new Ctx();
    rc = init_ctx(*cur().gta, m, &q2, 1, 1);
    if (rc) {
      free_all();
      return rc;
    }
  }
  return 0;
}

static int init_ctx(Ctx &c, const UmtMesh *m, const UmtQuad *q, int ngr, int flags) {
  if (!m || !q || ngr <= 0 || q->nangles <= 0 || !q->omega || !q->weight)
    return set_error(UMT_ERR_ARG, "umt103_init: null mesh/quadrature or bad sizes");
  if (m->maxcf > UMT_MAXCF || m->maxFaces > UMT_MAXFACES || m->maxcf <= 0)
    return set_error(UMT_ERR_ARG, "umt103_init: maxcf must be <= %d and maxFaces <= %d", UMT_MAXCF, UMT_MAXFACES);
  if (m->index_base != 0 && m->index_base != 1) return set_error(UMT_ERR_ARG, "index_base must be 0 or 1");
  const int nz = m->nzones, nc = m->ncornr, nb = m->nbelem, A = q->nangles, G = ngr;
  if (nz <= 0 || nc <= 0 || nb < 0) return set_error(UMT_ERR_ARG, "bad mesh sizes");
  if ((size_t)A * nz >= (1ull << 31)) return set_error(UMT_ERR_ARG, "nangles*nzones must be < 2^31");
  if (nc >= (1 << 28)) return set_error(UMT_ERR_ARG, "ncornr must be < 2^28");
  if (!m->px && !(m->A_fp && m->A_ez && m->Volume))
    return set_error(UMT_ERR_ARG, "either px or A_fp/A_ez/Volume must be given");
  const int base = m->index_base;
  // host-side validation of sizes and index ranges
  for (int z = 0; z < nz; ++z) {
    if (m->numCorner[z] < 1 || m->numCorner[z] > UMT_MAXCORNER)
      return set_error(UMT_ERR_ARG, "zone %d has %d corners (1..%d supported)", z, m->numCorner[z], UMT_MAXCORNER);
    if (m->zoneFaces[z] < 1 || m->zoneFaces[z] > m->maxFaces)
      return set_error(UMT_ERR_ARG, "zone %d has %d faces", z, m->zoneFaces[z]);
    if (m->cOffSet[z] < 0 || m->cOffSet[z] + m->numCorner[z] > nc)
      return set_error(UMT_ERR_ARG, "zone %d corner range out of bounds", z);
  }
  c.nz = nz; c.nc = nc; c.nb = nb; c.A = A; c.G = G; c.flags = (flags & 3) ? (flags & 3) : 3;
  invalidate_graphs(c);                                   // a fresh graph generation
  UMT_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
  UMT_CUDA(cudaEventCreate(&c.ev0));
  UMT_CUDA(cudaEventCreate(&c.ev1));
  UMT_CUDA(cudaEventCreate(&c.evMid));
  TRY(dalloc(&c.status, 1));
  UMT_CUDA(cudaMemset(c.status, 0, sizeof(unsigned)));

  // ---- mesh, converted to 0-based, padded to UMT_MAXCF / UMT_MAXFACES ----
  const int mcf = m->maxcf, mf = m->maxFaces;
  std::vector<int> cfp((size_t)nc * UMT_MAXCF, 0), cez((size_t)nc * UMT_MAXCF, 0), ctf((size_t)nc * UMT_MAXCF, 0);
  std::vector<int> zo((size_t)nz * UMT_MAXFACES, -1), fo((size_t)nz * UMT_MAXFACES, -1);
  std::vector<int> ncfv(m->nCFaces, m->nCFaces + nc);
  std::vector<int> c2z(nc, -1);
  for (int z = 0; z < nz; ++z)
    for (int k = 0; k < m->numCorner[z]; ++k) c2z[m->cOffSet[z] + k] = z;
  for (int cc = 0; cc < nc; ++cc) {
    if (ncfv[cc] < 1 || ncfv[cc] > mcf) return set_error(UMT_ERR_ARG, "corner %d has %d corner faces", cc, ncfv[cc]);
    const int z = c2z[cc];
    if (z < 0) return set_error(UMT_ERR_ARG, "corner %d belongs to no zone", cc);
    for (int k = 0; k < ncfv[cc]; ++k) {
      const int vfp = m->cFP[(size_t)cc * mcf + k] - base;
      const int vez = m->cEZ[(size_t)cc * mcf + k] - base;
      const int vtf = m->CToFace[(size_t)cc * mcf + k] - base;
      if (vfp < 0 || vfp >= nc + nb) return set_error(UMT_ERR_ARG, "cFP out of range at corner %d", cc);
      if (vez < 0 || vez >= m->numCorner[z]) return set_error(UMT_ERR_ARG, "cEZ out of range at corner %d", cc);
      if (vtf < 0 || vtf >= m->zoneFaces[z]) return set_error(UMT_ERR_ARG, "CToFace out of range at corner %d", cc);
      cfp[(size_t)cc * UMT_MAXCF + k] = vfp;
      cez[(size_t)cc * UMT_MAXCF + k] = vez;
      ctf[(size_t)cc * UMT_MAXCF + k] = vtf;
    }
  }
  for (int z = 0; z < nz; ++z)
    for (int f = 0; f < m->zoneFaces[z]; ++f) {
      const int v = m->zoneOpp[(size_t)z * mf + f];
      const int zz = (v >= base) ? v - base : -1;
      if (zz >= nz) return set_error(UMT_ERR_ARG, "zoneOpp out of range at zone %d", z);
      zo[(size_t)z * UMT_MAXFACES + f] = zz;
      fo[(size_t)z * UMT_MAXFACES + f] = zz >= 0 ? m->faceOpp[(size_t)z * mf + f] - base : -1;
    }
  std::vector<int> bdy(m->bdyToC, m->bdyToC + nb);
  for (auto &v : bdy) { v -= base; if (v < 0 || v >= nc) return set_error(UMT_ERR_ARG, "bdyToC out of range"); }

  TRY(upload_ints(&c.numCorner, m->numCorner, nz, 0));
  TRY(upload_ints(&c.cOffSet, m->cOffSet, nz, 0));
  TRY(upload_ints(&c.zoneFaces, m->zoneFaces, nz, 0));
  TRY(upload_ints(&c.zoneOpp, zo.data(), zo.size(), 0));
  TRY(upload_ints(&c.faceOpp, fo.data(), fo.size(), 0));
  TRY(upload_ints(&c.nCFaces, ncfv.data(), nc, 0));
  TRY(upload_ints(&c.cFP, cfp.data(), cfp.size(), 0));
  TRY(upload_ints(&c.cEZ, cez.data(), cez.size(), 0));
  TRY(upload_ints(&c.CToFace, ctf.data(), ctf.size(), 0));
  TRY(upload_ints(&c.bdyToC, bdy.data(), nb, 0));
  TRY(upload_ints(&c.cToZone, c2z.data(), nc, 0));

  const size_t nA = (size_t)nc * UMT_MAXCF * 3;
  TRY(dalloc(&c.A_fp, nA)); TRY(dalloc(&c.A_ez, nA)); TRY(dalloc(&c.Volume, nc));
  TRY(dalloc(&c.VolumeZone, nz)); TRY(dalloc(&c.A_bdy, (size_t)nb * 3));
  if (m->px) {
    TRY(dalloc(&c.px, (size_t)nc * 3));
    TRY(dalloc(&c.Afp_raw, nA));
    UMT_CUDA(cudaMemcpy(c.px, m->px, (size_t)nc * 3 * sizeof(double), cudaMemcpyHostToDevice));
  }
  if (m->A_fp && m->A_ez && m->Volume) {
    std::vector<double> afp(nA, 0.0), aez(nA, 0.0);
    for (int cc = 0; cc < nc; ++cc)
      for (int k = 0; k < ncfv[cc]; ++k)
        for (int d = 0; d < 3; ++d) {
          afp[((size_t)cc * UMT_MAXCF + k) * 3 + d] = m->A_fp[((size_t)cc * mcf + k) * 3 + d];
          aez[((size_t)cc * UMT_MAXCF + k) * 3 + d] = m->A_ez[((size_t)cc * mcf + k) * 3 + d];
        }
    UMT_CUDA(cudaMemcpy(c.A_fp, afp.data(), nA * sizeof(double), cudaMemcpyHostToDevice));
    UMT_CUDA(cudaMemcpy(c.A_ez, aez.data(), nA * sizeof(double), cudaMemcpyHostToDevice));
    UMT_CUDA(cudaMemcpy(c.Volume, m->Volume, nc * sizeof(double), cudaMemcpyHostToDevice));
    std::vector<double> vz(nz, 0.0), ab((size_t)nb * 3, 0.0);
    for (int z = 0; z < nz; ++z)
      for (int k = 0; k < m->numCorner[z]; ++k) vz[z] += m->Volume[m->cOffSet[z] + k];
    for (int cc = 0; cc < nc; ++cc)
      for (int k = 0; k < ncfv[cc]; ++k) {
        const int v = cfp[(size_t)cc * UMT_MAXCF + k];
        if (v >= nc)
          for (int d = 0; d < 3; ++d) ab[(size_t)(v - nc) * 3 + d] = afp[((size_t)cc * UMT_MAXCF + k) * 3 + d];
      }
    UMT_CUDA(cudaMemcpy(c.VolumeZone, vz.data(), nz * sizeof(double), cudaMemcpyHostToDevice));
    UMT_CUDA(cudaMemcpy(c.A_bdy, ab.data(), ab.size() * sizeof(double), cudaMemcpyHostToDevice));
  } else {
    TRY(launch_geometry(c));
  }

  // ---- quadrature ----
  c.h_omega.assign(q->omega, q->omega + 3 * (size_t)A);
  c.h_weight.assign(q->weight, q->weight + A);
  TRY(dalloc(&c.omega, 3 * (size_t)A)); TRY(dalloc(&c.weight, A));
  UMT_CUDA(cudaMemcpy(c.omega, q->omega, 3 * (size_t)A * sizeof(double), cudaMemcpyHostToDevice));
  UMT_CUDA(cudaMemcpy(c.weight, q->weight, (size_t)A * sizeof(double), cudaMemcpyHostToDevice));
  {
    std::vector<float> w32(q->weight, q->weight + A);
    TRY(dalloc(&c.weight32, A));
    UMT_CUDA(cudaMemcpy(c.weight32, w32.data(), (size_t)A * sizeof(float), cudaMemcpyHostToDevice));
  }

  // ---- projections (FP64 always: the schedule is decided in FP64) ----
  const size_t nP = (size_t)A * nc * UMT_MAXCF;
  TRY(dalloc(&c.afp64, nP)); TRY(dalloc(&c.aez64, nP));
  if (c.flags & 2) { TRY(dalloc(&c.afp32, nP)); TRY(dalloc(&c.aez32, nP)); }
  TRY(launch_projections(c));

  // ---- schedule ----
  Schedule &s = c.sch;
  const size_t nAZ = (size_t)A * nz;
  TRY(dalloc(&s.items, nAZ)); TRY(dalloc(&s.items2, nAZ)); TRY(dalloc(&s.stageCount, nz + 2)); TRY(dalloc(&s.stageOffset, nz + 2));
  TRY(dalloc(&s.need, nAZ)); TRY(dalloc(&s.exitMask, (nAZ + 3) & ~(size_t)3)); TRY(dalloc(&s.bad, nAZ));
  TRY(dalloc(&s.needInit, nAZ)); TRY(dalloc(&c.dep, nAZ)); TRY(dalloc(&c.ticket, 1));
  TRY(dalloc(&s.order, nAZ)); TRY(dalloc(&s.level, nAZ)); TRY(dalloc(&s.nHyper, A));
  TRY(dalloc(&s.processed, 1)); TRY(dalloc(&s.cycZ, nAZ));
  TRY(build_schedule(c));

  // ---- state ----
  const size_t ncG = (size_t)nc * G, nzG = (size_t)nz * G, psiN = (size_t)A * ncG, psiBN = (size_t)A * nb * G;
  TRY(dalloc(&c.Sigt, nzG)); TRY(dalloc(&c.SigS, nzG));
  TRY(dalloc(&c.STotal, ncG)); TRY(dalloc(&c.Phi, ncG));
  UMT_CUDA(cudaMemset(c.Sigt, 0, nzG * sizeof(double)));
  UMT_CUDA(cudaMemset(c.SigS, 0, nzG * sizeof(double)));
  UMT_CUDA(cudaMemset(c.STotal, 0, ncG * sizeof(double)));
  UMT_CUDA(cudaMemset(c.Phi, 0, ncG * sizeof(double)));
  if (c.flags & 1) {
    for (int i = 0; i < 2; ++i) { TRY(dalloc(&c.psi64[i], psiN)); UMT_CUDA(cudaMemset(c.psi64[i], 0, psiN * 8)); }
    TRY(dalloc(&c.psiB64, psiBN)); UMT_CUDA(cudaMemset(c.psiB64, 0, psiBN * 8));
  }
  if (c.flags & 2) {
    TRY(dalloc(&c.Sigt32, nzG)); TRY(dalloc(&c.STotal32, ncG));
    for (int i = 0; i < 2; ++i) { TRY(dalloc(&c.psi32[i], psiN)); UMT_CUDA(cudaMemset(c.psi32[i], 0, psiN * 4)); }
    TRY(dalloc(&c.psiB32, psiBN)); UMT_CUDA(cudaMemset(c.psiB32, 0, psiBN * 4));
    TRY(dalloc(&c.psibOut, 1)); UMT_CUDA(cudaMemset(c.psibOut, 0, sizeof(double *)));
    TRY(dalloc(&c.phiOut, 1)); UMT_CUDA(cudaMemset(c.phiOut, 0, sizeof(double *)));
  }
  TRY(cycle_from_psi(c));
  UMT_CUDA(cudaDeviceSynchronize());
  c.ready = true;
  return 0;
}

int umt103_set_materials(const double *sigt, const double *sigs, double tau) {
  Ctx &c = cur();
  if (!c.ready) return set_error(UMT_ERR_STATE, "umt103_init not called");
  if (!sigt) return set_error(UMT_ERR_ARG, "sigt is required");
  const size_t nzG = (size_t)c.nz * c.G;
  for (size_t i = 0; i < nzG; ++i)
    if (!(sigt[i] > 0.0)) return set_error(UMT_ERR_ARG, "sigt must be > 0 (element %zu)", i);
  UMT_CUDA(cudaMemcpy(c.Sigt, sigt, nzG * 8, cudaMemcpyHostToDevice));
  if (sigs) UMT_CUDA(cudaMemcpy(c.SigS, sigs, nzG * 8, cudaMemcpyHostToDevice));
  else UMT_CUDA(cudaMemset(c.SigS, 0, nzG * 8));
  if (c.tau != tau) invalidate_graphs(c);   // tau is a captured kernel argument
  c.tau = tau;
  return 0;
}

__global__ void k_d2f(size_t n, const double *x, float *y) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] = (float)x[i];
}
__global__ void k_f2d(size_t n, const float *x, double *y) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] = (double)x[i];
}

// PsiB rows (direction a, boundary element b; G values each) as the FP32
// sweep kernels classify them: a row is exiting when the FP32 projection
// Omega_a.A_fp of b's corner face is > 0 (the sweep writes it), every other
// row is left as it is (the sweep reads it when the projection is < 0).
// out == 0: every non-exiting row, FP64 -> psiB32; out == 1: every exiting
// row, psiB32 -> FP64.  src/dst may be page-locked host memory.
__global__ void k_psib_rows(int A, int nb, int nc, int G, const int *bFace, const float *afp32, const double *src,
                            float *psiB32, double *dst, int out) {
  const size_t n = (size_t)A * nb * G;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const size_t row = i / (size_t)G;
    const int a = (int)(row / (size_t)nb), b = (int)(row - (size_t)a * nb);
    const int bf = bFace[b];
    const bool exiting = bf >= 0 && afp32[(size_t)a * nc * UMT_MAXCF + bf] > 0.f;
    if (out == 0 && !exiting) psiB32[i] = (float)src[i];
    if (out == 1 && exiting) dst[i] = (double)psiB32[i];
  }
}

__global__ void k_count_exit_rows(int A, int nb, int nc, const int *bFace, const float *afp32,
                                  unsigned long long *count) {
  const size_t n = (size_t)A * nb;
  unsigned long long k = 0;
  for (size_t r = blockIdx.x * (size_t)blockDim.x + threadIdx.x; r < n; r += (size_t)gridDim.x * blockDim.x) {
    const int a = (int)(r / (size_t)nb), b = (int)(r - (size_t)a * nb);
    const int bf = bFace[b];
    k += (bf >= 0 && afp32[(size_t)a * nc * UMT_MAXCF + bf] > 0.f) ? 1 : 0;
  }
  if (k) atomicAdd(count, k);
}

__global__ void k_set_word(double **word, double *value) { *word = value; }

// The device address of page-locked host memory, or null for pageable memory.
static double *mapped_host(double *p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) { cudaGetLastError(); return nullptr; }
  if (at.type != cudaMemoryTypeHost || !at.devicePointer) return nullptr;
  return (double *)at.devicePointer;
}

int umt103_set_psi(const double *Psi, const double *PsiB) {
  Ctx &c = cur();
  if (!c.ready) return set_error(UMT_ERR_STATE, "umt103_init not called");
  const size_t psiN = (size_t)c.A * c.nc * c.G, psiBN = (size_t)c.A * c.nb * c.G;
  double *tmp = nullptr;
  TRY(dalloc(&tmp, std::max(psiN, psiBN)));
  auto put = [&](const double *h, size_t n, double *d64, float *d32) -> int {
    if (h) UMT_CUDA(cudaMemcpy(tmp, h, n * 8, cudaMemcpyHostToDevice));
    else UMT_CUDA(cudaMemset(tmp, 0, n * 8));
    if (d64) UMT_CUDA(cudaMemcpy(d64, tmp, n * 8, cudaMemcpyDeviceToDevice));
    if (d32) k_d2f<<<4096, 256>>>(n, tmp, d32);
    UMT_CUDA(cudaDeviceSynchronize());
    return 0;
  };
  int rc = put(Psi, psiN, c.psi64[c.cur64], c.psi32[c.cur32]);
  if (!rc) rc = put(PsiB, psiBN, c.psiB64, c.psiB32);
  cudaFree(tmp);
  if (!rc) rc = cycle_from_psi(c);               // the cycle list starts from the saved flux
  return rc;
}

int umt103_get_psi(double *Psi, double *PsiB, int precision) {
  Ctx &c = cur();
  if (!c.ready) return set_error(UMT_ERR_STATE, "umt103_init not called");
  const size_t psiN = (size_t)c.A * c.nc * c.G, psiBN = (size_t)c.A * c.nb * c.G;
  if (precision != UMT_FP64 && precision != UMT_FP32) return set_error(UMT_ERR_ARG, "precision must be UMT_FP64 or UMT_FP32");
  if (precision == UMT_FP64) {
    if (!c.psi64[0]) return set_error(UMT_ERR_STATE, "FP64 flux not allocated");
    if (Psi) UMT_CUDA(cudaMemcpy(Psi, c.psi64[c.cur64], psiN * 8, cudaMemcpyDeviceToHost));
    if (PsiB) UMT_CUDA(cudaMemcpy(PsiB, c.psiB64, psiBN * 8, cudaMemcpyDeviceToHost));
    return 0;
  }
  if (!c.psi32[0]) return set_error(UMT_ERR_STATE, "FP32 flux not allocated");
  double *tmp = nullptr;
  TRY(dalloc(&tmp, std::max(psiN, psiBN)));
  if (Psi) { k_f2d<<<4096, 256>>>(psiN, c.psi32[c.cur32], tmp); cudaMemcpy(Psi, tmp, psiN * 8, cudaMemcpyDeviceToHost); }
  if (PsiB) { k_f2d<<<4096, 256>>>(psiBN, c.psiB32, tmp); cudaMemcpy(PsiB, tmp, psiBN * 8, cudaMemcpyDeviceToHost); }
  cudaError_t e = cudaDeviceSynchronize();
  cudaFree(tmp);
  if (e != cudaSuccess) return set_error(UMT_ERR_CUDA, "get_psi: %s", cudaGetErrorString(e));
  return 0;
}

int umt103_set_source(const double *STotal) {
  Ctx &c = cur();
  if (!c.ready) return set_error(UMT_ERR_STATE, "umt103_init not called");
  const size_t ncG = (size_t)c.nc * c.G;
  if (STotal) UMT_CUDA(cudaMemcpy(c.STotal, STotal, ncG * 8, cudaMemcpyHostToDevice));
  else UMT_CUDA(cudaMemset(c.STotal, 0, ncG * 8));
  return 0;
}

static int sweep_core(int savePsi, int precision) {
  Ctx &c = cur();
  if (c.rz) return set_error(UMT_ERR_STATE, "the context holds an RZ problem: use umt103_sweep_rz");
  if (precision != UMT_FP64 && precision != UMT_FP32) return set_error(UMT_ERR_ARG, "precision must be UMT_FP64 or UMT_FP32");
  if (precision == UMT_FP64 && !c.psi64[0]) return set_error(UMT_ERR_STATE, "FP64 flux not allocated");
  if (precision == UMT_FP32 && !c.psi32[0]) return set_error(UMT_ERR_STATE, "FP32 flux not allocated");
  UMT_CUDA(cudaEventRecord(c.ev0, c.stream));
  {
    // a held item (umt103_hold_item) is enqueued for this sweep only, outside the graphs
    const bool graphs = c.useGraphs;
    if (c.holdItem >= 0) c.useGraphs = false;
    const int rc = launch_sweep_once(c, precision, true);
    c.useGraphs = graphs;
    c.holdItem = -1;
    TRY(rc);
  }
  UMT_CUDA(cudaEventRecord(c.ev1, c.stream));
  UMT_CUDA(cudaStreamSynchronize(c.stream));
  cudaEventElapsedTime(&c.lastMs, c.ev0, c.ev1);
  // stage kernels only: the FP32 path records evMid twice (after the source
  // conversion and after the last stage); the second record wins for the
  // tally split, the first is folded into the step time
  cudaEventElapsedTime(&c.lastTallyMs, c.evMid, c.ev1);
  c.lastKernMs = c.lastMs - c.lastTallyMs;
  if (savePsi) {
    if (precision == UMT_FP64) c.cur64 = 1 - c.cur64;
    else c.cur32 = 1 - c.cur32;
  }
  unsigned st = 0;
  UMT_CUDA(cudaMemcpy(&st, c.status, sizeof(st), cudaMemcpyDeviceToHost));
  if (st) UMT_CUDA(cudaMemset(c.status, 0, sizeof(unsigned)));   // reported once; the context stays usable
  if (st & UMT_DEV_BOUNDS) return set_error(UMT_ERR_BOUNDS, "device bounds check");
  if (st & UMT_DEV_TIMEOUT) return set_error(UMT_ERR_TIMEOUT, "device wait timed out");
  return 0;
}

int umt103_sweep_resident(int savePsi, int precision) {
  if (!cur().ready) return set_error(UMT_ERR_STATE, "umt103_init not called");
  return sweep_core(savePsi, precision);
}

int umt103_get_phi(double *PhiTotal) {
  Ctx &c = cur();
  if (!c.ready) return set_error(UMT_ERR_STATE, "umt103_init not called");
  if (!PhiTotal) return set_error(UMT_ERR_ARG, "null PhiTotal");
  UMT_CUDA(cudaMemcpy(PhiTotal, c.Phi, (size_t)c.nc * c.G * 8, cudaMemcpyDeviceToHost));
  return 0;
}

// FP64 staging buffer for the FP32 path's PsiB conversions, allocated on the
// first call that needs it and kept with the context (a per-call
// allocation and free would synchronise the device every sweep).
static int staging64(Ctx &c, size_t n, double **out) {
  if (c.stage64N < n) {
    dfree(c.stage64);
    c.stage64N = 0;
    TRY(dalloc(&c.stage64, n));
    c.stage64N = n;
  }
  *out = c.stage64;
  return 0;
}

int umt103_sweep(const double *STotal, int savePsi, double *PhiTotal_out, double *PsiB_inout, int precision) {
  Ctx &c = cur();
  if (!c.ready) return set_error(UMT_ERR_STATE, "umt103_init not called");
  if (c.rz) return set_error(UMT_ERR_STATE, "the context holds an RZ problem: use umt103_sweep_rz");
  if (precision != UMT_FP64 && precision != UMT_FP32) return set_error(UMT_ERR_ARG, "precision must be UMT_FP64 or UMT_FP32");
  if (precision == UMT_FP64 && !c.psi64[0]) return set_error(UMT_ERR_STATE, "FP64 flux not allocated");
  if (precision == UMT_FP32 && !c.psi32[0]) return set_error(UMT_ERR_STATE, "FP32 flux not allocated");
  const size_t ncG = (size_t)c.nc * c.G, psiBN = (size_t)c.A * c.nb * c.G;
  // FP32: only the PsiB rows a sweep reads go in and only the rows it writes
  // come out, so the caller's array keeps its other rows bit for bit.
  // Page-locked host memory is read and written by the kernels directly;
  // pageable memory goes through the FP64 staging buffer, which keeps the
  // input rows.  The incoming rows are converted into the device copy, not
  // read from host memory by the stage kernels (that put the link's latency
  // on every boundary item's dependency chain and was slower).  With the
  // zone-program kernel that copy runs in stage-ordered chunks beside the
  // stages, the exiting rows go to the FP64 array in chunks after the stages
  // that write them, and the tally writes PhiTotal straight to a page-locked
  // destination.  A page-locked STotal is converted in stage-ordered chunks
  // beside the stages too, instead of being copied whole before the first
  // stage.
  double *psibHost = nullptr, *psibFP64 = nullptr, *phiHost = nullptr, *srcHost = nullptr;
  bool psibWT = false, wt = false, prog = false;
  if (precision == UMT_FP32 && (PsiB_inout || PhiTotal_out)) {
    TRY(fp32_program_path(c, &prog));
    if (PsiB_inout) {
      TRY(ensure_bface(c));
      psibHost = mapped_host(PsiB_inout);
      psibFP64 = psibHost;
      if (!psibFP64) {
        TRY(staging64(c, psiBN, &psibFP64));
        UMT_CUDA(cudaMemcpyAsync(psibFP64, PsiB_inout, psiBN * 8, cudaMemcpyHostToDevice, c.stream));
      }
      psibWT = prog && ((uintptr_t)psibFP64 & 15u) == 0;      // the kernel's FP64 accesses are 16-byte
    }
    if (PhiTotal_out) {
      phiHost = mapped_host(PhiTotal_out);
      if ((uintptr_t)phiHost & 15u) phiHost = nullptr;
    }
    wt = psibWT || phiHost;
    // the host-facing graph copies the rows the sweep reads in stage-ordered
    // chunks beside the stages (psib.cu); otherwise they go in first
    if (wt) TRY(ensure_psib_order(c));
    if (wt && prog) {
      TRY(ensure_src_order(c));
      srcHost = STotal ? mapped_host(const_cast<double *>(STotal)) : nullptr;   // read only
      if ((uintptr_t)srcHost & 15u) srcHost = nullptr;
    }
    if (PsiB_inout && !psibWT)
      k_psib_rows<<<4096, 256, 0, c.stream>>>(c.A, c.nb, c.nc, c.G, c.bFace, c.afp32, psibFP64, c.psiB32, nullptr, 0);
    if (wt) {
      k_set_word<<<1, 1, 0, c.stream>>>(c.psibIn, psibWT ? psibFP64 : nullptr);
      k_set_word<<<1, 1, 0, c.stream>>>(c.psibOut, psibWT ? psibFP64 : nullptr);
      k_set_word<<<1, 1, 0, c.stream>>>(c.phiOut, phiHost);
      if (c.srcIn) k_set_word<<<1, 1, 0, c.stream>>>(c.srcIn, srcHost);
    }
    UMT_CUDA(cudaGetLastError());
  } else if (PsiB_inout) {
    UMT_CUDA(cudaMemcpyAsync(c.psiB64, PsiB_inout, psiBN * 8, cudaMemcpyHostToDevice, c.stream));
  }
  // the device's FP64 source: copied here, or filled from srcHost by the chunks
  if (!srcHost) {
    if (STotal) UMT_CUDA(cudaMemcpyAsync(c.STotal, STotal, ncG * 8, cudaMemcpyHostToDevice, c.stream));
    else UMT_CUDA(cudaMemsetAsync(c.STotal, 0, ncG * 8, c.stream));
  }
  c.wantExitsThrough = wt;
  c.wantSrcChunks = wt && prog;
  const int rcs = sweep_core(savePsi, precision);
  const bool wrote = psibWT && c.exitsThrough;
  c.wantExitsThrough = false;
  c.wantSrcChunks = false;
  if (wt) {                                        // resident sweeps touch no host memory
    k_set_word<<<1, 1, 0, c.stream>>>(c.psibIn, nullptr);
    k_set_word<<<1, 1, 0, c.stream>>>(c.psibOut, nullptr);
    k_set_word<<<1, 1, 0, c.stream>>>(c.phiOut, nullptr);
    if (c.srcIn) k_set_word<<<1, 1, 0, c.stream>>>(c.srcIn, nullptr);
  }
  TRY(rcs);
  if (PhiTotal_out && !phiHost) UMT_CUDA(cudaMemcpyAsync(PhiTotal_out, c.Phi, ncG * 8, cudaMemcpyDeviceToHost, c.stream));
  if (PsiB_inout) {
    if (precision == UMT_FP64) {
      UMT_CUDA(cudaMemcpyAsync(PsiB_inout, c.psiB64, psiBN * 8, cudaMemcpyDeviceToHost, c.stream));
    } else {
      if (!wrote)
        k_psib_rows<<<4096, 256, 0, c.stream>>>(c.A, c.nb, c.nc, c.G, c.bFace, c.afp32, nullptr, c.psiB32, psibFP64, 1);
      UMT_CUDA(cudaGetLastError());
      if (!psibHost) UMT_CUDA(cudaMemcpyAsync(PsiB_inout, psibFP64, psiBN * 8, cudaMemcpyDeviceToHost, c.stream));
    }
  }
  UMT_CUDA(cudaStreamSynchronize(c.stream));
  return 0;
}

double umt103_last_sweep_ms(void) { return cur().lastMs; }

int umt103_last_timing(double *out3) {
  if (!out3) return set_error(UMT_ERR_ARG, "null output");
  out3[0] = cur().lastMs; out3[1] = cur().lastKernMs; out3[2] = cur().lastTallyMs;
  return 0;
}

int umt103_launches_per_sweep(int precision) {
  if (precision != 0 && precision != 1) return set_error(UMT_ERR_ARG, "precision");
  return cur().launchesPerSweep[precision];
}

int umt103_hold_item(int item) {
  Ctx &c = cur();
  if (!c.ready) return set_error(UMT_ERR_STATE, "umt103_init not called");
  if (item < -1 || item >= c.A * c.nz) return set_error(UMT_ERR_ARG, "item out of range");
  c.holdItem = item;
  return 0;
}

int umt103_psib_rows(long long *exiting, long long *total) {
  Ctx &c = cur();
  if (!c.ready) return set_error(UMT_ERR_STATE, "umt103_init not called");
  if (!exiting || !total) return set_error(UMT_ERR_ARG, "null output");
  if (!c.afp32) return set_error(UMT_ERR_STATE, "FP32 flux not allocated");
  if (c.rz) return set_error(UMT_ERR_STATE, "the context holds an RZ problem");
  TRY(ensure_bface(c));
  unsigned long long *cnt = nullptr;
  TRY(dalloc(&cnt, 1));
  cudaMemset(cnt, 0, sizeof(unsigned long long));
  k_count_exit_rows<<<1024, 256>>>(c.A, c.nb, c.nc, c.bFace, c.afp32, cnt);
  unsigned long long h = 0;
  cudaMemcpy(&h, cnt, sizeof(h), cudaMemcpyDeviceToHost);
  const cudaError_t e = cudaGetLastError();
  cudaFree(cnt);
  if (e != cudaSuccess) return set_error(UMT_ERR_CUDA, "psib_rows: %s", cudaGetErrorString(e));
  *exiting = (long long)h;
  *total = (long long)c.A * c.nb;
  return 0;
}

int umt103_set_gta(int max_krylov, double tol, int spectrum) {
  Ctx &c = cur();
  if (!c.ready) return set_error(UMT_ERR_STATE, "umt103_init not called");
  if (max_krylov < 1 || !(tol > 0.0) || spectrum < 0 || spectrum > 1)
    return set_error(UMT_ERR_ARG, "bad GTA options");
  c.gtaMaxKrylov = max_krylov; c.gtaTol = tol; c.gtaSpectrum = spectrum;
  return 0;
}

int umt103_set_gta_solver(int solver) {
  Ctx &c = cur();
  if (!c.ready) return set_error(UMT_ERR_STATE, "umt103_init not called");
  if (solver != UMT_GTA_TSA && solver != UMT_GTA_ZONE)
    return set_error(UMT_ERR_ARG, "GTA solver must be UMT_GTA_TSA (1) or UMT_GTA_ZONE (2)");
  c.gtaSolver = solver;
  return 0;
}

int umt103_set_sweep_mode(int mode) {
  Ctx &c = cur();
  if (!c.ready) return set_error(UMT_ERR_STATE, "umt103_init not called");
  if (mode < 0 || mode > 2) return set_error(UMT_ERR_ARG, "sweep mode must be 0, 1 or 2");
  if (mode == 1 && c.sch.nCyc > 0)
    return set_error(UMT_ERR_CYCLE, "the persistent sweep (mode 1) does not run meshes with a cycle list");
  if (c.sweepMode != mode) invalidate_graphs(c);
  c.sweepMode = mode;
  return 0;
}

int umt103_set_group_tile(int lanes_per_zone, int groups_per_lane) {
  Ctx &c = cur();
  if (!c.ready) return set_error(UMT_ERR_STATE, "umt103_init not called");
  invalidate_graphs(c);
  if (lanes_per_zone == 0 && groups_per_lane == 0) { c.tileGT = 0; c.tileGPL = 0; return 0; }
  if (!sweep32_supported(c.G, lanes_per_zone, groups_per_lane))
    return set_error(UMT_ERR_ARG, "group tile %d x %d does not cover G=%d", lanes_per_zone, groups_per_lane, c.G);
  c.tileGT = lanes_per_zone; c.tileGPL = groups_per_lane;
  return 0;
}

int umt103_select_device(int device) {
  int n = 0;
  UMT_CUDA(cudaGetDeviceCount(&n));
  if (device < 0 || device >= n) return set_error(UMT_ERR_ARG, "device %d of %d", device, n);
  UMT_CUDA(cudaSetDevice(device));
  return 0;
}

int umt103_schedule_info(int angle, int *nHyperPlanes, int *numCycles) {
  Ctx &c = cur();
  if (!c.ready) return set_error(UMT_ERR_STATE, "umt103_init not called");
  if (angle < 0 || angle >= c.A) return set_error(UMT_ERR_ARG, "angle out of range");
  int h = 0;
  UMT_CUDA(cudaMemcpy(&h, c.sch.nHyper + angle, sizeof(int), cudaMemcpyDeviceToHost));
  if (nHyperPlanes) *nHyperPlanes = h;
  if (numCycles)
    *numCycles = c.sch.hCycOff.empty() ? 0 : (int)(c.sch.hCycOff[angle + 1] - c.sch.hCycOff[angle]);
  return 0;
}

int umt103_get_schedule(int *level, int *nHyperPlanes) {
  Ctx &c = cur();
  if (!c.ready) return set_error(UMT_ERR_STATE, "umt103_init not called");
  if (level) UMT_CUDA(cudaMemcpy(level, c.sch.level, (size_t)c.A * c.nz * sizeof(int), cudaMemcpyDeviceToHost));
  if (nHyperPlanes) UMT_CUDA(cudaMemcpy(nHyperPlanes, c.sch.nHyper, c.A * sizeof(int), cudaMemcpyDeviceToHost));
  return 0;
}

int umt103_get_geometry(double *A_fp, double *A_ez, double *Volume) {
  Ctx &c = cur();
  if (!c.ready) return set_error(UMT_ERR_STATE, "umt103_init not called");
  const size_t nA = (size_t)c.nc * UMT_MAXCF * 3;
  if (A_fp) UMT_CUDA(cudaMemcpy(A_fp, c.A_fp, nA * 8, cudaMemcpyDeviceToHost));
  if (A_ez) UMT_CUDA(cudaMemcpy(A_ez, c.A_ez, nA * 8, cudaMemcpyDeviceToHost));
  if (Volume) UMT_CUDA(cudaMemcpy(Volume, c.Volume, (size_t)c.nc * 8, cudaMemcpyDeviceToHost));
  return 0;
}

// The grey correction of rt/GTASolver.F90:42-425 (the BiCGStab branch with
// GreySweep, rt/GreySweep.F90): A = I - M with M the grey operator (grey S2
// sweep plus stretched-TSA sweep, gta_op); the initial residual is M applied
// to the grey source alone; inner products are weighted by sigma_s,grey V
// (scat_prod) and the shadow product is their plain sum (scat_prod1); the
// iteration stops when the zone-averaged correction changes by less than
// tol relative to the zone energy plus correction (pointwise and L2), or
// after max_krylov iterations.  Then phi_g += chi_g x (rt/addGreyCorrections.F90).
// With UMT_GTA_ZONE the operator is GreySweepNEW's (rt/GreySweep.F90:12-47,
// rt/GTASolver.F90:158-174): one grey sweep, then the per-zone direct solve
// (gta_op_zone), in place of the grey and stretched sweeps.
// Vectors (FP64, device) in c.gtaVec: 0 x (GreyCorrection), 1 r, 3 d, 4 Ad,
// 5 As, 7 R (grey source).  apply=false leaves PhiTotal unchanged.
static int gta_solve(Ctx &c, int maxit, double tol, int *greySweeps, bool apply = true) {
  const int n = c.nc;
  double *V = c.gtaVec;
  double *x = V, *r = V + (size_t)n, *d = V + 3 * (size_t)n, *Ad = V + 4 * (size_t)n, *As = V + 5 * (size_t)n;
  const double small = 1.0e-150;                  // adqtSmall, mods/constant_mod.F90:51
  const bool zoneSolve = c.gtaSolver == UMT_GTA_ZONE;
  auto op = [&](const double *P, double *out, bool withSource) -> int {
    *greySweeps += zoneSolve ? 1 : 2;
    return zoneSolve ? gta_op_zone(c, P, out, withSource) : gta_op(c, P, out, withSource);
  };
  TRY(gta_prepare(c));
  if (zoneSolve) TRY(gta_prepare_zone(c));
  UMT_CUDA(cudaMemsetAsync(x, 0, (size_t)n * 8, c.stream));
  TRY(op(nullptr, r, true));                      // CGResidual: M with the grey source, from zero
  UMT_CUDA(cudaMemcpyAsync(d, r, (size_t)n * 8, cudaMemcpyDeviceToDevice, c.stream));
  double h[2];
  TRY(gta_sdot2(c, r, nullptr, nullptr, nullptr, h));
  double rrOld = h[0];
  int nGrey = 1;
  for (int it = 0;; ++it) {
    if (std::fabs(rrOld) < small) {
      if (nGrey <= 2) UMT_CUDA(cudaMemcpyAsync(x, r, (size_t)n * 8, cudaMemcpyDeviceToDevice, c.stream));
      break;
    }
    nGrey += 2;
    TRY(op(d, Ad, false));                        // Ad = d - M d
    TRY(gta_axpbypcz(c, n, 1.0, d, -1.0, Ad, 0.0, nullptr));
    TRY(gta_sdot2(c, Ad, nullptr, nullptr, nullptr, h));
    const double dAd = h[0];
    if (std::fabs(dAd) < small) break;
    const double alpha = rrOld / dAd;
    TRY(gta_axpbypcz(c, n, -alpha, Ad, 1.0, r, 0.0, nullptr));          // r -= alpha Ad
    TRY(op(r, As, false));                        // As = r - M r
    TRY(gta_axpbypcz(c, n, 1.0, r, -1.0, As, 0.0, nullptr));
    TRY(gta_sdot2(c, As, r, As, As, h));
    const double omegaNum = h[0], omegaDen = h[1];
    if (std::fabs(omegaDen) < small || std::fabs(omegaNum) < small) {
      TRY(gta_axpbypcz(c, n, alpha, d, 1.0, x, 0.0, nullptr));
      break;
    }
    const double omega = omegaNum / omegaDen;
    TRY(gta_axpbypcz(c, n, alpha, d, 1.0, x, omega, r));                // x += alpha d + omega r
    TRY(gta_axpbypcz(c, n, -omega, As, 1.0, r, 0.0, nullptr));         // r -= omega As
    TRY(gta_sdot2(c, r, nullptr, nullptr, nullptr, h));
    const double rr = h[0];
    const double beta = (rr * alpha) / (rrOld * omega);
    TRY(gta_axpbypcz(c, n, 1.0, r, beta, d, -beta * omega, Ad));       // d = r + beta (d - omega Ad)
    double rel = 0.0;
    TRY(gta_converge(c, x, &rel));
    if (rel < tol || it + 1 >= maxit) break;
    rrOld = rr;
  }
  return apply ? gta_correct(c, x) : 0;
}

static int gta_alloc(Ctx &c) {
  if (!c.gta) return set_error(UMT_ERR_STATE, "GTA context not created (init flag 8 set)");
  if (!c.gtaChi) TRY(dalloc(&c.gtaChi, (size_t)c.nz * c.G));
  if (!c.gtaVec) {
    TRY(dalloc(&c.gtaVec, 8 * (size_t)c.nc));
    UMT_CUDA(cudaMemset(c.gtaVec, 0, 8 * (size_t)c.nc * 8));
  }
  if (!c.gtaSigS) TRY(dalloc(&c.gtaSigS, c.nz));
  if (!c.gtaZ) TRY(dalloc(&c.gtaZ, 5 * (size_t)c.nz));
  if (!c.red) TRY(dalloc(&c.red, 16));
  if (c.gtaSolver == UMT_GTA_ZONE && !c.gtaTT) {
    TRY(dalloc(&c.gtaTT, 8 * (size_t)c.nc));
    TRY(dalloc(&c.gtaLU, 8 * (size_t)c.nc));
  }
  return 0;
}

int umt103_gta_correction(const double *PhiPrev, double *correction, double *chi, int *grey_sweeps) {
  Ctx &c = cur();
  if (!c.ready) return set_error(UMT_ERR_STATE, "umt103_init not called");
  if (c.rz) return set_error(UMT_ERR_STATE, "the context holds an RZ problem");
  if (!PhiPrev || !correction) return set_error(UMT_ERR_ARG, "null PhiPrev or correction");
  TRY(gta_alloc(c));
  const size_t ncG = (size_t)c.nc * c.G;
  if (!c.PhiPrev) TRY(dalloc(&c.PhiPrev, ncG));
  UMT_CUDA(cudaMemcpy(c.PhiPrev, PhiPrev, ncG * 8, cudaMemcpyHostToDevice));
  int gs = 0;
  TRY(gta_solve(c, c.gtaMaxKrylov, c.gtaTol, &gs, false));
  UMT_CUDA(cudaStreamSynchronize(c.stream));
  UMT_CUDA(cudaMemcpy(correction, c.gtaVec, (size_t)c.nc * 8, cudaMemcpyDeviceToHost));
  if (chi) UMT_CUDA(cudaMemcpy(chi, c.gtaChi, (size_t)c.nz * c.G * 8, cudaMemcpyDeviceToHost));
  if (grey_sweeps) *grey_sweeps = gs;
  return 0;
}

// ---------------------------------------------------------------------------
// Source iteration as one CUDA graph launch: a conditional WHILE node whose
// body is build-source -> sweep -> change norm (-> distance to phi_ref) ->
// k_si_decide, which counts the iteration, forms the convergence criterion
// on the device and sets the loop condition.  The host waits once, at the
// end.  Used for plain iterations (no GTA, no learned step: those decide on
// the host); a context where the graph cannot be built keeps the host loop.
// ---------------------------------------------------------------------------
struct SIState {
  int it, maxit, conv, useRef;
  double tol, rel, dist;
};

__global__ void k_si_reset(SIState *s, int maxit, double tol, int useRef) {
  s->it = 0; s->maxit = maxit; s->conv = 0; s->useRef = useRef;
  s->tol = tol; s->rel = 1.0; s->dist = -1.0;
}

__global__ void k_si_decide(cudaGraphConditionalHandle h, SIState *s, const double *red) {
  const double rel = red[1] > 0.0 ? sqrt(red[0] / red[1]) : 0.0;
  double crit = rel;
  if (s->useRef) {
    crit = red[9] > 0.0 ? sqrt(red[8] / red[9]) : 0.0;
    s->dist = crit;
  }
  s->rel = rel;
  s->it += 1;
  s->conv = crit < s->tol ? 1 : 0;
  cudaGraphSetConditional(h, (!s->conv && s->it < s->maxit) ? 1u : 0u);
}

// Builds (once per precision, buffer parity and criterion) and returns the
// graph; 1 when this context cannot use one.
static int si_graph(Ctx &c, int prec, const double *q, bool useRef, cudaGraphExec_t *out) {
  const int cur = prec == UMT_FP64 ? c.cur64 : c.cur32;
  cudaGraphExec_t &ex = c.siGraph[prec][cur][useRef ? 1 : 0];
  if (ex) { *out = ex; return 0; }
  if (c.siGraphState < 0) return 1;
  if (prec == UMT_FP32) {                          // one-time FP32 preparation, outside any capture
    bool prog = false;
    TRY(fp32_program_path(c, &prog));
  }
  cudaGraph_t g = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraphConditionalHandle h = 0;
  cudaError_t e = cudaGraphCreate(&g, 0);
  if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  if (e == cudaSuccess) e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np);
  int rc = 0;
  if (e == cudaSuccess) {
    cudaGraph_t body = np.conditional.phGraph_out[0];
    e = cudaStreamBeginCaptureToGraph(c.stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      const bool graphs = c.useGraphs;
      c.useGraphs = false;                         // enqueue the sweep's kernels into the body
      c.inSIGraph = true;
      rc = launch_build_source(c, q);
      if (!rc) rc = launch_sweep_once(c, prec, true);
      if (!rc) rc = launch_change_norm(c, c.PhiPrev, c.red, c.siDelta, c.siDeltaPrev);
      if (!rc && useRef) rc = launch_distance(c, c.siRef, c.red + 8);
      if (!rc) {
        k_si_decide<<<1, 1, 0, c.stream>>>(h, (SIState *)c.siState, c.red);
        if (cudaGetLastError() != cudaSuccess) rc = set_error(UMT_ERR_CUDA, "si graph: decide launch");
      }
      c.inSIGraph = false;
      c.useGraphs = graphs;
      cudaGraph_t got = nullptr;
      const cudaError_t e2 = cudaStreamEndCapture(c.stream, &got);
      if (e == cudaSuccess) e = e2;
    }
  }
  if (!rc && e == cudaSuccess) e = cudaGraphInstantiate(&exec, g, 0);
  if (g) cudaGraphDestroy(g);
  if (rc) { cudaGetLastError(); return rc; }
  if (e != cudaSuccess || !exec) {
    // conditional bodies refuse some node kinds; this context keeps the host loop
    cudaGetLastError();
    c.siGraphState = -1;
    return 1;
  }
  c.siGraphState = 1;
  ex = exec;
  *out = exec;
  return 0;
}

// Mixed-precision source iteration (UMT_MIXED): FP64 residual sweeps, FP32
// correction solves, the learned step inside the correction solves.
struct MixedStats { int outer = 0, fp32 = 0, fp64 = 0, kept = 0, rejected = 0; double rel = 1.0; bool conv = false; };

static int mixed_iterate(Ctx &c, const UmtSIParams *prm, const double *q, const double *ref, MixedStats &st) {
  const size_t ncG = (size_t)c.nc * c.G, psiBN = (size_t)c.A * c.nb * c.G;
  if (!c.psi64[0] || !c.psi32[0]) return set_error(UMT_ERR_STATE, "UMT_MIXED needs both the FP64 and the FP32 flux");
  if (!c.mixX) TRY(dalloc(&c.mixX, ncG));
  if (!c.mixR) TRY(dalloc(&c.mixR, ncG));
  if (!c.mixD) TRY(dalloc(&c.mixD, ncG));
  if (!c.psiB32h) {
    TRY(dalloc(&c.psiB32h, psiBN));
    UMT_CUDA(cudaMemset(c.psiB32h, 0, psiBN * sizeof(float)));
  }
  const int maxit = prm->max_iters > 0 ? prm->max_iters : 50;
  const double innerTol = prm->inner_tol > 0.0 ? prm->inner_tol : 1e-3;
  const int innerMax = prm->inner_max > 0 ? prm->inner_max : 500;
  const int learnEvery = prm->learn_every;
  const int learnStart = std::max(prm->learn_start, 2);
  if (prm->warm_start) UMT_CUDA(cudaMemcpyAsync(c.mixX, c.Phi, ncG * 8, cudaMemcpyDeviceToDevice, c.stream));
  else UMT_CUDA(cudaMemsetAsync(c.mixX, 0, ncG * 8, c.stream));
  struct Homog {                                  // the homogeneous FP32 sweeps end with the call
    Ctx &c;
    ~Homog() { c.homog32 = false; }
  } homogGuard{c};
  double h[3];
  auto fetch2 = [&](const double *dev) -> int {
    UMT_CUDA(cudaMemcpyAsync(h, dev, 3 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    UMT_CUDA(cudaStreamSynchronize(c.stream));
    return 0;
  };
  while (st.outer < maxit) {
    ++st.outer;
    // exact residual of the current iterate: one FP64 sweep
    c.homog32 = false;
    TRY(launch_build_source_vec(c, c.mixX, q));
    TRY(launch_sweep_once(c, UMT_FP64, true));
    ++st.fp64;
    TRY(launch_residual(c, c.mixX, c.mixR, c.red));
    TRY(fetch2(c.red));
    st.rel = h[1] > 0.0 ? std::sqrt(h[0] / h[1]) : 0.0;
    double crit = st.rel;
    if (ref) {                                    // T(X) is the better iterate: measure it
      TRY(launch_distance(c, ref, c.red + 8));
      TRY(fetch2(c.red + 8));
      crit = h[1] > 0.0 ? std::sqrt(h[0] / h[1]) : 0.0;
    }
    if (crit < prm->rel_tol) {
      UMT_CUDA(cudaMemcpyAsync(c.mixX, c.Phi, ncG * 8, cudaMemcpyDeviceToDevice, c.stream));
      st.conv = true;
      break;
    }
    // correction D = K D + R by FP32 source iteration from D = R
    c.homog32 = true;
    UMT_CUDA(cudaMemcpyAsync(c.mixD, c.mixR, ncG * 8, cudaMemcpyDeviceToDevice, c.stream));
    UMT_CUDA(cudaMemcpyAsync(c.siDelta, c.mixR, ncG * 8, cudaMemcpyDeviceToDevice, c.stream));
    UMT_CUDA(cudaMemsetAsync(c.siDeltaPrev, 0, ncG * 8, c.stream));
    int plain = 1;
    bool pending = false;
    double rBefore = 0.0;
    for (int j = 1; j < innerMax; ++j) {
      TRY(launch_build_source_vec(c, c.mixD, nullptr));
      TRY(launch_sweep_once(c, UMT_FP32, true));
      ++st.fp32;
      TRY(launch_inner_update(c, c.mixR, c.mixD, c.siDelta, c.siDeltaPrev, c.red));
      TRY(fetch2(c.red));
      const double dAbs = std::sqrt(h[2]);            // amplification-weighted change
      const double relIn = h[1] > 0.0 ? std::sqrt(h[0] / h[1]) : 0.0;
      if (pending) {
        pending = false;
        if (dAbs < rBefore) {
          ++st.kept;
        } else {
          ++st.rejected;
          UMT_CUDA(cudaMemcpyAsync(c.mixD, c.siKeep, ncG * 8, cudaMemcpyDeviceToDevice, c.stream));
          plain = 0;
          continue;
        }
      }
      if (relIn < innerTol) break;
      ++plain;
      if (learnEvery > 0 && j + 1 >= learnStart && plain >= std::max(learnEvery, 2)) {
        UMT_CUDA(cudaMemcpyAsync(c.siKeep, c.mixD, ncG * 8, cudaMemcpyDeviceToDevice, c.stream));
        TRY(mlp_correct(c, c.mixD, c.siDelta, c.siDeltaPrev));
        rBefore = dAbs;
        pending = true;
        plain = 0;
      }
    }
    if (pending) {                                // unchecked: undo
      UMT_CUDA(cudaMemcpyAsync(c.mixD, c.siKeep, ncG * 8, cudaMemcpyDeviceToDevice, c.stream));
      ++st.rejected;
    }
    c.homog32 = false;
    TRY(gta_axpbypcz(c, (int)ncG, 1.0, c.mixD, 1.0, c.mixX, 0.0, nullptr));     // X += D
    if (ref) {
      TRY(launch_distance(c, ref, c.red + 8, c.mixX));
      TRY(fetch2(c.red + 8));
      if ((h[1] > 0.0 ? std::sqrt(h[0] / h[1]) : 0.0) < prm->rel_tol) { st.conv = true; break; }
    }
  }
  UMT_CUDA(cudaMemcpyAsync(c.Phi, c.mixX, ncG * 8, cudaMemcpyDeviceToDevice, c.stream));
  UMT_CUDA(cudaMemcpyAsync(c.PhiPrev, c.mixX, ncG * 8, cudaMemcpyDeviceToDevice, c.stream));
  if (learnEvery > 0) TRY(mlp_status());
  return 0;
}

int umt103_source_iterate(const UmtSIParams *prm, UmtSIResult *res) {
  Ctx &c = cur();
  if (!c.ready) return set_error(UMT_ERR_STATE, "umt103_init not called");
  if (c.rz) return set_error(UMT_ERR_STATE, "the context holds an RZ problem: use umt103_sweep_rz");
  if (!prm || !res) return set_error(UMT_ERR_ARG, "null params/result");
  const int prec = prm->precision;
  if (prec != UMT_FP64 && prec != UMT_FP32 && prec != UMT_MIXED) return set_error(UMT_ERR_ARG, "precision");
  if (prec == UMT_MIXED && prm->use_gta) return set_error(UMT_ERR_ARG, "UMT_MIXED does not combine with GTA");
  if (prm->use_gta) TRY(gta_alloc(c));
  int greySweeps = 0;
  const size_t ncG = (size_t)c.nc * c.G, nzG = (size_t)c.nz * c.G;
  if (!c.PhiPrev) TRY(dalloc(&c.PhiPrev, ncG));
  if (!c.red) TRY(dalloc(&c.red, 16));
  const int learnEvery = prm->learn_every;
  if (learnEvery < 0) return set_error(UMT_ERR_ARG, "learn_every must be >= 0");
  if (learnEvery > 0 && !mlp_ready_for(c.G))
    return set_error(UMT_ERR_STATE, "learned correction requested but no model for G=%d (umt103_mlp_init)", c.G);
  // the last two changes of PhiTotal (features of the learned step, and the
  // training snapshots of umt103_mlp_collect)
  if (!c.siDelta) TRY(dalloc(&c.siDelta, ncG));
  if (!c.siDeltaPrev) TRY(dalloc(&c.siDeltaPrev, ncG));
  if (learnEvery > 0 && !c.siKeep) TRY(dalloc(&c.siKeep, ncG));
  UMT_CUDA(cudaMemsetAsync(c.siDelta, 0, ncG * 8, c.stream));
  UMT_CUDA(cudaMemsetAsync(c.siDeltaPrev, 0, ncG * 8, c.stream));
  double *ref = nullptr;                          // device copy of phi_ref (this call only)
  if (prm->phi_ref) {
    TRY(dalloc(&ref, ncG));
    if (cudaMemcpy(ref, prm->phi_ref, ncG * 8, cudaMemcpyHostToDevice) != cudaSuccess) {
      cudaFree(ref);
      return set_error(UMT_ERR_CUDA, "phi_ref upload failed");
    }
  }
  struct RefGuard { double *p; ~RefGuard() { if (p) cudaFree(p); } } refGuard{ref};
  const double *q = nullptr;
  if (prm->q_ext) {
    if (!c.qExt) TRY(dalloc(&c.qExt, nzG));
    UMT_CUDA(cudaMemcpy(c.qExt, prm->q_ext, nzG * 8, cudaMemcpyHostToDevice));
    q = c.qExt;
  }
  const int maxit = prm->max_iters > 0 ? prm->max_iters : 50;
  if (!prm->warm_start) UMT_CUDA(cudaMemsetAsync(c.Phi, 0, ncG * 8, c.stream));
  UMT_CUDA(cudaMemcpyAsync(c.PhiPrev, c.Phi, ncG * 8, cudaMemcpyDeviceToDevice, c.stream));
  cudaEvent_t t0, t1;
  UMT_CUDA(cudaEventCreate(&t0)); UMT_CUDA(cudaEventCreate(&t1));
  UMT_CUDA(cudaEventRecord(t0, c.stream));
  int it = 0, sweeps = 0, kept = 0, rejected = 0, plain = 0;
  const int learnStart = std::max(prm->learn_start, 2);
  double rel = 1.0, rBefore = 0.0;
  bool conv = false, pending = false;
  bool viaGraph = false;
  const bool mixed = prec == UMT_MIXED;
  int fp64Sweeps = 0;
  if (mixed) {
    MixedStats ms;
    TRY(mixed_iterate(c, prm, q, ref, ms));
    it = ms.outer; sweeps = ms.fp32 + ms.fp64; fp64Sweeps = ms.fp64; rel = ms.rel; conv = ms.conv;
    kept = ms.kept; rejected = ms.rejected;
  }
  if (!mixed && !prm->use_gta && learnEvery == 0 && c.useGraphs && c.siGraphState >= 0) {
    if (!c.siState) TRY(dalloc((SIState **)&c.siState, 1));
    if (ref && !c.siRef) TRY(dalloc(&c.siRef, ncG));
    cudaGraphExec_t ex = nullptr;
    const int grc = si_graph(c, prec, q, ref != nullptr, &ex);
    if (grc < 0) return grc;
    if (grc == 0) {
      viaGraph = true;
      if (ref) UMT_CUDA(cudaMemcpyAsync(c.siRef, ref, ncG * 8, cudaMemcpyDeviceToDevice, c.stream));
      k_si_reset<<<1, 1, 0, c.stream>>>((SIState *)c.siState, maxit, prm->rel_tol, ref ? 1 : 0);
      UMT_CUDA(cudaGetLastError());
      UMT_CUDA(cudaEventRecord(t0, c.stream));   // timing starts at the graph launch
      UMT_CUDA(cudaGraphLaunch(ex, c.stream));
      SIState st;
      UMT_CUDA(cudaMemcpyAsync(&st, c.siState, sizeof(st), cudaMemcpyDeviceToHost, c.stream));
      UMT_CUDA(cudaStreamSynchronize(c.stream));
      it = st.it; sweeps = st.it; rel = st.rel; conv = st.conv != 0;
    }
  }
  while (!viaGraph && !mixed && it < maxit) {
    ++it;
    TRY(launch_build_source(c, q));
    TRY(launch_sweep_once(c, prec, true));
    ++sweeps;
    if (prm->use_gta) TRY(gta_solve(c, c.gtaMaxKrylov, c.gtaTol, &greySweeps));
    TRY(launch_change_norm(c, c.PhiPrev, c.red, c.siDelta, c.siDeltaPrev, learnEvery > 0));
    double h[3];
    UMT_CUDA(cudaMemcpyAsync(h, c.red, 3 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    UMT_CUDA(cudaStreamSynchronize(c.stream));
    rel = h[1] > 0.0 ? std::sqrt(h[0] / h[1]) : 0.0;
    const double rAbs = std::sqrt(h[2]);          // amplification-weighted change (learned guard)
    double dist = -1.0;                           // relative distance to phi_ref
    if (ref) {
      TRY(launch_distance(c, ref, c.red + 8));
      UMT_CUDA(cudaMemcpyAsync(h, c.red + 8, 2 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
      UMT_CUDA(cudaStreamSynchronize(c.stream));
      dist = h[1] > 0.0 ? std::sqrt(h[0] / h[1]) : 0.0;
    }
    if (pending) {
      // The sweep after a learned correction is its check: the correction
      // stays only if the iteration residual dropped below the one before it.
      // The residual is weighted per zone and group by 1/(1 - c), the factor
      // by which it understates the error where scattering dominates; an
      // unweighted norm would reject corrections that remove slowly decaying
      // error in thick scattering zones at the price of smaller, quickly
      // damped errors in thin ones.
      pending = false;
      if (rAbs < rBefore) {
        ++kept;
      } else {
        ++rejected;
        UMT_CUDA(cudaMemcpyAsync(c.Phi, c.siKeep, ncG * 8, cudaMemcpyDeviceToDevice, c.stream));
        UMT_CUDA(cudaMemcpyAsync(c.PhiPrev, c.siKeep, ncG * 8, cudaMemcpyDeviceToDevice, c.stream));
        plain = 0;
        rel = 1.0;
        continue;
      }
    }
    if ((ref ? dist : rel) < prm->rel_tol) { conv = true; break; }
    ++plain;
    // two plain iterations since the last correction give the change ratio
    if (learnEvery > 0 && it >= learnStart && plain >= std::max(learnEvery, 2)) {
      UMT_CUDA(cudaMemcpyAsync(c.siKeep, c.Phi, ncG * 8, cudaMemcpyDeviceToDevice, c.stream));
      TRY(mlp_correct(c, c.Phi, c.siDelta, c.siDeltaPrev));
      UMT_CUDA(cudaMemcpyAsync(c.PhiPrev, c.Phi, ncG * 8, cudaMemcpyDeviceToDevice, c.stream));
      rBefore = rAbs;
      pending = true;
      plain = 0;
    }
  }
  if (pending) {                                  // the last correction was never checked: undo it
    UMT_CUDA(cudaMemcpyAsync(c.Phi, c.siKeep, ncG * 8, cudaMemcpyDeviceToDevice, c.stream));
    ++rejected;
  }
  if (learnEvery > 0 && !mixed) TRY(mlp_status());
  if (prec == UMT_FP64) fp64Sweeps = sweeps;
  if (prm->save_psi) {
    const int sp = mixed ? UMT_FP64 : prec;     // the mixed iterate is FP64-accurate
    TRY(launch_build_source(c, q));
    TRY(launch_sweep_once(c, sp, true));
    ++sweeps;
    if (sp == UMT_FP64) { c.cur64 = 1 - c.cur64; ++fp64Sweeps; } else c.cur32 = 1 - c.cur32;
  }
  UMT_CUDA(cudaEventRecord(t1, c.stream));
  UMT_CUDA(cudaStreamSynchronize(c.stream));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, t0, t1);
  cudaEventDestroy(t0); cudaEventDestroy(t1);
  res->iterations = it; res->sweeps = sweeps; res->rel_change = rel; res->seconds = ms * 1e-3;
  res->grey_sweeps = greySweeps;
  res->learned_kept = kept;
  res->learned_rejected = rejected;
  res->fp64_sweeps = fp64Sweeps;
  return conv ? 0 : set_error(UMT_ERR_NOTCONV, "not converged after %d iterations (rel change %.3e)", it, rel);
}

// ---- source iteration one step at a time, for a caller that owns the
// collective (angle sharding: each rank sweeps its directions, then sums
// PhiTotal over ranks in place on the device) ----
int umt103_phi_device(double **phi, long long *count) {
  Ctx &c = cur();
  if (!c.ready) return set_error(UMT_ERR_STATE, "umt103_init not called");
  if (!phi) return set_error(UMT_ERR_ARG, "null output");
  *phi = c.Phi;
  if (count) *count = (long long)c.nc * c.G;
  return 0;
}

int umt103_set_external_source(const double *q_ext) {
  Ctx &c = cur();
  if (!c.ready) return set_error(UMT_ERR_STATE, "umt103_init not called");
  const size_t nzG = (size_t)c.nz * c.G;
  if (!q_ext) { dfree(c.qExt); return 0; }
  if (!c.qExt) TRY(dalloc(&c.qExt, nzG));
  UMT_CUDA(cudaMemcpy(c.qExt, q_ext, nzG * 8, cudaMemcpyHostToDevice));
  return 0;
}

int umt103_si_step(int precision) {
  Ctx &c = cur();
  if (!c.ready) return set_error(UMT_ERR_STATE, "umt103_init not called");
  if (c.rz) return set_error(UMT_ERR_STATE, "the context holds an RZ problem");
  if (precision != UMT_FP64 && precision != UMT_FP32) return set_error(UMT_ERR_ARG, "precision");
  if (precision == UMT_FP64 && !c.psi64[0]) return set_error(UMT_ERR_STATE, "FP64 flux not allocated");
  if (precision == UMT_FP32 && !c.psi32[0]) return set_error(UMT_ERR_STATE, "FP32 flux not allocated");
  TRY(launch_build_source(c, c.qExt));
  TRY(launch_sweep_once(c, precision, true));
  UMT_CUDA(cudaStreamSynchronize(c.stream));
  return 0;
}

int umt103_si_change(double *rel) {
  Ctx &c = cur();
  if (!c.ready) return set_error(UMT_ERR_STATE, "umt103_init not called");
  if (!rel) return set_error(UMT_ERR_ARG, "null output");
  const size_t ncG = (size_t)c.nc * c.G;
  if (!c.red) TRY(dalloc(&c.red, 16));
  if (!c.PhiPrev) {
    TRY(dalloc(&c.PhiPrev, ncG));
    UMT_CUDA(cudaMemset(c.PhiPrev, 0, ncG * 8));
  }
  TRY(launch_change_norm(c, c.PhiPrev, c.red));
  double h[3];
  UMT_CUDA(cudaMemcpyAsync(h, c.red, 3 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  UMT_CUDA(cudaStreamSynchronize(c.stream));
  *rel = h[1] > 0.0 ? std::sqrt(h[0] / h[1]) : 0.0;
  return 0;
}

int umt103_tally(const double *siga, double speed_light, UmtEnergyTally *t) {
  if (!cur().ready) return set_error(UMT_ERR_STATE, "umt103_init not called");
  return umt103_tally_precision(siga, speed_light, cur().psi64[0] ? UMT_FP64 : UMT_FP32, t);
}

int umt103_tally_precision(const double *siga, double speed_light, int precision, UmtEnergyTally *t) {
  Ctx &c = cur();
  if (!c.ready) return set_error(UMT_ERR_STATE, "umt103_init not called");
  if (c.rz) return set_error(UMT_ERR_STATE, "umt103_tally: the context holds an RZ problem");
  if (precision != UMT_FP64 && precision != UMT_FP32) return set_error(UMT_ERR_ARG, "precision must be UMT_FP64 or UMT_FP32");
  if (precision == UMT_FP64 && !c.psi64[0]) return set_error(UMT_ERR_STATE, "FP64 flux not allocated");
  if (precision == UMT_FP32 && !c.psi32[0]) return set_error(UMT_ERR_STATE, "FP32 flux not allocated");
  if (!t || !(speed_light > 0.0)) return set_error(UMT_ERR_ARG, "bad tally arguments");
  if (!c.red) TRY(dalloc(&c.red, 16));
  const size_t nzG = (size_t)c.nz * c.G;
  double *dsiga = nullptr;
  if (siga) {
    TRY(dalloc(&dsiga, nzG));
    UMT_CUDA(cudaMemcpy(dsiga, siga, nzG * 8, cudaMemcpyHostToDevice));
  }
  int rc = launch_energy(c, dsiga, precision, c.red);
  double h[4] = {0, 0, 0, 0};
  if (!rc) {
    cudaError_t e = cudaMemcpyAsync(h, c.red, 4 * sizeof(double), cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess) rc = set_error(UMT_ERR_CUDA, "tally: %s", cudaGetErrorString(e));
  }
  if (dsiga) cudaFree(dsiga);
  if (rc) return rc;
  t->EnergyRadiation = h[0] / speed_light;
  t->PowerAbsorbed = h[1];
  t->PowerEscape = h[2];
  t->PowerIncident = h[3];
  t->Balance = 0.0;
  return 0;
}

}  // extern "C"

namespace umt {

// Context set-up and release for the other front ends of the library (the
// RZ entry points in rz.cu): the same validation, uploads, projections and
// device schedule as umt103_init, without the grey context.
int init_context(Ctx &c, const UmtMesh *m, const UmtQuad *q, int ngr, int flags) {
  return init_ctx(c, m, q, ngr, flags);
}
void release_current_context() { free_all(); }
int staging_buffer64(Ctx &c, size_t n, double **out) { return staging64(c, n, out); }

}  // namespace umt
