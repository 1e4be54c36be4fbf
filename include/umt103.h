/*
 * umt103.h -- C-ABI of the GB300 (sm_103a) upstream-corner-balance sweep.
 *
 * This library replaces Teton's sweep/solve path below ControlSweep
 * (src/teton/rt/ControlSweep.F90:15-81): the CPU SetSweep/SweepUCBxyz pair
 * (snac/SetSweep.F90:10, snac/SweepUCBxyz.F90:11), the OpenMP-offload
 * SetSweep_GPU (gpu/SetSweep_OMPOL.F90:12) and the CUDA gpu_sweepucbxyz
 * (gpu/GPU_SweepUCBxyz.cu:532-572, bound from gpu/SweepUCBxyzToGPU.F90:44-90),
 * plus the psi->phi tally getPhiTotal (control/getPhiTotal_OMPOL.F90:12) and
 * the source-iteration loop of rtmainsn/LinearSolver
 * (rt/rtmainsn.F90:167-246, rt/LinearSolver.F90:10-124).
 *
 * Conventions (all functions):
 *   - return 0 on success, a negative UMT_ERR_* code otherwise; nothing
 *     calls exit() or abort();
 *   - called from one host thread; the library owns every device buffer;
 *     host pointers are borrowed for the duration of the call only;
 *   - index arrays are 0-based or 1-based per UmtMesh.index_base (Fortran
 *     callers pass 1); the library converts once in umt103_init;
 *   - arrays are in Teton's memory order: Psi(G,ncornr,A) is [a][c][g],
 *     A_fp(3,maxcf,ncornr) is [c][cf][3], Sigt(G,nzones) is [z][g].
 */
#ifndef UMT103_H
#define UMT103_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
  UMT_OK = 0,
  UMT_ERR_ARG = -1,        /* bad argument or size                         */
  UMT_ERR_STATE = -2,      /* call order (e.g. sweep before init)          */
  UMT_ERR_CUDA = -3,       /* CUDA runtime error                           */
  UMT_ERR_CYCLE = -4,      /* a mesh cycle this path cannot carry (RZ, the
                              persistent sweep), or a cycle left unbroken */
  UMT_ERR_TIMEOUT = -5,    /* a bounded device wait gave up                */
  UMT_ERR_BOUNDS = -6,     /* device bounds check tripped                  */
  UMT_ERR_NOMEM = -7,      /* device allocation failed                     */
  UMT_ERR_NOTCONV = -8     /* iteration limit reached before convergence   */
};

/* precision of the angular-flux sweep; UMT_MIXED (source iteration only):
 * FP64 residual sweeps around FP32 correction solves */
enum { UMT_FP64 = 0, UMT_FP32 = 1, UMT_MIXED = 2 };

/*
 * Mesh in Teton's corner representation: what teton_setzone
 * (aux/setTetonZone.F90:10-202) stores in Geometry_mod.
 */
typedef struct UmtMesh {
  int index_base;          /* 0 (C) or 1 (Fortran)                          */
  int nzones, ncornr, nbelem;
  int maxcf;               /* corner faces per corner, must be <= 3         */
  int maxFaces;            /* row stride of zoneOpp/faceOpp, <= 6           */
  const int *numCorner;    /* [nzones] corners per zone (<= 8)              */
  const int *cOffSet;      /* [nzones] corners before this zone (a count)   */
  const int *zoneFaces;    /* [nzones]                                      */
  const int *zoneOpp;      /* [nzones*maxFaces] zone across face; < base => boundary */
  const int *faceOpp;      /* [nzones*maxFaces] face index in that zone     */
  const int *nCFaces;      /* [ncornr]                                      */
  const int *cFP;          /* [ncornr*maxcf] corner across FP face, or ncornr+b */
  const int *cEZ;          /* [ncornr*maxcf] zone-local corner across EZ face */
  const int *CToFace;      /* [ncornr*maxcf] zone-local face of the corner face */
  const int *bdyToC;       /* [nbelem] corner of each boundary element      */
  const double *px;        /* [ncornr*3] vertex of each corner, or NULL     */
  const double *A_fp;      /* [ncornr*maxcf*3] or NULL: computed on device  */
  const double *A_ez;      /* [ncornr*maxcf*3] or NULL: computed on device  */
  const double *Volume;    /* [ncornr] or NULL: computed on device          */
} UmtMesh;

/* Directions and weights (Quadrature_mod omega(3,A), weight(A)). */
typedef struct UmtQuad {
  int nangles;
  const double *omega;     /* [nangles*3] */
  const double *weight;    /* [nangles]   */
} UmtQuad;

/*
 * umt103_init: upload mesh and quadrature, compute corner geometry on the
 * device when not given (rt/geometryUCBxyz.F90:9-185) and build the sweep
 * schedule of every direction on the device (replaces rtorder/snnext,
 * rt/rtorder.F90:8-111, snac/snnext.F90:12-234, and findexit,
 * rt/findexit.F90:296-347).  Meshes with sweep cycles are ordered as the
 * reference orders them: faces of mixed sign and zones whose corners cannot
 * be ordered put corners on the direction's cycle list (snac/snneed.F90,
 * fixZone), and when a direction's wavefront stalls its remaining zones are
 * cut apart with the reference's strongly-connected-component breaker
 * (snac/cyclebreaker.F90, snac/sccsearch.F90) on the host; each sweep reads
 * the cycle-list corners from the previous sweep's values
 * (initFromCycleList / updateCycleList).  flags: bit0 = allocate the FP64
 * angular flux, bit1 = allocate the FP32 angular flux (both when 0).
 */
int umt103_init(const UmtMesh *mesh, const UmtQuad *quad, int ngr, int flags);

/* Release every device buffer of the current context (idempotent). */
void umt103_finalize(void);

/*
 * Several independent problems can be resident at once.  Context 0 always
 * exists; umt103_context_create adds one (empty until umt103_init), and every
 * other entry point acts on the context made current by umt103_context_select.
 * No reference counterpart: Teton keeps one problem in module state.
 */
int umt103_context_create(int *id);
int umt103_context_select(int id);
int umt103_context_current(void);
int umt103_context_destroy(int id);   /* id > 0; releases its buffers */

/*
 * One sweep of each listed context from a single CUDA graph launch: the
 * contexts' captured sweeps become independent child graphs, so problems of
 * different zone, group and direction counts run concurrently.  *ms (may be
 * NULL) receives the device time of the whole batch.  Each context's
 * PhiTotal is left on its device (umt103_get_phi after selecting it).  The
 * instantiated batch graph is kept for the same list, precision and buffer
 * parities until a listed context changes (materials, group tile, sweep
 * mode, re-initialisation), so a repeated batch costs one graph launch.
 * Every listed context's device status word is read and cleared after the
 * launch; a bounds or timeout flag returns UMT_ERR_BOUNDS / UMT_ERR_TIMEOUT
 * naming the context.  A context with a held work item (umt103_hold_item) or
 * an RZ problem is refused with UMT_ERR_STATE; a context listed twice with
 * UMT_ERR_ARG.
 */
int umt103_batch_sweep(const int *ids, int n, int precision, double *ms);

/* How umt103_batch_sweep builds its graph.  UMT_BATCH_GRAPHS (1, default):
 * each context's own sweep graph as a child node, so every problem's stages
 * advance at their own pace.  UMT_BATCH_MERGED (0): for FP32 contexts on the
 * zone-program kernel, every dependency stage of all the problems that share
 * a group tile is one kernel launch (problems of different tiles on parallel
 * streams), with each context's conversions, cycle rows and tally around
 * them; it holds those problems in lockstep and measured 5-22% slower; any
 * other batch falls back to the nested form.  Results are the same in both. */
#define UMT_BATCH_MERGED 0
#define UMT_BATCH_GRAPHS 1
int umt103_set_batch_mode(int mode);

/*
 * Materials: sigt = total opacity including tau, Sigt(G,nzones) as
 * setTotalOpacity builds it (control/setTotalOpacity.F90:52); sigs =
 * scattering opacity SigS(G,nzones) (may be NULL: no scattering); tau =
 * 1/(c*dt) multiplying the previous-cycle angular flux in the source
 * (snac/SweepUCBxyz.F90:121).
 */
int umt103_set_materials(const double *sigt, const double *sigs, double tau);

/*
 * Angular-flux state: Psi(G,ncornr,A) saved at the end of the last cycle
 * (Set%Psi) and PsiB(G,nbelem,A) (Set%PsiB).  Either may be NULL (zero).
 * Both precisions present are set from the FP64 input.
 */
int umt103_set_psi(const double *Psi, const double *PsiB);
int umt103_get_psi(double *Psi, double *PsiB, int precision);

/*
 * One full sweep of every direction and group (SetSweep + getPhiTotal):
 * source Q = STotal + tau*Psi; PhiTotal(G,ncornr) = sum_a w_a psi_a;
 * exiting boundary fluxes written into PsiB; with savePsi the new angular
 * flux becomes Psi.  STotal may be NULL (zero source, the mini-app case);
 * PhiTotal_out and PsiB_inout may be NULL (results stay on the device).
 * With UMT_FP32 only the PsiB rows the sweep reads are read and only the
 * rows it writes are written; the others keep their values bit for bit.
 * Host arrays in page-locked memory (16-byte aligned) are read and written
 * in place while the stages run; pageable ones are copied whole before and
 * after.  The results are the same either way.
 */
int umt103_sweep(const double *STotal, int savePsi, double *PhiTotal_out,
                 double *PsiB_inout, int precision);

/*
 * Device-resident variant for callers that keep everything in HBM: uses the
 * source last set with umt103_set_source (or zero) and leaves PhiTotal on
 * the device (read it with umt103_get_phi).
 */
int umt103_set_source(const double *STotal);
int umt103_sweep_resident(int savePsi, int precision);
int umt103_get_phi(double *PhiTotal);

/*
 * Source iteration one step at a time, for a caller that owns the collective:
 * with the directions split over ranks (one GPU each), every rank runs
 * umt103_si_step (STotal = wtiso (sigma_s PhiTotal + q) built on the device,
 * then a resident sweep of its directions), sums the device PhiTotal over
 * ranks in place (e.g. an NCCL all-reduce on the pointer umt103_phi_device
 * returns: nc*G FP64, valid until the context is released), and calls
 * umt103_si_change for the relative L2 change since its last call.  This is
 * the flux all-reduce of snac/SetSweep.F90:199 and rt/scat_prod.F90:81.
 * umt103_set_external_source uploads q [nzones*G] once (NULL: none).
 */
int umt103_phi_device(double **phi, long long *count);
int umt103_set_external_source(const double *q_ext);
int umt103_si_step(int precision);
int umt103_si_change(double *rel);

/* Source iteration (rtmainsn / LinearSolver / ConvergenceTest).
 *
 * UMT_MIXED is defect correction: each outer step is one FP64 sweep of the
 * current iterate X, giving the exact residual R = T(X) - X of the
 * source-iteration map T; the correction D solving D = K D + R (K: the
 * scattering sweep with no tau*psi_old term and no boundary inflow) is then
 * iterated with FP32 sweeps until its relative change is below inner_tol,
 * and X += D.  The FP32 rounding then limits only the correction, so the
 * iteration reaches FP64 accuracy where plain FP32 source iteration stalls
 * at an error of about (FP32 rounding) / (1 - c) in strongly scattering
 * zones.  The learned step (learn_every) acts on the inner iteration.  No
 * counterpart in the reference (FP64 throughout). */
typedef struct UmtSIParams {
  int precision;           /* UMT_FP64, UMT_FP32 or UMT_MIXED               */
  int max_iters;           /* outer iterations (default 50)                 */
  double rel_tol;          /* max relative change of zone phi               */
  int use_gta;             /* 1: grey transport acceleration after each sweep */
  const double *q_ext;     /* [nzones*G] isotropic external source, or NULL */
  int save_psi;            /* final savePsi sweep                           */
  int warm_start;          /* 1: start from the current PhiTotal, 0: from zero */
  int learn_every;         /* 0: off; else apply the learned correction after
                              every learn_every (>= 2) plain iterations; needs
                              umt103_mlp_init for this group count           */
  int learn_start;         /* first iteration that may be corrected (>= 2)  */
  const double *phi_ref;   /* [ncornr*G] or NULL: when given, stop when the
                              relative L2 distance of PhiTotal to it is below
                              rel_tol (time-to-converge measurements against a
                              known converged answer) instead of the change */
  double inner_tol;        /* UMT_MIXED: relative change ending a correction
                              solve (0: 1e-3)                                */
  int inner_max;           /* UMT_MIXED: FP32 sweeps per correction (0: 500) */
} UmtSIParams;

typedef struct UmtSIResult {
  int iterations;
  int sweeps;
  double rel_change;       /* last relative change of phi                   */
  double seconds;          /* device time                                   */
  int grey_sweeps;         /* GTA grey S2 sweeps performed                  */
  int learned_kept;        /* learned corrections kept (residual dropped)   */
  int learned_rejected;    /* learned corrections undone                    */
  int fp64_sweeps;         /* sweeps with the FP64 angular flux             */
} UmtSIResult;

int umt103_source_iterate(const UmtSIParams *params, UmtSIResult *result);

/* GTA options: BiCGStab iterations per correction (each costs two grey S2
 * sweeps; the reference's default grey budget is 21 sweeps,
 * mods/default_iter_controls_mod.F90:10-22), relative residual tolerance, and
 * the correction spectrum (0: shape of the scattering residual, 1: residual
 * weighted by 1/(1-c) per group). */
int umt103_set_gta(int max_krylov, double tol, int spectrum);

/* GTA solver (Teton's Size%useNewGTASolver, driver option gta_kernel):
 * UMT_GTA_TSA (1, the reference's default) applies the grey operator as a
 * grey S2 sweep plus a stretched-TSA sweep (rt/GreySweep.F90 GreySweep);
 * UMT_GTA_ZONE (2) as one grey sweep followed by a direct solve of each
 * zone's local scattering with the zone's transfer matrix
 * (rt/GreySweep.F90 GreySweepNEW, snac/InitSweepGreyUCBxyz.F90,
 * snac/UpdateScalarIntensity.F90).  Both feed the same BiCGStab
 * (rt/GTASolver.F90). */
#define UMT_GTA_TSA 1
#define UMT_GTA_ZONE 2
int umt103_set_gta_solver(int solver);

/* The grey correction of one source iteration, not applied: with the
 * context's current PhiTotal and the previous iterate PhiPrev [ncornr*G], the
 * spectrum chi [nzones*G] (may be NULL) and the grey correction [ncornr]
 * that umt103_source_iterate (use_gta) would add as phi_g += chi_g x
 * (rt/GTASolver.F90:42-425 with rt/GreySweep.F90, rt/addGreyCorrections.F90).
 * *grey_sweeps (may be NULL) receives the grey S2 sweeps it took. */
int umt103_gta_correction(const double *PhiPrev, double *correction, double *chi, int *grey_sweeps);

/*
 * Energy tallies of the last sweep (rtedit, aux/rtedit.F90:8-327, and
 * BoundaryEdit, control/BoundaryEdit.F90:9-215), accumulated in FP64.
 */
typedef struct UmtEnergyTally {
  double EnergyRadiation;   /* sum V*PhiTotal / c                           */
  double PowerEscape;       /* sum w (A_bdy.Omega>0) A_bdy.Omega psi         */
  double PowerIncident;     /* sum w (A_bdy.Omega<0) |A_bdy.Omega| psiB      */
  double PowerAbsorbed;     /* sum V sigma_a PhiTotal                        */
  double Balance;           /* reserved; always 0 (the host forms the balance
                               from the other four, as rtedit does)          */
} UmtEnergyTally;

int umt103_tally(const double *siga, double speed_light, UmtEnergyTally *tally);

/* Same, on the angular flux of the given precision (UMT_FP64 / UMT_FP32). */
int umt103_tally_precision(const double *siga, double speed_light, int precision,
                           UmtEnergyTally *tally);

/*
 * umt103_tally_noalloc: the energy edits of umt103_tally_precision for
 * callers that cannot let a library allocate device memory during a call --
 * host codes whose memory pool must account for every device byte, or runs
 * that have already reserved all free device memory, where an allocation
 * inside the library would fail or escape the pool.  No counterpart in the
 * reference (its edits run on the host, aux/rtedit.F90).
 *
 *   siga_dev    absorption opacity Siga(G,nzones) already in device memory,
 *               or NULL (PowerAbsorbed is then 0); nothing is copied;
 *   precision   UMT_FP64 or UMT_FP32 angular flux.
 *
 * It allocates nothing: the reduction works in a fixed scratch array that is
 * part of the loaded library (one copy on every GPU that loads it, held until
 * the process exits), and the result is summed in a fixed order, so repeated
 * calls give bit-identical results.  The scratch need not start at zero:
 * each call writes every value it later reads.  Limit: max(ncornr*G, nangles*nbelem)
 * must not exceed UMT_NOALLOC_MAX_BLOCKS*4096 elements (UMT_ERR_ARG with a
 * message otherwise).  Every call looks up the scratch address on the
 * current device (a lookup, not an allocation), so a primary context that
 * was reset and recreated is followed; make the first call on a device
 * before any stream capture, because that lookup may load the library's
 * device image.  An RZ context is refused (UMT_ERR_STATE).
 * All calls share the scratch: calls that overlap on the GPU (other threads,
 * other streams of the same device) race and must be serialised by the caller.
 */
#define UMT_NOALLOC_MAX_BLOCKS 32768
int umt103_tally_noalloc(const double *siga_dev, double speed_light, int precision,
                         UmtEnergyTally *tally);

/* ---------------------------------------------------------------------------
 * Learned acceleration of source iteration.  No counterpart in the reference
 * (Teton accelerates only with grey transport, rt/GTASolver.F90).
 *
 * One network per process: per zone, F = 4G+4 features (optical size
 * ln(sigma_t h), -ln(1-c), the ratio of the last two zone changes of phi, the
 * signed relative change, and zone size, corner count, corner-volume spread)
 * -> 3 hidden layers of 128 (ReLU) -> G outputs o; the corrected flux of each
 * corner is phi + exp(clamp(o, -12, 8)) * (phi - phi_prev).  Weights are
 * BF16 on the tensor cores with FP32 accumulation (FP32 master copy).  In
 * umt103_source_iterate (UmtSIParams.learn_every) a correction is kept only
 * if the next sweep's change of phi is smaller than the change before the
 * correction; otherwise the iterate is restored.
 * ------------------------------------------------------------------------- */
int umt103_mlp_init(int ngr, unsigned seed);          /* random weights; 1 <= ngr <= 60 */
void umt103_mlp_finalize(void);
int umt103_mlp_info(int *features, int *hidden, long long *nparams);
/* FP32 master parameters, in order W1[128][F], b1[128], W2[128][128], b2,
 * W3[128][128], b3, W4[G][128], b4[G] (row-major, out x in). */
int umt103_mlp_get_params(float *params);
int umt103_mlp_set_params(const float *params);
/* Outputs o [rows][G] of host features X [rows][F] (rounded to BF16). */
int umt103_mlp_forward(const float *X, int rows, float *Y);
/* Gradient of sum(dY * o) with respect to every parameter (rows a multiple
 * of 128), from the same kernels the training uses. */
int umt103_mlp_gradient(const float *X, const float *dY, int rows, float *grad);
/* Training set: umt103_mlp_collect appends the current context's zone
 * features after an (unconverged) umt103_source_iterate of two or more
 * iterations; umt103_mlp_set_targets(PhiStar) gives the converged PhiTotal
 * [ncornr][G] of that problem, which sets the targets of every snapshot
 * collected from it since the last call. */
int umt103_mlp_collect(int *rows_added);
int umt103_mlp_set_targets(const double *PhiStar);
int umt103_mlp_rows(long long *rows);
int umt103_mlp_clear(void);
/* Adam on random batches (batch a multiple of 128); loss[0..1] = fraction of
 * the targets' squared error left after the correction over the first and
 * last tenth of the steps. */
int umt103_mlp_train(int steps, int batch, float lr, float *loss);

/* Schedule statistics for one direction: its dependency stages and the
 * number of corners on its cycle list (ASet%numCycles, the corners whose
 * flux the sweep reads before it computes them and takes from the previous
 * sweep; control/constructDynMemory.F90:56-214). */
int umt103_schedule_info(int angle, int *nHyperPlanes, int *numCycles);

/* ---------------------------------------------------------------------------
 * 2-D cylindrical (RZ) geometry: the UCB sweep of snac/SweepUCBrz.F90 with
 * the angular-derivative (half-angle intensity PsiM) terms, FP64.
 * ------------------------------------------------------------------------- */

/* RZ mesh: polygonal zones in the (r, z) half-plane, two corner faces per
 * corner, Teton's RZ conventions (rt/geometryUCBrz.F90:48-150): a zone's
 * corners counter-clockwise; cEZ[2c] the previous and cEZ[2c+1] the next
 * corner of the zone (zone-local); corner face 0 on the edge to the next
 * vertex, face 1 on the edge from the previous one; cFP the corner at the
 * same vertex across that edge, or ncornr + b for boundary element b. */
typedef struct UmtMeshRZ {
  int index_base;            /* 0 or 1 (Fortran)                              */
  int nzones, ncornr, nbelem, maxFaces;
  const int *numCorner, *cOffSet, *zoneFaces;   /* [nzones]                   */
  const int *zoneOpp, *faceOpp;                 /* [nzones*maxFaces]          */
  const int *cFP, *cEZ, *CToFace;               /* [ncornr*2]                 */
  const int *bdyToC;                            /* [nbelem]                   */
  const double *px;                             /* [ncornr*2] (r, z)          */
} UmtMeshRZ;

/* RZ quadrature in sweep order (levels of fixed xi, each a starting
 * direction, the weighted directions, a finishing direction; rt/quadrz.F90)
 * with the angular coefficients of mods/AngleSet_mod.F90:335-346. */
typedef struct UmtQuadRZ {
  int nangles;
  const double *omega;                          /* [nangles*2] (mu, xi)       */
  const double *weight;                         /* [nangles]                  */
  const double *angDerivFac, *quadTauW1, *quadTauW2;   /* [nangles]           */
  const int *starting, *finishing;              /* [nangles] 0/1              */
} UmtQuadRZ;

/* Replaces the current context with an RZ problem: geometry (A_fp, A_ez,
 * Area, Volume, RadiusFP, RadiusEZ) and every direction's schedule are built
 * here; the directions of a level are swept in order (each needs the previous
 * one's PsiM), the levels concurrently.  flags: bit0 = FP64 angular flux,
 * bit1 = FP32 angular flux (0 = both), as for umt103_init; the FP32 path
 * needs ncornr + nbelem < 2^28. */
int umt103_init_rz(const UmtMeshRZ *mesh, const UmtQuadRZ *quad, int ngr, int flags);

/* One SetSweep of the RZ problem (snac/SetSweep.F90 with SweepUCBrz): same
 * arguments as umt103_sweep.  UMT_FP64 follows the reference's operation
 * order; UMT_FP32 keeps the flux in FP32 (tallies in FP64).  Finishing
 * directions receive PsiM, as in the reference.  umt103_set_materials /
 * umt103_set_psi / umt103_get_psi apply to the RZ context as to a 3-D one. */
int umt103_sweep_rz(const double *STotal, int savePsi, double *PhiTotal, double *PsiB_inout, int precision);

/* Copy out the RZ geometry: Area, Volume [ncornr], RadiusFP, RadiusEZ
 * [ncornr*2] (any pointer may be NULL). */
int umt103_get_geometry_rz(double *Area, double *Volume, double *RadiusFP, double *RadiusEZ);

/* Copy out the device-built schedule: level of each (angle, zone) [A][nzones]
 * and per-angle hyperplane counts. */
int umt103_get_schedule(int *level, int *nHyperPlanes);

/* Copy out the device geometry (A_fp, A_ez [ncornr*maxcf*3], Volume). */
int umt103_get_geometry(double *A_fp, double *A_ez, double *Volume);

/* Device time of the last umt103_sweep* call in milliseconds, or < 0. */
double umt103_last_sweep_ms(void);

/* Device times (ms) of the last sweep: [0] whole sweep, [1] the dependency-
 * stage sweep kernels, [2] the psi->phi tally.  No reference counterpart
 * (the reference accumulates wall time in SweepTimeCycle, rt/ControlSweep.F90). */
int umt103_last_timing(double *out3);

/* Group tile of the FP32 sweep: lanes_per_zone lanes share one (direction,
 * zone) pair and each lane carries groups_per_lane consecutive groups
 * (lanes_per_zone*groups_per_lane must equal the group count; 0,0 restores
 * the default).  Set by the autotuner (umt_gb300/autotune.py).  No reference
 * counterpart: the reference kernel fixes 4 groups x 32 zones per block
 * (gpu/GPU_SweepUCBxyz.cu:30-31). */
int umt103_set_group_tile(int lanes_per_zone, int groups_per_lane);

/* Autotuner (no reference counterpart): times every group tile the FP32
 * sweep supports on the current context's problem (reps timed sweeps after
 * one that captures the graph; the sweeps overwrite PhiTotal), keeps the
 * fastest, and caches it for the problem's shape (groups, directions, zones,
 * corners, sweep mode).  times (may be NULL) receives up to max_times
 * triples {lanes_per_zone, groups_per_lane, best ms}; *ntimes their count.
 * umt103_autotune_contexts tunes each listed context whose shape has no
 * cached tile and applies the cached tile to the others; umt103_batch_sweep
 * applies the cached tile of their shape to contexts with no tile set. */
int umt103_autotune(int reps, int *lanes_per_zone, int *groups_per_lane, double *times, int max_times,
                    int *ntimes);
int umt103_autotune_contexts(const int *ids, int n, int reps);

/* FP32 sweep kernel and scheduling.  Modes 0 and 2 launch one kernel per
 * dependency stage (the hyperplane loop of snac/SweepUCBxyz.F90:103, all
 * directions at once):
 *   0 (default) zone-program kernel: each (direction, zone) pair runs a
 *     compact list of its face operations built once on the device (group
 *     tiles with 2 or 4 groups per lane; other tiles, and geometry the
 *     program format cannot hold, fall back to mode 2);
 *   2 unrolled corner-slot kernel (every group tile; the fallback);
 *   1 one persistent launch in which each (direction, zone) pair starts as
 *     soon as its upwind zones have finished (bounded waits; a wait that
 *     gives up makes the sweep return UMT_ERR_TIMEOUT).  Slower than mode 0;
 *     kept as the one kernel whose blocks wait on one another, which the
 *     bounded-wait failure path (umt103_hold_item) exercises. */
int umt103_set_sweep_mode(int mode);

/* Number of kernels one sweep of the given precision launches (>= 0). */
int umt103_launches_per_sweep(int precision);

/* Failure-path test hook: the next sweep of the current context gives work
 * item `item` (direction * nzones + zone) one upwind dependency that nothing
 * satisfies (-1 clears).  In the persistent sweep mode (umt103_set_sweep_mode
 * 1) that item's bounded wait gives up, every waiting team drains, and the
 * call returns UMT_ERR_TIMEOUT; the device status is cleared once reported,
 * so the context stays usable.  Stage-launched modes ignore the hold.  No
 * counterpart in the reference. */
int umt103_hold_item(int item);

/* PsiB rows (direction, boundary element) of the current 3-D context: how
 * many the FP32 sweep writes (exiting faces) of the A*nbelem in all.  An FP32
 * umt103_sweep moves only the other rows host -> device and only the
 * exiting rows device -> host; the caller's PsiB keeps every row the sweep
 * does not write bit for bit (snac/SweepUCBxyz.F90 writes PsiB only on the
 * exit list).  No counterpart in the reference. */
int umt103_psib_rows(long long *exiting, long long *total);

/* Make `device` current for the calling thread before umt103_init (one
 * process per GPU; the reference binds ranks to GPUs the same way). */
int umt103_select_device(int device);

/* Last error text (static storage). */
const char *umt103_error_string(void);

#ifdef __cplusplus
}
#endif
#endif
