/*
 * vacgpu.h - C ABI of the GB300 TVDLF/Hancock engine for VAC 4.52.
 *
 * The library replaces the explicit time step of VAC's `program vac`
 * (src/vac.t:55-106): the dt selection (getdt_courant, src/vac.t:664-722),
 * the split twostep advance (advance/advance_expl/advect/advect1,
 * src/vac.t:223-572) with the Hancock predictor and TVDLF corrector
 * (src/vactvdlf.t:5-367), the ghost-cell fill (getboundary,
 * src/vacgrid.t:195-413) and the Powell/user source terms
 * (addsource2, src/vac.t:575-605).
 *
 * All entry points are plain C: POD arguments, host pointers, an int status
 * (0 = success, nonzero = error; the message is kept per thread and read with
 * vacgpu_last_error).  A nonzero status is where the Fortran host calls
 * die(message) (src/vacio.t:1108-1116).
 *
 * Arrays cross the boundary in VAC's own layout: column-major, ix1 fastest,
 * one contiguous block per variable, mesh cells only (ixM, no ghost layers),
 * exactly as readfileini_bin reads them (src/vacio.t:682-755) and
 * savefileout_bin writes them (src/vacio.t:1008-1047).  The library owns its
 * device copies; host arrays are never retained after a call returns.
 *
 * Threading: a handle is used by one host thread at a time (VAC itself is
 * single threaded, COMMON-block state, src/vacdef.t:78-175).  Distinct
 * handles are independent.
 */
#ifndef VACGPU_H
#define VACGPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define VACGPU_MAXNW 8      /* 3-D ideal MHD: rho, m1..m3, e, b1..b3          */
#define VACGPU_MAXB 6       /* 2*ndim default boundary regions (boundsetup)   */
#define VACGPU_MAXEQPAR 4
#define VACGPU_MAXSRCPAR 8

/* physics module (setvac -p=..., src/setvac:5-17) */
enum { VACGPU_PHYS_HD = 0, VACGPU_PHYS_MHD = 1 };

/* typelimiter(iw) (dwlimiter2, src/vacgrid.t:938-996) */
enum {
  VACGPU_LIM_MINMOD = 0,
  VACGPU_LIM_WOODWARD = 1,
  VACGPU_LIM_SUPERBEE = 2,
  VACGPU_LIM_VANLEER = 3,
  VACGPU_LIM_ALBADA = 4
};

/* typeB(iw,iB) (getboundary, src/vacgrid.t:195-413).  'fixed', 'fixed1'
 * and 'grad1' store their ghost values (grad1: ghost minus edge) at the
 * first ghost fill after vacgpu_upload and reuse them; 'cont1' extrapolates
 * linearly every time; 'symm0' is 'symm' with zero flux of the variable
 * through the boundary face (setnoflux, src/vacgrid.t:416-454). */
enum {
  VACGPU_BC_CONT = 0,
  VACGPU_BC_PERIODIC = 1,
  VACGPU_BC_SYMM = 2,
  VACGPU_BC_ASYMM = 3,
  VACGPU_BC_FIXED = 4,
  VACGPU_BC_FIXED1 = 5,
  VACGPU_BC_CONT1 = 6,
  VACGPU_BC_GRAD1 = 7,
  VACGPU_BC_SYMM0 = 8,
  VACGPU_BC_SPECIAL = 9  /* user routine specialbound: vacgpu_register_bound */
};

/* typefull1 (src/vactvdlf.t:92-299): second order 'tvdlf' or 'tvdlf1'
 * (Lax-Friedrichs dissipation), 'tvdmu' or 'tvdmu1' (TVD-MUSCL: Roe
 * characteristic dissipation, src/vactvd.t:86-206, src/vacphys.mhdroe.t,
 * src/vacphys.hdroe.t).  The first order forms run as one substep. */
enum {
  VACGPU_TVDLF = 0,
  VACGPU_TVDLF1 = 1,
  VACGPU_TVDMU = 2,
  VACGPU_TVDMU1 = 3
};

/* typeentropy per characteristic wave (entropyfix, src/vactvd.t:422-451) */
enum {
  VACGPU_ENTROPY_NUL = 0,
  VACGPU_ENTROPY_HARTEN = 1,
  VACGPU_ENTROPY_POWELL = 2,
  VACGPU_ENTROPY_RATIO = 3,
  VACGPU_ENTROPY_YEE = 4
};

/* typelimited (src/vactvdlf.t:150-162) */
enum {
  VACGPU_LIMITED_ORIGINAL = 0,
  VACGPU_LIMITED_PREVIOUS = 1,
  VACGPU_LIMITED_PREDICTOR = 2
};

/* typedimsplit (src/vac.t:310-324) */
enum { VACGPU_SPLIT_XYYX = 0, VACGPU_SPLIT_XY = 1 };

/* Arithmetic of the device state.
 * FP64: every operation in IEEE double, in the reference's operation order
 *       (no FMA contraction), bit-compatible with the FP64 oracle.
 * MIXED: state, fluxes and wave speeds in FP32.  The thermal-pressure
 *       recovery p=(g-1)(e-m^2/2rho-B^2/2), where low-beta cells cancel, is
 *       evaluated by default in double-float arithmetic on the FP32 pipes
 *       (exact FMA products and compensated sums, 44+ significant bits;
 *       the result is within a few FP32 ulps of p itself, however much
 *       e and m^2/2rho+B^2/2 cancel), not on the FP64 pipe; the environment
 *       variable VACGPU_MIXED_PRESSURE=f64 selects native IEEE double
 *       instead (split kernels, slower on GB300's narrow FP64 pipe).  The
 *       conservation sums, dt and t+=dt are native FP64.  Tolerance of the
 *       state against the FP64 path: relative L1 <= 1e-5 per variable. */
enum { VACGPU_PREC_FP64 = 0, VACGPU_PREC_MIXED = 1 };

/* device source hooks standing in for specialsource/getdt_special
 * (src/vacnul.specialsource.t:9-71) */
enum {
  VACGPU_SRC_NONE = 0,
  /* uniform gravity, vacusr.gravity.t:24-75: dm_i/dt += rho*g_i,
   * de/dt += sum_i g_i*m_i; params = g_1..g_ndim */
  VACGPU_SRC_GRAVITY = 1
};

/* Run parameters: the par/DEFAULT + par/PROBLEM namelist values the path
 * reads (readparameters, src/vacio.t:5-531; par/DEFAULT:1-86) after VAC's
 * derived defaults are applied (typepred1='hancock' for tvdlf, dimsplit and
 * sourcesplit harmonisation, typelimited='previous' when unsplit). */
typedef struct vacgpu_params {
  int ndim;                     /* 1..3                                     */
  int ndir;                     /* ndim..3 vector components                */
  int physics;                  /* VACGPU_PHYS_*                            */
  int nw;                       /* HD: 2+ndir, MHD: 2+2*ndir                */
  int nx[3];                    /* mesh cells per dimension (ixM extent)    */
  int dixB;                     /* ghost layers; must be 2 (src/vacdef.t:24)*/
  double eqpar[VACGPU_MAXEQPAR];/* eqpar(gamma_)[, eqpar(eta_)]             */
  int typefull;                 /* VACGPU_TVDLF / _TVDLF1 / _TVDMU / _TVDMU1 */
  int typelimiter[VACGPU_MAXNW];/* VACGPU_LIM_* per variable                */
  int typelimited;              /* VACGPU_LIMITED_*                         */
  int dimsplit;                 /* 1 = dimensional splitting                */
  int typedimsplit;             /* VACGPU_SPLIT_*                           */
  int divbfix;                  /* Powell source (MHD only)                 */
  int sourceunsplit;            /* sources inside predictor/corrector       */
  double courantpar;            /* CFL number                               */
  double dtpar;                 /* >0: fixed dt                             */
  double smallpcoeff;           /* smallp = min(p)*smallpcoeff at 1st call  */
  double smallp;                /* <0: computed as in getpthermal           */
  int slowsteps;
  int dtcantgrow;
  int tmaxexact;
  int itmax;
  double tmax;
  double dtmin;
  int typeB[VACGPU_MAXB][VACGPU_MAXNW]; /* [iB][iw]; iB = 2*(idim-1)+upper */
  int precision;                /* VACGPU_PREC_*                            */
  /* positivity repair in getboundary (keeppositive, src/vacphys.t.mhd:9-53,
   * src/vacphys.t.hd:176-219, src/vacproc.positive.t:2-34)               */
  int smallfix;                 /* 1 = keeppositive before each ghost fill  */
  double smallrho;              /* -1: min(rho)*smallrhocoeff at 1st use    */
  double smallrhocoeff;
  double vacuumrho;             /* >=0: rho<smallrho becomes vacuum         */
  int useprimitive;             /* limit primitive variables (upwindLR,     */
                                /* src/vactvdlf.t:325-362)                  */
  /* resistive MHD, eqpar[1] = eqpar(eta_): > 0 constant eta, < 0 the     */
  /* specialeta hook's field (src/vacphys.mhdres.t)                        */
  int compactres;               /* 1: Laplacian form, 0: curl form          */
  double dtdiffpar;             /* diffusion dt limit dtdiffpar*dx^2/eta    */
  /* Roe dissipation of 'tvdmu'/'tvdmu1' (src/vactvd.t:86-206)             */
  int typeentropy[VACGPU_MAXNW];   /* VACGPU_ENTROPY_* per wave il          */
  double entropycoef[VACGPU_MAXNW];/* 'yee' lower limit of |a| per wave     */
  int divbwave;                 /* MHD: keep the div B wave (par/DEFAULT:47) */
} vacgpu_params;

typedef struct vacgpu_handle vacgpu_handle;

/* Fill *p with par/DEFAULT values for the given configuration
 * (par/DEFAULT:1-86 plus the readparameters defaults src/vacio.t:55-118:
 * typefull='tvdlf', typelimiter='minmod', typeB='cont'). */
void vacgpu_default_params(vacgpu_params* p, int ndim, int ndir, int physics,
                           const int* nx);

/* Validate parameters, allocate device state for one grid.
 * Replaces readparameters + boundsetup + startup (src/vacio.t:5-531,
 * src/vacgrid.t:9-160, src/vac.t:160-220). */
int vacgpu_create(const vacgpu_params* p, vacgpu_handle** out);

/* Mesh coordinates x(ixM^S,1:ndim) as read from the .ini file.
 * Replaces gridsetup1 (src/vacgrid.t:457-593): ghost coordinates are
 * extrapolated linearly, dx=(x_{i+1}-x_{i-1})/2, dvolume, volume.
 * The grid must be a Cartesian product grid (x_d depends on ix_d only). */
int vacgpu_set_grid(vacgpu_handle* h, const double* x);

/* Initial state w(ixM^S,1:nw) with its it and t (readfileini_bin,
 * src/vacio.t:682-755); ghost cells are filled as by the getboundary call
 * before the time loop (src/vac.t:54). */
int vacgpu_upload(vacgpu_handle* h, const double* w, int it, double t);

/* Current state w(ixM^S,1:nw) (what savefileout_bin writes,
 * src/vacio.t:1008-1047). */
int vacgpu_download(vacgpu_handle* h, double* w);

/* Asynchronous snapshots for VAC's save events (timetosave,
 * src/vac.t:56-58,631-661, which calls savefileout_bin,
 * src/vacio.t:1008-1047, and stops the run while it writes).
 * vacgpu_snapshot_begin enqueues a copy of the current state -- the state
 * after every step issued so far -- into snapshot slot `slot` (0 or 1) and
 * returns at once: the copy leaves the device on a copy stream of its own
 * while later vacgpu_step calls run.  vacgpu_snapshot_wait(h, slot, w)
 * waits for that copy and writes the snapshot to w in vacgpu_download's
 * layout, w(ixM^S,1:nw) (NULL w: no copy; vacgpu_snapshot_data gives the
 * snapshot in place).  A slot holds one
 * snapshot: a second begin on a pending slot is an error, as is a wait on
 * an empty one.  The caller keeps it and t of the snapshot (vacgpu_step
 * returns them).  The first begin of a slot allocates its device and
 * page-locked host buffers (8 bytes per mesh cell and variable each).
 * vacgpu_snapshot_wait may run on another host thread while this thread
 * calls vacgpu_step on the handle; no other call on the handle may run
 * concurrently with it. */
int vacgpu_snapshot_begin(vacgpu_handle* h, int slot);
int vacgpu_snapshot_wait(vacgpu_handle* h, int slot, double* w);
/* The page-locked host copy of slot's completed snapshot in
 * vacgpu_download's layout, valid from vacgpu_snapshot_wait until the next
 * vacgpu_snapshot_begin on that slot or vacgpu_destroy: a host that writes
 * the snapshot itself reads it there and saves the copy into its own array
 * (wait with w = NULL).  NULL (and the message) if the slot holds none. */
const double* vacgpu_snapshot_data(vacgpu_handle* h, int slot);

/* Advance: repeat the body of the time loop (src/vac.t:59-106) at most
 * maxsteps times.  Before each step the dt is chosen exactly as VAC does
 * (dtpar / getdt_courant / getdt_special / dtcantgrow / slowsteps /
 * tmaxexact) and the step is skipped and the call returns when
 * timetofinish (src/vac.t:608-628) holds or t >= tstop (the next save time
 * of the caller's timetosave).  dt, it and t stay on the device between
 * steps; *t, *it, *dt receive their values at return, *finished is set to 1
 * when timetofinish held.  The fused sweeps wait for their TMA copies with
 * a bounded wait (about 2^31 cycles); if one gives up, the tiles of that
 * sweep were not all written, the call fails with that message, the state
 * on the device is invalid, and every further vacgpu_step on the handle is
 * refused until vacgpu_upload gives it a new state. */
int vacgpu_step(vacgpu_handle* h, int maxsteps, double tstop, double* t,
                int* it, double* dt, int* finished);

/* Volume-averaged variables wmean(iw) = sum(dvolume*w)/volume over the mesh
 * in FP64 (savefilelog_default, src/vacio.t:1050-1105). */
int vacgpu_sums(vacgpu_handle* h, double* wmean);

/* Error counters nerror(1:4) (src/vacdef.t:54-55): toosmallp, toosmallr,
 * couranterr, poissonerr. */
int vacgpu_error_counts(vacgpu_handle* h, int* nerror);

/* specialbound (src/vacgrid.t:355-371; user routine
 * src/vacnul.specialbound.t:2-13): the ghost values of the variables whose
 * typeB is 'special'.  One region iB (0-based, 2*(idim-1)+upper) as the
 * hook sees it: its cells, the layout of the device state and the device
 * pointers the hook may read.  Element (gx,gy,gz) of variable iw is at
 * w[offset0 + gx*stride[0] + gy*stride[1] + gz*stride[2] + iw*var_stride]
 * (ghost-box coordinates, mesh cells 2..nx+1 in a used dimension). */
typedef struct vacgpu_region {
  int iB;                  /* region, 2*(idim-1)+upper                     */
  unsigned iw_mask;        /* bit iw set: variable iw is 'special' here    */
  int lo[3], hi[3];        /* the region's cells (inclusive)               */
  int nx[3];               /* mesh cells per dimension (1 if unused)       */
  int nG[3];               /* ghost-box extents                            */
  long long offset0;       /* element offset of ghost cell (0,0,0)         */
  long long stride[3];     /* element strides of the three dimensions      */
  long long var_stride;    /* element stride between variables             */
  int elem;                /* 8: double state (FP64), 4: float (mixed)     */
  const double* qt;        /* device: getboundary's time qt of this fill   */
                           /* (t; t+dt/2 after the predictor, t+dt after   */
                           /* the corrector, src/vac.t:567)                */
  const double* x[3];      /* device: cell centres along each dimension,   */
                           /* nG[d] values over the ghost box              */
} vacgpu_region;

/* The hook is called on the host while the engine issues a ghost fill --
 * also while it captures a CUDA graph -- once per region that has
 * 'special' variables, after the region's other variables are filled and
 * before the next region (getboundary's order).  It enqueues device work
 * on `stream` (a cudaStream_t) that writes the region's cells of the
 * variables in iw_mask, must not synchronise, and returns 0 (non-zero
 * fails the call that issued the fill). */
typedef int (*vacgpu_bound_fn)(void* user, void* w, const vacgpu_region* r,
                               void* stream);

/* Install the specialbound hook of the handle (NULL removes it).  A grid
 * with 'special' faces refuses to run without one ("Special boundary is
 * not defined", src/vacnul.specialbound.t:12). */
int vacgpu_register_bound(vacgpu_handle* h, vacgpu_bound_fn fn, void* user);

/* specialeta (src/vacphys.mhdres.t:26-30,127-129,271-273; eqpar(eta_) < 0):
 * the user's resistivity field.  The engine calls the hook on the host while
 * it issues a step (also under CUDA-graph capture) before each resistive
 * source evaluation -- the predictor's, from the state, and the
 * corrector's, from the predictor output -- and before the first step's dt
 * choice (getdt_res); the hook enqueues device work on `stream` that writes
 * eta, and gradeta for the compact form, on the cells of `box` (the mesh
 * and one layer around it in each used dimension).  Arrays share the
 * state's cell indexing (box.offset0, box.stride); box.qt points at the
 * time-loop t, box.iB is -1. */
typedef struct vacgpu_eta_args {
  vacgpu_region box;
  const void* w;            /* device: the state the source is evaluated on */
  const double* current[3]; /* device: J_1..J_3 on box (from idirmin on)    */
  int idirmin;              /* first J component set: 7-2*ndir              */
  double* eta;              /* device, out: eta on box                      */
  double* gradeta[3];       /* device, out (compactres, else NULL): d eta/dx_j */
} vacgpu_eta_args;
typedef int (*vacgpu_eta_fn)(void* user, const vacgpu_eta_args* e,
                             void* stream);

/* Install the specialeta hook (NULL removes it); a grid with
 * eqpar(eta_) < 0 refuses to run without one. */
int vacgpu_register_eta(vacgpu_handle* h, vacgpu_eta_fn fn, void* user);

/* Install a device source hook (specialsource + getdt_special,
 * src/vacnul.specialsource.t:9-71); VACGPU_SRC_NONE removes it. */
int vacgpu_register_source(vacgpu_handle* h, int source_id,
                           const double* params, int nparams);

/* specialsource (src/vac.t:575-605 calls it from addsource2; user routine
 * src/vacnul.specialsource.t:9-47): the user's source terms
 * w = w + qdt*S(wCT), added on the mesh cells of box before the physics
 * sources (resistivity, Powell's div B terms) of the same call.  The engine
 * calls the hook on the host while it issues a step (also while it captures
 * a CUDA graph) once per advect1 call: after the Hancock predictor (wCT = the
 * state, w = the predictor output, qtC = t) and after the corrector
 * (wCT = the predictor output, w = the new state, qtC = t+dt/2); onestep
 * schemes ('tvdlf1', 'tvdmu1') call it once with wCT = the state.  dt lives
 * on the device, so qdt, qtC and qt are device pointers the hook's kernels
 * read: *qdt = qdt*(idimmax-idimmin+1)/ndim of the call (src/vactvdlf.t:85,
 * 292), *box.qt = qt = t.  The hook enqueues device work on `stream` that
 * updates w on the cells of box (the arrays use box's indexing), must not
 * synchronise, and returns 0 (non-zero fails the call that issued it). */
typedef struct vacgpu_source_args {
  vacgpu_region box;       /* the mesh; box.qt: device pointer to qt        */
  const double* qdt;       /* device: the source's time step                */
  const double* qtC;       /* device: time of wCT                           */
  const void* wCT;         /* device: the time-centred state                */
  void* w;                 /* device, in/out: the state the source updates  */
  int nw, ndir;            /* variables: rho, m_1..m_ndir, e[, b_1..b_ndir] */
} vacgpu_source_args;
typedef int (*vacgpu_source_fn)(void* user, const vacgpu_source_args* s,
                                void* stream);

/* getdt_special (src/vac.t:66; user routine
 * src/vacnul.specialsource.t:50-71): the user's time-step limit.  Called
 * like the source hook, once per step before the step's dt is chosen
 * (unless dtpar > 0, when the step uses dtpar and the limit is not read);
 * it enqueues device work that stores its limit dt_mine in *dt (which the
 * engine sets to 1e99 before the call), and the step takes
 * dt = min(dt, dt_mine) after the CFL and resistive limits, as the
 * reference's "dt=min(dt,dt_mine)".  w: the state at the start of the
 * step on box (the mesh). */
typedef struct vacgpu_dtspecial_args {
  vacgpu_region box;
  const void* w;           /* device: the state                             */
  double* dt;              /* device, out: the user's dt limit              */
} vacgpu_dtspecial_args;
typedef int (*vacgpu_dtspecial_fn)(void* user, const vacgpu_dtspecial_args* a,
                                   void* stream);

/* Install the user's specialsource and getdt_special hooks (either may be
 * NULL; both NULL removes them).  They replace a built-in source of
 * vacgpu_register_source.  A grid with a source hook runs the split
 * predictor/corrector kernels (the hook reads the predictor output from
 * device memory). */
int vacgpu_register_source_fn(vacgpu_handle* h, vacgpu_source_fn src,
                              vacgpu_dtspecial_fn dt, void* user);

/* Run the handle's work on the caller's CUDA stream (a cudaStream_t passed
 * as void*; NULL returns to the handle's own stream).  No counterpart in the
 * reference (VAC has no device); it lets a host order the engine's kernels
 * with its own device work. */
int vacgpu_set_stream(vacgpu_handle* h, void* stream);

/* Kernel classes for vacgpu_kernel_stats. */
enum {
  VACGPU_K_PREDICT = 0, /* Hancock predictor (split kernels)              */
  VACGPU_K_CORRECT = 1, /* TVDLF corrector (split kernels)                */
  VACGPU_K_SWEEP = 2,   /* fused predictor+corrector sweep                */
  VACGPU_K_GHOST = 3,   /* ghost-cell fill                                */
  VACGPU_K_DT = 4,      /* cell-centred CFL / smallp passes               */
  VACGPU_K_CONTROL = 5, /* single-block time-loop kernels                 */
  VACGPU_K_NCLASS = 6
};

/* Device timing of the engine's kernels (no counterpart in the reference,
 * which times its advance loop with the host clock, src/vac.t:52,115).
 * enable=1 clears the statistics and brackets every following launch with
 * CUDA events on the handle's stream; enable=0 stops bracketing.  Launch
 * counts are kept whether or not timing is enabled. */
int vacgpu_timing(vacgpu_handle* h, int enable);

/* Launches of kernel class kclass since the last vacgpu_timing(h,1) (or
 * since creation) and, when timing was enabled, their summed device time in
 * milliseconds.  Synchronises the handle's stream. */
int vacgpu_kernel_stats(vacgpu_handle* h, int kclass, long long* launches,
                        double* ms);

/* ------------------------------------------------------------ batches --
 * Many independent grids of uneven sizes advanced together (each its own
 * VAC run: own state, dt, it, t).  No counterpart in the reference, which
 * advances one grid per process; the per-grid semantics are those of
 * vacgpu_step.  A batch runs the mixed-precision fused sweep: every grid
 * must have precision VACGPU_PREC_MIXED, dimsplit, ndir=ndim (2 or 3) and
 * share physics, method, limiters and itmax with the others; all grids
 * start from the same it. */
typedef struct vacgpu_batch vacgpu_batch;

/* n grids, params[i] for grid i (nx may differ). */
int vacgpu_batch_create(const vacgpu_params* params, int n,
                        vacgpu_batch** out);
/* vacgpu_set_grid / vacgpu_upload / vacgpu_download of grid i. */
int vacgpu_batch_set_grid(vacgpu_batch* b, int i, const double* x);
int vacgpu_batch_upload(vacgpu_batch* b, int i, const double* w, int it,
                        double t);
int vacgpu_batch_download(vacgpu_batch* b, int i, double* w);
/* Advance every grid by up to nsteps steps (vacgpu_step semantics per
 * grid).  The steps are captured once into a CUDA graph of batched launches
 * (persistent sweep kernels over the work list of all grids' tiles) and
 * replayed on later calls with the same nsteps and tstop, or, for 2-D
 * line-sweep batches where the tuner finds it faster, run as one
 * cooperative launch (itself captured and replayed) with grid-wide barriers
 * between the phases of each step.  The first call tunes the launch shape
 * (VACGPU_TUNE=0 skips tuning; VACGPU_ONELAUNCH=0 leaves the one-launch
 * form out of the trials, =1 takes it).  With 'xyyx' splitting every grid starts a
 * step with the sweep its own it selects: after a tstop that ended the
 * grids at different parities of it, 2-D batches continue correctly (one
 * launch, per-grid sweep order) and 3-D batches refuse the call. */
int vacgpu_batch_step(vacgpu_batch* b, int nsteps, double tstop);
/* t, it, dt and the finished flag of grid i. */
int vacgpu_batch_status(vacgpu_batch* b, int i, double* t, int* it,
                        double* dt, int* finished);
/* Run (or report) the launch-shape autotuner: persistent CTAs, work-list
 * order (0 round-robin over grids, 1 grid-major), rows per work item of the
 * 2-D line sweep (16, or -B for a guided list: items of B rows, then two
 * each of B/2, B/4 and B/8 rows per grid and strip at the end of the list,
 * B = 32 or 16; 0 for 3-D batches, which have one item shape), whether
 * the steps run as one cooperative launch (2-D line-sweep batches only;
 * ctas is then that launch's CTA count; 2 once a step call has captured
 * that launch into a CUDA graph, 1 otherwise, 0 for the graph of separate
 * launches) and the trial times
 * in ms of two steps, 24 doubles: per item shape, per CTA count (two
 * persistent counts, then one CTA per item), per order; then the one-launch
 * form per item shape and order (0 where not tried). */
int vacgpu_batch_tune(vacgpu_batch* b, int* ctas, int* order, int* rows, int* onelaunch,
                      double* ms);
void vacgpu_batch_destroy(vacgpu_batch* b);

/* ------------------------------------------------------------- server --
 * Continuous-batching request server (no counterpart in the reference).
 * A worker thread admits submitted solves in arrival order while their
 * device memory fits the HBM budget and fewer than max_active are running,
 * keeps each admitted solve's state on the device, and issues its steps in
 * chunks of steps_per_chunk (replayed CUDA graphs) on its own stream as
 * soon as its previous chunk finished, so the admitted solves overlap on
 * the GPU; a finished solve is copied back and its memory released for the
 * next one.  Each solve runs exactly as vacgpu_step would run it alone. */
typedef struct vacgpu_server vacgpu_server;

int vacgpu_server_create(double hbm_budget_bytes, int max_active,
                         int steps_per_chunk, vacgpu_server** out);
/* Queue a solve: grid x(ixM^S,1:ndim), state w(ixM^S,1:nw) at it=0, t=0,
 * advanced nsteps steps.  Thread safe; the inputs are copied. */
int vacgpu_server_submit(vacgpu_server* s, const vacgpu_params* p,
                         const double* x, const double* w, int nsteps,
                         long long* id);
/* 0: finished (state copied into w when w is not NULL, with its t, it and
 * the time from submission to result in seconds); 1: not finished after
 * waiting up to wait_s seconds; other nonzero: the solve failed. */
int vacgpu_server_result(vacgpu_server* s, long long id, double wait_s,
                         double* w, double* t, int* it, double* tts);
/* The time-to-solution of a finished solve split in two: queue_s from
 * submission to admission (waiting for a slot or for device memory),
 * service_s from admission (device allocation, upload, steps, download)
 * to the result.  0: finished; 1: not finished yet; other: error. */
int vacgpu_server_timing(vacgpu_server* s, long long id, double* queue_s,
                         double* service_s);
/* Queue length, running solves, finished solves, the largest number of
 * solves that ran at once, cell updates of finished solves and the time
 * from the first submission to the last completion. */
int vacgpu_server_stats(vacgpu_server* s, int* nqueued, int* nactive,
                        int* ndone, int* peak_active, double* cell_updates,
                        double* span_s);
void vacgpu_server_destroy(vacgpu_server* s);

/* Largest grid vacgpu_sweep_noalloc accepts, in cells including the ghost
 * layers (prod over the used dimensions of nx+4): 262144 cells, e.g. 508^2
 * in 2-D or 60^3 in 3-D.  Its scratch is two fixed 16 MiB FP64 device
 * arrays (8 variables: the predictor state and the corrector's face fluxes)
 * that every GPU which loads the library holds until exit. */
#define VACGPU_NOALLOC_MAX_GCELLS 262144

/* One dimensional sweep of the split twostep scheme in FP64 -- the Hancock
 * predictor over dt/2, the TVDLF corrector over dt, the unsplit sources of
 * both substeps and the ghost-cell fill of both results, exactly as one
 * advect(idim,idim) of vacgpu_step -- on device arrays the caller owns, and
 * without allocating device memory.  No counterpart in the reference (VAC
 * has no device and allocates nothing on one).
 *
 * It exists for callers that cannot call cudaMalloc: hosts that record the
 * call into their own CUDA graph or stream capture (where an allocation is
 * not allowed), hosts that own all device memory through their own pool,
 * and latency-bound loops where cudaMalloc/cudaFree would synchronise the
 * device.  The predictor's intermediate state and the CFL reduction slots
 * live in a static device array of the library instead; the caller passes
 * inputs and outputs.
 *
 *  p           run parameters (dimsplit, typelimited original or predictor,
 *              precision FP64; smallp >= 0 must be given, dtpar unused)
 *  w, wout     device FP64 arrays in VAC's full-grid layout w(ixG^T,nw),
 *              column-major, nx+4 cells per used dimension; w must hold
 *              valid ghost cells; wout receives mesh and ghost cells
 *              (w and wout must not overlap)
 *  dx0,dx1,dx2 device FP64 arrays of dx along each used dimension over the
 *              ghost-extended range (nx+4 values; what vacgpu_set_grid
 *              derives with gridsetup1); unused dimensions may be NULL
 *  dt          the time step (qdt of the corrector)
 *  idim        sweep direction, 0-based
 *  courantmax  device pointer (or NULL) receiving the corrector's
 *              max cmax*2/(dx_i+dx_i+1) over the faces of this sweep, the
 *              value VAC folds into dtcourant(idim) (src/vactvdlf.t:184-201)
 *  stream      cudaStream_t as void* (NULL = legacy default stream)
 *
 * The first call on a device resolves the scratch array's device address
 * (cudaGetSymbolAddress) for that device, with that device current; make
 * that first call before any stream capture.  Every call shares the one
 * scratch array, so calls that overlap on the GPU (different streams or
 * host threads) race: serialise them.  Grids larger than
 * VACGPU_NOALLOC_MAX_GCELLS are rejected with an error. */
int vacgpu_sweep_noalloc(const vacgpu_params* p, const double* w,
                         double* wout, const double* dx0, const double* dx1,
                         const double* dx2, double dt, int idim,
                         double* courantmax, void* stream);

/* Release the handle and its device memory. */
void vacgpu_destroy(vacgpu_handle* h);

/* Copy the calling thread's last error message into buf (NUL terminated);
 * returns its full length. */
int vacgpu_last_error(char* buf, int len);

/* Library version string. */
const char* vacgpu_version(void);

/* Diagnostic (no counterpart in the reference): the FP64 throughput of this
 * GPU's FP64 pipe, measured by timing a kernel of independent FP64
 * fused multiply-add chains on every SM with CUDA events on the given
 * stream (NULL: legacy default stream).  *flops_per_s receives 2 x DFMA/s.
 * The denominator of the plain FP64 path's FP64-pipe roofline. */
int vacgpu_measure_fp64_peak(double* flops_per_s, void* stream);

/* Diagnostic (no counterpart in the reference): runs out, on purpose, the
 * two kinds of bounded device wait the kernels use, each with a limit of
 * about 2^22 cycles: an mbarrier phase that no copy completes (the TMA
 * waits of the sweeps) and a grid-wide barrier that one CTA of a
 * cooperative launch never reaches (the one-launch batched step).
 * *mbar_timed_out and *grid_timed_out receive 1 when the wait gave up and
 * reported it, as designed; the context stays usable.  Nothing faults. */
int vacgpu_test_bounded_waits(int* mbar_timed_out, int* grid_timed_out);

#ifdef __cplusplus
}
#endif
#endif /* VACGPU_H */
