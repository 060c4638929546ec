/*
 * nhwave_gb300.h -- C-ABI of the GB300 (sm_103a) implementation of NHWAVE's
 * time-step hot path.
 *
 * Every entry point uses plain C types (no CUDA or torch types), returns an
 * int status (NHW_OK == 0) and never keeps a host pointer after it returns.
 * Host arrays use the reference's own memory layout: Fortran column-major
 * order over the ghosted local extents of module GLOBAL
 * (src/mod_global.F:212-243), i.e. element (i,j,k) with 1-based Fortran
 * indices sits at offset (i-1) + Mloc*((j-1) + Nloc*(k-1)), with
 *   Mloc = Mglob+4, Nloc = Nglob+4, Kloc = Kglob+4        (Nghost = 2)
 * and face arrays one longer in their face direction (Mloc1 = Mloc+1 ...),
 * exactly as allocated in src/initialize.F:1423-1643.
 *
 * The entry points replace, one for one, the argument-less subroutines that
 * program NHWAVE calls inside its time loop (src/nhwave.F:119-258):
 *
 *   nhw_estimate_dt        <- estimate_dt          src/nhwave.F:3694-3874
 *   nhw_update_bathymetry  <- update_bathymetry    src/nhwave.F:5755-6071 (RIGID_3D)
 *   nhw_update_wave_bc     <- update_wave_bc       src/nhwave.F:5514-5565 (the generators of enum nhw_wavemaker)
 *   nhw_update_mask        <- update_mask          src/nhwave.F:5403-5456
 *   nhw_update_vars        <- update_vars          src/nhwave.F:5459-5511
 *   nhw_source_terms       <- source_terms         src/source_terms.F:1-455 (internal makers + bed slope)
 *   nhw_fluxes             <- fluxes               src/nhwave.F:1686-1714
 *   nhw_eval_duvw          <- eval_duvw(ISTEP)     src/nhwave.F:539-1300 (inviscid path,
 *                             incl. poisson_solver src/pressure.F:63-245 and
 *                             generate_coef_rhs src/pressure.F:475-840)
 *   nhw_sponge_damping     <- sponge_damping       src/nhwave.F:6463-6502
 *   nhw_eval_turb          <- eval_turb(ISTEP)     src/nhwave.F:6544-6782 (IVTURB 1, 2, 3 with
 *                             kepsilon :11117-11524, 10 with kepsilon_3D :10030-11114,
 *                             20 with les_3D :8545-8729, 30 with les_dyn :7989-8542;
 *                             IHTURB 1, 2, >= 10;
 *                             viscous flow only, a no-op otherwise)
 *   nhw_step               <- one pass of the do-while body src/nhwave.F:119-258
 *   nhw_mass               <- statistics' MassVolume  src/nhwave.F:3139-3148
 *   nhw_statistics         <- statistics               src/nhwave.F:3118-3160
 *
 * Set-up (the work of read_bathymetry src/initialize.F:1734-2175, generate_grid
 * src/initialize.F:1647-1729 and initial src/initialize.F:2502-3408) is offered
 * by nhw_setup for callers without the Fortran driver; a Fortran driver that
 * runs its own set-up hands its arrays over with nhw_set_field instead.
 */
#ifndef NHWAVE_GB300_H
#define NHWAVE_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum nhw_status {
  NHW_OK = 0,
  NHW_ERR_ARG = 1,           /* null pointer, bad size or bad field id            */
  NHW_ERR_UNSUPPORTED = 2,   /* option outside this path (viscous, open BC)       */
  NHW_ERR_CUDA = 3,          /* CUDA runtime error (message: nhw_last_error)      */
  NHW_ERR_NOMEM = 4,         /* device allocation failed                          */
  NHW_ERR_DT_MIN = 5,        /* dt < DT_MIN: the reference stops here             */
  NHW_ERR_KRYLOV_NOCONV = 6, /* Poisson solve reached ITMAX above TOL             */
  NHW_ERR_NAN = 7,           /* non-finite value in the Poisson residual          */
  NHW_ERR_TIMEOUT = 8,       /* a bounded device wait gave up                     */
  NHW_ERR_STATE = 9,         /* call out of order (e.g. step before set-up)       */
  NHW_ERR_CAPACITY = 10,     /* serving: HBM budget or slot table exhausted       */
  NHW_ERR_NOT_FOUND = 11     /* serving: unknown request id                       */
};

/* arithmetic form of the state arrays */
enum nhw_precision {
  NHW_FP64 = 0,     /* plain FP64 drop-in: every array and the Krylov solve in FP64   */
  NHW_FP32_IR = 1   /* FP32 3-D state, fluxes and Krylov inner iterations; FP64 2-D
                       depth/eta/mask fields, FP64 Poisson residual + refinement     */
};

/* INT_*: internal source strip (src/source_terms.F); LEF_*, WAV_CUR and
 * FOCUSED: waves fed through the west boundary, which then needs BC_X0 = 3:
 * linear, solitary, second-order Stokes, cnoidal, linear on a current ramped
 * up over TRAMP, a focused group of NWAVE linear components, and the S2 tide
 * (src/waves.F:92-170, 518-560, 638-756, 808-903; src/nhwave.F:5715-5750).
 * RIG_LIN: a linear wave fed through the east boundary, which then needs
 * BC_Xn = 3 (src/waves.F:762-803).  FLUX_LR: a log-profile current in through
 * the west side (BC_X0 = 3) and out through the east side (BC_Xn = 3) at the
 * same volume flux, with the east values radiated as in the Orlanski
 * condition (flux_left_right_boundary, src/nhwave.F:5566-5712; it uses Zob
 * and TRAMP).  LEF_JON / LEF_TMA: irregular waves through the west side
 * (BC_X0 = 3), NUMFREQ linear components of a JONSWAP spectrum (TMA: times
 * the finite-depth factor) of significant height HM0 and peak period TP
 * (src/initialize.F:880-941, src/waves.F:566-623).  LEF_SPC: irregular,
 * directional waves through the west side from a 2-D spectrum the driver
 * passes with nhw_set_wave_spectrum (the reference reads it from spc2d.txt,
 * src/initialize.F:782-830; src/waves.F:376-513).  INT_CON, INT_JON, INT_TMA,
 * INT_SPC, INT_IRR: the internal source strip fed by a cnoidal wave, by the
 * JONSWAP / TMA components of LEF_JON / LEF_TMA, by a 2-D spectrum of
 * densities (spc2d.txt) or by one of component amplitudes with their phases
 * (irr2d.txt), both passed with nhw_set_wave_spectrum (src/source_terms.F:
 * 71-340; src/initialize.F:835-876) */
enum nhw_wavemaker { NHW_WM_NONE = 0, NHW_WM_INT_LIN = 1, NHW_WM_INT_SOL = 2, NHW_WM_LEF_LIN = 3,
                     NHW_WM_LEF_SOL = 4, NHW_WM_LEF_STK = 5, NHW_WM_LEF_CON = 6, NHW_WM_WAV_CUR = 7,
                     NHW_WM_FOCUSED = 8, NHW_WM_LEF_TID = 9, NHW_WM_RIG_LIN = 10, NHW_WM_FLUX_LR = 11,
                     NHW_WM_LEF_JON = 12, NHW_WM_LEF_TMA = 13, NHW_WM_LEF_SPC = 14, NHW_WM_INT_CON = 15,
                     NHW_WM_INT_JON = 16, NHW_WM_INT_TMA = 17, NHW_WM_INT_SPC = 18, NHW_WM_INT_IRR = 19 };
enum nhw_slide     { NHW_SLIDE_NONE = 0, NHW_SLIDE_RIGID_3D = 1 };
enum nhw_depth_type { NHW_DEPTH_CELL_CENTER = 0, NHW_DEPTH_CELL_GRID = 1 };

/*
 * Run-time parameters: the input.txt keys that the path reads
 * (src/initialize.F:141-1321), parsed to double exactly as Get_Float_Val
 * does (src/mod_util.F:138).  Names follow the input.txt keys.
 */
typedef struct nhw_params {
  int32_t Mglob, Nglob, Kglob;             /* Mglob Nglob Kglob                       */
  double  dx, dy;                          /* DX DY                                   */
  int32_t ivgrd;  double grd_r;            /* IVGRD GRD_R                             */
  double  dt_ini, dt_min, dt_max;          /* DT_INI DT_MIN DT_MAX                    */
  double  total_time; int32_t sim_steps;   /* TOTAL_TIME SIM_STEPS                    */
  double  cfl;                             /* CFL                                     */
  int32_t froude_cap_on; double froude_cap;/* -DFROUDE_CAP build flag, FROUDE_CAP     */
  double  min_dep;                         /* MinDep                                  */
  int32_t non_hydro;                       /* NON_HYDRO                               */
  int32_t time_order;                      /* 1,2,3 <- TIME_ORDER FIRST/SECOND/THIRD  */
  int32_t hllc;                            /* HLLC: 1 HLLC face fluxes, 0 HLL          */
  int32_t viscous_flow;                    /* VISCOUS_FLOW: 1 needs IVTURB = IHTURB = 1
                                              (constant eddy viscosities)             */
  int32_t barotropic;                      /* BAROTROPIC; 0 runs the same path: the
                                              density is Rho0 everywhere (no salinity,
                                              temperature, sediment or bubbles), so the
                                              baroclinic gradient is zero            */
  int32_t itmax; double tol;               /* ITMAX TOL                               */
  int32_t bc_x0, bc_xn, bc_y0, bc_yn;      /* BC_X0 BC_Xn BC_Y0 BC_Yn: 1 free-slip wall,
                                              2 no-slip wall, 5 wall friction; BC_X0 = 3
                                              inflow with a LEF_* wavemaker or FLUX_LR;
                                              BC_Xn = 3 inflow/outflow with RIG_LIN or
                                              FLUX_LR; BC_Xn = 6 Orlanski radiation
                                              (open east side)                        */
  int32_t bc_z0;                           /* BC_Z0: 1 free-slip bed, 2 no-slip,
                                              5 friction law (Ibot, Cd0, Zob)          */
  double  visc;                            /* VISCOSITY (initial Cmu)                 */
  double  slat;                            /* slat -> fcor                            */
  double  wind_u, wind_v;                  /* WindU WindV (Iws = 1)                   */
  int32_t depth_type;                      /* DEPTH_TYPE                              */
  int32_t wavemaker;                       /* WAVEMAKER                               */
  double  amp_wave, per_wave, dep_wave, theta_wave, cur_wave; /* AMP PER DEP THETA CUR */
  double  xsource_west, xsource_east, ysource_suth, ysource_nrth;
  int32_t sponge_on;                       /* SPONGE_ON                               */
  double  sponge_west_width, sponge_east_width, sponge_south_width, sponge_north_width;
  double  tramp;                           /* TRAMP                                   */
  int32_t slide_type;                      /* SlideType (-DLANDSLIDE build)            */
  double  slide_t, slide_l, slide_w, slide_angle, slope_angle, slide_x0, slide_y0;
  double  slide_ut, slide_a0;              /* SlideUt SlideA0                         */
  int32_t precision;                       /* enum nhw_precision                      */
  int32_t device;                          /* CUDA device ordinal of the handle       */
  int32_t precond;                         /* Poisson preconditioner: 0 multigrid V-cycle,
                                              1 vertical-line (tridiagonal) only     */
  float   mg_weight;                       /* multigrid coarse-correction weight (0: 1.0) */
  int32_t krylov_kernel;                   /* inner Krylov solver of the pressure solve:
                                              0: BiCGSTAB, one launch per phase, loops
                                              in graph conditional nodes (fastest);
                                              1: BiCGSTAB, the whole solve in one
                                              persistent cooperative launch;
                                              2: GMRES as in the reference's HYPRE
                                              path (cycles of up to 16 iterations,
                                              one V-cycle each), one launch per phase.
                                              1 and 2 need the multigrid preconditioner;
                                              without it BiCGSTAB runs phase by phase */
  int32_t mg_coarse_sweeps;                /* red-black sweeps on the coarsest level (0: 2) */
  int32_t mg_cta_columns;                  /* levels with at most this many columns run in
                                              one thread block (0: 64)                */
  int32_t mg_aggregate;                    /* multigrid aggregates of n x n columns (0: 2) */
  int32_t test_barrier_extra;              /* test hook, 0 in use: the persistent solve's
                                              grid barrier also waits for this many blocks
                                              that do not exist, so its bounded wait runs
                                              out and the solve reports NHW_ERR_TIMEOUT */
  /* viscous flow (read when viscous_flow = 1; src/initialize.F:357, 385-392) */
  int32_t ivturb, ihturb;                  /* IVTURB IHTURB: 1 constant viscosity,
                                              2 subgrid model; IVTURB 3 / 10 2-D /
                                              3-D k-epsilon, 20 / 30 Smagorinsky /
                                              dynamic LES; IHTURB
                                              >= 10 takes CmuHt = CmuVt                */
  int32_t rng;                             /* RNG: seeding viscosity of the first stage */
  double  cvs, chs;                        /* Cvs Chs: vertical / horizontal eddy
                                              viscosity of IVTURB = 1 / IHTURB = 1, the
                                              subgrid models' coefficients with 2; Cvs
                                              the Smagorinsky constant of IVTURB = 20 */
  double  schmidt;                         /* Schmidt                                 */
  double  viscous_number;                  /* VISCOUS_NUMBER: dt limit of the explicit
                                              horizontal viscous terms                */
  /* bed friction of BC_Z0 = 5 (src/initialize.F:466-468) */
  int32_t ibot;                            /* Ibot: 1 drag coefficient Cd0, 2 roughness Zob */
  double  cd0, zob;                        /* Cd0 Zob                                 */
  /* FOCUSED wave group (src/initialize.F:709-781): NWAVE >= 2 components of
     frequencies spread over normalized_delta_f around f_center, focusing at
     x_breaking, t_breaking; amplitude Slope_group/NWAVE/k (k_center when
     Component_Amp_Type = 1); depth_comp; sd_return (read with AMP for the
     LEF_ / WAV_ makers only, so 0 for FOCUSED inputs) */
  int32_t nwave, component_amp_type;
  double  k_center, f_center, x_breaking, t_breaking, slope_group, normalized_delta_f, depth_comp;
  double  sd_return;
  /* JONSWAP / TMA spectrum of LEF_JON / LEF_TMA (src/initialize.F:880-941):
     significant height Hm0, peak period Tp, NumFreq components at the
     centres of NumFreq equal bands over [Freq_Min, Freq_Max] (NumFreq <= 500,
     the reference's MaxNumFreq).  The reference draws each component's phase
     with the compiler's rand(); here they come from wave_seed (a SplitMix64
     stream: phase_i = 2 pi u_i) unless nhw_set_wave_phases gives them. */
  double  hm0, tp, freq_min, freq_max;
  int32_t numfreq, wave_seed;
  /* k-epsilon closure of IVTURB = 10 (src/initialize.F:388): PRODTYPE 1
     production from the vertical shear of U and V, 2 from the vertical
     shear, otherwise (3 in every example input) the full 3-D production */
  int32_t prod_type;
} nhw_params;

/* Scalars the driver reads back after a step (module GLOBAL scalars). */
typedef struct nhw_scalars {
  double  time;          /* TIME                                          */
  double  dt;            /* dt                                            */
  double  dt_old;        /* dt_old                                        */
  int32_t run_step;      /* RUN_STEP                                      */
  int32_t last_krylov_iters;   /* inner iterations of the last Poisson solve */
  int64_t total_krylov_iters;  /* since set-up                              */
  int64_t poisson_solves;      /* since set-up                              */
  double  last_rel_residual;   /* FP64 ||b-Ax||/||b|| of the last solve     */
  int32_t last_refinements;    /* FP64 refinement sweeps of the last solve  */
  int32_t status;              /* sticky device status (enum nhw_status)    */
} nhw_scalars;

/* Field ids for nhw_get_field / nhw_set_field.  Shapes are the reference's
 * ghosted allocations; integer fields are int32, all others double. */
enum nhw_field {
  /* 2-D cell (Mloc,Nloc) */
  NHW_F_D = 0, NHW_F_D0, NHW_F_ETA, NHW_F_ETA0, NHW_F_HC, NHW_F_HC0,
  NHW_F_DELXH, NHW_F_DELYH, NHW_F_DELXETA, NHW_F_DELYETA, NHW_F_DELTH, NHW_F_DELT2H,
  NHW_F_SOURCEX, NHW_F_SOURCEY, NHW_F_SOURCEC, NHW_F_SPONGE, NHW_F_R1,
  /* 2-D x faces (Mloc1,Nloc) */
  NHW_F_HFX, NHW_F_HFX0, NHW_F_ETAXL, NHW_F_ETAXR,
  /* 2-D y faces (Mloc,Nloc1) */
  NHW_F_HFY, NHW_F_HFY0, NHW_F_ETAYL, NHW_F_ETAYR,
  /* 2-D int (Mloc,Nloc) */
  NHW_F_MASK, NHW_F_MASK_STRUCT, NHW_F_MASK9,
  /* 3-D cell (Mloc,Nloc,Kloc) */
  NHW_F_U, NHW_F_V, NHW_F_W, NHW_F_DU, NHW_F_DV, NHW_F_DW,
  NHW_F_DU0, NHW_F_DV0, NHW_F_DW0, NHW_F_P,
  /* 3-D z faces (Mloc,Nloc,Kloc1) */
  NHW_F_OMEGA,
  /* 3-D x faces (Mloc1,Nloc,Kloc) */
  NHW_F_EX, NHW_F_FX, NHW_F_GX, NHW_F_HX,
  /* 3-D y faces (Mloc,Nloc1,Kloc) */
  NHW_F_EY, NHW_F_FY, NHW_F_GY, NHW_F_HY,
  /* 3-D z faces (Mloc,Nloc,Kloc1) */
  NHW_F_FZ, NHW_F_GZ, NHW_F_HZ,
  /* 3-D cell (Mloc,Nloc,Kloc): eddy viscosities of eval_turb (viscous flow only) */
  NHW_F_CMUVT, NHW_F_CMUHT,
  /* 3-D cell (Mloc,Nloc,Kloc): k-epsilon state (viscous flow only) */
  NHW_F_TKE, NHW_F_EPS, NHW_F_DTKE, NHW_F_DEPS,
  NHW_F_COUNT
};

typedef struct nhw_handle nhw_handle;

/* ------------------------------------------------------------- lifecycle */
/* Validate parameters, size and allocate the device state (index +
 * allocate_variables, src/initialize.F:1339-1643).  One CUDA stream per
 * handle; one host thread per handle. */
int nhw_create(const nhw_params* params, nhw_handle** out);
int nhw_destroy(nhw_handle* h);
/* Device memory (bytes) a handle created with these parameters holds, found
 * without allocating: the admission test of a memory-budgeted request loop.
 * Needs the CUDA device (kernel occupancy is part of the plan). */
int nhw_device_bytes(const nhw_params* params, int64_t* bytes);

/* Set-up without the Fortran driver: generate_grid + read_bathymetry (from
 * `depth`, Mglob x Nglob for CELL_CENTER, (Mglob+1) x (Nglob+1) for
 * CELL_GRID, i fastest, as the rows of depth.txt) + initial (eta0/uvw0 may be
 * NULL for a state at rest; uvw0 holds U, V then W, each Mglob x Nglob x
 * Kglob with i fastest, as uvw0.txt).  src/initialize.F:1647-2175, 2502-3408 */
int nhw_setup(nhw_handle* h, const double* depth, const double* eta0, const double* uvw0);

/* Copy one whole ghosted field between host and device (Fortran layout). */
int nhw_get_field(nhw_handle* h, int field, void* host);
int nhw_set_field(nhw_handle* h, int field, const void* host);
/* Shape of a field: dims[0..2] (dims[2] == 1 for 2-D), elem_bytes. */
int nhw_field_shape(const nhw_handle* h, int field, int32_t dims[3], int32_t* elem_bytes);

int nhw_get_scalars(nhw_handle* h, nhw_scalars* out);
int nhw_set_time(nhw_handle* h, double time, double dt, int32_t run_step);
/* Phases (radians) of the n = NumFreq components of a JONSWAP / TMA maker, in
 * place of the ones drawn from wave_seed: the reference's RanPhs
 * (src/initialize.F:937-940), for a driver that wants its own draw.  Call
 * it after nhw_setup (which sets the seeded phases); they apply from the
 * next update_wave_bc (LEF_) or source_terms (INT_).  NHW_ERR_ARG unless
 * the handle runs LEF_JON, LEF_TMA, INT_JON or INT_TMA with n components. */
int nhw_set_wave_phases(nhw_handle* h, int32_t n, const double* phases);
/* The 2-D spectrum of LEF_SPC, as the reference reads it from spc2d.txt
 * (src/initialize.F:783-830): numfreq >= 2 frequencies freq[] (Hz), numdir >= 2
 * directions dire[] (degrees from the x axis), and the spectral densities
 * spc2d[] and phases[] (radians) laid out as the Fortran arrays
 * Wave_Spc2d(NumDir, NumFreq) and Random_Phs(NumDir, NumFreq), direction
 * fastest, numfreq * numdir <= 12,000.  phases may be NULL: they are then drawn from
 * wave_seed (the reference draws them with the compiler's rand()).  Call it
 * after nhw_create and before the first step; the library copies the data.
 * A checkpoint does not hold the spectrum: after nhw_load_state pass it
 * again.  INT_SPC takes the same data; INT_IRR takes component amplitudes
 * in spc2d[] (the reference's irr2d.txt, src/initialize.F:835-876) and its
 * phases, which are then required.  The internal makers snap each direction
 * to the nearest one that the channel width repeats (src/source_terms.F:
 * 94-136), which needs |direction| <= 90 degrees.  NHW_ERR_ARG unless the
 * handle runs LEF_SPC, INT_SPC or INT_IRR. */
int nhw_set_wave_spectrum(nhw_handle* h, int32_t numfreq, int32_t numdir, const double* freq,
                          const double* dire, const double* spc2d, const double* phases);

/* ------------------------------------------- the reference's subroutines */
int nhw_estimate_dt(nhw_handle* h);
int nhw_update_bathymetry(nhw_handle* h);
int nhw_update_wave_bc(nhw_handle* h);
int nhw_update_mask(nhw_handle* h);
int nhw_update_vars(nhw_handle* h);
int nhw_source_terms(nhw_handle* h);
int nhw_fluxes(nhw_handle* h);
int nhw_eval_duvw(nhw_handle* h, int32_t istep);
int nhw_sponge_damping(nhw_handle* h);
int nhw_eval_turb(nhw_handle* h, int32_t istep);

/* One full time step (estimate_dt ... last RK stage).  The first call
 * captures the step into a CUDA graph whose pressure-solve loops run on the
 * device (conditional nodes); later calls replay it, with one host round trip
 * per call.  Returns the step's first non-OK pressure status, or DT_MIN.
 * Writes TIME, dt and RUN_STEP if non-NULL. */
int nhw_step(nhw_handle* h, double* time, double* dt, int32_t* run_step);
/* Up to nsteps steps while TIME < TOTAL_TIME and RUN_STEP < SIM_STEPS (the
 * reference's do-while condition, src/nhwave.F:119).  The test runs on the
 * device in a gated copy of the step graph, so steps go out in batches
 * without a host round trip each.  Stops at DT_MIN or at a step whose
 * pressure solve went non-finite; ITMAX without convergence does not stop
 * it.  *steps_done counts the steps taken (plus the one that hit DT_MIN). */
int nhw_run(nhw_handle* h, int32_t nsteps, int32_t* steps_done);

/* Checkpoint / resume.  The reference's hot start rereads f15.6 text files
 * written at output intervals (src/nhwave.F:3513-3690), which loses bits;
 * these three calls save and restore a scenario's complete state instead, so
 * a resumed run continues bit for bit: every array a step reads before it
 * writes it (grids, 2-D fields, masks, 3-D fields, P) and the device scalars
 * (TIME, dt, RUN_STEP, solver counters).  The buffer is host memory of
 * nhw_checkpoint_bytes bytes.  nhw_load_state needs a handle created with the
 * same parameters and set up from the same inputs (nhw_setup), as the
 * reference's hot start rereads input.txt and the depth file; a checkpoint of
 * another grid, precision or library build is rejected with NHW_ERR_ARG. */
int nhw_checkpoint_bytes(nhw_handle* h, int64_t* bytes);
int nhw_save_state(nhw_handle* h, void* host, int64_t bytes);
int nhw_load_state(nhw_handle* h, const void* host, int64_t bytes);

/* FP64 device reduction of statistics' MassVolume = sum(D*dx*dy). */
int nhw_mass(nhw_handle* h, double* mass);

/* The figures statistics prints (src/nhwave.F:3118-3160) over the interior,
 * reduced on the device in FP64: MassVolume = sum D dx dy; Energy = sum over
 * cells of CellMass (g (D sigc_k - Hc) + |u|^2 / 2), CellMass =
 * Rho0 dsig_k D dx dy (potential energy measured from z = 0); MaxEta, MinEta;
 * the largest |U|, |V|, |W|.  The sums are taken in a fixed block order, not
 * the reference's loop order. */
typedef struct nhw_stats {
  double mass_volume, energy, max_eta, min_eta, max_u, max_v, max_w;
} nhw_stats;
int nhw_statistics(nhw_handle* h, nhw_stats* out);

/* Wait for the handle's stream. */
int nhw_synchronize(nhw_handle* h);

/* Run nsteps full steps (no TOTAL_TIME / SIM_STEPS test) and report the
 * device time of the whole sequence, from CUDA events recorded on the
 * handle's stream before the first and after the last kernel. */
int nhw_run_timed(nhw_handle* h, int32_t nsteps, double* device_ms);

/* Per-kernel timing with CUDA events on the handle's stream (on = 1 starts a
 * fresh record, 0 stops).  The report lists, one line per kernel,
 * "name launches total_ms", plus a first line "launches N" counting every
 * kernel the handle launched since set-up (counted whether or not timing is
 * on).  Returns the bytes written (without the terminating NUL). */
int nhw_profile(nhw_handle* h, int32_t on);
int nhw_profile_report(nhw_handle* h, char* buf, int32_t buflen);

/* Device microseconds of one level-0 multigrid half-sweep, the largest
 * kernel of a non-hydrostatic step, on this handle's current operator (call
 * it after a step).  Events around single launches add several microseconds
 * to each, so the launches are timed in bulk: a CUDA graph of `reps` rounds,
 * each a write of `flush_bytes` bytes (0: none; more than the 129 MB L2
 * evicts it) followed by the four level-0 half-sweeps of a V-cycle, minus a
 * graph of the writes alone.  Overwrites a preconditioner scratch vector,
 * no state.  NHW_ERR_STATE for a hydrostatic handle or one not set up. */
int nhw_time_smoother(nhw_handle* h, int32_t reps, int64_t flush_bytes, double* us_per_launch);

/* sizeof(nhw_params) and sizeof(nhw_scalars) as compiled into the library,
 * for bindings to check their struct images (no GPU needed). */
int nhw_abi_sizes(int32_t* params_bytes, int32_t* scalars_bytes);

/* Human-readable text of a status code, and the last CUDA error text. */
const char* nhw_status_string(int status);
const char* nhw_last_error(void);

/* --------------------------------------------------------------- ensembles
 * Many scenarios advanced together.  The reference runs one scenario per
 * program; an ensemble takes set-up handles (same device, precision,
 * TIME_ORDER and NON_HYDRO; the multigrid preconditioner) and advances all of
 * them one step per CUDA graph launch: every member's step kernels on a
 * branch of their own, and per RK stage the pressure solves of all members in
 * one persistent cooperative launch (more than one when the members need more
 * blocks than the GPU holds at once).  A member whose run is over (TIME >=
 * TOTAL_TIME or RUN_STEP >= SIM_STEPS) or that stopped at DT_MIN is skipped
 * on the device.  A member's results do not depend on the other members.
 * Members stay owned by the caller: destroy the ensemble before them, and do
 * not step a member on its own while it belongs to a live ensemble. */
typedef struct nhw_ensemble nhw_ensemble;
typedef struct nhw_ensemble_opts {
  int32_t cells_per_block;   /* unknowns per block of a member's solve (0: 16384)  */
  int32_t block_rows;        /* solve blocks are 32 x block_rows threads: 8 or 16  */
  int32_t coarse_sweeps;     /* red-black sweeps on the coarsest level (0: 2)      */
  int32_t solver;            /* 0: every member's phase-by-phase solve on its own
                                branch, loops in conditional nodes; 1: the solves
                                of all members as groups of persistent launches */
  int32_t reserved[4];
} nhw_ensemble_opts;
typedef struct nhw_ensemble_info {
  int32_t members;
  int32_t solve_launches_per_stage;   /* persistent-solve launches per RK stage  */
  int32_t blocks_per_launch;          /* blocks of the largest of them           */
  int32_t max_resident_blocks;        /* blocks the GPU holds at once            */
  int64_t kernels_per_step;           /* kernel launches of a step outside the
                                         members' own solver loops               */
  int64_t cells;                      /* interior cells over all members         */
  nhw_ensemble_opts opts;             /* settings in use                         */
  int64_t kernels_launched;           /* all kernel launches so far, loops
                                         counted from the device's counters      */
} nhw_ensemble_info;

int nhw_ensemble_create(nhw_handle* const* members, int32_t n, const nhw_ensemble_opts* opts,
                        nhw_ensemble** out);
/* nsteps ensemble steps; returns the worst member status (DT_MIN, NAN, TIMEOUT) */
int nhw_ensemble_step(nhw_ensemble* e, int32_t nsteps);
/* nsteps ensemble steps timed with CUDA events on the ensemble's stream */
int nhw_ensemble_run_timed(nhw_ensemble* e, int32_t nsteps, double* device_ms);
/* Autotuner: times candidate settings (solver form, cells per block, block
 * height, coarse sweeps) on real ensemble steps -- the members advance by steps_per_trial
 * steps per candidate -- and keeps the fastest; writes it to *chosen. */
int nhw_ensemble_tune(nhw_ensemble* e, int32_t steps_per_trial, nhw_ensemble_opts* chosen);
int nhw_ensemble_get_info(nhw_ensemble* e, nhw_ensemble_info* out);
int nhw_ensemble_destroy(nhw_ensemble* e);

/* ------------------------------------------------ allocation-free variant
 * No counterpart in the reference: an addition for callers that cannot let a
 * library allocate device memory.  Such a caller -- a host model whose fields
 * live in device memory owned by the OpenACC / CUDA Fortran runtime or by a
 * framework's caching allocator -- cannot use nhw_create, which allocates a
 * scenario arena, because cudaMalloc and cudaFree synchronise the device
 * (stalling its other streams) and draw on a memory budget it fixes up front.
 *
 * nhw_estimate_dt_noalloc computes what nhw_estimate_dt computes, the new
 * time step dt = min(1.05 dt_old, CFL * Courant bound, DT_MAX), on the
 * caller's device arrays, and writes it to dt_out[0] (device memory) on
 * `stream` (a cudaStream_t; NULL = the default stream).  It returns once the
 * work is queued.  U, V, W are (Mglob+4, Nglob+4, Kglob+4), D is
 * (Mglob+4, Nglob+4) and dsig (Kglob+4), all FP64 in the reference's ghosted
 * Fortran layout (column-major, two ghost cells a side).  Every array must be
 * device memory of the current device, or managed memory; host memory and
 * another GPU's memory are refused with NHW_ERR_ARG.  A NaN candidate is
 * skipped, as the reference's `if (x < tmp2) tmp2 = x` skips it.  The caller checks
 * dt against DT_MIN.  A viscous run (VISCOUS_FLOW) also takes the minimum
 * with VISCOUS_NUMBER * min(dx^2, dy^2) / (|CmuHt| + 1e-16), which this call
 * leaves to the caller (src/nhwave.F:3812-3832).
 *
 * It allocates nothing.  Its reduction scratch is a fixed 65,792-byte device
 * array inside the library, present on every GPU that loads the library
 * until the process exits, which caps a call at Mglob*Nglob*Kglob <=
 * 16,777,216 interior cells; larger grids are rejected with NHW_ERR_ARG and
 * an nhw_last_error() message.  All calls share that one array: calls whose
 * work overlaps on the GPU (different streams, threads or processes sharing
 * a context) race and give wrong results, so order them, e.g. on one stream.
 * The first call on each device looks the array's address up
 * (cudaGetSymbolAddress) and keeps it; make that first call before any
 * stream capture begins. */
int nhw_estimate_dt_noalloc(const double* U, const double* V, const double* W, const double* D,
                            const double* dsig, int32_t Mglob, int32_t Nglob, int32_t Kglob, double dx,
                            double dy, double cfl, double dt_old, double dt_max, double* dt_out,
                            void* stream);

#ifdef __cplusplus
}
#endif
#endif /* NHWAVE_GB300_H */
