// state.h -- device-side state of one NHWAVE scenario.
//
// Layout in HBM: every array of a scenario uses the same padded, ghosted,
// i-fastest layout, 0-based:
//     2-D  (i, j)     -> i + sy*j                 i in [0, Mloc], j in [0, Nloc]
//     3-D  (i, j, k)  -> i + sy*j + sz*k          k in [0, Kloc]
// with sy = Mloc+1 and sz = sy*(Nloc+1), so cell, x-face, y-face and z-face
// arrays (the reference's (Mloc,Nloc,Kloc), (Mloc1,Nloc,Kloc), (Mloc,Nloc1,Kloc)
// and (Mloc,Nloc,Kloc1) allocations, src/initialize.F:1423-1643) share one index
// formula; Fortran (i,j,k) is (i-1, j-1, k-1) here.  Interior cells are
// i in [IB, IE] = [2, M+1] (likewise j, k); face f lies between cells f-1 and f.
//
// 2-D fields (depth, elevation, masks, bathymetry derivatives) are always FP64;
// 3-D fields use the scenario's storage type T (double for the plain FP64
// form, float for the FP32+IR form).  Poisson vectors use a compact interior
// ordering  ic = (i-IB) + M*((j-JB) + N*(k-KB)).
#pragma once
#include <cstdint>
#include <cstddef>

namespace nhw {

constexpr int NG = 2;          // Nghost (src/mod_global.F:35)
constexpr int KMAX = 64;       // largest Kglob a column kernel holds in registers/local memory
constexpr int NCOEF = 15;      // Poisson stencil entries (src/pressure.F:276-278)

// Constants of module GLOBAL (src/mod_global.F:21-30): default-real literals,
// i.e. rounded to single precision then widened.
constexpr double kPi = (double)3.141592653f;
constexpr double kSmall = (double)1.0e-16f;
constexpr double kOrlSmall = (double)1.e-16f;   // the Orlanski boundary's 1.e-16 (default real)
constexpr double kKappa = (double)0.41f;        // von Karman constant (default real parameter)
constexpr double kLarge = 10000000.0;
constexpr double kGrav = (double)9.81f;
constexpr double kRho0 = 1000.0;

// Per-scenario scalars that live on the device (written by kernels).
struct DevScal {
  double time, dt, dt_old;
  int32_t run_step, status;
  unsigned long long dtmin_bits;   // estimate_dt minimum (bit pattern of a positive double)
  double source_area;
  // Krylov state
  double rho, alpha, omega, beta;
  double red[8];                    // reduction results
  double bnorm, relres, relres64;
  int32_t it, conv, ir, itmax_in;
  double tol_in;
  double rho_dt, dt_rho;            // Rho0/dt and dt/Rho0 of the current dt (set where dt is set)
  unsigned int counter[4];          // last-block-done counters
  int64_t total_it, solves;
  // Poisson refinement state, decided on the device (so that a captured step
  // can loop without the host): see k_res64 in krylov.cuh
  int32_t ir_go, ir_count, inner_total, pstat, zero_x;
  int32_t step_status;              // first non-OK Poisson status of the current step
  int32_t worst;                    // largest status code since the host last cleared it
  int32_t step_go;                  // set by k_dt_finalize: the step proceeds
  int64_t total_ir;                 // refinement sweeps, cumulative
  // grid barrier of the persistent solve (psolve.cuh)
  unsigned int bar_count, bar_gen;
  int32_t bar_err;
  int32_t sig_set, pad3_;           // viscous flow: the sigma slopes have been formed once
  unsigned long long htmax_bits;    // estimate_dt: largest |CmuHt| of the interior (bit pattern)
  double gm_inv;                    // GMRES: 1 / ||w|| of the vector the next iteration normalises
};

template <class T>
struct Dev {
  // dimensions (interior M x N x K; ghosted Mloc x Nloc x Kloc)
  int M, N, K, Mloc, Nloc, Kloc;
  int sy;            // j stride
  long long sz;      // k stride
  int IB, IE, JB, JE, KB, KE;   // interior bounds (inclusive), 0-based
  int neq;           // M*N*K
  int col_chunks, col_kc;   // column-walk matvecs: chunks per column, levels per chunk
  // parameters
  double dx, dy, min_dep, cfl, dt_min, dt_max, fcor, froude_cap;
  double cxx, cyy;                 // Poisson in-level couplings -1/dx^2, -1/dy^2
  int froude_on, non_hydro, sponge_on, it_order;
  int hllc;                        // HLLC face fluxes (ADV_HLLC) instead of HLL
  int bc_x0, bc_xn, bc_y0, bc_yn;
  double tol, tol_floor;          // outer Poisson tolerance (TOL); floor of the inner one
  int itmax, max_ir;               // ITMAX over all inner iterations; refinement sweeps
  double total_time;               // TOTAL_TIME and SIM_STEPS, for the gated run graph
  int sim_steps;
  // graph_mode = 1 in kernels captured into a step graph: they do nothing
  // unless k_dt_finalize let the step proceed (sc->step_go), and the
  // phase-by-phase solver sets the conditions of its loop nodes through the
  // handles.  Eagerly launched kernels have graph_mode = 0.
  int graph_mode;
  unsigned long long h_go, h_ir, h_inner;
  double visc_top;                 // inviscid path: Small + 0.5*(Cmu+CmuR+CmuVt+Cmu+CmuR+CmuVt), CmuVt = 0
  // viscous flow: Cmu = Visc (every cell); CmuVt, CmuHt per cell (below),
  // Cmut_min from initial, then what eval_turb sets -- Cvs / Chs (IVTURB,
  // IHTURB = 1) or the subgrid models (2); Schmidt; VISCOUS_NUMBER.
  // viscous = 0 on the inviscid path, where CmuVt = CmuHt = 0.
  int viscous, ivturb, ihturb;
  double v_cmu, v_cmut0, v_cvs, v_chs, v_schmidt, v_number;
  // k-epsilon closure (IVTURB = 10): RNG variant, PRODTYPE, Dmin = 2 MinDep;
  // ke_quiet: an INT_, LEF_ or FOCUSED maker, whose source region is kept
  // free of turbulence
  int ke_rng, ke_prod, ke_quiet;
  // LES closure (IVTURB = 20): a LEF_ maker (first column kept laminar), an
  // INT_ maker (source region kept laminar)
  int les_lef, les_int;
  double ke_dmin;
  // bed (BC_Z0): 1 free slip, 2 no slip, 5 friction law with Ibot 1 (Cd0) or 2 (Zob)
  int bc_z0, ibot;
  double cd0, zob;
  double alpha[3], beta[3];        // SSP-RK coefficients
  // wavemaker (INT_LIN / INT_SOL): host-computed constants
  int wavemaker;
  double wm_segma, wm_celerity, wm_amp, wm_wnumy, wm_xw, wm_xe, wm_ys, wm_yn;
  double wm_atmp, wm_xstart;
  int wm_i0, wm_i1;                // interior i range of the source strip (xc is monotonic)
  // waves through the west boundary (BC_X0 = 3): LEF_LIN / LEF_SOL /
  // LEF_STK / LEF_CON constants (host-computed, src/waves.F:92-170,
  // 518-560, 808-903) and the boundary values of the step
  int lef;                         // 0 none, else the nhw_wavemaker (3 .. 6)
  double lef_amp, lef_dep, lef_per, lef_segma, lef_wn, lef_shd, lef_stokes, lef_sinth, lef_costh;
  double lef_cel, lef_atmp, lef_xstart, lef_c2;
  double lef_e2, lef_u2;                           // LEF_STK second-order amplitudes
  double con_mod, con_len, con_ytr, con_ck, con_x0;   // LEF_CON: m, L, trough, K(m), start phase
  // FOCUSED: components Amp_i, k_i, f_i ([nwave] each, host-computed), focus
  // point and time, depth_comp, sd_return
  const double* foc;
  int nwave;
  // LEF_JON / LEF_TMA: [6][njon] components (Wh, 2 pi f, k, Stokes drift,
  // phase, sinh(k h)), host-computed
  const double* jon;
  int njon;
  double foc_xb, foc_tb, foc_dc, foc_sd;
  double *Ein, *Din;               // [Nloc] Ein_X0, Din_X0
  double *Uin, *Vin, *Win;         // [Kloc][Nloc] Uin_X0 .. (index j + Nloc*k)
  // the east side open to a boundary condition (BC_Xn = 3): RIG_LIN or
  // FLUX_LR (0: none); its values of the step (src/nhwave.F:5514-5712), and
  // FLUX_LR's outflow velocity of this and the previous step (checkpointed)
  int east;
  double *Ein_xn, *Din_xn;         // [Nloc] Ein_Xn, Din_Xn
  double *Uin_xn, *Vin_xn, *Win_xn;  // [Kloc][Nloc] Uin_Xn ..
  double *Uxni, *Uxni0;            // [Kloc][Nloc] Uin_Xni, Uin_Xni0
  // sponge current
  double cur_wave, tramp;
  // rigid slide (RIGID_3D)
  int slide;
  double sl_e, sl_kb, sl_kw, sl_cosa, sl_sina, sl_cosslope, sl_s0, sl_t0, sl_T, sl_x0, sl_y0;
  // 1-D grid
  const double *sig, *dsig, *sigc, *xc, *yc;
  // 2-D FP64 fields
  double *D, *D0, *Eta, *Eta0, *Hc, *Hc0, *Ho;
  double* Eta00;               // east boundary of BC_Xn = 6 or 3 only, else nullptr
  // viscous flow only, else nullptr: D, DelxEta, DelyEta, DelxH, DelyH as of
  // the last sigma_transform, from which the viscous terms form DelxSc /
  // DelySc (cell levels) and DelxSl / DelySl (faces) of that moment
  double *scD, *scEx, *scEy, *scHx, *scHy;
  T *CmuVt, *CmuHt;                // viscous flow: eddy viscosities per cell (ghosted 3-D), else nullptr
  double *Hfx, *Hfy, *Hfx0, *Hfy0, *DelxH, *DelyH, *DeltH, *DeltHo, *Delt2H;
  double *DelxEta, *DelyEta, *SourceX, *SourceY, *SourceC, *Sponge, *R1, *Wsx, *Wsy;
  double *EtaxL, *EtaxR, *EtayL, *EtayR;
  double *zUL, *zVL, *zWL, *zUR, *zVR, *zWR;   // vel_bc face states at the surface / bed
  double *cf_hx, *cf_ex, *cf_hy, *cf_ey, *cf_invD;  // per column: DelxH/D, DelxEta/D, ..., 1/D
  // per sigma level k: 1/(2dx(dsig_k+dsig_k-1)), 1/(2dy(..)), 1/(h_k dsig_k), 1/(h_k dsig_k-1),
  // 1/h_k with h_k = (dsig_k+dsig_k-1)/2, 1/dsig_k
  const double *lv_x, *lv_y, *lv_up, *lv_dn, *lv_h, *lv_ds;
  const double* lv_fint;   // dsig_k / (dsig_k + dsig_k-1): weight of level k-1 at face k
  // per sigma level k in the storage type T, [3][Kloc]: 1/dsig_k, sigc_k - sigc_k-1,
  // dsig_k / 2 -- each formed in FP64 on the host and rounded once, as the
  // kernels formed them per cell before
  const T* lvT;
  double i2dx, i2dy;       // 0.5/dx, 0.5/dy
  // the spacings in the storage type, rounded once: dx, dx/2, 1/dx (and y)
  T dxT, hdxT, idxT, dyT, hdyT, idyT;
  // FP32+IR form with HLL: 2-D face states of the x / y faces in the storage
  // type, [6][sy*(Nloc+1)] (the size of a 2-D field) at the face's right cell
  // (OpFacePrep), else nullptr
  T *fxT, *fyT;
  int *Mask, *MaskT, *Mask_Struct, *Mask9;
  // 3-D fields (storage type T); P is FP64 in both forms
  T *U, *V, *W, *DU, *DV, *DW, *DU0, *DV0, *DW0, *Omega;
  T *Ex, *Fx, *Gx, *Hx, *Ey, *Fy, *Gy, *Hy, *Fz, *Gz, *Hz;
  double* P;
  // Poisson: FP64 operator (compact 7-slot form, see krylov.cuh) + rhs
  double* coef64;     // [7][neq]
  double* rhs64;      // [neq]
  double* xsol64;     // [neq]  FP64 solution (= P interior)
  double* res64;      // [neq]  FP64 residual for refinement
  // Krylov working vectors in the inner precision T (compact interior order)
  T* coefT;           // [7][neq] (aliases coef64 when T == double)
  T *lcp, *linv;      // line preconditioner factors [neq]
  T* sp0;             // colour-split copy of the level-0 smoother's operator (MGL::sp), or nullptr
  T *kx, *kr, *kr0, *kp, *kph, *kv, *ks, *ksh, *kt;
  // velocities of the last two steps, read by the Orlanski boundary
  // (BC_Xn = 6) only, else nullptr
  T *U0, *V0, *W0, *U00, *V00, *W00;
  // explicit viscous terms of the stage (viscous flow only, else nullptr):
  // Diffxx, Diffxy (into R2), Diffyx, Diffyy (R3), Diffzx, Diffzy (R4)
  T *Dxx, *Dxy, *Dyx, *Dyy, *Dzx, *Dzy;
  // k-epsilon (IVTURB = 10, else nullptr): tke, epsilon, their depth
  // integrals and the step's starting integrals (checkpointed state); the
  // limited horizontal slopes of U, V (from get_Omega) and W (from fluxes)
  // the production reads; the floored surface values of tke and epsilon
  T *Tke, *Eps, *DTke, *DEps, *DTke0, *DEps0;
  T *keDxU, *keDyU, *keDxV, *keDyV, *keDxW, *keDyW;
  double *keTopK, *keTopE;
  // dynamic LES (IVTURB = 30, else nullptr): 31 scratch fields of ld_n cells
  T* ld;
  long long ld_n;
  // GMRES (krylov.cuh): basis V [kGmMax+1][neq], preconditioned basis Z
  // [kGmMax][neq], Hessenberg / rotations / g / y in FP64 (gm), the current
  // column, y and 1/||w|| in T (gmT), wide reduction partials; nullptr unless
  // the GMRES solver is on
  T *gmV, *gmZ, *gmT;
  double *gm, *gm_part;
  double* partials;   // reduction partials [nblocks * 8]
  DevScal* sc;
};

// -------------------------------------------------------------- indexing
template <class T>
__host__ __device__ __forceinline__ long long i2(const Dev<T>& S, int i, int j) {
  return (long long)i + (long long)S.sy * j;
}
template <class T>
__host__ __device__ __forceinline__ long long i3(const Dev<T>& S, int i, int j, int k) {
  return (long long)i + (long long)S.sy * j + S.sz * k;
}
template <class T>
__host__ __device__ __forceinline__ int ic_of(const Dev<T>& S, int i, int j, int k) {
  return (i - S.IB) + S.M * ((j - S.JB) + S.N * (k - S.KB));
}

}  // namespace nhw
