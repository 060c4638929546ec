// nhw_oracle.cpp -- TEST INFRASTRUCTURE, not product code.
//
// A plain single-threaded FP64 C++ restatement of NHWAVE's time-step hot path,
// written loop by loop after the reference Fortran so that each routine can be
// checked against its source lines.  Only tests/, __graft_entry__.smoke() and
// bench.py's CPU-baseline leg load it, and only as the checker / CPU baseline.
//
// Parity status: the reference is Fortran, no Fortran compiler is installed
// where this file is compiled and run, and the reference ships no golden
// outputs; this restatement is therefore "parity unpinned" against the
// reference binary.  It is pinned instead by known-answer tests (lake at rest, mass conservation,
// mirror symmetry, linear dispersion, hand-computed limiter / HLL / Poisson
// coefficients, boundary-wave formulas, elliptic functions against scipy,
// viscous decay rates) in tests/test_oracle.py.
//
// Reference routines restated here (file:line in the reference project):
//   generate_grid              src/initialize.F:1647-1729
//   read_bathymetry            src/initialize.F:1734-2175 (CELL_CENTER/CELL_GRID, RIGID_3D slide)
//   initial                    src/initialize.F:2502-3408 (non-optional parts)
//   calculate_sponge           src/nhwave.F:6405-6460
//   estimate_dt                src/nhwave.F:3694-3874
//   update_bathymetry RIGID_3D src/nhwave.F:5755-5857, 6024-6071
//   update_mask / update_vars  src/nhwave.F:5403-5511
//   update_wind (Iws=1)        src/nhwave.F:5333-5400
//   source_terms               src/source_terms.F:1-67, 418-455; wave_dispersion src/waves.F:61-91
//   fluxes & co.               src/nhwave.F:1686-2351, 2354-2552, 2673-2776, 2813-2906
//   eval_duvw                  src/nhwave.F:539-1300 (with the implicit vertical viscous step)
//   diffusion                  src/nhwave.F:6785-7141
//   trig                       src/nhwave.F:13182-13224
//   eval_turb (IVTURB 1, 2, 3, 10, 20, 30; IHTURB 1, 2, >= 10) src/nhwave.F:6544-6782
//   les_3D                     src/nhwave.F:8545-8729
//   kepsilon (2-D, IVTURB = 3) src/nhwave.F:11117-11524
//   les_dyn, filter            src/nhwave.F:7989-8410, 8412-8542
//   kepsilon_3D                src/nhwave.F:10030-11114, adv_scalar_hlpa 7604-7806,
//                              hlpa 7809-7847, flux_scalar_bc 7850-7986
//   get_UVW / vel_bc / KBC     src/nhwave.F:1651-1683, 4416-5117 (walls 1/2/5, inflow,
//                              Orlanski east side, bed stress)
//   update_wave_bc             src/nhwave.F:5514-5565, 5715-5750; src/waves.F:92-370,
//                              518-560, 638-756, 808-903; components src/initialize.F:709-781
//   interpolate_velocity_to_faces src/nhwave.F:1332-1368
//   get_Omega                  src/nhwave.F:1411-1648
//   wl_bc / phi_2D_coll        src/nhwave.F:5119-5330
//   projection_corrector       src/nhwave.F:487-536
//   poisson_solver             src/pressure.F:63-245 (solver replaced, see below)
//   generate_coef_rhs          src/pressure.F:475-840
//   sponge_damping             src/nhwave.F:6463-6502
//   sigma_transform            src/nhwave.F:6505-6541
//   statistics                 src/nhwave.F:3118-3160
//
// Arithmetic: IEEE FP64 with the reference's evaluation order written out
// (left-to-right products and quotients, explicit parentheses) and built with
// -ffp-contract=off.  Default-real literals of the reference (Grav=9.81,
// pi, Small=1e-16, 1.05, 1e-6, 1/3, 2/3, 0.717, dsig=1.0/float(Kglob) ...)
// are rounded to single precision and widened, as the reference's double build
// does with empty FFLAGS (src/Makefile.farber.mpif90:40).
//
// The Poisson system is solved by restarted GMRES with a vertical-line
// (tridiagonal) right preconditioner -- a solver of this file's own, standing in
// for NSPCG (src/nspcg.f) / HYPRE GMRES+SMG (src/pressure.F:260-462) -- with the
// same stopping test as HYPRE (||b-Ax||_2 <= TOL*||b||_2) and the previous P as
// the initial guess (src/pressure.F:104-113, 386-397).

#include "../include/nhwave_gb300.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

namespace {

// reference parameters (src/mod_global.F:21-35): default-real literals
const double pi = (double)3.141592653f;
const double Small = (double)1.0e-16f;
const double Large = 10000000.0;
const double Grav = (double)9.81f;
const double Zero = 0.0;
const double Rho0 = 1000.0;
const double kOrlSmall = (double)1.e-16f;   // the Orlanski boundary's 1.e-16 (default real)
const double Kappa = (double)0.41f;         // von Karman constant (default real parameter)
const int Nghost = 2;

// ---------------------------------------------------------------- cnoidal
// cnoidal_cn, cnoidal_ck, cnoidal_ce (src/waves.F:225-370): the AGM
// sequence of the parameter m, stopped when |c| < 1.0e-15 (default real) or
// after 1000 terms; K = (pi/2)/a_N with a default-real pi literal;
// E = K (1 - sum 2^(n-2) c_n^2); cn by descending Landen steps from
// phi_N = 2^(N-1) a_N u.
const double CnPi = (double)3.1415926535897932384626f;
int agm_terms(double mod, double* a, double* c) {
  double a0 = 1.0, b0 = std::sqrt(1.0 - mod), c0 = std::sqrt(mod);
  int n = 1;
  a[n] = a0; c[n] = c0;
  while (!(std::fabs(c0) < (double)1.0e-15f || n > 1000)) {
    n = n + 1;
    const double a1 = (a0 + b0) / 2.0, b1 = std::sqrt(a0 * b0), c1 = (a0 - b0) / 2.0;
    a0 = a1; b0 = b1; c0 = c1;
    a[n] = a0; c[n] = c0;
  }
  return n;
}
double cnoidal_cn(double u, double mod) {
  std::vector<double> a(1002), c(1002), y(1002);
  const int n = agm_terms(mod, a.data(), c.data());
  y[n] = std::pow(2.0, n - 1) * a[n] * u;
  for (int i = n - 1; i >= 1; --i) y[i] = (y[i + 1] + std::asin(c[i + 1] / a[i + 1] * std::sin(y[i + 1]))) / 2.0;
  return std::cos(y[1]);
}
double cnoidal_ck(double mod) {
  std::vector<double> a(1002), c(1002);
  const int n = agm_terms(mod, a.data(), c.data());
  return CnPi / 2.0 / a[n];
}
double cnoidal_ce(double mod) {
  std::vector<double> a(1002), c(1002);
  const int n = agm_terms(mod, a.data(), c.data());
  const double ck = CnPi / 2.0 / a[n];
  double sum = 0.0;
  for (int k1 = 1; k1 <= n; ++k1) sum = sum + std::pow(2.0, k1 - 2) * (c[k1] * c[k1]);
  return ck * (1.0 - sum);
}
// cnoidal (src/waves.F:184-220): Newton iteration for m from 0.99999999,
// then the wave length l, the trough level x2 and, when asked for, the
// celerity c (the boundary does not use it; INT_CON does).  False when m
// leaves (0, 1], where the reference's square roots turn to NaN.
bool cnoidal(double height, double depth, double period, double& l, double& x2, double& mod,
             double* c = nullptr) {
  mod = 0.99999999;
  int n = 0;
  while (true) {
    n = n + 1;
    if (!(mod > 0.0 && mod <= 1.0)) return false;
    const double xa = mod * depth + 2.0 * height - mod * height - 3.0 * height * cnoidal_ce(mod) / cnoidal_ck(mod) -
                      16.0 * (depth * depth * depth) * (mod * mod) * (cnoidal_ck(mod) * cnoidal_ck(mod)) / 3.0 / Grav /
                          height / (period * period);
    if (std::fabs(xa) <= (double)1.0e-8f || n > 1000) break;
    const double ck = cnoidal_ck(mod), ce = cnoidal_ce(mod);
    const double xb = depth - height +
                      3.0 * height / 2.0 / mod / (1.0 - mod) / (ck * ck) *
                          ((1.0 - mod) * (ck * ck) + ce * ce - 2.0 * (1.0 - mod) * ck * ce) -
                      16.0 * (depth * depth * depth) * mod * ck / 3.0 / Grav / (1.0 - mod) / height /
                          (period * period) * ((1.0 - mod) * ck + ce);
    mod = mod - xa / xb;
  }
  if (!(mod > 0.0 && mod <= 1.0)) return false;
  l = 4.0 * cnoidal_ck(mod) * depth * std::sqrt(mod * depth / height / 3.0);
  const double xtemp = -mod + 2.0 - 3.0 * cnoidal_ce(mod) / cnoidal_ck(mod);
  if (c) *c = std::sqrt(Grav * depth * (1.0 + height / depth / mod * xtemp));
  x2 = height / mod * (1.0 - mod - cnoidal_ce(mod) / cnoidal_ck(mod));
  return std::isfinite(l) && std::isfinite(x2);
}

inline double dmax(double a, double b) { return a > b ? a : b; }
inline double dmin(double a, double b) { return a < b ? a : b; }

struct A1 {
  std::vector<double> v;
  void init(int n) { v.assign(n, 0.0); }
  double& operator()(int i) { return v[i - 1]; }
};
struct A2 {
  int n1 = 0, n2 = 0;
  std::vector<double> v;
  void init(int a, int b) { n1 = a; n2 = b; v.assign((size_t)a * b, 0.0); }
  double& operator()(int i, int j) { return v[(size_t)(i - 1) + (size_t)n1 * (j - 1)]; }
  void fill(double x) { std::fill(v.begin(), v.end(), x); }
};
struct I2 {
  int n1 = 0, n2 = 0;
  std::vector<int32_t> v;
  void init(int a, int b) { n1 = a; n2 = b; v.assign((size_t)a * b, 0); }
  int32_t& operator()(int i, int j) { return v[(size_t)(i - 1) + (size_t)n1 * (j - 1)]; }
};
struct A3 {
  int n1 = 0, n2 = 0, n3 = 0;
  std::vector<double> v;
  void init(int a, int b, int c) { n1 = a; n2 = b; n3 = c; v.assign((size_t)a * b * c, 0.0); }
  double& operator()(int i, int j, int k) {
    return v[(size_t)(i - 1) + (size_t)n1 * ((size_t)(j - 1) + (size_t)n2 * (k - 1))];
  }
  void fill(double x) { std::fill(v.begin(), v.end(), x); }
};

// LIMITER, van Leer (src/nhwave.F:2889-2906)
inline double LIMITER(double A, double B) {
  return (A * std::fabs(B) + std::fabs(A) * B) / (std::fabs(A) + std::fabs(B));
}

struct Model {
  nhw_params p;
  int Mloc, Nloc, Kloc, Mloc1, Nloc1, Kloc1;
  int Ibeg, Iend, Iend1, Jbeg, Jend, Jend1, Kbeg, Kend, Kend1;
  double dx, dy, dt = 0, dt_old = 0, TIME = 0, MinDep, fcor;
  int RUN_STEP = 0, It_Order = 3;
  double ALPHA[3], BETA[3];
  int last_iters = 0, last_refine = 0;
  int64_t total_iters = 0, solves = 0;
  double last_relres = 0;
  int status = NHW_OK;

  A1 x, xc, y, yc, sig, dsig, sigc;
  A2 Hc, Hc0, Ho, Hfx, Hfy, Hfx0, Hfy0, DeltH, DeltHo, Delt2H, DelxH, DelyH;
  A2 D, D0, Eta, Eta0, Eta00, SourceX, SourceY, SourceC, DxL, DxR, DyL, DyR;
  A2 EtaxL, EtaxR, EtayL, EtayR, DelxEta, DelyEta, Sponge, Wsx, Wsy, R1s;
  I2 Mask, Mask_Struct, Mask9;
  // west-boundary inflow (Ein_X0, Din_X0, Uin_X0, Vin_X0, Win_X0; src/mod_global.F)
  A1 Ein_X0, Din_X0;
  A2 Uin_X0, Vin_X0, Win_X0;
  // east-boundary inflow/outflow (Ein_Xn ... Win_Xn) and the FLUX_LR outflow
  // velocities of this and the previous call (Uin_Xni, Uin_Xni0; zero at
  // start, src/initialize.F:2688-2689)
  A1 Ein_Xn, Din_Xn;
  A2 Uin_Xn, Vin_Xn, Win_Xn, Uin_Xni, Uin_Xni0;
  A3 U, V, W, DU, DV, DW, DU0, DV0, DW0, P, Omega, Uf, Vf, Wf;
  A3 U0, V0, W0, U00, V00, W00;   // earlier time levels, read by the Orlanski boundary
  A3 UxL, UxR, VxL, VxR, WxL, WxR, DUxL, DUxR, DVxL, DVxR, DWxL, DWxR;
  A3 UyL, UyR, VyL, VyR, WyL, WyR, DUyL, DUyR, DVyL, DVyR, DWyL, DWyR;
  A3 UzL, UzR, VzL, VzR, WzL, WzR;
  A3 SxL, SxR, SxS, SyL, SyR, SyS;
  A3 ExL, ExR, FxL, FxR, GxL, GxR, HxL, HxR, EyL, EyR, FyL, FyR, GyL, GyR, HyL, HyR;
  A3 Ex, Ey, Fx, Fy, Fz, Gx, Gy, Gz, Hx, Hy, Hz;
  A3 DelxU, DelyU, DelzU, DelxV, DelyV, DelzV, DelxW, DelyW, DelzW;
  A3 DelxDU, DelyDU, DelxDV, DelyDV, DelxDW, DelyDW, DelxSc, DelySc;
  // Poisson system (Coef(neqns,15), Rhs(neqns); src/mod_global.F:239-243)
  int neqns = 0;
  std::vector<double> Coef, Rhs;
  // Cmu = Visc and CmuR = 0 in every cell (no sediment rheology), so they
  // are scalars here; CmuVt and CmuHt are zero on the inviscid path
  // (src/initialize.F:2663-2668), Cmut_min in every cell from initial with
  // VISCOUS_FLOW (:3172-3195), then what eval_turb sets (src/nhwave.F:
  // 6544-6782): Cvs / Chs, or the subgrid models of IVTURB / IHTURB = 2.
  double Cmu = 0, CmuR = 0;
  A3 CmuVt, CmuHt;
  // k-epsilon state (src/mod_global.F:229): Tke, Eps and their depth
  // integrals DTke, DEps with the step's starting values DTke0, DEps0;
  // seeded by initial with Tke_min, Eps_min (src/initialize.F:3172-3193)
  A3 Tke, Eps, DTke, DEps, DTke0, DEps0;
  const double Tke_min = (double)1.e-9f, Eps_min = (double)1.e-9f;
  double Cmut_min = 0.0;
  // viscous flow: face sigma slopes (sigma_transform) and the explicit
  // viscous terms of diffusion (src/nhwave.F:6785-7141)
  A3 DelxSl, DelySl, Diffxx, Diffxy, Diffyx, Diffyy, Diffzx, Diffzy;

  // ------------------------------------------------------------ index/alloc
  int create(const nhw_params& q) {
    p = q;
    if (p.Mglob < 1 || p.Nglob < 1 || p.Kglob < 1 || !(p.dx > 0) || !(p.dy > 0)) return NHW_ERR_ARG;
    // BAROTROPIC = F: baropg_z (src/nhwave.F:13038-13179) of the uniform
    // density Rho0 (no salinity, temperature, sediment or bubbles) gives
    // DRhoX = DRhoY = 0, so the flag runs the same path
    // IVTURB 1, 2, 10 (k-epsilon) and IHTURB 1, 2, >= 10 (CmuHt = CmuVt)
    if (p.viscous_flow &&
        !(p.ivturb == 1 || p.ivturb == 2 || p.ivturb == 3 || p.ivturb == 10 || p.ivturb == 20 || p.ivturb == 30))
      return NHW_ERR_UNSUPPORTED;
    if (p.viscous_flow && !(p.ihturb == 1 || p.ihturb == 2 || p.ihturb >= 10)) return NHW_ERR_UNSUPPORTED;
    if (p.viscous_flow && (!(p.schmidt != 0.0) || !(p.viscous_number > 0.0))) return NHW_ERR_ARG;
    for (int b : {p.bc_y0, p.bc_yn})
      if (b != 1 && b != 2 && b != 5) return NHW_ERR_UNSUPPORTED;
    const bool east_in = p.wavemaker == NHW_WM_RIG_LIN || p.wavemaker == NHW_WM_FLUX_LR;
    // 6: Orlanski; 3: inflow/outflow of RIG_LIN and FLUX_LR
    if (p.bc_xn != 1 && p.bc_xn != 2 && p.bc_xn != 5 && p.bc_xn != 6 && !(p.bc_xn == 3 && east_in))
      return NHW_ERR_UNSUPPORTED;
    const bool lef = (p.wavemaker >= NHW_WM_LEF_LIN && p.wavemaker <= NHW_WM_LEF_TID) ||
                     p.wavemaker == NHW_WM_FLUX_LR || p.wavemaker == NHW_WM_LEF_JON ||
                     p.wavemaker == NHW_WM_LEF_TMA || p.wavemaker == NHW_WM_LEF_SPC;
    const bool jon = p.wavemaker == NHW_WM_LEF_JON || p.wavemaker == NHW_WM_LEF_TMA ||
                     p.wavemaker == NHW_WM_INT_JON || p.wavemaker == NHW_WM_INT_TMA;
    if (jon && (!(p.hm0 > 0) || !(p.tp > 0) || !(p.freq_min > 0) || !(p.freq_max > p.freq_min) || p.numfreq < 1 ||
                p.numfreq > 500 || !(p.dep_wave > 0)))
      return NHW_ERR_ARG;
    if ((p.wavemaker == NHW_WM_INT_SPC || p.wavemaker == NHW_WM_INT_IRR) && !(p.dep_wave > 0)) return NHW_ERR_ARG;
    if (!(p.bc_x0 == 1 || p.bc_x0 == 2 || p.bc_x0 == 5 || (p.bc_x0 == 3 && lef))) return NHW_ERR_UNSUPPORTED;
    if (p.wavemaker == NHW_WM_FLUX_LR && !(p.zob > 0.0)) return NHW_ERR_ARG;
    if (jon) jonswap_spectrum();
    if (p.wavemaker == NHW_WM_FOCUSED) {   // components (src/initialize.F:742-781)
      if (p.nwave < 2 || p.nwave > 12000 || !(p.f_center > 0) || !(p.depth_comp > 0)) return NHW_ERR_ARG;
      const int nw = p.nwave;
      Amp_i.assign(nw, 0.0); k_i.assign(nw, 0.0); f_i.assign(nw, 0.0);
      for (int n = 1; n <= nw; ++n) {
        f_i[n - 1] = p.f_center - 0.5 * p.normalized_delta_f * p.f_center +
                     (n - 1.0) * p.normalized_delta_f * p.f_center / (nw - 1.0);
        const double period_i = 1.0 / f_i[n - 1];
        const double segmasqr = (2.0 * pi / period_i) * (2.0 * pi / period_i);
        const double ctmp = std::sqrt(Grav * p.depth_comp);
        const double xltmp = ctmp * period_i;
        double xxk = 2.0 * pi / xltmp;
        int it = 0;
        while (true) {
          const double Fk = Grav * xxk * std::tanh(xxk * p.depth_comp) - segmasqr;
          if (std::fabs(Fk) <= (double)1.0e-6f || it > 1000) break;
          const double Fkdif = Grav * xxk * p.depth_comp *
                                   (1.0 - std::tanh(xxk * p.depth_comp) * std::tanh(xxk * p.depth_comp)) +
                               Grav * std::tanh(xxk * p.depth_comp);
          xxk = xxk - Fk / Fkdif;
          it = it + 1;
        }
        k_i[n - 1] = xxk;
      }
      for (int n = 0; n < nw; ++n)
        Amp_i[n] = p.component_amp_type == 1 ? p.slope_group / nw / p.k_center : p.slope_group / nw / k_i[n];
    }
    if (p.wavemaker == NHW_WM_LEF_CON || p.wavemaker == NHW_WM_INT_CON) {   // the reference stops when these fail
      double l, x2, m, xs;
      if (!(p.amp_wave > 0) || !cnoidal(p.amp_wave, p.dep_wave, p.per_wave, l, x2, m) ||
          !cnoidal_start(x2, m, xs))
        return NHW_ERR_ARG;
    }
    // bed: 1 free slip, 2 no slip, 5 friction law with Ibot 1 (Cd0) or 2 (Zob)
    if (p.bc_z0 != 1 && p.bc_z0 != 2 && p.bc_z0 != 5) return NHW_ERR_UNSUPPORTED;
    const bool fric = p.bc_z0 == 5 || p.bc_x0 == 5 || p.bc_xn == 5 || p.bc_y0 == 5 || p.bc_yn == 5;
    if (fric && p.ibot != 1 && p.ibot != 2) return NHW_ERR_UNSUPPORTED;
    if (fric && p.ibot == 2 && !(p.zob > 0.0)) return NHW_ERR_ARG;
    // index (src/initialize.F:1339-1419), serial build
    Mloc = p.Mglob + 2 * Nghost; Nloc = p.Nglob + 2 * Nghost; Kloc = p.Kglob + 2 * Nghost;
    Mloc1 = Mloc + 1; Nloc1 = Nloc + 1; Kloc1 = Kloc + 1;
    Ibeg = Nghost + 1; Iend = Mloc - Nghost; Iend1 = Mloc1 - Nghost;
    Jbeg = Nghost + 1; Jend = Nloc - Nghost; Jend1 = Nloc1 - Nghost;
    Kbeg = Nghost + 1; Kend = Kloc - Nghost; Kend1 = Kloc1 - Nghost;
    dx = p.dx; dy = p.dy; MinDep = p.min_dep;
    fcor = 2.0 * (double)7.29e-5f * std::sin(p.slat);  // src/initialize.F:494
    x.init(Mloc1); xc.init(Mloc); y.init(Nloc1); yc.init(Nloc);
    Ein_X0.init(Nloc); Din_X0.init(Nloc);
    for (A2* a : {&Uin_X0, &Vin_X0, &Win_X0}) a->init(Nloc, Kloc);
    Ein_Xn.init(Nloc); Din_Xn.init(Nloc);
    for (A2* a : {&Uin_Xn, &Vin_Xn, &Win_Xn, &Uin_Xni, &Uin_Xni0}) a->init(Nloc, Kloc);
    sig.init(Kloc1); dsig.init(Kloc); sigc.init(Kloc);
    for (A2* a : {&Hc, &Hc0, &Ho, &DeltH, &DeltHo, &Delt2H, &DelxH, &DelyH, &D, &D0, &Eta, &Eta0, &Eta00,
                  &SourceX, &SourceY, &SourceC, &DelxEta, &DelyEta, &Sponge, &Wsx, &Wsy, &R1s})
      a->init(Mloc, Nloc);
    for (A2* a : {&Hfx, &Hfx0, &DxL, &DxR, &EtaxL, &EtaxR}) a->init(Mloc1, Nloc);
    for (A2* a : {&Hfy, &Hfy0, &DyL, &DyR, &EtayL, &EtayR}) a->init(Mloc, Nloc1);
    Mask.init(Mloc, Nloc); Mask_Struct.init(Mloc, Nloc); Mask9.init(Mloc, Nloc);
    for (A3* a : {&U, &V, &W, &DU, &DV, &DW, &DU0, &DV0, &DW0, &U0, &V0, &W0, &U00, &V00, &W00, &P, &DelxU,
                  &DelyU, &DelzU, &DelxV,
                  &DelyV, &DelzV, &DelxW, &DelyW, &DelzW, &DelxDU, &DelyDU, &DelxDV, &DelyDV,
                  &DelxDW, &DelyDW, &DelxSc, &DelySc, &CmuVt, &CmuHt})
      a->init(Mloc, Nloc, Kloc);
    for (A3* a : {&Omega, &Uf, &Vf, &Wf, &UzL, &UzR, &VzL, &VzR, &WzL, &WzR, &Fz, &Gz, &Hz})
      a->init(Mloc, Nloc, Kloc1);
    if (p.viscous_flow) {
      DelxSl.init(Mloc, Nloc, Kloc1); DelySl.init(Mloc, Nloc, Kloc1);
      for (A3* a : {&Diffxx, &Diffxy, &Diffyx, &Diffyy, &Diffzx, &Diffzy}) a->init(Mloc, Nloc, Kloc);
      for (A3* a : {&Tke, &Eps, &DTke, &DEps, &DTke0, &DEps0}) a->init(Mloc, Nloc, Kloc);
    }
    for (A3* a : {&UxL, &UxR, &VxL, &VxR, &WxL, &WxR, &DUxL, &DUxR, &DVxL, &DVxR, &DWxL, &DWxR,
                  &SxL, &SxR, &SxS, &ExL, &ExR, &FxL, &FxR, &GxL, &GxR, &HxL, &HxR, &Ex, &Fx,
                  &Gx, &Hx})
      a->init(Mloc1, Nloc, Kloc);
    for (A3* a : {&UyL, &UyR, &VyL, &VyR, &WyL, &WyR, &DUyL, &DUyR, &DVyL, &DVyR, &DWyL, &DWyR,
                  &SyL, &SyR, &SyS, &EyL, &EyR, &FyL, &FyR, &GyL, &GyR, &HyL, &HyR, &Ey, &Fy,
                  &Gy, &Hy})
      a->init(Mloc, Nloc1, Kloc);
    neqns = p.Mglob * p.Nglob * p.Kglob;
    Coef.assign((size_t)neqns * 15, 0.0);
    Rhs.assign(neqns, 0.0);
    return NHW_OK;
  }

  // -------------------------------------------------------- generate_grid
  void generate_grid() {
    x(Ibeg) = Zero;
    for (int i = Ibeg + 1; i <= Mloc1; ++i) { x(i) = x(i - 1) + dx; xc(i - 1) = x(i - 1) + 0.5 * dx; }
    for (int i = Ibeg - 1; i >= Ibeg - Nghost; --i) { x(i) = x(i + 1) - dx; xc(i) = x(i + 1) - 0.5 * dx; }
    y(Jbeg) = Zero;
    for (int j = Jbeg + 1; j <= Nloc1; ++j) { y(j) = y(j - 1) + dy; yc(j - 1) = y(j - 1) + 0.5 * dy; }
    for (int j = Jbeg - 1; j >= Jbeg - Nghost; --j) { y(j) = y(j + 1) - dy; yc(j) = y(j + 1) - 0.5 * dy; }
    if (p.ivgrd == 2) {
      dsig(Kbeg) = (p.grd_r - 1.0) / (std::pow(p.grd_r, (double)(float)p.Kglob) - 1.0);
      for (int k = Kbeg + 1; k <= Kend; ++k) dsig(k) = dsig(k - 1) * p.grd_r;
      for (int k = 1; k <= Nghost; ++k) dsig(Kbeg - k) = dsig(Kbeg + k - 1);
      for (int k = 1; k <= Nghost; ++k) dsig(Kend + k) = dsig(Kend - k + 1);
    } else {
      const double d = (double)(1.0f / (float)p.Kglob);  // 1.0/float(Kglob) in default real
      for (int k = 1; k <= Kloc; ++k) dsig(k) = d;
    }
    sig(Kbeg) = Zero;
    for (int k = Kbeg + 1; k <= Kloc1; ++k) { sig(k) = sig(k - 1) + dsig(k - 1); sigc(k - 1) = sig(k - 1) + 0.5 * dsig(k - 1); }
    for (int k = Kbeg - 1; k >= 1; --k) { sig(k) = sig(k + 1) - dsig(k); sigc(k) = sig(k + 1) - 0.5 * dsig(k); }
  }

  // ---------------------------------------------------------- phi_2D_coll
  void phi_2D_coll(A2& phi) {
    for (int j = Jbeg; j <= Jend; ++j)
      for (int i = 1; i <= Nghost; ++i) phi(i, j) = phi(Ibeg + Nghost - i, j);
    for (int j = Jbeg; j <= Jend; ++j)
      for (int i = 1; i <= Nghost; ++i) phi(Iend + i, j) = phi(Iend - i + 1, j);
    for (int i = 1; i <= Mloc; ++i)
      for (int j = 1; j <= Nghost; ++j) phi(i, j) = phi(i, Jbeg + Nghost - j);
    for (int i = 1; i <= Mloc; ++i)
      for (int j = 1; j <= Nghost; ++j) phi(i, Jend + j) = phi(i, Jend - j + 1);
  }

  // ------------------------------------------------------ read_bathymetry
  void slide_shape_rigid3d(double x0, double y0) {
    const double e = (double)0.717f;
    const double alpha0 = p.slide_angle * pi / 180.;
    const double kb = 2.0 * std::acosh(1.0 / e) / p.slide_l;
    const double kw = 2.0 * std::acosh(1.0 / e) / p.slide_w;
    for (int j = Jbeg; j <= Jend; ++j)
      for (int i = Ibeg; i <= Iend; ++i) {
        double xt = (xc(i) - x0) * std::cos(alpha0) + (yc(j) - y0) * std::sin(alpha0);
        double yt = -((xc(i) - x0) * std::sin(alpha0)) + (yc(j) - y0) * std::cos(alpha0);
        double zt = p.slide_t / (1 - e) * (1.0 / std::cosh(kb * xt) / std::cosh(kw * yt) - e);
        Hc(i, j) = Hc0(i, j) - dmax(0.0, zt);
      }
  }

  void read_bathymetry(const double* depth) {
    Hc.fill(0.0);
    const int Mg = p.Mglob, Ng = p.Nglob;
    if (p.depth_type == NHW_DEPTH_CELL_GRID) {
      auto HG = [&](int i, int j) { return depth[(size_t)(i - 1) + (size_t)(Mg + 1) * (j - 1)]; };
      auto Maskp = [&](int i, int j) { return HG(i, j) < -1000.0 ? 0 : 1; };
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i) {
          int ig = i - Nghost, jg = j - Nghost;
          int ms = Maskp(ig, jg) + Maskp(ig + 1, jg) + Maskp(ig, jg + 1) + Maskp(ig + 1, jg + 1);
          double num = HG(ig, jg) * Maskp(ig, jg) + HG(ig + 1, jg) * Maskp(ig + 1, jg) +
                       HG(ig, jg + 1) * Maskp(ig, jg + 1) + HG(ig + 1, jg + 1) * Maskp(ig + 1, jg + 1);
          // integer + default-real literal is evaluated in single precision
          Hc(i, j) = num / (double)((float)ms + 1.e-16f);
        }
    } else {
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i)
          Hc(i, j) = depth[(size_t)(i - Nghost - 1) + (size_t)Mg * (j - Nghost - 1)];
    }
    phi_2D_coll(Hc);
    Hc0 = Hc;
    if (p.slide_type == NHW_SLIDE_RIGID_3D) slide_shape_rigid3d(p.slide_x0, p.slide_y0);
    for (int j = 1; j <= Nloc; ++j)
      for (int i = 1; i <= Mloc; ++i) Mask_Struct(i, j) = 1;
    for (int j = Jbeg; j <= Jend; ++j)
      for (int i = Ibeg; i <= Iend; ++i)
        if (Hc(i, j) < -1000.0) Mask_Struct(i, j) = 0;
    for (int j = 1; j <= Nloc; ++j) {
      for (int i = 2; i <= Mloc; ++i) Hfx(i, j) = 0.5 * (Hc(i - 1, j) + Hc(i, j));
      Hfx(1, j) = Hc(1, j);
      Hfx(Mloc1, j) = Hc(Mloc, j);
    }
    Hfx0 = Hfx;
    for (int i = 1; i <= Mloc; ++i) {
      for (int j = 2; j <= Nloc; ++j) Hfy(i, j) = 0.5 * (Hc(i, j - 1) + Hc(i, j));
      Hfy(i, 1) = Hc(i, 1);
      Hfy(i, Nloc1) = Hc(i, Nloc);
    }
    Hfy0 = Hfy;
    for (int j = 1; j <= Nloc; ++j)
      for (int i = 1; i <= Mloc; ++i) {
        DelxH(i, j) = (Hfx(i + 1, j) - Hfx(i, j)) / dx;
        DelyH(i, j) = (Hfy(i, j + 1) - Hfy(i, j)) / dy;
      }
  }

  // -------------------------------------------------------------- initial
  void update_wind() {
    // Iws = 1 (src/nhwave.F:5343-5398); constant in time for a constant wind
    const double Cdsmin = (double)(1.e-3f * (0.61f + 0.063f * 6.0f));
    const double Cdsmax = (double)(1.e-3f * (0.61f + 0.063f * 50.0f));
    for (int j = Jbeg; j <= Jend; ++j)
      for (int i = Ibeg; i <= Iend; ++i) {
        double WdU = p.wind_u, WdV = p.wind_v;
        double Wds = std::sqrt(WdU * WdU + WdV * WdV);
        double Cds = (double)1.e-3f * ((double)0.61f + (double)0.063f * Wds);
        Cds = dmin(dmax(Cds, Cdsmin), Cdsmax);
        Wsx(i, j) = (double)0.001293f * Cds * WdU * Wds;
        Wsy(i, j) = (double)0.001293f * Cds * WdV * Wds;
      }
  }

  void calculate_sponge() {
    if (p.sponge_west_width > Zero)
      for (int j = 1; j <= Nloc; ++j)
        for (int i = 1; i <= Mloc; ++i)
          if (xc(i) <= p.sponge_west_width) {
            double t = (xc(i) - p.sponge_west_width) / p.sponge_west_width;
            Sponge(i, j) = std::sqrt(1.0 - dmin(t * t, 1.0));
          }
    if (p.sponge_east_width > Zero)
      for (int j = 1; j <= Nloc; ++j)
        for (int i = 1; i <= Mloc; ++i)
          if (xc(i) >= p.Mglob * dx - p.sponge_east_width) {
            double t = (xc(i) - (p.Mglob * dx - p.sponge_east_width)) / p.sponge_east_width;
            Sponge(i, j) = std::sqrt(1.0 - dmin(t * t, 1.0));
          }
    if (p.sponge_south_width > Zero)
      for (int j = 1; j <= Nloc; ++j)
        for (int i = 1; i <= Mloc; ++i)
          if (yc(j) <= p.sponge_south_width) {
            double t = (yc(j) - p.sponge_south_width) / p.sponge_south_width;
            Sponge(i, j) = std::sqrt(1.0 - dmin(t * t, 1.0));
          }
    if (p.sponge_north_width > Zero)
      for (int j = 1; j <= Nloc; ++j)
        for (int i = 1; i <= Mloc; ++i)
          if (yc(j) >= p.Nglob * dy - p.sponge_north_width) {
            double t = (yc(j) - (p.Nglob * dy - p.sponge_north_width)) / p.sponge_north_width;
            Sponge(i, j) = std::sqrt(1.0 - dmin(t * t, 1.0));
          }
  }

  void initial(const double* eta0, const double* uvw0) {
    TIME = Zero; RUN_STEP = 0; dt = p.dt_ini;
    Sponge.fill(1.0);
    Cmu = p.visc; CmuR = 0.0; CmuVt.fill(0.0); CmuHt.fill(0.0);
    Eta.fill(0.0);
    const int Mg = p.Mglob, Ng = p.Nglob, Kg = p.Kglob;
    if (eta0 || uvw0) {
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i) {
          size_t g = (size_t)(i - Nghost - 1) + (size_t)Mg * (j - Nghost - 1);
          if (eta0) Eta(i, j) = eta0[g];
          if (uvw0)
            for (int k = Kbeg; k <= Kend; ++k) {
              size_t g3 = g + (size_t)Mg * Ng * (k - Nghost - 1);
              U(i, j, k) = uvw0[g3];
              V(i, j, k) = uvw0[g3 + (size_t)Mg * Ng * Kg];
              W(i, j, k) = uvw0[g3 + 2 * (size_t)Mg * Ng * Kg];
            }
        }
    }
    for (int j = 1; j <= Nloc; ++j)
      for (int i = 1; i <= Mloc; ++i) {
        if ((Eta(i, j) + Hc(i, j)) <= MinDep) { Mask(i, j) = 0; Eta(i, j) = MinDep - Hc(i, j); }
        else Mask(i, j) = 1;
      }
    for (int j = 1; j <= Nloc; ++j)
      for (int i = 1; i <= Mloc; ++i) Mask(i, j) = Mask(i, j) * Mask_Struct(i, j);
    phi_2D_coll(Eta);
    Eta0 = Eta;
    compute_mask9();
    for (int j = 1; j <= Nloc; ++j)
      for (int i = 1; i <= Mloc; ++i) D(i, j) = dmax(Hc(i, j) + Eta(i, j), MinDep);
    update_wind();
    vel_bc();
    for (int k = 1; k <= Kloc; ++k)
      for (int j = 1; j <= Nloc; ++j)
        for (int i = 1; i <= Mloc; ++i) {
          DU(i, j, k) = D(i, j) * U(i, j, k) * Mask(i, j);
          DV(i, j, k) = D(i, j) * V(i, j, k) * Mask(i, j);
          DW(i, j, k) = D(i, j) * W(i, j, k) * Mask(i, j);
        }
    // seeding values (src/initialize.F:3172-3195), after vel_bc, which so
    // saw CmuVt = 0; DTke0 = DEps0 = 0 (:2950-2951)
    if (p.viscous_flow) {
      Cmut_min = (p.rng ? (double)8.5e-2f : (double)9.0e-2f) * (Tke_min * Tke_min) / Eps_min;
      CmuHt.fill(Cmut_min);
      CmuVt.fill(Cmut_min);
      Tke.fill(Tke_min);
      Eps.fill(Eps_min);
      for (int k = 1; k <= Kloc; ++k)
        for (int j = 1; j <= Nloc; ++j)
          for (int i = 1; i <= Mloc; ++i) {
            DTke(i, j, k) = D(i, j) * Tke(i, j, k) * Mask(i, j);
            DEps(i, j, k) = D(i, j) * Eps(i, j, k) * Mask(i, j);
          }
      DTke0.fill(0.0);
      DEps0.fill(0.0);
    }
    if (p.time_order == 3) {
      It_Order = 3;
      ALPHA[0] = 0.0; ALPHA[1] = (double)(3.0f / 4.0f); ALPHA[2] = (double)(1.0f / 3.0f);
      BETA[0] = 1.0; BETA[1] = (double)(1.0f / 4.0f); BETA[2] = (double)(2.0f / 3.0f);
    } else if (p.time_order == 2) {
      It_Order = 2;
      ALPHA[0] = 0.0; ALPHA[1] = (double)(1.0f / 2.0f); BETA[0] = 1.0; BETA[1] = (double)(1.0f / 2.0f);
    } else {
      It_Order = 1; ALPHA[0] = 0.0; BETA[0] = 1.0;
    }
    if (p.sponge_on) calculate_sponge();
  }

  void compute_mask9() {
    for (int j = Jbeg; j <= Jend; ++j)
      for (int i = Ibeg; i <= Iend; ++i)
        Mask9(i, j) = Mask(i, j) * Mask(i - 1, j) * Mask(i + 1, j) * Mask(i + 1, j + 1) * Mask(i, j + 1) *
                      Mask(i - 1, j + 1) * Mask(i + 1, j - 1) * Mask(i, j - 1) * Mask(i - 1, j - 1);
  }

  // ---------------------------------------------------------- estimate_dt
  int estimate_dt() {
    dt_old = dt;
    const double dt_growth = (double)1.05f * dt_old;
    double tmp2 = Large;
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i) {
          double tmp1 = std::fabs(U(i, j, k)) + std::sqrt(Grav * D(i, j));
          tmp1 = dmax(tmp1, Small);
          double dxonu = dx / tmp1;
          if (dxonu < tmp2) tmp2 = dxonu;
          tmp1 = std::fabs(V(i, j, k)) + std::sqrt(Grav * D(i, j));
          tmp1 = dmax(tmp1, Small);
          double dyonv = dy / tmp1;
          if (dyonv < tmp2) tmp2 = dyonv;
          tmp1 = dmax(std::fabs(W(i, j, k)), Small);
          double dzonw = dsig(k) * D(i, j) / tmp1;
          if (dzonw < tmp2) tmp2 = dzonw;
        }
    const double dt_courant = p.cfl * tmp2;
    // limit of the explicit viscous terms (src/nhwave.F:3812-3832)
    double dt_viscous = Large;
    if (p.viscous_flow) {
      tmp2 = Large;
      for (int k = Kbeg; k <= Kend; ++k)
        for (int j = Jbeg; j <= Jend; ++j)
          for (int i = Ibeg; i <= Iend; ++i) {
            double tmp1 = dx * dx / (std::fabs(CmuHt(i, j, k)) + (double)1.e-16f);
            if (tmp1 < tmp2) tmp2 = tmp1;
            tmp1 = dy * dy / (std::fabs(CmuHt(i, j, k)) + (double)1.e-16f);
            if (tmp1 < tmp2) tmp2 = tmp1;
          }
      dt_viscous = p.viscous_number * tmp2;
    }
    dt = dmin(dmin(dmin(dt_growth, dt_courant), dt_viscous), p.dt_max);
    if (dt < p.dt_min) return NHW_ERR_DT_MIN;
    TIME = TIME + dt;
    RUN_STEP = RUN_STEP + 1;
    return NHW_OK;
  }

  // ---------------------------------------------------- update_bathymetry
  double hc_ext(int i, int j) {
    // Hfx/Hfy below read Hc(Mloc+1,j) and Hc(i,Nloc+1): past the column, the
    // Fortran storage continues with Hc(1,j+1); past the array it is undefined
    // and taken as 0 here.  Only ghost-face values depend on it.
    if (i == Mloc + 1) { i = 1; ++j; }
    if (j > Nloc) return 0.0;
    return Hc(i, j);
  }

  void update_bathymetry() {
    Ho = Hc;
    if (p.slide_type == NHW_SLIDE_RIGID_3D) {
      const double alpha0 = p.slide_angle * pi / 180.;
      const double slope0 = p.slope_angle * pi / 180.;
      const double ut = p.slide_ut, a0 = p.slide_a0;
      const double t0 = ut / a0;
      const double s0 = ut * ut / a0;
      const double st = s0 * std::log(std::cosh(TIME / t0)) * std::cos(slope0);
      const double x0 = p.slide_x0 + st * std::cos(alpha0);
      const double y0 = p.slide_y0 + st * std::sin(alpha0);
      slide_shape_rigid3d(x0, y0);
    }
    phi_2D_coll(Hc);
    for (int j = 1; j <= Nloc; ++j) {
      for (int i = 2; i <= Mloc; ++i) Hfx(i, j) = 0.5 * (Hc(i, j) + hc_ext(i + 1, j));
      Hfx(1, j) = Hfx(2, j);
      Hfx(Mloc1, j) = Hfx(Mloc, j);
    }
    Hfx0 = Hfx;
    for (int i = 1; i <= Mloc; ++i) {
      for (int j = 2; j <= Nloc; ++j) Hfy(i, j) = 0.5 * (Hc(i, j) + hc_ext(i, j + 1));
      Hfy(i, 1) = Hfy(i, 2);
      Hfy(i, Nloc1) = Hfy(i, Nloc);
    }
    Hfy0 = Hfy;
    for (int j = 1; j <= Nloc; ++j)
      for (int i = 1; i <= Mloc; ++i) {
        DelxH(i, j) = (Hfx(i + 1, j) - Hfx(i, j)) / dx;
        DelyH(i, j) = (Hfy(i, j + 1) - Hfy(i, j)) / dy;
      }
    DeltHo = DeltH;
    for (int j = 1; j <= Nloc; ++j)
      for (int i = 1; i <= Mloc; ++i) DeltH(i, j) = (Hc(i, j) - Ho(i, j)) / dt;
    if (RUN_STEP > 2)
      for (int j = 1; j <= Nloc; ++j)
        for (int i = 1; i <= Mloc; ++i) Delt2H(i, j) = (DeltH(i, j) - DeltHo(i, j)) / dt;
  }

  // ---------------------------------------------------------- update_mask
  void update_mask() {
    I2 Masktmp = Mask;
    const double thr = (double)1.e-6f;
    for (int j = Jbeg; j <= Jend; ++j)
      for (int i = Ibeg; i <= Iend; ++i) {
        if (Mask_Struct(i, j) == 0) continue;
        if (Mask(i, j) == 0) {
          if (Mask(i - 1, j) == 1 && Eta(i - 1, j) > Eta(i, j) && D(i - 1, j) - MinDep > thr) Masktmp(i, j) = 1;
          if (Mask(i + 1, j) == 1 && Eta(i + 1, j) > Eta(i, j) && D(i + 1, j) - MinDep > thr) Masktmp(i, j) = 1;
          if (Mask(i, j - 1) == 1 && Eta(i, j - 1) > Eta(i, j) && D(i, j - 1) - MinDep > thr) Masktmp(i, j) = 1;
          if (Mask(i, j + 1) == 1 && Eta(i, j + 1) > Eta(i, j) && D(i, j + 1) - MinDep > thr) Masktmp(i, j) = 1;
        } else {
          if (std::fabs(D(i, j) - MinDep) <= thr) {
            Masktmp(i, j) = 0;
            Eta(i, j) = MinDep - Hc(i, j);
            D(i, j) = Eta(i, j) + Hc(i, j);
          }
        }
      }
    for (int j = 1; j <= Nloc; ++j)
      for (int i = 1; i <= Mloc; ++i) Mask(i, j) = Masktmp(i, j) * Mask_Struct(i, j);
    compute_mask9();
  }

  // update_vars (src/nhwave.F:5459-5511): the time levels the step reads.
  // Eta00, U00/V00/W00 and U0/V0/W0 feed only the Orlanski boundary, and
  // start as zero (the reference never initialises them)
  void update_vars() {
    Eta00 = Eta0; U00 = U0; V00 = V0; W00 = W0;
    D0 = D; Eta0 = Eta; U0 = U; V0 = V; W0 = W; DU0 = DU; DV0 = DV; DW0 = DW;
    if (p.viscous_flow) { DTke0 = DTke; DEps0 = DEps; }   // src/nhwave.F:5483-5484
  }

  // --------------------------------------------------------- source_terms
  double wave_dispersion(double Segma) {
    const double Dep = p.dep_wave;
    double Wn = (Segma * Segma) / (Grav * std::pow(std::tanh(Segma * Segma * Dep / Grav), 0.5));
    double error = 100.;
    while (error >= (double)1.0e-8f) {
      double Fk = Segma * Segma - Grav * Wn * std::tanh(Wn * Dep);
      double ch = std::cosh(Wn * Dep);
      double Fkdif = -(Grav * (std::tanh(Wn * Dep) + (Wn * Dep) / (ch * ch)));
      double Wn_new = Wn - Fk / Fkdif;
      error = std::fabs((Wn - Wn_new) / Wn);
      Wn = Wn_new;
    }
    return Wn;
  }

  // FOCUSED wave group components (src/initialize.F:742-781)
  std::vector<double> Amp_i, k_i, f_i;

  // JONSWAP / TMA spectrum (src/initialize.F:880-941): Freq(i) at the centres
  // of NumFreq bands over [Freq_Min, Freq_Max], Jon_Spc(i) scaled to
  // m0 = Hm0^2/16, and the phases RanPhs(i).  The reference draws RanPhs with
  // the compiler's rand(); here they are element i + 1 of a SplitMix64
  // stream from WAVE_SEED, times 2 pi, unless set_wave_phases gives them.
  std::vector<double> Freq, Jon_Spc, RanPhs;
  static double phase_of(int32_t seed, int i) {
    uint64_t z = (uint64_t)(uint32_t)seed + (uint64_t)(i + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * 0x1.0p-53 * 2.0 * pi;
  }
  void jonswap_spectrum() {
    const int NumFreq = p.numfreq;
    const double Dep_Wave = p.dep_wave;
    const double gam = (double)3.3f, sa = (double)0.07f, sb = (double)0.09f;
    const double Freq_Peak = 1.0 / p.tp;
    const double DFreq = (p.freq_max - p.freq_min) / NumFreq;
    Freq.assign(NumFreq, 0.0); Jon_Spc.assign(NumFreq, 0.0); RanPhs.assign(NumFreq, 0.0);
    for (int i = 1; i <= NumFreq; ++i) {
      Freq[i - 1] = p.freq_min + 0.5 * DFreq + (i - 1) * DFreq;
      const double Per_Wave = 1.0 / Freq[i - 1];
      const double Segma = 2.0 * pi / Per_Wave;
      const double Celerity = std::sqrt(Grav * Dep_Wave);
      const double Wave_Length = Celerity * Per_Wave;
      double Wave_Number = 2.0 * pi / Wave_Length;
      int Iter = 0;
      while (true) {
        const double Fk = Grav * Wave_Number * std::tanh(Wave_Number * Dep_Wave) - Segma * Segma;
        if (std::fabs(Fk) <= (double)1.0e-8f || Iter > 1000) break;
        const double th = std::tanh(Wave_Number * Dep_Wave);
        const double Fkdif = Grav * Wave_Number * Dep_Wave * (1.0 - th * th) + Grav * std::tanh(Wave_Number * Dep_Wave);
        Wave_Number = Wave_Number - Fk / Fkdif;
        Iter = Iter + 1;
      }
      const double F = Freq[i - 1], r = Freq_Peak / F;
      const double s2 = F < Freq_Peak ? sa * sa : sb * sb;
      Jon_Spc[i - 1] = (Grav * Grav) / ((F * F) * (F * F) * F) * std::exp(-1.25 * ((r * r) * (r * r))) *
                       std::pow(gam, std::exp(-0.5 * ((F / Freq_Peak - 1.0) * (F / Freq_Peak - 1.0)) / s2));
      if (p.wavemaker == NHW_WM_LEF_TMA || p.wavemaker == NHW_WM_INT_TMA) {
        const double th = std::tanh(Wave_Number * Dep_Wave);
        Jon_Spc[i - 1] = Jon_Spc[i - 1] * (th * th) /
                         (1.0 + 2 * Wave_Number * Dep_Wave / std::sinh(2. * Wave_Number * Dep_Wave));
      }
    }
    double SumInt = Zero;
    for (int i = 0; i < NumFreq; ++i) SumInt = SumInt + Jon_Spc[i] * DFreq;
    const double A_Jon = (p.hm0 * p.hm0) / 16.0 / SumInt;
    for (int i = 0; i < NumFreq; ++i) {
      Jon_Spc[i] = Jon_Spc[i] * A_Jon;
      RanPhs[i] = phase_of(p.wave_seed, i);
    }
  }

  // LEF_SPC's spectrum (src/initialize.F:783-830): Freq, Dire, Wave_Spc2d
  // and Random_Phs as (ndir, nfreq) arrays, direction fastest
  int NumFreq_s = 0, NumDir_s = 0;
  std::vector<double> Freq_s, Dire_s, Spc2d, Random_Phs;

  // random_wave_left_boundary (src/waves.F:376-513).  The angle adjustment
  // for periodic lateral sides is skipped by the reference's `goto 100`
  // (:398), so the direction is Dire itself.
  void random_left_boundary() {
    const int NumFreq = NumFreq_s, NumDir = NumDir_s;
    const double Dep_Wave = p.dep_wave;
    std::vector<double> Wtheta(NumFreq * NumDir), Wh(NumFreq * NumDir), Stokes_Drift(NumFreq * NumDir),
        Wnum(NumFreq * NumDir);
    auto at = [&](int nd, int nfq) { return (nd - 1) + NumDir * (nfq - 1); };
    for (int nfq = 1; nfq <= NumFreq; ++nfq)
      for (int nd = 1; nd <= NumDir; ++nd) {
        const double Per_Wave = 1.0 / Freq_s[nfq - 1];
        const double Segma = 2.0 * pi / Per_Wave;
        const double Wave_Number = wave_dispersion(Segma);
        const double Wave_Length = 2.0 * pi / Wave_Number;
        const double Angle = Dire_s[nd - 1] * pi / 180.;
        Wtheta[at(nd, nfq)] = Angle;
        double dfreq;
        if (nfq == 1) dfreq = Freq_s[1] - Freq_s[0];
        else if (nfq == NumFreq) dfreq = Freq_s[NumFreq - 1] - Freq_s[NumFreq - 2];
        else dfreq = 0.5 * (Freq_s[nfq] - Freq_s[nfq - 2]);
        dfreq = std::fabs(dfreq);
        double ddir;
        if (nd == 1) ddir = Dire_s[1] - Dire_s[0];
        else if (nd == NumDir) ddir = Dire_s[NumDir - 1] - Dire_s[NumDir - 2];
        else ddir = 0.5 * (Dire_s[nd] - Dire_s[nd - 2]);
        ddir = std::fabs(ddir);
        Wnum[at(nd, nfq)] = Wave_Number;
        Wh[at(nd, nfq)] = 2.0 * std::sqrt(2.0 * Spc2d[at(nd, nfq)] * dfreq * ddir);
        Stokes_Drift[at(nd, nfq)] =
            Grav * (Wh[at(nd, nfq)] * Wh[at(nd, nfq)]) / (Wave_Length / Per_Wave) / Dep_Wave / 8.0;
      }
    const double Fact = 1.0;
    for (int j = 1; j <= Nloc; ++j) {
      Ein_X0(j) = 0.0;
      for (int nfq = 1; nfq <= NumFreq; ++nfq)
        for (int nd = 1; nd <= NumDir; ++nd) {
          const int c = at(nd, nfq);
          const double Segma = 2.0 * pi * Freq_s[nfq - 1];
          const double Phs_Lag = yc(j) * std::sin(Wtheta[c]) * Wnum[c] + Random_Phs[c];
          Ein_X0(j) = Ein_X0(j) + 0.5 * Wh[c] * std::cos(pi / 2 - Segma * TIME + Phs_Lag);
        }
      Ein_X0(j) = Ein_X0(j) * std::tanh(TIME / 20.0);
      Din_X0(j) = Ein_X0(j) + Hfx(Ibeg, j);
    }
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j) {
        const double Zlev = sigc(k) * Din_X0(j);
        Uin_X0(j, k) = 0.0;
        Win_X0(j, k) = 0.0;
        Vin_X0(j, k) = 0.0;
        for (int nfq = 1; nfq <= NumFreq; ++nfq)
          for (int nd = 1; nd <= NumDir; ++nd) {
            const int c = at(nd, nfq);
            const double Segma = 2.0 * pi * Freq_s[nfq - 1];
            const double Phs_Lag = yc(j) * std::sin(Wtheta[c]) * Wnum[c] + Random_Phs[c];
            const double sh = std::sinh(Wnum[c] * Dep_Wave);
            const double arg = pi / 2 - Segma * TIME + Phs_Lag;
            Uin_X0(j, k) = Uin_X0(j, k) +
                           (0.5 * Wh[c] * Segma * std::cosh(Wnum[c] * Zlev) / sh * std::cos(arg) - Stokes_Drift[c] * Fact) *
                               std::cos(Wtheta[c]);
            Win_X0(j, k) = Win_X0(j, k) + 0.5 * Wh[c] * Segma * std::sinh(Wnum[c] * Zlev) / sh * std::sin(arg);
            Vin_X0(j, k) = Vin_X0(j, k) +
                           (0.5 * Wh[c] * Segma * std::cosh(Wnum[c] * Zlev) / sh * std::cos(arg) - Stokes_Drift[c] * Fact) *
                               std::sin(Wtheta[c]);
          }
      }
  }

  // jonswap_wave_left_boundary (src/waves.F:566-623).  The reference calls
  // wave_dispersion with three arguments where it takes two (src/waves.F:585),
  // which leaves its Wave_Number undefined; each component's wave number here
  // is wave_dispersion's, as random_wave_left_boundary computes it (:395).
  void jonswap_left_boundary() {
    const int NumFreq = p.numfreq;
    const double Dep_Wave = p.dep_wave;
    std::vector<double> Wh(NumFreq), Wnum(NumFreq), Stokes_Drift(NumFreq);
    const double dfreq = (p.freq_max - p.freq_min) / (double)(float)NumFreq;
    for (int n = 0; n < NumFreq; ++n) {
      const double Per_Wave = 1.0 / Freq[n];
      const double Segma = 2.0 * pi / Per_Wave;
      const double Wave_Number = wave_dispersion(Segma);
      const double Wave_Length = 2.0 * pi / Wave_Number;
      Wh[n] = 2.0 * std::sqrt(2.0 * Jon_Spc[n] * dfreq);
      Wnum[n] = Wave_Number;
      Stokes_Drift[n] = Grav * (Wh[n] * Wh[n]) / (Wave_Length / Per_Wave) / Dep_Wave / 8.0;
    }
    const double Fact = 1.0;
    for (int j = 1; j <= Nloc; ++j) {
      Ein_X0(j) = 0.0;
      for (int n = 0; n < NumFreq; ++n) {
        const double Segma = 2.0 * pi * Freq[n];
        Ein_X0(j) = Ein_X0(j) + 0.5 * Wh[n] * std::cos(pi / 2 - Segma * TIME + RanPhs[n]);
      }
      Din_X0(j) = Ein_X0(j) + Hfx(Ibeg, j);
    }
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j) {
        const double Zlev = sigc(k) * Din_X0(j);
        Uin_X0(j, k) = 0.0;
        Win_X0(j, k) = 0.0;
        Vin_X0(j, k) = 0.0;
        for (int n = 0; n < NumFreq; ++n) {
          const double Segma = 2.0 * pi * Freq[n];
          const double sh = std::sinh(Wnum[n] * Dep_Wave);
          Uin_X0(j, k) = Uin_X0(j, k) +
                         0.5 * Wh[n] * Segma * std::cosh(Wnum[n] * Zlev) / sh * std::cos(pi / 2 - Segma * TIME + RanPhs[n]) -
                         Stokes_Drift[n] * Fact;
          Win_X0(j, k) = Win_X0(j, k) +
                         0.5 * Wh[n] * Segma * std::sinh(Wnum[n] * Zlev) / sh * std::sin(pi / 2 - Segma * TIME + RanPhs[n]);
          Vin_X0(j, k) = 0.0;
        }
      }
  }

  // Start phase of the cnoidal boundary wave (src/waves.F:106-130):
  // bisection on [0, 1] for the zero crossing of the elevation.
  bool cnoidal_start(double Ytrough, double Mod1, double& Xstart) {
    double Zup = 1.0, Zlow = 0.0, Zmid = (Zup + Zlow) / 2.0;
    int nn = 0;
    while (true) {
      nn = nn + 1;
      const double cn = cnoidal_cn(Zmid * 0.5 * cnoidal_ck(Mod1), Mod1);
      const double Zero1 = Ytrough + p.amp_wave * (cn * cn);
      if (std::fabs(Zero1) <= (double)1.0e-6f) break;
      if (nn > 1000) return false;
      if (Zero1 < 0.0) {
        Zup = Zmid;
        Zmid = (Zup + Zlow) / 2.0;
      } else {
        Zlow = Zmid;
        Zmid = (Zup + Zlow) / 2.0;
      }
    }
    Xstart = Zmid;
    return true;
  }

  // ------------------------------------------------------ update_wave_bc
  // Linear (LEF_LIN, src/waves.F:808-855), solitary (LEF_SOL, :869-903),
  // second-order Stokes (LEF_STK, :518-560) and cnoidal (LEF_CON, :92-170)
  // waves fed through the west boundary (src/nhwave.F:5514-5565), evaluated
  // at the new TIME once per step.
  void update_wave_bc() {
    if (p.wavemaker == NHW_WM_LEF_LIN || p.wavemaker == NHW_WM_WAV_CUR) {
      // WAV_CUR (src/waves.F:706-756) is LEF_LIN plus the current
      // Ucur = tanh(TIME/TRamp) Cur_Wave in the horizontal velocities
      double Ucur = 0.0;
      if (p.wavemaker == NHW_WM_WAV_CUR) Ucur = (p.tramp > 0.0 ? std::tanh(TIME / p.tramp) : 1.0) * p.cur_wave;
      const double Segma = 2.0 * pi / p.per_wave;
      const double Wave_Number = wave_dispersion(Segma);
      const double Wave_Length = 2.0 * pi / Wave_Number;
      const double Stokes_Drift = Grav * (p.amp_wave * p.amp_wave) / (Wave_Length / p.per_wave) / p.dep_wave / 8.0;
      const double Fact = 1.0;
      const double th = p.theta_wave * pi / 180.;
      for (int j = 1; j <= Nloc; ++j) {
        const double Phs_Lag = yc(j) * std::sin(th) * Wave_Number;
        Ein_X0(j) = 0.5 * p.amp_wave * std::cos(pi / 2 - Segma * TIME + Phs_Lag);
        Din_X0(j) = Ein_X0(j) + Hfx(Ibeg, j);
      }
      const double shd = std::sinh(Wave_Number * p.dep_wave);
      for (int k = Kbeg; k <= Kend; ++k)
        for (int j = Jbeg; j <= Jend; ++j) {
          const double Phs_Lag = yc(j) * std::sin(th) * Wave_Number;
          const double Zlev = sigc(k) * Din_X0(j);
          const double cs = std::cos(pi / 2 - Segma * TIME + Phs_Lag);
          const double sn = std::sin(pi / 2 - Segma * TIME + Phs_Lag);
          Uin_X0(j, k) = (Ucur + 0.5 * p.amp_wave * Segma * std::cosh(Wave_Number * Zlev) / shd * cs - Stokes_Drift * Fact) *
                         std::cos(th);
          Win_X0(j, k) = 0.5 * p.amp_wave * Segma * std::sinh(Wave_Number * Zlev) / shd * sn;
          Vin_X0(j, k) = (Ucur + 0.5 * p.amp_wave * Segma * std::cosh(Wave_Number * Zlev) / shd * cs - Stokes_Drift * Fact) *
                         std::sin(th);
        }
    } else if (p.wavemaker == NHW_WM_LEF_SOL) {
      Uin_X0.fill(0.0); Vin_X0.fill(0.0); Win_X0.fill(0.0);
      const double A = p.amp_wave, Dep = p.dep_wave;
      const double Celerity = std::sqrt(Grav * Dep * (1.0 + A / Dep));
      for (int j = 1; j <= Nloc; ++j) {
        const double Atmp = std::sqrt((double)0.75f * A / (Dep * Dep * Dep));
        const double Xstart = 4.0 * Dep / std::sqrt(A / Dep);
        const double Xc = Xstart - Celerity * TIME;
        const double ch = std::cosh(Atmp * Xc), sh = std::sinh(Atmp * Xc);
        const double ch2 = ch * ch, ch3 = ch * ch2, ch4 = ch2 * ch2, ch5 = ch * ch4;
        Ein_X0(j) = A / ch2;
        Din_X0(j) = Ein_X0(j) + Hfx(Ibeg, j);
        const double C2 = std::sqrt(Grav * Dep);
        const double D2 = 2.0 * A * (Atmp * Atmp) * (2.0 * ch2 - 3.) / ch4;
        const double D1 = -2.0 * A * sh * Atmp / ch3;
        const double D3 = -8.0 * A * sh * (Atmp * Atmp * Atmp) * (ch2 - 3.) / ch5;
        if (j < Jbeg || j > Jend) continue;
        for (int k = Kbeg; k <= Kend; ++k) {
          const double Zlev = sigc(k) * Din_X0(j);
          const double E = Ein_X0(j);
          Uin_X0(j, k) = C2 * E / Dep *
                         (1.0 - 0.25 * E / Dep + Dep / 3.0 * (Dep / E) * (1.0 - 1.5 * (Zlev * Zlev) / (Dep * Dep)) * D2);
          Win_X0(j, k) = -C2 * Zlev / Dep *
                         ((1.0 - 0.5 * E / Dep) * D1 +
                          (double)(1.0f / 3.0f) * (Dep * Dep) * (1.0 - 0.5 * (Zlev * Zlev) / (Dep * Dep)) * D3);
          Vin_X0(j, k) = 0.0;
        }
      }
    } else if (p.wavemaker == NHW_WM_LEF_STK) {
      const double A = p.amp_wave, Dep = p.dep_wave;
      const double Segma = 2.0 * pi / p.per_wave;
      const double Wave_Number = wave_dispersion(Segma);
      const double sh = std::sinh(Wave_Number * Dep);
      for (int j = 1; j <= Nloc; ++j) {
        Ein_X0(j) = 0.5 * A * std::cos(pi / 2 - Segma * TIME) +
                    (A * A) * Wave_Number / 16. * std::cosh(Wave_Number * Dep) / (sh * sh * sh) *
                        (2.0 + std::cosh(2. * Wave_Number * Dep)) * std::cos(2. * (pi / 2 - Segma * TIME));
        Din_X0(j) = Ein_X0(j) + Hfx(Ibeg, j);
      }
      const double sh4 = (sh * sh) * (sh * sh);
      for (int k = Kbeg; k <= Kend; ++k)
        for (int j = Jbeg; j <= Jend; ++j) {
          const double Zlev = sigc(k) * Din_X0(j);
          Uin_X0(j, k) = 0.5 * A * Segma * std::cosh(Wave_Number * Zlev) / sh * std::cos(pi / 2 - Segma * TIME) +
                         3. / 16. * (A * A) * Segma * Wave_Number * std::cosh(2. * Wave_Number * Zlev) / sh4 *
                             std::cos(2. * (pi / 2 - Segma * TIME));
          Win_X0(j, k) = 0.5 * A * Segma * std::sinh(Wave_Number * Zlev) / sh * std::sin(pi / 2 - Segma * TIME) +
                         3. / 16. * (A * A) * Segma * Wave_Number * std::sinh(2. * Wave_Number * Zlev) / sh4 *
                             std::sin(2. * (pi / 2 - Segma * TIME));
          Vin_X0(j, k) = 0.0;
        }
    } else if (p.wavemaker == NHW_WM_LEF_TID) {   // tidal_wave_left_boundary (src/nhwave.F:5715-5750)
      const double period1 = 43200.;   // S2 (the first of the routine's eight periods)
      for (int j = 1; j <= Nloc; ++j) {
        Ein_X0(j) = 0.5 * p.amp_wave * std::cos(2.0 * pi / period1 * TIME - pi / 2.0);
        Din_X0(j) = Ein_X0(j) + Hfx(Ibeg, j);
      }
      for (int k = Kbeg; k <= Kend; ++k)
        for (int j = Jbeg; j <= Jend; ++j) {
          Uin_X0(j, k) = std::sqrt(Grav / Hfx(Ibeg, j)) * Ein_X0(j);
          Vin_X0(j, k) = 0.0;
          Win_X0(j, k) = 0.0;
        }
    } else if (p.wavemaker == NHW_WM_FOCUSED) {   // src/waves.F:638-692
      const int nw = p.nwave;
      const double tc = TIME - (double)(int)(TIME / 20.0) * 20.0;
      std::vector<double> Segma_i(nw), c_i(nw), eta_i(nw), Stokes_Drift_i(nw);
      for (int n = 0; n < nw; ++n) {
        Segma_i[n] = 2. * pi * f_i[n];
        c_i[n] = Segma_i[n] / k_i[n];
        eta_i[n] = Amp_i[n] * std::cos(-k_i[n] * p.x_breaking - Segma_i[n] * (tc - p.t_breaking));
        Stokes_Drift_i[n] = Grav * (Amp_i[n] * Amp_i[n]) / c_i[n] / p.depth_comp / 2.;
      }
      for (int j = 1; j <= Nloc; ++j) {
        Ein_X0(j) = Zero;
        for (int n = 0; n < nw; ++n) Ein_X0(j) = Ein_X0(j) + eta_i[n];
        Din_X0(j) = Ein_X0(j) + Hfx(Ibeg, j);
      }
      const double dc = p.depth_comp;
      for (int k = Kbeg; k <= Kend; ++k)
        for (int j = Jbeg; j <= Jend; ++j) {
          const double Zlev = sigc(k) * Din_X0(j);
          Uin_X0(j, k) = Zero;
          Win_X0(j, k) = Zero;
          for (int n = 0; n < nw; ++n) {
            const double ph = -k_i[n] * p.x_breaking - Segma_i[n] * (tc - p.t_breaking);
            Uin_X0(j, k) = Uin_X0(j, k) +
                           Grav * Amp_i[n] * k_i[n] / Segma_i[n] * std::cosh(k_i[n] * Zlev) /
                               std::cosh(k_i[n] * (dc + Ein_X0(j))) * std::cos(ph) -
                           Stokes_Drift_i[n] * (2 * k_i[n] * dc) / std::sinh(2 * k_i[n] * (dc + Ein_X0(j))) *
                               std::cosh(2 * k_i[n] * Zlev) * p.sd_return;
            Win_X0(j, k) = Win_X0(j, k) + Grav * Amp_i[n] * k_i[n] / Segma_i[n] * std::sinh(k_i[n] * Zlev) /
                                              std::cosh(k_i[n] * (dc + Ein_X0(j))) * std::sin(ph);
          }
          Vin_X0(j, k) = Zero;
        }
    } else if (p.wavemaker == NHW_WM_LEF_CON) {
      const double A = p.amp_wave, Dep = p.dep_wave;
      double Wave_Length = 0, Ytrough = 0, Mod1 = 0, Xstart = 0;
      cnoidal(A, Dep, p.per_wave, Wave_Length, Ytrough, Mod1);   // checked at create
      cnoidal_start(Ytrough, Mod1, Xstart);
      const double ck = cnoidal_ck(Mod1);
      for (int j = 1; j <= Nloc; ++j) {
        const double cn = cnoidal_cn(Xstart * 0.5 * ck + 2.0 * ck * (-(TIME / p.per_wave)), Mod1);
        Ein_X0(j) = Ytrough + A * (cn * cn);
        Din_X0(j) = Ein_X0(j) + Hfx(Ibeg, j);
      }
      const double Stokes_Drift = Grav * (A * A) / (Wave_Length / p.per_wave) / Dep / 8.0;
      const double Fact = 1.0;
      for (int k = Kbeg; k <= Kend; ++k)
        for (int j = Jbeg; j <= Jend; ++j) {
          const double Zlev = sigc(k) * Din_X0(j);
          const double Xcn = cnoidal_cn(Xstart * 0.5 * ck + 2.0 * ck * (-(TIME / p.per_wave)), Mod1);
          const double Xsn = std::sqrt(1.0 - Xcn * Xcn);
          const double Xdn = std::sqrt(1.0 - Mod1 * (1.0 - Xcn * Xcn));
          const double c2 = Xcn * Xcn, s2 = Xsn * Xsn, d2 = Xdn * Xdn, m2 = Mod1 * Mod1;
          Uin_X0(j, k) = std::sqrt(Grav * Dep) *
                             (-5. / 4. + 3. * (Dep + Ytrough) / 2.0 / Dep -
                              ((Dep + Ytrough) * (Dep + Ytrough)) / 4. / (Dep * Dep) +
                              (3. * A / 2. / Dep - (Dep + Ytrough) * A / 2. / (Dep * Dep)) * c2 -
                              (A * A) / 4. / (Dep * Dep) * (c2 * c2) -
                              8.0 * A * (ck * ck) / (Wave_Length * Wave_Length) * (Dep / 3 - (Zlev * Zlev) / 2 / Dep) *
                                  (-(m2 * s2 * c2) + c2 * d2 - s2 * d2)) -
                         Stokes_Drift * Fact;
          Win_X0(j, k) = std::sqrt(Grav * Dep) * Zlev * 2 * A * ck / Wave_Length / Dep *
                         (1 + (Dep + Ytrough) / Dep + A / Dep * c2 +
                          32 * (ck * ck) / 3 / (Wave_Length * Wave_Length) * ((Dep * Dep) - (Zlev * Zlev) / 2) *
                              (m2 * s2 - m2 * c2 - d2)) *
                         Xsn * Xcn * Xdn;
          Vin_X0(j, k) = 0.0;
        }
    }
    if (p.wavemaker == NHW_WM_LEF_JON || p.wavemaker == NHW_WM_LEF_TMA) jonswap_left_boundary();
    if (p.wavemaker == NHW_WM_LEF_SPC && NumFreq_s > 0) random_left_boundary();
    if (p.wavemaker == NHW_WM_RIG_LIN) right_boundary_linear();
    if (p.wavemaker == NHW_WM_FLUX_LR) flux_left_right();
  }

  // linear_wave_right_boundary (src/waves.F:762-803): the linear wave of
  // LEF_LIN given to the east side (BC_Xn = 3), with the same phase and sign
  // convention as the west one
  void right_boundary_linear() {
    const double Segma = 2.0 * pi / p.per_wave;
    const double Wave_Number = wave_dispersion(Segma);
    const double Wave_Length = 2.0 * pi / Wave_Number;
    const double Stokes_Drift = Grav * (p.amp_wave * p.amp_wave) / (Wave_Length / p.per_wave) / p.dep_wave / 8.0;
    const double Fact = 1.0;
    const double th = p.theta_wave * pi / 180.;
    for (int j = 1; j <= Nloc; ++j) {
      const double Phs_Lag = yc(j) * std::sin(th) * Wave_Number;
      Ein_Xn(j) = 0.5 * p.amp_wave * std::cos(pi / 2 - Segma * TIME + Phs_Lag);
      Din_Xn(j) = Ein_Xn(j) + Hfx(Iend1, j);
    }
    const double shd = std::sinh(Wave_Number * p.dep_wave);
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j) {
        const double Phs_Lag = yc(j) * std::sin(th) * Wave_Number;
        const double Zlev = sigc(k) * Din_Xn(j);
        const double cs = std::cos(pi / 2 - Segma * TIME + Phs_Lag), sn = std::sin(pi / 2 - Segma * TIME + Phs_Lag);
        Uin_Xn(j, k) = (0.5 * p.amp_wave * Segma * std::cosh(Wave_Number * Zlev) / shd * cs - Stokes_Drift * Fact) *
                       std::cos(th);
        Win_Xn(j, k) = 0.5 * p.amp_wave * Segma * std::sinh(Wave_Number * Zlev) / shd * sn;
        Vin_Xn(j, k) = (0.5 * p.amp_wave * Segma * std::cosh(Wave_Number * Zlev) / shd * cs - Stokes_Drift * Fact) *
                       std::sin(th);
      }
  }

  // flux_left_right_boundary (src/nhwave.F:5566-5712) without its sediment
  // and salinity parts: a logarithmic current of depth-mean 0.115 m/s into
  // the west side at eta = 0, ramped up by tanh(TIME/TRamp); its volume flux
  // FluxL leaves through the east side, whose eta, V and W are radiated from
  // the last two steps and whose U mixes the interior value with the outflow
  // velocity FluxL/(Din_Xn dy Nglob) of this call and the previous one
  void flux_left_right() {
    const double Uavg_Left = (double)0.115f;
    double FluxL = 0.0;
    const double Ramp = p.tramp > 0.0 ? std::tanh(TIME / p.tramp) : 1.0;
    for (int j = 1; j <= Nloc; ++j) {
      Ein_X0(j) = 0.0;
      Din_X0(j) = Ein_X0(j) + Hfx(Ibeg, j);
    }
    const double Ufric = Uavg_Left * Kappa / (std::log(30. * Din_X0(Jbeg) / p.zob));
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j) {
        const double Zlev1 = sigc(k) * Din_X0(j);
        Uin_X0(j, k) = Ufric / Kappa * std::log(30. * Zlev1 / p.zob) * Ramp;
        FluxL = FluxL + dsig(k) * Din_X0(j) * dy * Uin_X0(j, k);
        Win_X0(j, k) = 0.0;
        Vin_X0(j, k) = 0.0;
      }
    auto cg = [&](double a, double b, double c) {   // Cg = -(a - b + 1e-16)/(b - c + 1e-16) in [0, 1]
      const double Cg = -(a - b + kOrlSmall) / (b - c + kOrlSmall);
      return dmax(dmin(Cg, 1.0), 0.0);
    };
    for (int j = 1; j <= Nloc; ++j) {
      const double Cg = cg(Eta0(Iend, j), Eta00(Iend, j), Eta00(Iend - 1, j));
      Ein_Xn(j) = (Cg * Eta0(Iend, j) + (1.0 - Cg) * Eta0(Iend + 1, j) + Eta(Iend, j)) / 2.0;
      Din_Xn(j) = Hfx(Iend + 1, j) + Ein_Xn(j);
    }
    Uin_Xni0 = Uin_Xni;
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j) {
        Uin_Xni(j, k) = FluxL / (Din_Xn(j) * dy * (double)(float)p.Nglob);
        double Cg = cg(U0(Iend, j, k), U00(Iend, j, k), U00(Iend - 1, j, k));
        Uin_Xn(j, k) = (Cg * U(Iend, j, k) + Uin_Xni0(j, k) - Cg * Uin_Xni(j, k) + U(Iend, j, k)) / 2.0;
        Cg = cg(V0(Iend, j, k), V00(Iend, j, k), V00(Iend - 1, j, k));
        Vin_Xn(j, k) = (Cg * V0(Iend, j, k) + (1.0 - Cg) * V0(Iend + 1, j, k) + V(Iend, j, k)) / 2.0;
        Cg = cg(W0(Iend, j, k), W00(Iend, j, k), W00(Iend - 1, j, k));
        Win_Xn(j, k) = (Cg * W0(Iend, j, k) + (1.0 - Cg) * W0(Iend + 1, j, k) + W(Iend, j, k)) / 2.0;
      }
  }

  double source_area() {
    double Source_Area = 0.0;
    for (int i = Ibeg; i <= Iend; ++i)
      if (xc(i) >= p.xsource_west && xc(i) <= p.xsource_east) Source_Area = Source_Area + dx * D(i, Jbeg + 1);
    return Source_Area;
  }

  // The direction of an internal maker's component snapped to one that the
  // channel width repeats (src/source_terms.F:94-136 for INT_SPC, 203-247 for
  // INT_IRR, which keeps a zero direction).  The reference's search has no
  // bound; a direction beyond 90 degrees never ends it, and is refused here
  // (false).
  bool snap_angle(double& Angle, double Wave_Number, bool irr) const {
    const double width = p.Nglob * dy;
    const long kMax = 10000000;
    double tmp1 = Wave_Number, tmp2, tmp3, tmp4;
    long nk = 0;
    if (Angle > Zero) {
      tmp3 = Zero;
      while (tmp3 < Angle) {
        nk = nk + 1;
        if (nk > kMax) return false;
        tmp2 = nk * 2.0 * pi / width;
        if (tmp2 >= tmp1) tmp3 = 0.5 * pi - Small;
        else tmp3 = std::asin(tmp2 / tmp1);
      }
      tmp4 = std::asin((nk - 1) * 2.0 * pi / width / tmp1);
      if (std::fabs(tmp4 - Angle) < std::fabs(Angle - tmp3)) Angle = tmp4;
      else Angle = tmp3;
    } else if (!irr || Angle < Zero) {
      tmp3 = Zero;
      while (tmp3 > Angle) {
        nk = nk + 1;
        if (nk > kMax) return false;
        tmp2 = nk * 2.0 * pi / width;
        if (tmp2 >= tmp1) tmp3 = -0.5 * pi + Small;
        else tmp3 = -std::asin(tmp2 / tmp1);
      }
      tmp4 = std::asin((nk - 1) * 2.0 * pi / width / tmp1);
      if (std::fabs(tmp4 - Angle) < std::fabs(Angle - tmp3)) Angle = tmp4;
      else Angle = tmp3;
    } else {
      Angle = 0.0;
    }
    return true;
  }

  // INT_SPC (src/source_terms.F:71-191) and INT_IRR (:194-302); INT_IRR's
  // eta_mean is never read by the reference (a zero module variable)
  bool internal_spectral_source() {
    const bool irr = p.wavemaker == NHW_WM_INT_IRR;
    const int NumFreq = NumFreq_s, NumDir = NumDir_s;
    const double eta_mean = 0.0;
    const double Source_Area = source_area();
    auto at = [&](int nd, int nfq) { return (nd - 1) + NumDir * (nfq - 1); };
    for (int j = Jbeg; j <= Jend; ++j)
      for (int i = Ibeg; i <= Iend; ++i) {
        SourceC(i, j) = Zero;
        if (!(xc(i) >= p.xsource_west && xc(i) <= p.xsource_east && yc(j) >= p.ysource_suth &&
              yc(j) <= p.ysource_nrth))
          continue;
        for (int nfreq = 1; nfreq <= NumFreq; ++nfreq)
          for (int ndir = 1; ndir <= NumDir; ++ndir) {
            const double Per_Wave = 1.0 / Freq_s[nfreq - 1];
            const double Segma = 2.0 * pi / Per_Wave;
            const double Wave_Number = wave_dispersion(Segma);
            const double Wave_Length = 2.0 * pi / Wave_Number;
            const double Celerity = Wave_Length / Per_Wave;
            double Angle = Dire_s[ndir - 1] * pi / 180.;
            if (!snap_angle(Angle, Wave_Number, irr)) return false;
            const double WnumY = Wave_Number * std::sin(Angle);
            const double Phs_lag = (dy / 2.0 + yc(j)) * WnumY;
            const double ph = Random_Phs[at(ndir, nfreq)];
            if (irr) {
              const double Amp_Wave = 2.0 * Spc2d[at(ndir, nfreq)];
              if (nfreq == 1)
                SourceC(i, j) = SourceC(i, j) + 2 * Celerity / Source_Area *
                                                    (Amp_Wave / 2 * std::cos(pi / 2 - Segma * TIME + Phs_lag + ph) +
                                                     eta_mean);
              else
                SourceC(i, j) = SourceC(i, j) + Celerity * Amp_Wave / Source_Area *
                                                    std::cos(pi / 2 - Segma * TIME + Phs_lag + ph);
            } else {
              double dfreq;
              if (nfreq == 1) dfreq = Freq_s[1] - Freq_s[0];
              else if (nfreq == NumFreq) dfreq = Freq_s[NumFreq - 1] - Freq_s[NumFreq - 2];
              else dfreq = 0.5 * (Freq_s[nfreq] - Freq_s[nfreq - 2]);
              dfreq = std::fabs(dfreq);
              double ddir;
              if (ndir == 1) ddir = Dire_s[1] - Dire_s[0];
              else if (ndir == NumDir) ddir = Dire_s[NumDir - 1] - Dire_s[NumDir - 2];
              else ddir = 0.5 * (Dire_s[ndir] - Dire_s[ndir - 2]);
              ddir = std::fabs(ddir);
              const double Amp_Wave = 2.0 * std::sqrt(2.0 * Spc2d[at(ndir, nfreq)] * ddir * dfreq);
              SourceC(i, j) = SourceC(i, j) + Celerity * Amp_Wave / Source_Area *
                                                  std::cos(pi / 2 - Segma * TIME + Phs_lag + ph);
            }
          }
      }
    return true;
  }

  void source_terms() {
    if (p.wavemaker == NHW_WM_INT_LIN) {
      const double Segma = 2.0 * pi / p.per_wave;
      const double Wave_Number = wave_dispersion(Segma);
      const double Wave_Length = 2.0 * pi / Wave_Number;
      const double Celerity = Wave_Length / p.per_wave;
      const double WnumY = Wave_Number * std::sin(p.theta_wave * pi / 180.);
      const double Source_Area = source_area();
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i)
          if (xc(i) >= p.xsource_west && xc(i) <= p.xsource_east && yc(j) >= p.ysource_suth &&
              yc(j) <= p.ysource_nrth) {
            double Phs_lag = yc(j) * WnumY;
            SourceC(i, j) = Celerity * p.amp_wave / Source_Area * std::cos(pi / 2 - Segma * TIME + Phs_lag);
          }
    } else if (p.wavemaker == NHW_WM_INT_SOL) {
      const double A = p.amp_wave, Dep = p.dep_wave;
      const double Celerity = std::sqrt(Grav * Dep * (1.0 + A / Dep));
      const double Atmp = std::sqrt((double)0.75f * A / (Dep * Dep * Dep));
      const double Xstart = 4.0 * Dep / std::sqrt(A / Dep);
      const double Source_Area = source_area();
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i)
          if (xc(i) >= p.xsource_west && xc(i) <= p.xsource_east && yc(j) >= p.ysource_suth &&
              yc(j) <= p.ysource_nrth) {
            double ch = std::cosh(Atmp * (Xstart - Celerity * TIME));
            SourceC(i, j) = 2.0 * Celerity / Source_Area * A / (ch * ch);
          }
    } else if (p.wavemaker == NHW_WM_INT_SPC || p.wavemaker == NHW_WM_INT_IRR) {
      if (!internal_spectral_source()) status = NHW_ERR_ARG;
    } else if (p.wavemaker == NHW_WM_INT_JON || p.wavemaker == NHW_WM_INT_TMA) {
      // src/source_terms.F:305-340
      const double Source_Area = source_area();
      const double DFreq = (p.freq_max - p.freq_min) / (double)(float)p.numfreq;
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i) {
          SourceC(i, j) = Zero;
          if (xc(i) >= p.xsource_west && xc(i) <= p.xsource_east && yc(j) >= p.ysource_suth &&
              yc(j) <= p.ysource_nrth)
            for (int nfreq = 1; nfreq <= p.numfreq; ++nfreq) {
              const double Per_Wave = 1.0 / Freq[nfreq - 1];
              const double Segma = 2.0 * pi / Per_Wave;
              const double Wave_Number = wave_dispersion(Segma);
              const double Wave_Length = 2.0 * pi / Wave_Number;
              const double Celerity = Wave_Length / Per_Wave;
              const double Amp_Wave = 2.0 * std::sqrt(2.0 * Jon_Spc[nfreq - 1] * DFreq);
              SourceC(i, j) = SourceC(i, j) + Celerity * Amp_Wave / Source_Area *
                                                  std::cos(pi / 2 - Segma * TIME + RanPhs[nfreq - 1]);
            }
        }
    } else if (p.wavemaker == NHW_WM_INT_CON) {
      // src/source_terms.F:343-395
      double Wave_Length = 0, Ytrough = 0, Mod1 = 0, Celerity = 0, Xstart = 0;
      cnoidal(p.amp_wave, p.dep_wave, p.per_wave, Wave_Length, Ytrough, Mod1, &Celerity);
      cnoidal_start(Ytrough, Mod1, Xstart);
      const double Source_Area = source_area();
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i)
          if (xc(i) >= p.xsource_west && xc(i) <= p.xsource_east && yc(j) >= p.ysource_suth &&
              yc(j) <= p.ysource_nrth) {
            const double cn = cnoidal_cn(Xstart * 0.5 * cnoidal_ck(Mod1) +
                                             2.0 * cnoidal_ck(Mod1) * (-(TIME / p.per_wave)), Mod1);
            SourceC(i, j) = 2.0 * Celerity / Source_Area * (Ytrough + p.amp_wave * (cn * cn));
          }
    }
    for (int j = Jbeg; j <= Jend; ++j)
      for (int i = Ibeg; i <= Iend; ++i) {
        SourceX(i, j) = Grav * 0.5 * (EtaxL(i + 1, j) + EtaxR(i, j)) * (Hfx0(i + 1, j) - Hfx0(i, j)) / dx * Mask(i, j);
        SourceY(i, j) = Grav * 0.5 * (EtayL(i, j + 1) + EtayR(i, j)) * (Hfy0(i, j + 1) - Hfy0(i, j)) / dy * Mask(i, j);
      }
  }

  // ------------------------------------------------------------ delxyzFun
  void delxFun_2D(A2& Din, A2& Dout) {
    for (int i = 2; i <= Mloc - 1; ++i)
      for (int j = 1; j <= Nloc; ++j) {
        if (Mask(i, j) == 0) Dout(i, j) = Zero;
        else {
          double T1 = (Din(i + 1, j) - Din(i, j)) / dx, T2 = (Din(i, j) - Din(i - 1, j)) / dx;
          Dout(i, j) = (std::fabs(T1) + std::fabs(T2)) < Small ? Zero : LIMITER(T1, T2);
        }
      }
    for (int j = 1; j <= Nloc; ++j) {
      Dout(1, j) = (Din(2, j) - Din(1, j)) / dx;
      Dout(Mloc, j) = (Din(Mloc, j) - Din(Mloc - 1, j)) / dx;
    }
  }
  void delyFun_2D(A2& Din, A2& Dout) {
    for (int i = 1; i <= Mloc; ++i)
      for (int j = 2; j <= Nloc - 1; ++j) {
        if (Mask(i, j) == 0) Dout(i, j) = Zero;
        else {
          double T1 = (Din(i, j + 1) - Din(i, j)) / dy, T2 = (Din(i, j) - Din(i, j - 1)) / dy;
          Dout(i, j) = (std::fabs(T1) + std::fabs(T2)) < Small ? Zero : LIMITER(T1, T2);
        }
      }
    for (int i = 1; i <= Mloc; ++i) {
      Dout(i, 1) = (Din(i, 2) - Din(i, 1)) / dy;
      Dout(i, Nloc) = (Din(i, Nloc) - Din(i, Nloc - 1)) / dy;
    }
  }
  // delxFun_3D / delxFun1_3D (same body over Kloc or Kloc1 levels)
  void delxFun_3D(A3& Din, A3& Dout) {
    const int L = Din.n3;
    for (int i = 2; i <= Mloc - 1; ++i)
      for (int j = 1; j <= Nloc; ++j)
        for (int k = 1; k <= L; ++k) {
          if (Mask(i, j) == 0) Dout(i, j, k) = Zero;
          else {
            double T1 = (Din(i + 1, j, k) - Din(i, j, k)) / dx, T2 = (Din(i, j, k) - Din(i - 1, j, k)) / dx;
            Dout(i, j, k) = (std::fabs(T1) + std::fabs(T2)) < Small ? Zero : LIMITER(T1, T2);
          }
        }
    for (int j = 1; j <= Nloc; ++j)
      for (int k = 1; k <= L; ++k) {
        Dout(1, j, k) = (Din(2, j, k) - Din(1, j, k)) / dx;
        Dout(Mloc, j, k) = (Din(Mloc, j, k) - Din(Mloc - 1, j, k)) / dx;
      }
  }
  void delyFun_3D(A3& Din, A3& Dout) {
    const int L = Din.n3;
    for (int i = 1; i <= Mloc; ++i)
      for (int j = 2; j <= Nloc - 1; ++j)
        for (int k = 1; k <= L; ++k) {
          if (Mask(i, j) == 0) Dout(i, j, k) = Zero;
          else {
            double T1 = (Din(i, j + 1, k) - Din(i, j, k)) / dy, T2 = (Din(i, j, k) - Din(i, j - 1, k)) / dy;
            Dout(i, j, k) = (std::fabs(T1) + std::fabs(T2)) < Small ? Zero : LIMITER(T1, T2);
          }
        }
    for (int i = 1; i <= Mloc; ++i)
      for (int k = 1; k <= L; ++k) {
        Dout(i, 1, k) = (Din(i, 2, k) - Din(i, 1, k)) / dy;
        Dout(i, Nloc, k) = (Din(i, Nloc, k) - Din(i, Nloc - 1, k)) / dy;
      }
  }
  void delzFun_3D(A3& Din, A3& Dout) {
    for (int i = 1; i <= Mloc; ++i)
      for (int j = 1; j <= Nloc; ++j)
        for (int k = 2; k <= Kloc - 1; ++k) {
          double T1 = (Din(i, j, k + 1) - Din(i, j, k)) / (sigc(k + 1) - sigc(k));
          double T2 = (Din(i, j, k) - Din(i, j, k - 1)) / (sigc(k) - sigc(k - 1));
          Dout(i, j, k) = (std::fabs(T1) + std::fabs(T2)) < Small ? Zero : LIMITER(T1, T2);
        }
    for (int i = 1; i <= Mloc; ++i)
      for (int j = 1; j <= Nloc; ++j) {
        Dout(i, j, 1) = (Din(i, j, 2) - Din(i, j, 1)) / (0.5 * (dsig(1) + dsig(2)));
        Dout(i, j, Kloc) = (Din(i, j, Kloc) - Din(i, j, Kloc - 1)) / (0.5 * (dsig(Kloc - 1) + dsig(Kloc)));
      }
  }

  void delxyzFun() {
    delxFun_2D(Eta, DelxEta);
    delxFun_3D(U, DelxU); delxFun_3D(V, DelxV); delxFun_3D(W, DelxW);
    delxFun_3D(DU, DelxDU); delxFun_3D(DV, DelxDV); delxFun_3D(DW, DelxDW);
    delyFun_2D(Eta, DelyEta);
    delyFun_3D(U, DelyU); delyFun_3D(V, DelyV); delyFun_3D(W, DelyW);
    delyFun_3D(DU, DelyDU); delyFun_3D(DV, DelyDV); delyFun_3D(DW, DelyDW);
    delzFun_3D(U, DelzU); delzFun_3D(V, DelzV); delzFun_3D(W, DelzW);
  }

  // ----------------------------------------------------------- construct_*
  void construct_2D_x(A2& Vin, A2& Din, A2& OutL, A2& OutR) {
    OutL.fill(0.0); OutR.fill(0.0);
    for (int i = Ibeg; i <= Iend1; ++i)
      for (int j = Jbeg; j <= Jend; ++j) {
        OutL(i, j) = Vin(i - 1, j) + 0.5 * dx * Din(i - 1, j);
        OutR(i, j) = Vin(i, j) - 0.5 * dx * Din(i, j);
      }
  }
  void construct_3D_x(A3& Vin, A3& Din, A3& OutL, A3& OutR) {
    OutL.fill(0.0); OutR.fill(0.0);
    for (int i = Ibeg; i <= Iend1; ++i)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int k = Kbeg; k <= Kend; ++k) {
          OutL(i, j, k) = Vin(i - 1, j, k) + 0.5 * dx * Din(i - 1, j, k);
          OutR(i, j, k) = Vin(i, j, k) - 0.5 * dx * Din(i, j, k);
        }
  }
  void construct_2D_y(A2& Vin, A2& Din, A2& OutL, A2& OutR) {
    OutL.fill(0.0); OutR.fill(0.0);
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend1; ++j) {
        OutL(i, j) = Vin(i, j - 1) + 0.5 * dy * Din(i, j - 1);
        OutR(i, j) = Vin(i, j) - 0.5 * dy * Din(i, j);
      }
  }
  void construct_3D_y(A3& Vin, A3& Din, A3& OutL, A3& OutR) {
    OutL.fill(0.0); OutR.fill(0.0);
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend1; ++j)
        for (int k = Kbeg; k <= Kend; ++k) {
          OutL(i, j, k) = Vin(i, j - 1, k) + 0.5 * dy * Din(i, j - 1, k);
          OutR(i, j, k) = Vin(i, j, k) - 0.5 * dy * Din(i, j, k);
        }
  }
  void construct_3D_z(A3& Vin, A3& Din, A3& OutL, A3& OutR) {
    OutL.fill(0.0); OutR.fill(0.0);
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int k = Kbeg; k <= Kend1; ++k) {
          OutL(i, j, k) = Vin(i, j, k - 1) + 0.5 * dsig(k - 1) * Din(i, j, k - 1);
          OutR(i, j, k) = Vin(i, j, k) - 0.5 * dsig(k) * Din(i, j, k);
        }
  }
  void KBC_surface() {
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend; ++j)
        WzL(i, j, Kend1) = (Eta(i, j) - Eta0(i, j)) / dt + DelxEta(i, j) * UzL(i, j, Kend1) +
                           DelyEta(i, j) * VzL(i, j, Kend1);
  }
  void KBC_bottom() {
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend; ++j)
        WzR(i, j, Kbeg) = -DeltH(i, j) - DelxH(i, j) * UzR(i, j, Kbeg) - DelyH(i, j) * VzR(i, j, Kbeg);
  }

  double hydro(double eta, double h0) { return 0.5 * Grav * (eta * eta + 2.0 * eta * h0); }

  void construction() {
    construct_2D_x(Eta, DelxEta, EtaxL, EtaxR);
    construct_3D_x(U, DelxU, UxL, UxR); construct_3D_x(V, DelxV, VxL, VxR);
    construct_3D_x(W, DelxW, WxL, WxR); construct_3D_x(DU, DelxDU, DUxL, DUxR);
    construct_3D_x(DV, DelxDV, DVxL, DVxR); construct_3D_x(DW, DelxDW, DWxL, DWxR);
    for (int j = Jbeg; j <= Jend; ++j)
      for (int i = Ibeg; i <= Iend1; ++i) {
        DxL(i, j) = EtaxL(i, j) + Hfx(i, j);
        DxR(i, j) = EtaxR(i, j) + Hfx(i, j);
      }
    for (double& v : DxL.v) v = dmax(v, MinDep);
    for (double& v : DxR.v) v = dmax(v, MinDep);
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i) {
          if (Mask(i, j) == 1 && Mask(i + 1, j) == 0) {
            EtaxL(i + 1, j) = Eta(i, j); DxL(i + 1, j) = D(i, j); Hfx0(i + 1, j) = Hc(i, j);
            DUxL(i + 1, j, k) = Zero; DVxL(i + 1, j, k) = Zero; DWxL(i + 1, j, k) = Zero;
            UxL(i + 1, j, k) = Zero; VxL(i + 1, j, k) = Zero; WxL(i + 1, j, k) = Zero;
          } else if (Mask(i, j) == 1 && Mask(i - 1, j) == 0) {
            EtaxR(i, j) = Eta(i, j); DxR(i, j) = D(i, j); Hfx0(i, j) = Hc(i, j);
            DUxR(i, j, k) = Zero; DVxR(i, j, k) = Zero; DWxR(i, j, k) = Zero;
            UxR(i, j, k) = Zero; VxR(i, j, k) = Zero; WxR(i, j, k) = Zero;
          } else if (Mask(i, j) == 0) {
            EtaxL(i + 1, j) = Eta(i, j); DxL(i + 1, j) = D(i, j);
            DUxL(i + 1, j, k) = Zero; DVxL(i + 1, j, k) = Zero; DWxL(i + 1, j, k) = Zero;
            UxL(i + 1, j, k) = Zero; VxL(i + 1, j, k) = Zero; WxL(i + 1, j, k) = Zero;
            EtaxR(i, j) = Eta(i, j); DxR(i, j) = D(i, j);
            DUxR(i, j, k) = Zero; DVxR(i, j, k) = Zero; DWxR(i, j, k) = Zero;
            UxR(i, j, k) = Zero; VxR(i, j, k) = Zero; WxR(i, j, k) = Zero;
          }
        }
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend1; ++i) {
          ExL(i, j, k) = DUxL(i, j, k);
          ExR(i, j, k) = DUxR(i, j, k);
          FxL(i, j, k) = DUxL(i, j, k) * UxL(i, j, k) + hydro(EtaxL(i, j), Hfx0(i, j));
          FxR(i, j, k) = DUxR(i, j, k) * UxR(i, j, k) + hydro(EtaxR(i, j), Hfx0(i, j));
          GxL(i, j, k) = DxL(i, j) * UxL(i, j, k) * VxL(i, j, k);
          GxR(i, j, k) = DxR(i, j) * UxR(i, j, k) * VxR(i, j, k);
          HxL(i, j, k) = DxL(i, j) * UxL(i, j, k) * WxL(i, j, k);
          HxR(i, j, k) = DxR(i, j) * UxR(i, j, k) * WxR(i, j, k);
        }
    construct_2D_y(Eta, DelyEta, EtayL, EtayR);
    construct_3D_y(U, DelyU, UyL, UyR); construct_3D_y(V, DelyV, VyL, VyR);
    construct_3D_y(W, DelyW, WyL, WyR); construct_3D_y(DU, DelyDU, DUyL, DUyR);
    construct_3D_y(DV, DelyDV, DVyL, DVyR); construct_3D_y(DW, DelyDW, DWyL, DWyR);
    for (int j = Jbeg; j <= Jend1; ++j)
      for (int i = Ibeg; i <= Iend; ++i) {
        DyL(i, j) = EtayL(i, j) + Hfy(i, j);
        DyR(i, j) = EtayR(i, j) + Hfy(i, j);
      }
    for (double& v : DyL.v) v = dmax(v, MinDep);
    for (double& v : DyR.v) v = dmax(v, MinDep);
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i) {
          if (Mask(i, j) == 1 && Mask(i, j + 1) == 0) {
            EtayL(i, j + 1) = Eta(i, j); DyL(i, j + 1) = D(i, j); Hfy0(i, j + 1) = Hc(i, j);
            DUyL(i, j + 1, k) = Zero; DVyL(i, j + 1, k) = Zero; DWyL(i, j + 1, k) = Zero;
            UyL(i, j + 1, k) = Zero; VyL(i, j + 1, k) = Zero; WyL(i, j + 1, k) = Zero;
          } else if (Mask(i, j) == 1 && Mask(i, j - 1) == 0) {
            EtayR(i, j) = Eta(i, j); DyR(i, j) = D(i, j); Hfy0(i, j) = Hc(i, j);
            DUyR(i, j, k) = Zero; DVyR(i, j, k) = Zero; DWyR(i, j, k) = Zero;
            UyR(i, j, k) = Zero; VyR(i, j, k) = Zero; WyR(i, j, k) = Zero;
          } else if (Mask(i, j) == 0) {
            EtayL(i, j + 1) = Eta(i, j); DyL(i, j + 1) = D(i, j);
            DUyL(i, j + 1, k) = Zero; DVyL(i, j + 1, k) = Zero; DWyL(i, j + 1, k) = Zero;
            UyL(i, j + 1, k) = Zero; VyL(i, j + 1, k) = Zero; WyL(i, j + 1, k) = Zero;
            EtayR(i, j) = Eta(i, j); DyR(i, j) = D(i, j);
            DUyR(i, j, k) = Zero; DVyR(i, j, k) = Zero; DWyR(i, j, k) = Zero;
            UyR(i, j, k) = Zero; VyR(i, j, k) = Zero; WyR(i, j, k) = Zero;
          }
        }
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend1; ++j)
        for (int i = Ibeg; i <= Iend; ++i) {
          EyL(i, j, k) = DVyL(i, j, k);
          EyR(i, j, k) = DVyR(i, j, k);
          FyL(i, j, k) = DyL(i, j) * UyL(i, j, k) * VyL(i, j, k);
          FyR(i, j, k) = DyR(i, j) * UyR(i, j, k) * VyR(i, j, k);
          GyL(i, j, k) = DVyL(i, j, k) * VyL(i, j, k) + hydro(EtayL(i, j), Hfy0(i, j));
          GyR(i, j, k) = DVyR(i, j, k) * VyR(i, j, k) + hydro(EtayR(i, j), Hfy0(i, j));
          HyL(i, j, k) = DyL(i, j) * VyL(i, j, k) * WyL(i, j, k);
          HyR(i, j, k) = DyR(i, j) * VyR(i, j, k) * WyR(i, j, k);
        }
    construct_3D_z(U, DelzU, UzL, UzR); construct_3D_z(V, DelzV, VzL, VzR);
    construct_3D_z(W, DelzW, WzL, WzR);
    KBC_surface();
    KBC_bottom();
  }

  // ------------------------------------------------------------ wave_speed
  void wave_speed() {
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend1; ++i) {
          if (Mask(i - 1, j) == 1 && Mask(i, j) == 1) {
            double L = std::sqrt(Grav * std::fabs(DxL(i, j))), R = std::sqrt(Grav * std::fabs(DxR(i, j)));
            double S = 0.5 * (L + R) + 0.25 * (UxL(i, j, k) - UxR(i, j, k));
            double US = 0.5 * (UxL(i, j, k) + UxR(i, j, k)) + L - R;
            SxL(i, j, k) = dmin(UxL(i, j, k) - L, US - S);
            SxR(i, j, k) = dmax(UxR(i, j, k) + R, US + S);
            SxS(i, j, k) = US;
          } else if (Mask(i - 1, j) == 0 && Mask(i, j) == 1) {
            double R = std::sqrt(Grav * std::fabs(DxR(i, j)));
            SxL(i, j, k) = UxR(i, j, k) - 2.0 * R;
            SxR(i, j, k) = UxR(i, j, k) + R;
            SxS(i, j, k) = SxL(i, j, k);
          } else if (Mask(i - 1, j) == 1 && Mask(i, j) == 0) {
            double L = std::sqrt(Grav * std::fabs(DxL(i, j)));
            SxL(i, j, k) = UxL(i, j, k) - L;
            SxR(i, j, k) = UxL(i, j, k) + 2.0 * L;
            SxS(i, j, k) = SxR(i, j, k);
          }
        }
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend1; ++j)
        for (int i = Ibeg; i <= Iend; ++i) {
          if (Mask(i, j - 1) == 1 && Mask(i, j) == 1) {
            double L = std::sqrt(Grav * std::fabs(DyL(i, j))), R = std::sqrt(Grav * std::fabs(DyR(i, j)));
            double S = 0.5 * (L + R) + 0.25 * (VyL(i, j, k) - VyR(i, j, k));
            double US = 0.5 * (VyL(i, j, k) + VyR(i, j, k)) + L - R;
            SyL(i, j, k) = dmin(VyL(i, j, k) - L, US - S);
            SyR(i, j, k) = dmax(VyR(i, j, k) + R, US + S);
            SyS(i, j, k) = US;
          } else if (Mask(i, j - 1) == 0 && Mask(i, j) == 1) {
            double R = std::sqrt(Grav * std::fabs(DyR(i, j)));
            SyL(i, j, k) = VyR(i, j, k) - 2.0 * R;
            SyR(i, j, k) = VyR(i, j, k) + R;
            SyS(i, j, k) = SyL(i, j, k);
          } else if (Mask(i, j - 1) == 1 && Mask(i, j) == 0) {
            double L = std::sqrt(Grav * std::fabs(DyL(i, j)));
            SyL(i, j, k) = VyL(i, j, k) - L;
            SyR(i, j, k) = VyL(i, j, k) + 2.0 * L;
            SyS(i, j, k) = SyR(i, j, k);
          }
        }
  }

  // HLL (src/nhwave.F:2741-2776) over a whole face array; UL/UR given per face
  void HLL(A3& SL, A3& SR, A3& FL, A3& FR, A3* UL3, A3* UR3, A2* UL2, A2* UR2, A3& FOUT) {
    for (int k = 1; k <= FOUT.n3; ++k)
      for (int j = 1; j <= FOUT.n2; ++j)
        for (int i = 1; i <= FOUT.n1; ++i) {
          double sl = SL(i, j, k), sr = SR(i, j, k);
          if (sl >= Zero) FOUT(i, j, k) = FL(i, j, k);
          else if (sr <= Zero) FOUT(i, j, k) = FR(i, j, k);
          else {
            double ul = UL3 ? (*UL3)(i, j, k) : (*UL2)(i, j);
            double ur = UR3 ? (*UR3)(i, j, k) : (*UR2)(i, j);
            double f = sr * FL(i, j, k) - sl * FR(i, j, k) + sl * sr * (ur - ul);
            if (std::fabs(sr - sl) < Small) f = f / Small;
            else f = f / (sr - sl);
            FOUT(i, j, k) = f;
          }
        }
  }

  void fluxes_at_faces_HLL() {
    HLL(SxL, SxR, ExL, ExR, nullptr, nullptr, &DxL, &DxR, Ex);
    HLL(SyL, SyR, EyL, EyR, nullptr, nullptr, &DyL, &DyR, Ey);
    HLL(SxL, SxR, FxL, FxR, &DUxL, &DUxR, nullptr, nullptr, Fx);
    HLL(SyL, SyR, FyL, FyR, &DUyL, &DUyR, nullptr, nullptr, Fy);
    HLL(SxL, SxR, GxL, GxR, &DVxL, &DVxR, nullptr, nullptr, Gx);
    HLL(SyL, SyR, GyL, GyR, &DVyL, &DVyR, nullptr, nullptr, Gy);
    HLL(SxL, SxR, HxL, HxR, &DWxL, &DWxR, nullptr, nullptr, Hx);
    HLL(SyL, SyR, HyL, HyR, &DWyL, &DWyR, nullptr, nullptr, Hy);
    for (int k = Kbeg + 1; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i) {
          double om = Omega(i, j, k);
          Fz(i, j, k) = 0.5 * (om * (UzL(i, j, k) + UzR(i, j, k)) - std::fabs(om) * (UzR(i, j, k) - UzL(i, j, k)));
          Gz(i, j, k) = 0.5 * (om * (VzL(i, j, k) + VzR(i, j, k)) - std::fabs(om) * (VzR(i, j, k) - VzL(i, j, k)));
          Hz(i, j, k) = 0.5 * (om * (WzL(i, j, k) + WzR(i, j, k)) - std::fabs(om) * (WzR(i, j, k) - WzL(i, j, k)));
        }
  }

  // HLLC (src/nhwave.F:2779-2810): left/right/star states of one face
  static double HLLC(double sl, double sr, double ss, double fl, double fr, double ul, double uls, double ur,
                     double urs) {
    if (sl >= Zero) return fl;
    if (sr <= Zero) return fr;
    if (ss >= Zero) return fl + sl * (uls - ul);
    return fr + sr * (urs - ur);
  }
  // fluxes_at_faces_HLLC (src/nhwave.F:2555-2670).  The reference forms every
  // star state as DxL*(SxL-UxL+Small)/(SxL-SxS+Small) times a factor; the
  // common product is formed once here, with the same operations in the same
  // order.
  void fluxes_at_faces_HLLC() {
    for (int k = 1; k <= Kloc; ++k)
      for (int j = 1; j <= Nloc; ++j)
        for (int i = 1; i <= Mloc1; ++i) {
          const double sl = SxL(i, j, k), sr = SxR(i, j, k), ss = SxS(i, j, k);
          const double dl = DxL(i, j), dr = DxR(i, j);
          const double ls = dl * (sl - UxL(i, j, k) + Small) / (sl - ss + Small);
          const double rs = dr * (sr - UxR(i, j, k) + Small) / (sr - ss + Small);
          Ex(i, j, k) = HLLC(sl, sr, ss, ExL(i, j, k), ExR(i, j, k), dl, ls, dr, rs);
          Fx(i, j, k) = HLLC(sl, sr, ss, FxL(i, j, k), FxR(i, j, k), DUxL(i, j, k), ls * ss, DUxR(i, j, k), rs * ss);
          Gx(i, j, k) = HLLC(sl, sr, ss, GxL(i, j, k), GxR(i, j, k), DVxL(i, j, k), ls * VxL(i, j, k), DVxR(i, j, k),
                             rs * VxR(i, j, k));
          Hx(i, j, k) = HLLC(sl, sr, ss, HxL(i, j, k), HxR(i, j, k), DWxL(i, j, k), ls * WxL(i, j, k), DWxR(i, j, k),
                             rs * WxR(i, j, k));
        }
    for (int k = 1; k <= Kloc; ++k)
      for (int j = 1; j <= Nloc1; ++j)
        for (int i = 1; i <= Mloc; ++i) {
          const double sl = SyL(i, j, k), sr = SyR(i, j, k), ss = SyS(i, j, k);
          const double dl = DyL(i, j), dr = DyR(i, j);
          const double ls = dl * (sl - VyL(i, j, k) + Small) / (sl - ss + Small);
          const double rs = dr * (sr - VyR(i, j, k) + Small) / (sr - ss + Small);
          Ey(i, j, k) = HLLC(sl, sr, ss, EyL(i, j, k), EyR(i, j, k), dl, ls, dr, rs);
          Fy(i, j, k) = HLLC(sl, sr, ss, FyL(i, j, k), FyR(i, j, k), DUyL(i, j, k), ls * UyL(i, j, k), DUyR(i, j, k),
                             rs * UyR(i, j, k));
          Gy(i, j, k) = HLLC(sl, sr, ss, GyL(i, j, k), GyR(i, j, k), DVyL(i, j, k), ls * ss, DVyR(i, j, k), rs * ss);
          Hy(i, j, k) = HLLC(sl, sr, ss, HyL(i, j, k), HyR(i, j, k), DWyL(i, j, k), ls * WyL(i, j, k), DWyR(i, j, k),
                             rs * WyR(i, j, k));
        }
    for (int k = Kbeg + 1; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i) {
          double om = Omega(i, j, k);
          Fz(i, j, k) = 0.5 * (om * (UzL(i, j, k) + UzR(i, j, k)) - std::fabs(om) * (UzR(i, j, k) - UzL(i, j, k)));
          Gz(i, j, k) = 0.5 * (om * (VzL(i, j, k) + VzR(i, j, k)) - std::fabs(om) * (VzR(i, j, k) - VzL(i, j, k)));
          Hz(i, j, k) = 0.5 * (om * (WzL(i, j, k) + WzR(i, j, k)) - std::fabs(om) * (WzR(i, j, k) - WzL(i, j, k)));
        }
  }

  void flux_bc() {
    for (int j = Jbeg; j <= Jend; ++j)
      for (int k = Kbeg; k <= Kend; ++k) {  // walls: Bc 1, 2 (5); inflow: Bc 3 (src/nhwave.F:2375-2387)
        if (p.bc_x0 == 3) {
          Ex(Ibeg, j, k) = Din_X0(j) * Uin_X0(j, k);
          Fx(Ibeg, j, k) = Din_X0(j) * Uin_X0(j, k) * Uin_X0(j, k) + hydro(Ein_X0(j), Hfx0(Ibeg, j));
          Gx(Ibeg, j, k) = Din_X0(j) * Uin_X0(j, k) * Vin_X0(j, k);
          Hx(Ibeg, j, k) = Din_X0(j) * Uin_X0(j, k) * Win_X0(j, k);
        } else {
          Ex(Ibeg, j, k) = Zero; Fx(Ibeg, j, k) = hydro(EtaxR(Ibeg, j), Hfx0(Ibeg, j));
          Gx(Ibeg, j, k) = Zero; Hx(Ibeg, j, k) = Zero;
        }
        if (p.bc_xn == 3) {   // inflow/outflow (src/nhwave.F:2411-2416)
          Ex(Iend1, j, k) = Din_Xn(j) * Uin_Xn(j, k);
          Fx(Iend1, j, k) = Din_Xn(j) * Uin_Xn(j, k) * Uin_Xn(j, k) + hydro(Ein_Xn(j), Hfx0(Iend1, j));
          Gx(Iend1, j, k) = Din_Xn(j) * Uin_Xn(j, k) * Vin_Xn(j, k);
          Hx(Iend1, j, k) = Din_Xn(j) * Uin_Xn(j, k) * Win_Xn(j, k);
        } else if (p.bc_xn != 6) {   // an open (Orlanski) east face keeps its Riemann fluxes
          Ex(Iend1, j, k) = Zero; Fx(Iend1, j, k) = hydro(EtaxL(Iend1, j), Hfx0(Iend1, j));
          Gx(Iend1, j, k) = Zero; Hx(Iend1, j, k) = Zero;
        }
      }
    for (int i = Ibeg; i <= Iend; ++i)
      for (int k = Kbeg; k <= Kend; ++k) {
        Ey(i, Jbeg, k) = Zero; Fy(i, Jbeg, k) = Zero;
        Gy(i, Jbeg, k) = hydro(EtayR(i, Jbeg), Hfy0(i, Jbeg)); Hy(i, Jbeg, k) = Zero;
        Ey(i, Jend1, k) = Zero; Fy(i, Jend1, k) = Zero;
        Gy(i, Jend1, k) = hydro(EtayL(i, Jend1), Hfy0(i, Jend1)); Hy(i, Jend1, k) = Zero;
      }
    for (int j = Jbeg; j <= Jend; ++j)
      for (int i = Ibeg; i <= Iend; ++i) {
        Fz(i, j, Kbeg) = Zero; Gz(i, j, Kbeg) = Zero; Hz(i, j, Kbeg) = Zero;
        Fz(i, j, Kend1) = Zero; Gz(i, j, Kend1) = Zero; Hz(i, j, Kend1) = Zero;
      }
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg - 1; j <= Jend + 1; ++j)
        for (int i = Ibeg - 1; i <= Iend + 1; ++i)
          if (Mask(i, j) == 0) {
            Ex(i, j, k) = Zero;
            Fx(i, j, k) = (i == Ibeg) ? Zero : hydro(EtaxL(i, j), Hfx0(i, j)) * Mask(i - 1, j);
            Gx(i, j, k) = Zero; Hx(i, j, k) = Zero;
            Ex(i + 1, j, k) = Zero;
            Fx(i + 1, j, k) = (i == Iend) ? Zero : hydro(EtaxR(i + 1, j), Hfx0(i + 1, j)) * Mask(i + 1, j);
            Gx(i + 1, j, k) = Zero; Hx(i + 1, j, k) = Zero;
            Ey(i, j, k) = Zero; Fy(i, j, k) = Zero;
            Gy(i, j, k) = (j == Jbeg) ? Zero : hydro(EtayL(i, j), Hfy0(i, j)) * Mask(i, j - 1);
            Hy(i, j, k) = Zero;
            Ey(i, j + 1, k) = Zero; Fy(i, j + 1, k) = Zero;
            Gy(i, j + 1, k) = (j == Jend) ? Zero : hydro(EtayR(i, j + 1), Hfy0(i, j + 1)) * Mask(i, j + 1);
            Hy(i, j + 1, k) = Zero;
          }
  }

  void fluxes() {
    delxyzFun();
    construction();
    wave_speed();
    if (p.hllc) fluxes_at_faces_HLLC();   // src/nhwave.F:1705-1709
    else fluxes_at_faces_HLL();
    flux_bc();
  }

  // -------------------------------------------------------------- wl_bc
  void wl_bc() {
    for (int j = Jbeg; j <= Jend; ++j) {
      if (p.bc_x0 == 3 && p.wavemaker == NHW_WM_LEF_TID)   // tide: D = Din from the first interior column out (src/nhwave.F:5145-5148)
        for (int i = 0; i <= Nghost; ++i) D(Ibeg - i, j) = Din_X0(j);
      else if (p.bc_x0 == 3)   // inflow (src/nhwave.F:5148-5157)
        for (int i = 1; i <= Nghost; ++i) D(Ibeg - i, j) = 2.0 * Din_X0(j) - D(Ibeg + i - 1, j);
      else
        for (int i = 1; i <= Nghost; ++i) D(Ibeg - i, j) = D(Ibeg + i - 1, j);
      if (p.bc_xn == 6 || p.bc_xn == 3)   // Orlanski radiation (src/nhwave.F:5182-5206)
        for (int i = 1; i <= Nghost; ++i) {
          double Cg = -(Eta0(Iend + i - 1, j) - Eta00(Iend + i - 1, j) + kOrlSmall) /
                      (Eta00(Iend + i - 1, j) - Eta00(Iend + i - 2, j) + kOrlSmall);
          Cg = dmax(dmin(Cg, 1.0), 0.0);
          Eta(Iend + i, j) = Cg * Eta0(Iend + i - 1, j) + (1.0 - Cg) * Eta0(Iend + i, j);
          D(Iend + i, j) = Hc(Iend + i, j) + Eta(Iend + i, j);
        }
      else
        for (int i = 1; i <= Nghost; ++i) D(Iend + i, j) = D(Iend - i + 1, j);
    }
    for (int i = 1; i <= Mloc; ++i)
      for (int j = 1; j <= Nghost; ++j) D(i, j) = D(i, Jbeg + Nghost - j);
    for (int i = 1; i <= Mloc; ++i)
      for (int j = 1; j <= Nghost; ++j) D(i, Jend + j) = D(i, Jend - j + 1);
  }

  void sigma_transform() {
    for (int k = 1; k <= Kloc; ++k)
      for (int j = 1; j <= Nloc; ++j)
        for (int i = 1; i <= Mloc; ++i) {
          DelxSc(i, j, k) = (1.0 - sigc(k)) / D(i, j) * DelxH(i, j) - sigc(k) / D(i, j) * DelxEta(i, j);
          DelySc(i, j, k) = (1.0 - sigc(k)) / D(i, j) * DelyH(i, j) - sigc(k) / D(i, j) * DelyEta(i, j);
        }
    if (!p.viscous_flow) return;   // DelxSl / DelySl feed only the viscous terms
    for (int k = 1; k <= Kloc1; ++k)
      for (int j = 1; j <= Nloc; ++j)
        for (int i = 1; i <= Mloc; ++i) {
          DelxSl(i, j, k) = (1.0 - sig(k)) / D(i, j) * DelxH(i, j) - sig(k) / D(i, j) * DelxEta(i, j);
          DelySl(i, j, k) = (1.0 - sig(k)) / D(i, j) * DelyH(i, j) - sig(k) / D(i, j) * DelyEta(i, j);
        }
  }

  // -------------------------------------------------------------- diffusion
  // Explicit part of the viscous terms (src/nhwave.F:6785-7141), with the
  // cells' CmuHt: Diffxx/Diffxy enter R2, Diffyx/Diffyy R3, Diffzx/Diffzy
  // R4 (the reference also forms Diffxz/Diffyz, which nothing reads).
  // The sigma slopes are those of the last sigma_transform; D is the
  // current one.  Every bracket keeps the reference's evaluation order.
  void diffusion() {
    for (A3* a : {&Diffxx, &Diffxy, &Diffyx, &Diffyy, &Diffzx, &Diffzy}) a->fill(0.0);
    const double Schmidt = p.schmidt;
    // face viscosity between cells a and b, and cell viscosity
    auto nuF = [&](double ha, double hb) { return 0.5 * (Cmu + Cmu) + 0.5 * (ha + hb) / Schmidt; };
    auto nuC = [&](int ii, int jj, int kk) { return Cmu + CmuHt(ii, jj, kk) / Schmidt; };
    for (int k = Kbeg; k <= Kend; ++k) {
      const double L1top = dsig(k + 1) / (dsig(k) + dsig(k + 1)), L2top = dsig(k) / (dsig(k) + dsig(k + 1));
      const double L1bot = dsig(k) / (dsig(k) + dsig(k - 1)), L2bot = dsig(k - 1) / (dsig(k) + dsig(k - 1));
      const double dsigck = (dsig(k) + dsig(k + 1)) / 2.0, dsigck1 = (dsig(k - 1) + dsig(k)) / 2.0;
      const double ac = -dsigck / (dsigck + dsigck1) / dsigck1;
      const double bc = (dsigck - dsigck1) / (dsigck * dsigck1);
      const double gc = dsigck1 / (dsigck + dsigck1) / dsigck;
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i) {
          if (Mask(i, j) == 0) continue;
          const double Dc = D(i, j);
          const double nuH_top = (L1top * Cmu + L2top * Cmu) + (L1top * CmuHt(i, j, k) + L2top * CmuHt(i, j, k + 1)) / Schmidt;
          const double nuH_bot = (L1bot * Cmu + L2bot * Cmu) + (L1bot * CmuHt(i, j, k - 1) + L2bot * CmuHt(i, j, k)) / Schmidt;
          const double H = CmuHt(i, j, k);
          const double nuE = nuF(CmuHt(i + 1, j, k), H), nuW = nuF(H, CmuHt(i - 1, j, k));
          const double nuN = nuF(CmuHt(i, j + 1, k), H), nuS = nuF(H, CmuHt(i, j - 1, k));
          const double cE = nuC(i + 1, j, k), cW = nuC(i - 1, j, k), cN = nuC(i, j + 1, k), cS = nuC(i, j - 1, k);
          const double cD = nuC(i, j, k - 1), c0 = nuC(i, j, k), cU = nuC(i, j, k + 1);
          // three-level sums  a F(k-1) G(k-1) + b F(k) G(k) + c F(k+1) G(k+1)
          auto s3 = [&](A3& F, A3& G, int ii, int jj) {
            return ac * F(ii, jj, k - 1) * G(ii, jj, k - 1) + bc * F(ii, jj, k) * G(ii, jj, k) +
                   gc * F(ii, jj, k + 1) * G(ii, jj, k + 1);
          };
          // lead + a (Sx DV + Sy DU)(k-1) + ..., summed left to right: the
          // cross-slope sums of Diffxy / Diffyx
          auto s3x = [&](double lead, int ii, int jj) {
            return lead + ac * (DelxSc(ii, jj, k - 1) * DV(ii, jj, k - 1) + DelySc(ii, jj, k - 1) * DU(ii, jj, k - 1)) +
                   bc * (DelxSc(ii, jj, k) * DV(ii, jj, k) + DelySc(ii, jj, k) * DU(ii, jj, k)) +
                   gc * (DelxSc(ii, jj, k + 1) * DV(ii, jj, k + 1) + DelySc(ii, jj, k + 1) * DU(ii, jj, k + 1));
          };
          // a (W Sx + F/D)(k-1) + ...: Diffzx / Diffzy
          auto s3w = [&](A3& Sl, A3& F, int ii, int jj) {
            return ac * (DW(ii, jj, k - 1) * Sl(ii, jj, k - 1) + F(ii, jj, k - 1) / Dc) +
                   bc * (DW(ii, jj, k) * Sl(ii, jj, k) + F(ii, jj, k) / Dc) +
                   gc * (DW(ii, jj, k + 1) * Sl(ii, jj, k + 1) + F(ii, jj, k + 1) / Dc);
          };
          // vertical coefficients of the d/dsigma[nu Sl d/dsigma] terms
          auto vco = [&](A3& Sl, double& cA, double& cB, double& cC) {
            const double Pq = nuH_top * Sl(i, j, k + 1) - nuH_bot * Sl(i, j, k);
            const double Sq = nuH_top * Sl(i, j, k + 1) + nuH_bot * Sl(i, j, k);
            cA = Pq * ac / dsig(k) + Sq / dsigck1 / (dsigck + dsigck1);
            cB = Pq * bc / dsig(k) - Sq / dsigck1 / dsigck;
            cC = Pq * gc / dsig(k) + Sq / dsigck / (dsigck + dsigck1);
          };
          double xA, xB, xC, yA, yB, yC;
          vco(DelxSl, xA, xB, xC);
          vco(DelySl, yA, yB, yC);
          // d/dx[2 nu d/dx DU] + d/dx[2 nu d/dsigma(DU Sx)] + d/dsigma[2 nu Sx d/dx DU]
          Diffxx(i, j, k) =
              (2.0 * nuE * (DU(i + 1, j, k) - DU(i, j, k)) / dx - 2.0 * nuW * (DU(i, j, k) - DU(i - 1, j, k)) / dx) / dx +
              (2.0 * cE * s3(DU, DelxSc, i + 1, j) - 2.0 * cW * s3(DU, DelxSc, i - 1, j)) / 2.0 / dx +
              (ac * 2.0 * cD * DelxSc(i, j, k - 1) * (DU(i + 1, j, k - 1) - DU(i - 1, j, k - 1)) / 2.0 / dx +
               bc * 2.0 * c0 * DelxSc(i, j, k) * (DU(i + 1, j, k) - DU(i - 1, j, k)) / 2.0 / dx +
               gc * 2.0 * cU * DelxSc(i, j, k + 1) * (DU(i + 1, j, k + 1) - DU(i - 1, j, k + 1)) / 2.0 / dx);
          auto mixed = [&](int kk) {   // d/dy DU + d/dx DV at level kk
            return (DU(i, j + 1, kk) - DU(i, j - 1, kk)) / 2.0 / dy + (DV(i + 1, j, kk) - DV(i - 1, j, kk)) / 2.0 / dx;
          };
          Diffxy(i, j, k) =
              (nuN * (DU(i, j + 1, k) - DU(i, j, k)) / dy - nuS * (DU(i, j, k) - DU(i, j - 1, k)) / dy) / dy +
              (cN * s3x((DV(i + 1, j + 1, k) - DV(i - 1, j + 1, k)) / 2.0 / dx, i, j + 1) -
               cS * s3x((DV(i + 1, j - 1, k) - DV(i - 1, j - 1, k)) / 2.0 / dx, i, j - 1)) /
                  2.0 / dy +
              (ac * cD * DelySc(i, j, k - 1) * mixed(k - 1) + bc * c0 * DelySc(i, j, k) * mixed(k) +
               gc * cU * DelySc(i, j, k + 1) * mixed(k + 1)) +
              (yA * DelxSc(i, j, k - 1) * DV(i, j, k - 1) + yB * DelxSc(i, j, k) * DV(i, j, k) +
               yC * DelxSc(i, j, k + 1) * DV(i, j, k + 1));
          Diffyx(i, j, k) =
              (nuE * (DV(i + 1, j, k) - DV(i, j, k)) / dx - nuW * (DV(i, j, k) - DV(i - 1, j, k)) / dx) / dx +
              (cE * s3x((DU(i + 1, j + 1, k) - DU(i + 1, j - 1, k)) / 2.0 / dy, i + 1, j) -
               cW * s3x((DU(i - 1, j + 1, k) - DU(i - 1, j - 1, k)) / 2.0 / dy, i - 1, j)) /
                  2.0 / dx +
              (ac * cD * DelxSc(i, j, k - 1) * mixed(k - 1) + bc * c0 * DelxSc(i, j, k) * mixed(k) +
               gc * cU * DelxSc(i, j, k + 1) * mixed(k + 1)) +
              (xA * DelySc(i, j, k - 1) * DU(i, j, k - 1) + xB * DelySc(i, j, k) * DU(i, j, k) +
               xC * DelySc(i, j, k + 1) * DU(i, j, k + 1));
          Diffyy(i, j, k) =
              (2.0 * nuN * (DV(i, j + 1, k) - DV(i, j, k)) / dy - 2.0 * nuS * (DV(i, j, k) - DV(i, j - 1, k)) / dy) / dy +
              (2.0 * cN * s3(DV, DelySc, i, j + 1) - 2.0 * cS * s3(DV, DelySc, i, j - 1)) / 2.0 / dy +
              (ac * 2.0 * cD * DelySc(i, j, k - 1) * (DV(i, j + 1, k - 1) - DV(i, j - 1, k - 1)) / 2.0 / dy +
               bc * 2.0 * c0 * DelySc(i, j, k) * (DV(i, j + 1, k) - DV(i, j - 1, k)) / 2.0 / dy +
               gc * 2.0 * cU * DelySc(i, j, k + 1) * (DV(i, j + 1, k + 1) - DV(i, j - 1, k + 1)) / 2.0 / dy);
          Diffzx(i, j, k) =
              (nuE * (DW(i + 1, j, k) - DW(i, j, k)) / dx - nuW * (DW(i, j, k) - DW(i - 1, j, k)) / dx) / dx +
              (cE * s3w(DelxSc, DU, i + 1, j) - cW * s3w(DelxSc, DU, i - 1, j)) / 2.0 / dx +
              (ac * cD * DelxSc(i, j, k - 1) * (DW(i + 1, j, k - 1) - DW(i - 1, j, k - 1)) / 2.0 / dx +
               bc * c0 * DelxSc(i, j, k) * (DW(i + 1, j, k) - DW(i - 1, j, k)) / 2.0 / dx +
               gc * cU * DelxSc(i, j, k + 1) * (DW(i + 1, j, k + 1) - DW(i - 1, j, k + 1)) / 2.0 / dx) +
              (xA * DU(i, j, k - 1) / Dc + xB * DU(i, j, k) / Dc + xC * DU(i, j, k + 1) / Dc);
          Diffzy(i, j, k) =
              (nuN * (DW(i, j + 1, k) - DW(i, j, k)) / dy - nuS * (DW(i, j, k) - DW(i, j - 1, k)) / dy) / dy +
              (cN * s3w(DelySc, DV, i, j + 1) - cS * s3w(DelySc, DV, i, j - 1)) / 2.0 / dy +
              (ac * cD * DelySc(i, j, k - 1) * (DW(i, j + 1, k - 1) - DW(i, j - 1, k - 1)) / 2.0 / dy +
               bc * c0 * DelySc(i, j, k) * (DW(i, j + 1, k) - DW(i, j - 1, k)) / 2.0 / dy +
               gc * cU * DelySc(i, j, k + 1) * (DW(i, j + 1, k + 1) - DW(i, j - 1, k + 1)) / 2.0 / dy) +
              (yA * DV(i, j, k - 1) / Dc + yB * DV(i, j, k) / Dc + yC * DV(i, j, k + 1) / Dc);
        }
    }
  }

  // trig (src/nhwave.F:13182-13224): tridiagonal solve by forward
  // elimination and back substitution
  static void trig(const std::vector<double>& a, const std::vector<double>& b, const std::vector<double>& c,
                   const std::vector<double>& r, std::vector<double>& x, int n) {
    std::vector<double> bp(n), rp(n);
    bp[0] = b[0];
    rp[0] = r[0];
    for (int q = 1; q < n; ++q) {
      const double coeff = a[q] / bp[q - 1];
      bp[q] = b[q] - coeff * c[q - 1];
      rp[q] = r[q] - coeff * rp[q - 1];
    }
    x[n - 1] = rp[n - 1] / bp[n - 1];
    for (int q = n - 2; q >= 0; --q) x[q] = (rp[q] - c[q] * x[q + 1]) / bp[q];
  }

  // Implicit vertical viscous step of eval_duvw for one column
  // (src/nhwave.F:690-822 DU, 850-1010 DV, 1012-1182 DW): on entry F holds
  // DU + dt R2 (the explicit update), on exit the solution.  which = 0 DU,
  // 1 DV, 2 DW.  The bed enters DU and DV: no slip (BC_Z0 = 2) in the first
  // diagonal, the friction law (5) in the first right-hand side.
  void vertical_viscous(int i, int j, int which) {
    const int n = Kend - Kbeg + 1;
    std::vector<double> A(n), B(n), C(n), Rhs(n), X(n);
    const double Schmidt = p.schmidt, Dc = D(i, j);
    // face viscosity between levels k1 and k2 (Cmu and CmuR uniform)
    auto nuz = [&](int k1, int k2) {
      return 0.5 * (((Cmu + Cmu) + CmuR) + CmuR) + 0.5 * (CmuVt(i, j, k1) + CmuVt(i, j, k2)) / Schmidt;
    };
    A3& F = which == 0 ? DU : which == 1 ? DV : DW;
    for (int k = Kbeg; k <= Kend; ++k) {
      const int q = k - Kbeg;
      A[q] = k == Kbeg ? 0.0 : -dt / (Dc * Dc) * nuz(k - 1, k) / (0.5 * dsig(k) * (dsig(k) + dsig(k - 1)));
      C[q] = k == Kend ? 0.0 : -dt / (Dc * Dc) * nuz(k, k + 1) / (0.5 * dsig(k) * (dsig(k) + dsig(k + 1)));
      if (which < 2) {
        if (k == Kbeg && p.bc_z0 == 2)
          B[q] = 1.0 - C[q] + dt / (Dc * Dc) * (Cmu + CmuR + CmuVt(i, j, k) / Schmidt) / (0.5 * dsig(k) * dsig(k));
        else
          B[q] = 1.0 - A[q] - C[q];
        if (k == Kbeg && p.bc_z0 == 5) {
          const double Dz1 = 0.5 * Dc * dsig(Kbeg);
          double Cdrag = p.cd0;
          if (p.ibot != 1) {
            const double lg = 1. / Kappa * std::log(30.0 * Dz1 / p.zob);
            Cdrag = 1. / (lg * lg);
          }
          const double Ustar2 = Cdrag * std::sqrt(U(i, j, k) * U(i, j, k) + V(i, j, k) * V(i, j, k)) *
                                (which == 0 ? U(i, j, k) : V(i, j, k));
          Rhs[q] = F(i, j, k) - dt * Ustar2 / dsig(k);
        } else if (k == Kend) {
          Rhs[q] = F(i, j, k) + dt * (which == 0 ? Wsx(i, j) : Wsy(i, j)) / dsig(k);
        } else {
          Rhs[q] = F(i, j, k);
        }
      } else if (k == Kbeg) {
        B[q] = 1.0 - C[q] + dt / (Dc * Dc) * nuz(k - 1, k) / (0.25 * dsig(k) * (dsig(k) + dsig(k - 1)));
        const double Wbot = -DeltH(i, j) - U(i, j, Kbeg) * DelxH(i, j) - V(i, j, Kbeg) * DelyH(i, j);
        Rhs[q] = F(i, j, k) + dt / Dc * nuz(k - 1, k) / (0.25 * dsig(k) * (dsig(k) + dsig(k - 1))) * Wbot;
      } else if (k == Kend) {
        B[q] = 1.0 - A[q] + dt / (Dc * Dc) * nuz(k, k + 1) / (0.25 * dsig(k) * (dsig(k) + dsig(k + 1)));
        const double Wtop = (Eta(i, j) - Eta0(i, j)) / dt + U(i, j, Kend) * DelxEta(i, j) + V(i, j, Kend) * DelyEta(i, j);
        Rhs[q] = F(i, j, k) + dt / Dc * nuz(k, k + 1) / (0.25 * dsig(k) * (dsig(k) + dsig(k + 1))) * Wtop;
      } else {
        B[q] = 1.0 - A[q] - C[q];
        Rhs[q] = F(i, j, k);
      }
    }
    trig(A, B, C, Rhs, X, n);
    for (int k = Kbeg; k <= Kend; ++k) F(i, j, k) = X[k - Kbeg];
  }

  // ------------------------------------------------------- get_UVW/vel_bc
  // Wall friction factor of a BC = 5 side (src/nhwave.F:4486-4493): h is the
  // grid spacing across the wall, a and b the tangential velocities of the
  // first interior cell, ht its CmuHt
  double wall_phi(double h, double a, double b, double ht) const {
    double Cdrag = p.cd0;
    if (p.ibot != 1) {
      const double lg = 1. / Kappa * std::log(30.0 * h / 2.0 / p.zob);
      Cdrag = 1. / (lg * lg);
    }
    const double Phi = h * Cdrag * std::sqrt(a * a + b * b) / (Cmu + ht);
    return dmin(Phi, 2.0);
  }

  void vel_bc() {
    const int sx0 = p.bc_x0 == 1 ? 1 : -1, sxn = p.bc_xn == 1 ? 1 : -1;
    const int sy0 = p.bc_y0 == 1 ? 1 : -1, syn = p.bc_yn == 1 ? 1 : -1;
    // Wall friction (BC = 5): tangential ghosts (1 - Phi) times the mirror;
    // the ghost momenta take D(i,j) with the ghost offset for i (x sides) or j
    // (y sides), as the reference writes them (src/nhwave.F:4486-4500,
    // 4583-4598, 4676-4691, 4737-4752)
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j) {
        if (p.bc_x0 == 5) {
          const double Phi = wall_phi(dx, V(Ibeg, j, k), W(Ibeg, j, k), CmuHt(Ibeg, j, k));
          for (int i = 1; i <= Nghost; ++i) {
            U(Ibeg - i, j, k) = -U(Ibeg + i - 1, j, k);
            V(Ibeg - i, j, k) = (1.0 - Phi) * V(Ibeg + i - 1, j, k);
            W(Ibeg - i, j, k) = (1.0 - Phi) * W(Ibeg + i - 1, j, k);
            DU(Ibeg - i, j, k) = D(i, j) * U(Ibeg - i, j, k);
            DV(Ibeg - i, j, k) = D(i, j) * V(Ibeg - i, j, k);
            DW(Ibeg - i, j, k) = D(i, j) * W(Ibeg - i, j, k);
          }
        }
        if (p.bc_xn == 5) {
          const double Phi = wall_phi(dx, V(Iend, j, k), W(Iend, j, k), CmuHt(Iend, j, k));
          for (int i = 1; i <= Nghost; ++i) {
            U(Iend + i, j, k) = -U(Iend - i + 1, j, k);
            V(Iend + i, j, k) = (1.0 - Phi) * V(Iend - i + 1, j, k);
            W(Iend + i, j, k) = (1.0 - Phi) * W(Iend - i + 1, j, k);
            DU(Iend + i, j, k) = D(i, j) * U(Iend + i, j, k);
            DV(Iend + i, j, k) = D(i, j) * V(Iend + i, j, k);
            DW(Iend + i, j, k) = D(i, j) * W(Iend + i, j, k);
          }
        }
      }
    for (int k = Kbeg; k <= Kend; ++k)
      for (int i = Ibeg; i <= Iend; ++i) {
        if (p.bc_y0 == 5) {
          const double Phi = wall_phi(dy, U(i, Jbeg, k), W(i, Jbeg, k), CmuHt(i, Jbeg, k));
          for (int j = 1; j <= Nghost; ++j) {
            U(i, Jbeg - j, k) = (1.0 - Phi) * U(i, Jbeg + j - 1, k);
            V(i, Jbeg - j, k) = -V(i, Jbeg + j - 1, k);
            W(i, Jbeg - j, k) = (1.0 - Phi) * W(i, Jbeg + j - 1, k);
            DU(i, Jbeg - j, k) = D(i, j) * U(i, Jbeg - j, k);
            DV(i, Jbeg - j, k) = D(i, j) * V(i, Jbeg - j, k);
            DW(i, Jbeg - j, k) = D(i, j) * W(i, Jbeg - j, k);
          }
        }
        if (p.bc_yn == 5) {
          const double Phi = wall_phi(dy, U(i, Jend, k), W(i, Jend, k), CmuHt(i, Jend, k));
          for (int j = 1; j <= Nghost; ++j) {
            U(i, Jend + j, k) = (1.0 - Phi) * U(i, Jend - j + 1, k);
            V(i, Jend + j, k) = -V(i, Jend - j + 1, k);
            W(i, Jend + j, k) = (1.0 - Phi) * W(i, Jend - j + 1, k);
            DU(i, Jend + j, k) = D(i, j) * U(i, Jend + j, k);
            DV(i, Jend + j, k) = D(i, j) * V(i, Jend + j, k);
            DW(i, Jend + j, k) = D(i, j) * W(i, Jend + j, k);
          }
        }
      }
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = 1; i <= Nghost; ++i) {
          if (p.bc_x0 == 5) break;
          if (p.bc_x0 == 3) {   // inflow (src/nhwave.F:4468-4476)
            U(Ibeg - i, j, k) = 2.0 * Uin_X0(j, k) - U(Ibeg + i - 1, j, k);
            V(Ibeg - i, j, k) = 2.0 * Vin_X0(j, k) - V(Ibeg + i - 1, j, k);
            W(Ibeg - i, j, k) = 2.0 * Win_X0(j, k) - W(Ibeg + i - 1, j, k);
            DU(Ibeg - i, j, k) = 2.0 * Din_X0(j) * Uin_X0(j, k) - DU(Ibeg + i - 1, j, k);
            DV(Ibeg - i, j, k) = 2.0 * Din_X0(j) * Vin_X0(j, k) - DV(Ibeg + i - 1, j, k);
            DW(Ibeg - i, j, k) = 2.0 * Din_X0(j) * Win_X0(j, k) - DW(Ibeg + i - 1, j, k);
            continue;
          }
          U(Ibeg - i, j, k) = -U(Ibeg + i - 1, j, k);
          V(Ibeg - i, j, k) = sx0 * V(Ibeg + i - 1, j, k);
          W(Ibeg - i, j, k) = sx0 * W(Ibeg + i - 1, j, k);
          DU(Ibeg - i, j, k) = -DU(Ibeg + i - 1, j, k);
          DV(Ibeg - i, j, k) = sx0 * DV(Ibeg + i - 1, j, k);
          DW(Ibeg - i, j, k) = sx0 * DW(Ibeg + i - 1, j, k);
        }
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = 1; i <= Nghost; ++i) {
          if (p.bc_xn == 5) break;
          if (p.bc_xn == 3) {   // inflow/outflow (src/nhwave.F:4547-4572)
            auto cgf = [&](A3& X0, A3& X00) {
              const double Cg = -(X0(Iend + i - 1, j, k) - X00(Iend + i - 1, j, k) + kOrlSmall) /
                                (X00(Iend + i - 1, j, k) - X00(Iend + i - 2, j, k) + kOrlSmall);
              return dmax(dmin(Cg, 1.0), 0.0);
            };
            double Cg = cgf(U0, U00);
            if (i == 1)
              U(Iend + i, j, k) = Cg * U(Iend + i - 1, j, k) + Uin_Xni0(j, k) - Cg * Uin_Xni(j, k);
            else
              U(Iend + i, j, k) = Cg * U(Iend + i - 1, j, k) + (1.0 - Cg) * U(Iend + i, j, k);
            Cg = cgf(V0, V00);
            V(Iend + i, j, k) = Cg * V0(Iend + i - 1, j, k) + (1.0 - Cg) * V0(Iend + i, j, k);
            Cg = cgf(W0, W00);
            W(Iend + i, j, k) = Cg * W0(Iend + i - 1, j, k) + (1.0 - Cg) * W0(Iend + i, j, k);
            DU(Iend + i, j, k) = 2.0 * Din_Xn(j) * Uin_Xn(j, k) - DU(Iend - i + 1, j, k);
            DV(Iend + i, j, k) = 2.0 * Din_Xn(j) * Vin_Xn(j, k) - DV(Iend - i + 1, j, k);
            DW(Iend + i, j, k) = 2.0 * Din_Xn(j) * Win_Xn(j, k) - DW(Iend - i + 1, j, k);
            continue;
          }
          if (p.bc_xn == 6) {   // Orlanski radiation (src/nhwave.F:4599-4621)
            auto orl = [&](A3& X0, A3& X00) {
              double Cg = -(X0(Iend + i - 1, j, k) - X00(Iend + i - 1, j, k) + kOrlSmall) /
                          (X00(Iend + i - 1, j, k) - X00(Iend + i - 2, j, k) + kOrlSmall);
              Cg = dmax(dmin(Cg, 1.0), 0.0);
              return Cg * X0(Iend + i - 1, j, k) + (1.0 - Cg) * X0(Iend + i, j, k);
            };
            U(Iend + i, j, k) = orl(U0, U00);
            V(Iend + i, j, k) = orl(V0, V00);
            W(Iend + i, j, k) = orl(W0, W00);
            DU(Iend + i, j, k) = D(Iend + i, j) * U(Iend + i, j, k);
            DV(Iend + i, j, k) = D(Iend + i, j) * V(Iend + i, j, k);
            DW(Iend + i, j, k) = D(Iend + i, j) * W(Iend + i, j, k);
            continue;
          }
          U(Iend + i, j, k) = -U(Iend - i + 1, j, k);
          V(Iend + i, j, k) = sxn * V(Iend - i + 1, j, k);
          W(Iend + i, j, k) = sxn * W(Iend - i + 1, j, k);
          DU(Iend + i, j, k) = -DU(Iend - i + 1, j, k);
          DV(Iend + i, j, k) = sxn * DV(Iend - i + 1, j, k);
          DW(Iend + i, j, k) = sxn * DW(Iend - i + 1, j, k);
        }
    for (int k = Kbeg; k <= Kend; ++k)
      for (int i = Ibeg; i <= Iend; ++i)
        for (int j = 1; j <= Nghost; ++j) {
          if (p.bc_y0 == 5) break;
          U(i, Jbeg - j, k) = sy0 * U(i, Jbeg + j - 1, k);
          V(i, Jbeg - j, k) = -V(i, Jbeg + j - 1, k);
          W(i, Jbeg - j, k) = sy0 * W(i, Jbeg + j - 1, k);
          DU(i, Jbeg - j, k) = sy0 * DU(i, Jbeg + j - 1, k);
          DV(i, Jbeg - j, k) = -DV(i, Jbeg + j - 1, k);
          DW(i, Jbeg - j, k) = sy0 * DW(i, Jbeg + j - 1, k);
        }
    for (int k = Kbeg; k <= Kend; ++k)
      for (int i = Ibeg; i <= Iend; ++i)
        for (int j = 1; j <= Nghost; ++j) {
          if (p.bc_yn == 5) break;
          U(i, Jend + j, k) = syn * U(i, Jend - j + 1, k);
          V(i, Jend + j, k) = -V(i, Jend - j + 1, k);
          W(i, Jend + j, k) = syn * W(i, Jend - j + 1, k);
          DU(i, Jend + j, k) = syn * DU(i, Jend - j + 1, k);
          DV(i, Jend + j, k) = -DV(i, Jend - j + 1, k);
          DW(i, Jend + j, k) = syn * DW(i, Jend - j + 1, k);
        }
    A3 DelxUzL, DelxVzL, DelxWzL, DelyUzL, DelyVzL, DelyWzL;
    for (A3* a : {&DelxUzL, &DelxVzL, &DelxWzL, &DelyUzL, &DelyVzL, &DelyWzL}) a->init(Mloc, Nloc, Kloc1);
    delzFun_3D(U, DelzU); delzFun_3D(V, DelzV); delzFun_3D(W, DelzW);
    construct_3D_z(U, DelzU, UzL, UzR); construct_3D_z(V, DelzV, VzL, VzR);
    construct_3D_z(W, DelzW, WzL, WzR);
    KBC_surface();
    KBC_bottom();
    delxFun_3D(UzL, DelxUzL); delxFun_3D(VzL, DelxVzL); delxFun_3D(WzL, DelxWzL);
    delyFun_3D(UzL, DelyUzL); delyFun_3D(VzL, DelyVzL); delyFun_3D(WzL, DelyWzL);
    // bed-face slopes, read by the stress ghosts of BC_Z0 = 2, 5
    A3 DelxUzR, DelxVzR, DelxWzR, DelyUzR, DelyVzR, DelyWzR;
    if (p.bc_z0 != 1) {
      for (A3* a : {&DelxUzR, &DelxVzR, &DelxWzR, &DelyUzR, &DelyVzR, &DelyWzR}) a->init(Mloc, Nloc, Kloc1);
      delxFun_3D(UzR, DelxUzR); delxFun_3D(VzR, DelxVzR); delxFun_3D(WzR, DelxWzR);
      delyFun_3D(UzR, DelyUzR); delyFun_3D(VzR, DelyVzR); delyFun_3D(WzR, DelyWzR);
    }
    const double MinDepBC = (double)0.01f;
    for (int j = Jbeg; j <= Jend; ++j)
      for (int i = Ibeg; i <= Iend; ++i) {
        const double visc_top =
            Small + 0.5 * (Cmu + CmuR + CmuVt(i, j, Kend) + Cmu + CmuR + CmuVt(i, j, Kend + 1));
        const double visc_bot = Cmu + CmuR + CmuVt(i, j, Kbeg);
        const double dxe = DelxEta(i, j), dye = DelyEta(i, j), Dij = D(i, j);
        const double Atop = std::sqrt(1.0 + dxe * dxe + dye * dye);
        const double Fext_Wind1 = 1.0 / Atop * ((1 - dxe * dxe) * Wsx(i, j) - dxe * dye * Wsy(i, j));
        const double Fext_Wind2 = 1.0 / Atop * ((1 - dye * dye) * Wsy(i, j) - dxe * dye * Wsx(i, j));
        // bed stress (src/nhwave.F:4806-4847)
        const double dxh = DelxH(i, j), dyh = DelyH(i, j);
        const double Abot = std::sqrt(1.0 + dxh * dxh + dyh * dyh), Bbot = std::sqrt(1.0 + dxh * dxh);
        double Fext_Bot1 = 0.0, Fext_Bot2 = 0.0;
        if (p.bc_z0 != 1) {
          const double DUprime = (DU(i, j, Kbeg) - dxh * DW(i, j, Kbeg)) / Bbot;
          // the reference's "DU(i,j,Kbeg)* +(1.0+DelxH**2)*DV(i,j,Kbeg)" multiplies
          // the two terms (a unary plus after '*'), so on a flat bed DVprime is 0
          const double DVprime =
              (-(dxh * dyh * DU(i, j, Kbeg) * ((1.0 + dxh * dxh) * DV(i, j, Kbeg))) - dyh * DW(i, j, Kbeg)) / Abot / Bbot;
          const double DUmag = std::sqrt(DUprime * DUprime + DVprime * DVprime);
          const double Dz1 = 0.5 * Dij * dsig(Kbeg) / Abot;
          const double Z0 = p.zob / 30.0;
          double Cdrag = p.ibot == 1 ? p.cd0 : (Kappa / std::log(Dz1 / Z0)) * (Kappa / std::log(Dz1 / Z0));
          Cdrag = dmin(Cdrag, visc_bot / Dz1 / (DUmag + Small) * Dij);
          double TauBot1 = Zero, TauBot2 = Zero;
          if (p.bc_z0 == 2) {
            TauBot1 = DUprime / Dij / Dz1 * visc_bot;
            TauBot2 = DVprime / Dij / Dz1 * visc_bot;
          } else if (p.bc_z0 == 5) {
            TauBot1 = Cdrag * DUprime * DUmag / (Dij * Dij);
            TauBot2 = Cdrag * DVprime * DUmag / (Dij * Dij);
          }
          Fext_Bot1 = Bbot * TauBot1;
          Fext_Bot2 = (dxh * dyh * TauBot1 + Abot * TauBot2) / Bbot;
        }
        for (int k = 1; k <= Nghost; ++k) {
          // bottom
          DW(i, j, Kbeg - k) = 2.0 * Dij * WzR(i, j, Kbeg) - DW(i, j, Kbeg + k - 1);
          if (p.bc_z0 == 1) {   // free slip
            DU(i, j, Kbeg - k) = DU(i, j, Kbeg + k - 1);
            DV(i, j, Kbeg - k) = DV(i, j, Kbeg + k - 1);
          } else {   // stress ghosts (src/nhwave.F:4869-4903)
            const double dsb = sigc(Kbeg + k - 1) - sigc(Kbeg - k);
            const double vb = Small + Cmu + CmuR + CmuVt(i, j, Kbeg);
            DU(i, j, Kbeg - k) = DU(i, j, Kbeg + k - 1) -
                dsb * (Fext_Bot1 * (Dij * Dij / Abot / vb) +
                       dxh * (DW(i, j, Kbeg + k - 1) - Dij * WzR(i, j, Kbeg)) / (dsb / 2.0) +
                       Dij * Dij / (Abot * Abot) *
                           (-2.0 * dxh * DelxUzR(i, j, Kbeg) - (1.0 - dxh * dxh) * DelxWzR(i, j, Kbeg) -
                            dyh * (DelyUzR(i, j, Kbeg) + DelxVzR(i, j, Kbeg) - dxh * DelyWzR(i, j, Kbeg))));
            const double DUbot_old = 2.0 * Dij * UzR(i, j, Kbeg) - DU(i, j, Kbeg + k - 1);
            if (DUbot_old > 0.) DU(i, j, Kbeg - k) = dmin(3.0 * DUbot_old, dmax(-1.0 * DUbot_old, DU(i, j, Kbeg - k)));
            else if (DUbot_old < 0.) DU(i, j, Kbeg - k) = dmax(3.0 * DUbot_old, dmin(-1.0 * DUbot_old, DU(i, j, Kbeg - k)));
            if (Dij < MinDepBC) DU(i, j, Kbeg - k) = DU(i, j, Kbeg + k - 1);
            DV(i, j, Kbeg - k) = DV(i, j, Kbeg + k - 1) -
                dsb * (Fext_Bot2 * (Dij * Dij / Abot / vb) +
                       dyh * (DW(i, j, Kbeg + k - 1) - Dij * WzR(i, j, Kbeg)) / (dsb / 2.0) +
                       Dij * Dij / (Abot * Abot) *
                           (-2.0 * dyh * DelyVzR(i, j, Kbeg) - (1.0 - dyh * dyh) * DelyWzR(i, j, Kbeg) -
                            dxh * (DelxVzR(i, j, Kbeg) + DelyUzR(i, j, Kbeg) - dyh * DelxWzR(i, j, Kbeg))));
            const double DVbot_old = 2.0 * Dij * VzR(i, j, Kbeg) - DV(i, j, Kbeg + k - 1);
            if (DVbot_old > 0.) DV(i, j, Kbeg - k) = dmin(3.0 * DVbot_old, dmax(-1.0 * DVbot_old, DV(i, j, Kbeg - k)));
            else if (DVbot_old < 0.) DV(i, j, Kbeg - k) = dmax(3.0 * DVbot_old, dmin(-1.0 * DVbot_old, DV(i, j, Kbeg - k)));
            if (Dij < MinDepBC) DV(i, j, Kbeg - k) = DV(i, j, Kbeg + k - 1);
          }
          // surface
          const double dsg = sigc(Kend + k) - sigc(Kend - k + 1);
          DW(i, j, Kend + k) = 2.0 * Dij * WzL(i, j, Kend1) - DW(i, j, Kend - k + 1);
          DU(i, j, Kend + k) = DU(i, j, Kend - k + 1) +
              dsg * (Fext_Wind1 * (Dij * Dij / Atop / visc_top) -
                     dxe * (Dij * WzL(i, j, Kend1) - DW(i, j, Kend - k + 1)) / (dsg / 2.0) +
                     Dij * Dij / (Atop * Atop) *
                         (+2.0 * dxe * DelxUzL(i, j, Kend1) - (1.0 - dxe * dxe) * DelxWzL(i, j, Kend1) +
                          dye * (DelyUzL(i, j, Kend1) + DelxVzL(i, j, Kend1) + dxe * DelyWzL(i, j, Kend1))));
          const double DUtop_old = 2.0 * Dij * UzL(i, j, Kend1) - DU(i, j, Kend - k + 1);
          if (DUtop_old > 0.) DU(i, j, Kend + k) = dmin(3.0 * DUtop_old, dmax(-1.0 * DUtop_old, DU(i, j, Kend + k)));
          else if (DUtop_old < 0.) DU(i, j, Kend + k) = dmax(3.0 * DUtop_old, dmin(-1.0 * DUtop_old, DU(i, j, Kend + k)));
          if (Dij < MinDepBC) DU(i, j, Kend + k) = DU(i, j, Kend - k + 1);
          DV(i, j, Kend + k) = DV(i, j, Kend - k + 1) +
              dsg * (Fext_Wind2 * (Dij * Dij / Atop / visc_top) -
                     dye * (Dij * WzL(i, j, Kend1) - DW(i, j, Kend - k + 1)) / (dsg / 2.0) +
                     Dij * Dij / (Atop * Atop) *
                         (+2.0 * dye * DelyVzL(i, j, Kend1) - (1.0 - dye * dye) * DelyWzL(i, j, Kend1) +
                          dxe * (DelxVzL(i, j, Kend1) + DelyUzL(i, j, Kend1) + dye * DelxWzL(i, j, Kend1))));
          const double DVtop_old = 2.0 * Dij * VzL(i, j, Kend1) - DV(i, j, Kend - k + 1);
          if (DVtop_old > 0.) DV(i, j, Kend + k) = dmin(3.0 * DVtop_old, dmax(-1.0 * DVtop_old, DV(i, j, Kend + k)));
          else if (DVtop_old < 0.) DV(i, j, Kend + k) = dmax(3.0 * DVtop_old, dmin(-1.0 * DVtop_old, DV(i, j, Kend + k)));
          if (Dij < MinDepBC) DV(i, j, Kend + k) = DV(i, j, Kend - k + 1);
          U(i, j, Kbeg - k) = DU(i, j, Kbeg - k) / Dij;
          V(i, j, Kbeg - k) = DV(i, j, Kbeg - k) / Dij;
          W(i, j, Kbeg - k) = DW(i, j, Kbeg - k) / Dij;
          U(i, j, Kend + k) = DU(i, j, Kend + k) / Dij;
          V(i, j, Kend + k) = DV(i, j, Kend + k) / Dij;
          W(i, j, Kend + k) = DW(i, j, Kend + k) / Dij;
        }
      }
  }

  void get_UVW() {
    for (int j = Jbeg; j <= Jend; ++j)
      for (int i = Ibeg; i <= Iend; ++i)
        for (int k = Kbeg; k <= Kend; ++k) {
          U(i, j, k) = DU(i, j, k) / D(i, j);
          V(i, j, k) = DV(i, j, k) / D(i, j);
          W(i, j, k) = DW(i, j, k) / D(i, j);
        }
    vel_bc();
  }

  void interpolate_velocity_to_faces() {
    for (int k = 2; k <= Kloc; ++k)
      for (int j = 1; j <= Nloc; ++j)
        for (int i = 1; i <= Mloc; ++i) {
          double f = dsig(k) / (dsig(k) + dsig(k - 1));
          Uf(i, j, k) = (1.0 - f) * U(i, j, k) + f * U(i, j, k - 1);
          Vf(i, j, k) = (1.0 - f) * V(i, j, k) + f * V(i, j, k - 1);
          Wf(i, j, k) = (1.0 - f) * W(i, j, k) + f * W(i, j, k - 1);
        }
    for (int j = 1; j <= Nloc; ++j)
      for (int i = 1; i <= Mloc; ++i) {
        Uf(i, j, 1) = U(i, j, 1); Vf(i, j, 1) = V(i, j, 1); Wf(i, j, 1) = W(i, j, 1);
        Uf(i, j, Kloc1) = U(i, j, Kloc); Vf(i, j, Kloc1) = V(i, j, Kloc); Wf(i, j, Kloc1) = W(i, j, Kloc);
      }
  }

  // ---------------------------------------------------- generate_coef_rhs
  int idx(int i, int j, int k) { return (i - Ibeg) + p.Mglob * ((j - Jbeg) + p.Nglob * (k - Kbeg)); }
  double& C(int ic, int n) { return Coef[(size_t)(n - 1) * neqns + ic]; }

  void generate_coef_rhs() {
    A3 DelxS, DelyS, DelzS, A1s;
    for (A3* a : {&DelxS, &DelyS, &DelzS, &A1s}) a->init(Mloc, Nloc, Kloc1);
    for (int k = Kbeg; k <= Kend1; ++k)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i) {
          DelxS(i, j, k) = (1. - sig(k)) / D(i, j) * DelxH(i, j) - sig(k) / D(i, j) * DelxEta(i, j);
          DelyS(i, j, k) = (1. - sig(k)) / D(i, j) * DelyH(i, j) - sig(k) / D(i, j) * DelyEta(i, j);
          DelzS(i, j, k) = 1. / D(i, j);
          A1s(i, j, k) = DelxS(i, j, k) * DelxS(i, j, k) + DelyS(i, j, k) * DelyS(i, j, k) +
                         DelzS(i, j, k) * DelzS(i, j, k);
        }
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i) {
          const double hk = 0.5 * (dsig(k) + dsig(k - 1));
          Rhs[idx(i, j, k)] =
              -((Uf(i + 1, j, k) - Uf(i - 1, j, k)) / (2.0 * dx) + (U(i, j, k) - U(i, j, k - 1)) / hk * DelxS(i, j, k) +
                (Vf(i, j + 1, k) - Vf(i, j - 1, k)) / (2.0 * dy) + (V(i, j, k) - V(i, j, k - 1)) / hk * DelyS(i, j, k) +
                (W(i, j, k) - W(i, j, k - 1)) / hk * DelzS(i, j, k) - SourceC(i, j)) *
              Rho0 / dt;
        }
    std::fill(Coef.begin(), Coef.end(), 0.0);
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i) {
          const int ic = idx(i, j, k);
          const double s = dsig(k) + dsig(k - 1), hk = 0.5 * (dsig(k) + dsig(k - 1));
          const double a1 = A1s(i, j, k);
          C(ic, 1) = 2. / (dx * dx) + 2. / (dy * dy) + a1 / (hk * dsig(k)) + a1 / (hk * dsig(k - 1));
          C(ic, 2) = -1. / (dx * dx);
          C(ic, 3) = -1. / (dy * dy);
          C(ic, 4) = DelyS(i, j - 1, k) / (2. * dy * s) + DelyS(i, j, k) / (2. * dy * s);
          C(ic, 5) = DelxS(i - 1, j, k) / (2. * dx * s) + DelxS(i, j, k) / (2. * dx * s);
          C(ic, 6) = -a1 / (hk * dsig(k));
          C(ic, 7) = -(DelxS(i + 1, j, k) / (2. * dx * s) + DelxS(i, j, k) / (2. * dx * s));
          C(ic, 8) = -(DelyS(i, j + 1, k) / (2. * dy * s) + DelyS(i, j, k) / (2. * dy * s));
          C(ic, 9) = -1. / (dx * dx);
          C(ic, 10) = -1. / (dy * dy);
          C(ic, 11) = DelyS(i, j + 1, k) / (2. * dy * s) + DelyS(i, j, k) / (2. * dy * s);
          C(ic, 12) = DelxS(i + 1, j, k) / (2. * dx * s) + DelxS(i, j, k) / (2. * dx * s);
          C(ic, 13) = -a1 / (hk * dsig(k - 1));
          C(ic, 14) = -(DelxS(i - 1, j, k) / (2. * dx * s) + DelxS(i, j, k) / (2. * dx * s));
          C(ic, 15) = -(DelyS(i, j - 1, k) / (2. * dy * s) + DelyS(i, j, k) / (2. * dy * s));
        }
    auto fold = [&](int ic, int dst, int src) { C(ic, dst) = C(ic, dst) + C(ic, src); };
    for (int k = Kbeg; k <= Kend; ++k)  // left
      for (int j = Jbeg; j <= Jend; ++j) {
        int ic = idx(Ibeg, j, k);
        fold(ic, 1, 9); fold(ic, 6, 5); fold(ic, 13, 14);
        C(ic, 9) = Zero; C(ic, 5) = Zero; C(ic, 14) = Zero;
      }
    for (int k = Kbeg; k <= Kend; ++k)  // right
      for (int j = Jbeg; j <= Jend; ++j) {
        int ic = idx(Iend, j, k);
        fold(ic, 1, 2); fold(ic, 6, 7); fold(ic, 13, 12);
        C(ic, 2) = Zero; C(ic, 7) = Zero; C(ic, 12) = Zero;
      }
    for (int k = Kbeg; k <= Kend; ++k)  // front
      for (int i = Ibeg; i <= Iend; ++i) {
        int ic = idx(i, Jbeg, k);
        fold(ic, 1, 10); fold(ic, 6, 4); fold(ic, 13, 15);
        C(ic, 10) = Zero; C(ic, 4) = Zero; C(ic, 15) = Zero;
      }
    for (int k = Kbeg; k <= Kend; ++k)  // back
      for (int i = Ibeg; i <= Iend; ++i) {
        int ic = idx(i, Jend, k);
        fold(ic, 1, 3); fold(ic, 6, 8); fold(ic, 13, 11);
        C(ic, 3) = Zero; C(ic, 8) = Zero; C(ic, 11) = Zero;
      }
    for (int j = Jbeg; j <= Jend; ++j)  // bottom (Neumann)
      for (int i = Ibeg; i <= Iend; ++i) {
        int ic = idx(i, j, Kbeg);
        if (p.slide_type == NHW_SLIDE_RIGID_3D)
          Rhs[ic] = Rhs[ic] + Rho0 * (dsig(Kbeg) + dsig(Kbeg - 1)) *
                                  (C(ic, 13) * D(i, j) * Delt2H(i, j) + C(ic, 12) * D(i + 1, j) * Delt2H(i + 1, j) +
                                   C(ic, 11) * D(i, j + 1) * Delt2H(i, j + 1) + C(ic, 14) * D(i - 1, j) * Delt2H(i - 1, j) +
                                   C(ic, 15) * D(i, j - 1) * Delt2H(i, j - 1));
        fold(ic, 6, 13); fold(ic, 7, 12); fold(ic, 8, 11); fold(ic, 5, 14); fold(ic, 4, 15);
        C(ic, 13) = Zero; C(ic, 12) = Zero; C(ic, 11) = Zero; C(ic, 14) = Zero; C(ic, 15) = Zero;
      }
    for (int j = Jbeg; j <= Jend; ++j)  // top (Dirichlet)
      for (int i = Ibeg; i <= Iend; ++i) {
        int ic = idx(i, j, Kend);
        C(ic, 4) = Zero; C(ic, 5) = Zero; C(ic, 6) = Zero; C(ic, 7) = Zero; C(ic, 8) = Zero;
      }
  }

  // ------------------------------------------- Poisson solve (oracle's own)
  // stencil offsets of src/pressure.F:276-278 (diagonals 1..15)
  const int OFF[15][3] = {{0, 0, 0},  {1, 0, 0},  {0, 1, 0},   {0, -1, 1}, {-1, 0, 1},
                          {0, 0, 1},  {1, 0, 1},  {0, 1, 1},   {-1, 0, 0}, {0, -1, 0},
                          {0, 1, -1}, {1, 0, -1}, {0, 0, -1},  {-1, 0, -1}, {0, -1, -1}};

  void matvec(const std::vector<double>& xv, std::vector<double>& yv) {
    const int M = p.Mglob, N = p.Nglob, K = p.Kglob;
    for (int k = 0; k < K; ++k)
      for (int j = 0; j < N; ++j)
        for (int i = 0; i < M; ++i) {
          int ic = i + M * (j + N * k);
          double s = 0.0;
          for (int n = 0; n < 15; ++n) {
            int ii = i + OFF[n][0], jj = j + OFF[n][1], kk = k + OFF[n][2];
            if (ii < 0 || ii >= M || jj < 0 || jj >= N || kk < 0 || kk >= K) continue;
            s += Coef[(size_t)n * neqns + ic] * xv[ii + M * (jj + N * kk)];
          }
          yv[ic] = s;
        }
  }
  // vertical-line preconditioner: tridiagonal (Coef 13, 1, 6) per column
  void precond(const std::vector<double>& r, std::vector<double>& z) {
    const int M = p.Mglob, N = p.Nglob, K = p.Kglob, MN = M * N;
    std::vector<double> cp(K), dp(K);
    for (int c = 0; c < MN; ++c) {
      for (int k = 0; k < K; ++k) {
        int ic = c + MN * k;
        double a = k > 0 ? Coef[(size_t)12 * neqns + ic] : 0.0;
        double b = Coef[ic];
        double cc = k < K - 1 ? Coef[(size_t)5 * neqns + ic] : 0.0;
        double den = b - (k > 0 ? a * cp[k - 1] : 0.0);
        cp[k] = cc / den;
        dp[k] = (r[ic] - (k > 0 ? a * dp[k - 1] : 0.0)) / den;
      }
      for (int k = K - 1; k >= 0; --k) {
        int ic = c + MN * k;
        z[ic] = dp[k] - (k < K - 1 ? cp[k] * z[ic + MN] : 0.0);
      }
    }
  }
  static double dot(const std::vector<double>& a, const std::vector<double>& b) {
    double s = 0.0;
    for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
    return s;
  }

  // restarted GMRES(m), right preconditioned; returns status
  int solve(std::vector<double>& xsol) {
    const int n = neqns, m = 40;
    const double bnorm = std::sqrt(dot(Rhs, Rhs));
    last_iters = 0;
    if (bnorm == 0.0) { std::fill(xsol.begin(), xsol.end(), 0.0); last_relres = 0.0; return NHW_OK; }
    std::vector<double> r(n), w(n), z(n);
    std::vector<std::vector<double>> Vb(m + 1, std::vector<double>(n)), Zb(m, std::vector<double>(n));
    std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1);
    int it = 0;
    double relres = 0.0;
    while (true) {
      matvec(xsol, w);
      for (int i = 0; i < n; ++i) r[i] = Rhs[i] - w[i];
      double beta = std::sqrt(dot(r, r));
      relres = beta / bnorm;
      if (!(relres == relres)) { last_relres = relres; return NHW_ERR_NAN; }
      if (relres <= p.tol || it >= p.itmax) break;
      for (int i = 0; i < n; ++i) Vb[0][i] = r[i] / beta;
      std::fill(g.begin(), g.end(), 0.0);
      g[0] = beta;
      int j = 0;
      for (; j < m && it < p.itmax; ++j) {
        ++it;
        precond(Vb[j], Zb[j]);
        matvec(Zb[j], w);
        for (int i2 = 0; i2 <= j; ++i2) {
          double h = dot(w, Vb[i2]);
          H[(size_t)i2 * m + j] = h;
          for (int q = 0; q < n; ++q) w[q] -= h * Vb[i2][q];
        }
        double hn = std::sqrt(dot(w, w));
        H[(size_t)(j + 1) * m + j] = hn;
        if (hn != 0.0)
          for (int q = 0; q < n; ++q) Vb[j + 1][q] = w[q] / hn;
        for (int i2 = 0; i2 < j; ++i2) {
          double a = H[(size_t)i2 * m + j], b = H[(size_t)(i2 + 1) * m + j];
          H[(size_t)i2 * m + j] = cs[i2] * a + sn[i2] * b;
          H[(size_t)(i2 + 1) * m + j] = -sn[i2] * a + cs[i2] * b;
        }
        double a = H[(size_t)j * m + j], b = H[(size_t)(j + 1) * m + j];
        double den = std::sqrt(a * a + b * b);
        cs[j] = den == 0.0 ? 1.0 : a / den;
        sn[j] = den == 0.0 ? 0.0 : b / den;
        H[(size_t)j * m + j] = den;
        H[(size_t)(j + 1) * m + j] = 0.0;
        g[j + 1] = -sn[j] * g[j];
        g[j] = cs[j] * g[j];
        if (std::fabs(g[j + 1]) / bnorm <= p.tol * 0.5 || hn == 0.0) { ++j; break; }
      }
      // back-substitution and update x += Z y
      std::vector<double> yv(j, 0.0);
      for (int i2 = j - 1; i2 >= 0; --i2) {
        double s = g[i2];
        for (int q = i2 + 1; q < j; ++q) s -= H[(size_t)i2 * m + q] * yv[q];
        yv[i2] = s / H[(size_t)i2 * m + i2];
      }
      for (int i2 = 0; i2 < j; ++i2)
        for (int q = 0; q < n; ++q) xsol[q] += yv[i2] * Zb[i2][q];
    }
    last_iters = it;
    last_relres = relres;
    total_iters += it;
    ++solves;
    return relres <= p.tol ? NHW_OK : NHW_ERR_KRYLOV_NOCONV;
  }

  int poisson_solver() {
    generate_coef_rhs();
    std::vector<double> Phi(neqns);
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i) Phi[idx(i, j, k)] = P(i, j, k);
    int st = solve(Phi);
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i) P(i, j, k) = Phi[idx(i, j, k)];
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = 1; i <= Nghost; ++i) {
          P(Ibeg - i, j, k) = P(Ibeg + i - 1, j, k);
          P(Iend + i, j, k) = P(Iend - i + 1, j, k);
        }
    for (int k = Kbeg; k <= Kend; ++k)
      for (int i = Ibeg; i <= Iend; ++i)
        for (int j = 1; j <= Nghost; ++j) {
          P(i, Jbeg - j, k) = P(i, Jbeg + j - 1, k);
          P(i, Jend + j, k) = P(i, Jend - j + 1, k);
        }
    return st;
  }

  void projection_corrector() {
    A3 DelxP, DelyP, DelzP;
    for (A3* a : {&DelxP, &DelyP, &DelzP}) a->init(Mloc, Nloc, Kloc);
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i) {
          DelxP(i, j, k) = 0.5 * ((P(i + 1, j, k) - P(i - 1, j, k)) / (2. * dx) +
                                  (P(i + 1, j, k + 1) - P(i - 1, j, k + 1)) / (2. * dx));
          DelyP(i, j, k) = 0.5 * ((P(i, j + 1, k) - P(i, j - 1, k)) / (2. * dy) +
                                  (P(i, j + 1, k + 1) - P(i, j - 1, k + 1)) / (2. * dy));
          DelzP(i, j, k) = (P(i, j, k + 1) - P(i, j, k)) / dsig(k);
        }
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i) {
          if (Mask(i, j) == 0) continue;
          DU(i, j, k) = DU(i, j, k) - D(i, j) * dt / Rho0 * (DelxP(i, j, k) + DelzP(i, j, k) * DelxSc(i, j, k));
          DV(i, j, k) = DV(i, j, k) - D(i, j) * dt / Rho0 * (DelyP(i, j, k) + DelzP(i, j, k) * DelySc(i, j, k));
          DW(i, j, k) = DW(i, j, k) - dt / Rho0 * DelzP(i, j, k);
        }
  }

  // ------------------------------------------------------------ get_Omega
  void get_Omega() {
    delxFun_2D(Eta, DelxEta); delyFun_2D(Eta, DelyEta);
    delxFun_3D(U, DelxU); delxFun_3D(V, DelxV); delyFun_3D(U, DelyU); delyFun_3D(V, DelyV);
    delxFun_3D(DU, DelxDU); delxFun_3D(DV, DelxDV); delyFun_3D(DU, DelyDU); delyFun_3D(DV, DelyDV);
    construct_2D_x(Eta, DelxEta, EtaxL, EtaxR); construct_2D_y(Eta, DelyEta, EtayL, EtayR);
    construct_3D_x(U, DelxU, UxL, UxR); construct_3D_x(V, DelxV, VxL, VxR);
    construct_3D_y(U, DelyU, UyL, UyR); construct_3D_y(V, DelyV, VyL, VyR);
    construct_3D_x(DU, DelxDU, DUxL, DUxR); construct_3D_x(DV, DelxDV, DVxL, DVxR);
    construct_3D_y(DU, DelyDU, DUyL, DUyR); construct_3D_y(DV, DelyDV, DVyL, DVyR);
    for (int j = Jbeg; j <= Jend; ++j)
      for (int i = Ibeg; i <= Iend1; ++i) { DxL(i, j) = EtaxL(i, j) + Hfx(i, j); DxR(i, j) = EtaxR(i, j) + Hfx(i, j); }
    for (double& v : DxL.v) v = dmax(v, MinDep);
    for (double& v : DxR.v) v = dmax(v, MinDep);
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i) {
          if (Mask(i, j) == 1 && Mask(i + 1, j) == 0) {
            EtaxL(i + 1, j) = Eta(i, j); DxL(i + 1, j) = D(i, j); DUxL(i + 1, j, k) = Zero;
          } else if (Mask(i, j) == 1 && Mask(i - 1, j) == 0) {
            EtaxR(i, j) = Eta(i, j); DxR(i, j) = D(i, j); DUxR(i, j, k) = Zero;
          } else if (Mask(i, j) == 0) {
            EtaxL(i + 1, j) = Eta(i, j); DxL(i + 1, j) = D(i, j); DUxL(i + 1, j, k) = Zero; DVxL(i + 1, j, k) = Zero;
            EtaxR(i, j) = Eta(i, j); DxR(i, j) = D(i, j); DUxR(i, j, k) = Zero;
          }
        }
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend1; ++i) { ExL(i, j, k) = DUxL(i, j, k); ExR(i, j, k) = DUxR(i, j, k); }
    for (int j = Jbeg; j <= Jend1; ++j)
      for (int i = Ibeg; i <= Iend; ++i) { DyL(i, j) = EtayL(i, j) + Hfy(i, j); DyR(i, j) = EtayR(i, j) + Hfy(i, j); }
    for (double& v : DyL.v) v = dmax(v, MinDep);
    for (double& v : DyR.v) v = dmax(v, MinDep);
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i) {
          if (Mask(i, j) == 1 && Mask(i, j + 1) == 0) {
            EtayL(i, j + 1) = Eta(i, j); DyL(i, j + 1) = D(i, j); DVyL(i, j + 1, k) = Zero;
          } else if (Mask(i, j) == 1 && Mask(i, j - 1) == 0) {
            EtayR(i, j) = Eta(i, j); DyR(i, j) = D(i, j); DVyR(i, j, k) = Zero;
          } else if (Mask(i, j) == 0) {
            EtayL(i, j + 1) = Eta(i, j); DyL(i, j + 1) = D(i, j); DVyL(i, j + 1, k) = Zero;
            EtayR(i, j) = Eta(i, j); DyR(i, j) = D(i, j); DVyR(i, j, k) = Zero;
          }
        }
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend1; ++j)
        for (int i = Ibeg; i <= Iend; ++i) { EyL(i, j, k) = DVyL(i, j, k); EyR(i, j, k) = DVyR(i, j, k); }
    wave_speed();
    HLL(SxL, SxR, ExL, ExR, nullptr, nullptr, &DxL, &DxR, Ex);
    HLL(SyL, SyR, EyL, EyR, nullptr, nullptr, &DyL, &DyR, Ey);
    for (int j = Jbeg; j <= Jend; ++j)
      for (int k = Kbeg; k <= Kend; ++k) {   // src/nhwave.F:1558-1580
        Ex(Ibeg, j, k) = p.bc_x0 == 3 ? Din_X0(j) * Uin_X0(j, k) : Zero;
        if (p.bc_xn == 3) Ex(Iend1, j, k) = Din_Xn(j) * Uin_Xn(j, k);   // src/nhwave.F:1580-1581
        else if (p.bc_xn != 6) Ex(Iend1, j, k) = Zero;
      }
    for (int i = Ibeg; i <= Iend; ++i)
      for (int k = Kbeg; k <= Kend; ++k) { Ey(i, Jbeg, k) = Zero; Ey(i, Jend1, k) = Zero; }
    Omega.fill(0.0);
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int k = Kbeg + 1; k <= Kend1; ++k) {
          Omega(i, j, k) = Omega(i, j, k - 1) - dsig(k - 1) * (R1s(i, j) + (Ex(i + 1, j, k - 1) - Ex(i, j, k - 1)) / dx +
                                                              (Ey(i, j + 1, k - 1) - Ey(i, j, k - 1)) / dy);
          if (Mask(i, j) == 0) Omega(i, j, k) = Zero;
        }
  }

  // ------------------------------------------------------------ eval_duvw
  int eval_duvw(int ISTEP) {
    const double al = ALPHA[ISTEP - 1], be = BETA[ISTEP - 1];
    int st = NHW_OK;
    if (p.viscous_flow) diffusion();
    R1s.fill(0.0);
    for (int j = Jbeg; j <= Jend; ++j)
      for (int i = Ibeg; i <= Iend; ++i) {
        if (Mask(i, j) == 0) continue;
        for (int k = Kbeg; k <= Kend; ++k)
          R1s(i, j) = R1s(i, j) - 1.0 / dx * (Ex(i + 1, j, k) - Ex(i, j, k)) * dsig(k) -
                      1.0 / dy * (Ey(i, j + 1, k) - Ey(i, j, k)) * dsig(k);
        R1s(i, j) = R1s(i, j) + D(i, j) * SourceC(i, j);
        D(i, j) = al * D0(i, j) + be * (D(i, j) + dt * R1s(i, j));
      }
    for (double& v : D.v) v = dmax(v, MinDep);
    wl_bc();
    for (int j = 1; j <= Nloc; ++j)
      for (int i = 1; i <= Mloc; ++i) Eta(i, j) = D(i, j) - Hc(i, j);
    delxFun_2D(Eta, DelxEta);
    delyFun_2D(Eta, DelyEta);
    sigma_transform();
    A3 R2, R3, R4;
    R2.init(Mloc, Nloc, Kloc); R3.init(Mloc, Nloc, Kloc); R4.init(Mloc, Nloc, Kloc);
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend; ++j) {
        if (Mask(i, j) == 0) continue;
        for (int k = Kbeg; k <= Kend; ++k) {
          R2(i, j, k) = -1.0 / dx * (Fx(i + 1, j, k) - Fx(i, j, k)) - 1.0 / dy * (Fy(i, j + 1, k) - Fy(i, j, k)) -
                        1.0 / dsig(k) * (Fz(i, j, k + 1) - Fz(i, j, k)) + fcor * DV(i, j, k) + SourceX(i, j);
          R3(i, j, k) = -1.0 / dx * (Gx(i + 1, j, k) - Gx(i, j, k)) - 1.0 / dy * (Gy(i, j + 1, k) - Gy(i, j, k)) -
                        1.0 / dsig(k) * (Gz(i, j, k + 1) - Gz(i, j, k)) - fcor * DU(i, j, k) + SourceY(i, j);
          R4(i, j, k) = -1.0 / dx * (Hx(i + 1, j, k) - Hx(i, j, k)) - 1.0 / dy * (Hy(i, j + 1, k) - Hy(i, j, k)) -
                        1.0 / dsig(k) * (Hz(i, j, k + 1) - Hz(i, j, k));
          if (p.viscous_flow) {   // + Diffxx + Diffxy etc. (src/nhwave.F:642-679)
            R2(i, j, k) = R2(i, j, k) + Diffxx(i, j, k) + Diffxy(i, j, k);
            R3(i, j, k) = R3(i, j, k) + Diffyx(i, j, k) + Diffyy(i, j, k);
            R4(i, j, k) = R4(i, j, k) + Diffzx(i, j, k) + Diffzy(i, j, k);
          }
        }
      }
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend; ++j) {
        if (Mask(i, j) == 0) continue;
        for (int k = Kbeg; k <= Kend; ++k) DU(i, j, k) = DU(i, j, k) + dt * R2(i, j, k);
      }
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend; ++j) {
        if (Mask(i, j) == 0) continue;
        for (int k = Kbeg; k <= Kend; ++k) DV(i, j, k) = DV(i, j, k) + dt * R3(i, j, k);
      }
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend; ++j) {
        if (Mask(i, j) == 0) continue;
        for (int k = Kbeg; k <= Kend; ++k) DW(i, j, k) = DW(i, j, k) + dt * R4(i, j, k);
      }
    if (p.viscous_flow)   // DU, DV, DW in turn, implicit in the vertical
      for (int which = 0; which < 3; ++which)
        for (int i = Ibeg; i <= Iend; ++i)
          for (int j = Jbeg; j <= Jend; ++j)
            if (Mask(i, j) != 0) vertical_viscous(i, j, which);
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i)
          if (Mask(i, j) == 0) { DU(i, j, k) = Zero; DV(i, j, k) = Zero; DW(i, j, k) = Zero; }
    if (p.non_hydro) {
      get_UVW();
      interpolate_velocity_to_faces();
      st = poisson_solver();
      projection_corrector();
    }
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i) {
          DU(i, j, k) = al * DU0(i, j, k) + be * DU(i, j, k);
          DV(i, j, k) = al * DV0(i, j, k) + be * DV(i, j, k);
          DW(i, j, k) = al * DW0(i, j, k) + be * DW(i, j, k);
          if (Mask(i, j) == 0) { DU(i, j, k) = Zero; DV(i, j, k) = Zero; DW(i, j, k) = Zero; }
        }
    if (p.froude_cap_on)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i) {
          double FroudeU = std::sqrt(Grav * D(i, j)) * p.froude_cap * D(i, j);
          if (Mask(i, j) > 0)
            for (int k = Kbeg; k <= Kend; ++k) {
              double DUU = std::sqrt(DU(i, j, k) * DU(i, j, k) + DV(i, j, k) * DV(i, j, k) + DW(i, j, k) * DW(i, j, k));
              if (DUU > FroudeU) {
                double Dangle = std::atan2(DV(i, j, k), DU(i, j, k));
                DU(i, j, k) = FroudeU * std::cos(Dangle);
                DV(i, j, k) = FroudeU * std::sin(Dangle);
                DW(i, j, k) = Zero;
              }
            }
        }
    get_UVW();
    get_Omega();
    return st;
  }

  // ------------------------------------------------------------ k-epsilon
  // HLPA upwinding of a face value (src/nhwave.F:7809-7847)
  static double hlpa(double Uw, double Fww, double Fw, double Fp, double Fe) {
    double h = 0.0;
    if (Uw >= Zero) {
      const double a = std::fabs(Fp - 2.0 * Fw + Fww) < std::fabs(Fp - Fww) ? 1.0 : 0.0;
      h = std::fabs(Fp - Fww) <= (double)1.e-16f ? Fw : Fw + a * (Fp - Fw) * (Fw - Fww) / (Fp - Fww);
    }
    if (Uw < Zero) {
      const double a = std::fabs(Fw - 2.0 * Fp + Fe) < std::fabs(Fw - Fe) ? 1.0 : 0.0;
      h = std::fabs(Fw - Fe) <= (double)1.e-16f ? Fp : Fp + a * (Fw - Fp) * (Fp - Fe) / (Fw - Fe);
    }
    return h;
  }
  // adv_scalar_hlpa (src/nhwave.F:7604-7806) with flux_scalar_bc (:7850-
  // 7986): R5 = -div(HLPA fluxes of Phi by Ex, Ey, Omega) + the horizontal
  // diffusion of Phi; IVAR 1 tke, 2 epsilon.  The boundary scalar of a
  // BC_X0 = 3 side is zero (no salinity or sediment).
  void adv_scalar_hlpa(A3& Phi, A3& R5, int IVAR) {
    A3 Scalx, Scaly, Scalz;
    Scalx.init(Mloc1, Nloc, Kloc); Scaly.init(Mloc, Nloc1, Kloc); Scalz.init(Mloc, Nloc, Kloc1);
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend + 1; ++i) {
          const double u = Ex(i, j, k);
          Scalx(i, j, k) = u * hlpa(u, Phi(i - 2, j, k), Phi(i - 1, j, k), Phi(i, j, k), Phi(i + 1, j, k));
        }
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend + 1; ++j)
        for (int i = Ibeg; i <= Iend; ++i) {
          const double v = Ey(i, j, k);
          Scaly(i, j, k) = v * hlpa(v, Phi(i, j - 2, k), Phi(i, j - 1, k), Phi(i, j, k), Phi(i, j + 1, k));
        }
    for (int k = Kbeg + 1; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i) {
          const double w = Omega(i, j, k);
          Scalz(i, j, k) = w * hlpa(w, Phi(i, j, k - 2), Phi(i, j, k - 1), Phi(i, j, k), Phi(i, j, k + 1));
        }
    // flux_scalar_bc
    for (int j = Jbeg; j <= Jend; ++j)
      for (int k = Kbeg; k <= Kend; ++k) {
        if (p.bc_x0 == 1 || p.bc_x0 == 2 || p.bc_x0 == 5) Scalx(Ibeg, j, k) = Zero;
        else if (p.bc_x0 == 3) Scalx(Ibeg, j, k) = Ex(Ibeg, j, k) * 0.0;
        Scalx(Iend1, j, k) = Zero;
      }
    for (int i = Ibeg; i <= Iend; ++i)
      for (int k = Kbeg; k <= Kend; ++k) {
        if (p.bc_y0 == 1 || p.bc_y0 == 2 || p.bc_y0 == 5) Scaly(i, Jbeg, k) = Zero;
        if (p.bc_yn == 1 || p.bc_yn == 2 || p.bc_yn == 5) Scaly(i, Jend1, k) = Zero;
      }
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i)
          if (Mask(i, j) == 0) {
            Scalx(i, j, k) = Zero; Scalx(i + 1, j, k) = Zero;
            Scaly(i, j, k) = Zero; Scaly(i, j + 1, k) = Zero;
          }
    for (int j = Jbeg; j <= Jend; ++j)
      for (int i = Ibeg; i <= Iend; ++i) { Scalz(i, j, Kbeg) = Zero; Scalz(i, j, Kend1) = Zero; }
    const double SchtH = IVAR == 1 ? (p.rng ? (double)0.72f : 1.0) : (p.rng ? (double)0.72f : (double)1.3f);
    R5.fill(0.0);
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i) {
          if (Mask(i, j) == 0) continue;
          auto nu = [&](double ha, double hb) { return 0.5 * (Cmu + Cmu) + 0.5 * (ha + hb) / SchtH; };
          const double Sdiffx =
              0.5 * (nu(CmuHt(i + 1, j, k), CmuHt(i, j, k)) * (D(i + 1, j) + D(i, j)) * (Phi(i + 1, j, k) - Phi(i, j, k)) -
                     nu(CmuHt(i, j, k), CmuHt(i - 1, j, k)) * (D(i, j) + D(i - 1, j)) * (Phi(i, j, k) - Phi(i - 1, j, k))) /
              (dx * dx);
          const double Sdiffy =
              0.5 * (nu(CmuHt(i, j + 1, k), CmuHt(i, j, k)) * (D(i, j + 1) + D(i, j)) * (Phi(i, j + 1, k) - Phi(i, j, k)) -
                     nu(CmuHt(i, j, k), CmuHt(i, j - 1, k)) * (D(i, j) + D(i, j - 1)) * (Phi(i, j, k) - Phi(i, j - 1, k))) /
              (dy * dy);
          R5(i, j, k) = -(1.0 / dx * (Scalx(i + 1, j, k) - Scalx(i, j, k))) - 1.0 / dy * (Scaly(i, j + 1, k) - Scaly(i, j, k)) -
                        1.0 / dsig(k) * (Scalz(i, j, k + 1) - Scalz(i, j, k)) + Sdiffx + Sdiffy;
        }
  }
  // Shear production of the nonlinear k-epsilon model (ke_model = 2, Lin
  // and Liu 1998; src/nhwave.F:10139-10274) at one cell: the Reynolds
  // stresses from the velocity gradient G (limited horizontal slopes plus
  // the sigma-slope terms) contracted with G per PRODTYPE (1: vertical
  // shear of U, V; 2: vertical shear; otherwise full 3-D).  (2./3.) and
  // (1./3.) are default-real quotients.
  static double ke_production(const double G[3][3], double tk, double ep, int prod_type) {
    const double c23 = (double)(2.0f / 3.0f), c13 = (double)(1.0f / 3.0f);
    double smax = Zero;
    for (int n = 0; n < 3; ++n)
      if (std::fabs(G[n][n]) > smax) smax = std::fabs(G[n][n]);
    smax = smax * tk / ep;
    const double c_d = c23 * (1.0 / ((double)7.4f + 2.0 * smax));
    double dmx = Zero;
    for (int n = 0; n < 3; ++n)
      for (int m = 0; m < 3; ++m)
        if (std::fabs(G[n][m]) > dmx) dmx = std::fabs(G[n][m]);
    dmx = dmx * tk / ep;
    const double c_1 = 1.0 / ((double)185.2f + 3.0 * (dmx * dmx));
    const double c_2 = -(1.0 / (58.5 + 2.0 * (dmx * dmx)));
    const double c_3 = 1.0 / ((double)370.4f + 3.0 * (dmx * dmx));
    const double tk2 = tk * tk, tk3 = tk * tk * tk, ep2 = ep * ep;
    double RS[3][3];
    for (int n = 0; n < 3; ++n)
      for (int m = 0; m < 3; ++m) {
        const double dl = n == m ? 1.0 : 0.0;
        double r = c_d * tk2 / ep * (G[n][m] + G[m][n]) - c23 * tk * dl;
        for (int l = 0; l < 3; ++l) {
          r = r + c_1 * tk3 / ep2 * (G[n][l] * G[l][m] + G[m][l] * G[l][n]);
          for (int g = 0; g < 3; ++g) r = r - c23 * c_1 * tk3 / ep2 * G[l][g] * G[g][l] * dl;
        }
        for (int g = 0; g < 3; ++g) {
          r = r + c_2 * tk3 / ep2 * G[n][g] * G[m][g];
          for (int l = 0; l < 3; ++l) r = r - c13 * c_2 * tk3 / ep2 * G[l][g] * G[l][g] * dl;
        }
        for (int g = 0; g < 3; ++g) {
          r = r + c_3 * tk3 / ep2 * G[g][n] * G[g][m];
          for (int l = 0; l < 3; ++l) r = r - c13 * c_3 * tk3 / ep2 * G[l][g] * G[l][g] * dl;
        }
        RS[n][m] = r;
      }
    double P = Zero;
    const int n1 = prod_type == 1 ? 2 : 3, m0 = (prod_type == 1 || prod_type == 2) ? 2 : 0;
    for (int n = 0; n < n1; ++n)
      for (int m = m0; m < 3; ++m) P = P + RS[n][m] * G[n][m];
    return P;
  }
  // kepsilon_3D (src/nhwave.F:10030-11114): the k-epsilon closure of
  // IVTURB = 10 with the nonlinear production, the RNG variant (RNG = T),
  // HLPA advection, implicit vertical diffusion, wall functions at the bed
  // and on friction walls (BC = 5), the gradient condition at the surface,
  // then CmuVt = cmiu k^2 / eps.  Barotropic: Rho = Rho0 everywhere
  // (src/initialize.F:2561), so the buoyancy production is zero.  The
  // reference leaves alpha_c, beta_c and gamma_c of its interior vertical
  // coefficients unset (locals never assigned); they are taken here as the
  // three-point weights the momentum equations use (src/nhwave.F:6826-6828).
  void kepsilon_3D(int istep) {
    const double Dmin = 2.0 * MinDep;
    const bool rng = p.rng != 0;
    const double c1e = rng ? (double)1.42f : (double)1.44f;
    double c2e = rng ? 0.0 : (double)1.92f;
    const double c3e = 0.0;
    const double cmiu = rng ? (double)0.085f : (double)0.09f;
    const double Sche = rng ? (double)0.72f : (double)1.3f, Schk = rng ? (double)0.72f : 1.0;
    A3 Tke_Old = Tke, Eps_Old = Eps;
    A3 Prod_s, R5;
    Prod_s.init(Mloc, Nloc, Kloc); R5.init(Mloc, Nloc, Kloc);
    auto ds = [&](int k) { return sigc(k + 1) - sigc(k - 1); };
    auto vel_grad = [&](int i, int j, int k, double G[3][3]) {
      const double dU = U(i, j, k + 1) - U(i, j, k - 1), dV = V(i, j, k + 1) - V(i, j, k - 1);
      const double dW = W(i, j, k + 1) - W(i, j, k - 1);
      G[0][0] = DelxU(i, j, k) + dU / ds(k) * DelxSc(i, j, k);
      G[0][1] = DelyU(i, j, k) + dU / ds(k) * DelySc(i, j, k);
      G[0][2] = 1.0 / D(i, j) * dU / ds(k);
      G[1][0] = DelxV(i, j, k) + dV / ds(k) * DelxSc(i, j, k);
      G[1][1] = DelyV(i, j, k) + dV / ds(k) * DelySc(i, j, k);
      G[1][2] = 1.0 / D(i, j) * dV / ds(k);
      G[2][0] = DelxW(i, j, k) + dW / ds(k) * DelxSc(i, j, k);
      G[2][1] = DelyW(i, j, k) + dW / ds(k) * DelySc(i, j, k);
      G[2][2] = 1.0 / D(i, j) * dW / ds(k);
    };
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int k = Kbeg; k <= Kend; ++k) {
          if (!(D(i, j) >= Dmin && Mask(i, j) == 1)) continue;
          double G[3][3];
          vel_grad(i, j, k, G);
          double P = ke_production(G, Tke_Old(i, j, k), Eps_Old(i, j, k), p.prod_type);
          if (k == Kend && P < 0.0) P = Zero;   // no negative production at the surface
          Prod_s(i, j, k) = P;
        }
    const double Prod_b = 0.0;
    // surface values of tke and epsilon (construct_3D_z, floored) and their
    // limited horizontal slopes, for the gradient condition at the surface
    A3 DelzTke, DelzEps, TkezL, TkezR, EpszL, EpszR, DelxTkezL, DelxEpszL, DelyTkezL, DelyEpszL;
    DelzTke.init(Mloc, Nloc, Kloc); DelzEps.init(Mloc, Nloc, Kloc);
    for (A3* a : {&TkezL, &TkezR, &EpszL, &EpszR, &DelxTkezL, &DelxEpszL, &DelyTkezL, &DelyEpszL})
      a->init(Mloc, Nloc, Kloc1);
    delzFun_3D(Tke_Old, DelzTke);
    delzFun_3D(Eps_Old, DelzEps);
    construct_3D_z(Tke_Old, DelzTke, TkezL, TkezR);
    construct_3D_z(Eps_Old, DelzEps, EpszL, EpszR);
    for (double& v : TkezL.v) v = dmax(v, Tke_min);
    for (double& v : TkezR.v) v = dmax(v, Tke_min);
    for (double& v : EpszL.v) v = dmax(v, Eps_min);
    for (double& v : EpszR.v) v = dmax(v, Eps_min);
    delxFun_3D(TkezL, DelxTkezL);
    delxFun_3D(EpszL, DelxEpszL);
    delyFun_3D(TkezL, DelyTkezL);
    delyFun_3D(EpszL, DelyEpszL);
    const int n = Kend - Kbeg + 1;
    std::vector<double> Ac(n), Bc(n), Cc(n), Rhs0(n), Xsol(n);
    // one column of the epsilon (eq = 2) or tke (eq = 1) equation
    auto column = [&](int i, int j, int eq) {
      A3& Old = eq == 2 ? Eps_Old : Tke_Old;
      A3& zL = eq == 2 ? EpszL : TkezL;
      A3& Dv = eq == 2 ? DEps : DTke;
      const double Sch = eq == 2 ? Sche : Schk;
      const double Dc = D(i, j);
      const double DxD = (DelxH(i, j) + DelxEta(i, j)) / Dc, DyD = (DelyH(i, j) + DelyEta(i, j)) / Dc;
      int q = 0;
      for (int k = Kbeg; k <= Kend; ++k) {
        const double L1top = dsig(k + 1) / (dsig(k) + dsig(k + 1)), L2top = dsig(k) / (dsig(k) + dsig(k + 1));
        const double L1bot = dsig(k) / (dsig(k) + dsig(k - 1)), L2bot = dsig(k - 1) / (dsig(k) + dsig(k - 1));
        const double dsigck = (dsig(k) + dsig(k + 1)) / 2.0, dsigck1 = (dsig(k - 1) + dsig(k)) / 2.0;
        const double alpha_c = -dsigck / (dsigck + dsigck1) / dsigck1;
        const double beta_c = (dsigck - dsigck1) / (dsigck * dsigck1);
        const double gamma_c = dsigck1 / (dsigck + dsigck1) / dsigck;
        const double nuV_top = (L1top * Cmu + L2top * Cmu) + (L1top * CmuR + L2top * CmuR) +
                               (L1top * CmuVt(i, j, k) + L2top * CmuVt(i, j, k + 1)) / Sch;
        const double nuH_top = (L1top * Cmu + L2top * Cmu) + (L1top * CmuR + L2top * CmuR) +
                               (L1top * CmuHt(i, j, k) + L2top * CmuHt(i, j, k + 1)) / Sch;
        const double nuV_bot = (L1bot * Cmu + L2bot * Cmu) + (L1bot * CmuR + L2bot * CmuR) +
                               (L1bot * CmuVt(i, j, k - 1) + L2bot * CmuVt(i, j, k)) / Sch;
        const double nuH_bot = (L1bot * Cmu + L2bot * Cmu) + (L1bot * CmuR + L2bot * CmuR) +
                               (L1bot * CmuHt(i, j, k - 1) + L2bot * CmuHt(i, j, k)) / Sch;
        double r = R5(i, j, k);
        if (eq == 2) r = r + c1e * Dc * (Prod_s(i, j, k) + c3e * Prod_b) * Eps_Old(i, j, k) / Tke_Old(i, j, k);
        else r = r + Dc * (Prod_s(i, j, k) + Prod_b) - DEps(i, j, k);
        if (k == Kbeg) {
          r = r - (-(nuH_bot * (DelxH(i, j) * DxD + DelyH(i, j) * DyD) * Old(i, j, k))) / dsig(k) +
              (dsig(k) - dsigck) / (dsig(k) * dsig(k) / 2.0 * (dsigck + dsig(k) / 2.0)) *
                  (nuH_top * (DelxSl(i, j, k + 1) * DelxH(i, j) + DelySl(i, j, k + 1) * DelyH(i, j)) + nuV_top / Dc) *
                  Old(i, j, k);
        } else if (k == Kend) {
          r = r + ((nuH_top * (DelxEta(i, j) * DelxEta(i, j) + DelyEta(i, j) * DelyEta(i, j)) + nuV_top) / (Dc * Dc) *
                       (Old(i, j, k + 1) - Old(i, j, k)) * Dc / dsigck -
                   nuH_top * (-(DelxEta(i, j) * DxD) - DelyEta(i, j) * DyD) * zL(i, j, k + 1)) /
                      dsig(k) +
              (dsig(k) - dsigck1) / (dsig(k) * dsig(k) / 2.0 * (dsigck1 + dsig(k) / 2.0)) *
                  (nuH_bot * (-(DelxSl(i, j, k) * DelxEta(i, j)) - DelySl(i, j, k) * DelyEta(i, j)) + nuV_bot / Dc) *
                  zL(i, j, k + 1);
        }
        // sigma-coupled vertical diffusion a . (nu_top Sl_top S_kk - nu_bot Sl_bot S_kk) + nu/D^2 at level kk
        auto top = [&](int kk) {
          return nuH_top * (DelxSl(i, j, k + 1) * DelxSc(i, j, kk) + DelySl(i, j, k + 1) * DelySc(i, j, kk)) +
                 nuV_top / (Dc * Dc);
        };
        auto bot = [&](int kk) {
          return nuH_bot * (DelxSl(i, j, k) * DelxSc(i, j, kk) + DelySl(i, j, k) * DelySc(i, j, kk)) +
                 nuV_bot / (Dc * Dc);
        };
        if (k == Kbeg) Ac[q] = 0.0;
        else if (k == Kend) Ac[q] = -dt * (3.0 / 2.0 * bot(k - 1) / (dsigck1 * (dsigck1 + dsig(k) / 2.0)));
        else
          Ac[q] = -dt * ((top(k - 1) - bot(k - 1)) * alpha_c / dsig(k) +
                         (top(k - 1) + bot(k - 1)) / (dsigck1 * (dsigck1 + dsigck)));
        if (k == Kbeg) Cc[q] = -dt * (3.0 / 2.0 * top(k + 1) / (dsigck * (dsigck + dsig(k) / 2.0)));
        else if (k == Kend) Cc[q] = 0.0;
        else
          Cc[q] = -dt * ((top(k + 1) - bot(k + 1)) * gamma_c / dsig(k) +
                         (top(k + 1) + bot(k + 1)) / (dsigck * (dsigck1 + dsigck)));
        double b0 = 1.0;
        if (eq == 2) {
          if (rng) {   // c2e of Yakhot et al. (1992) from the strain rate
            const double dUs = (U(i, j, k + 1) - U(i, j, k - 1)) / ds(k), dVs = (V(i, j, k + 1) - V(i, j, k - 1)) / ds(k);
            const double dWs = (W(i, j, k + 1) - W(i, j, k - 1)) / ds(k);
            const double S11 = DelxU(i, j, k) + dUs * DelxSc(i, j, k);
            const double S22 = DelyV(i, j, k) + dVs * DelySc(i, j, k);
            const double S33 = 1.0 / Dc * (W(i, j, k + 1) - W(i, j, k - 1)) / ds(k);
            const double S12 = 0.5 * (DelyU(i, j, k) + dUs * DelySc(i, j, k) + DelxV(i, j, k) + dVs * DelxSc(i, j, k));
            const double S13 = 0.5 * ((U(i, j, k + 1) - U(i, j, k - 1)) / ds(k) / Dc + DelxW(i, j, k) + dWs * DelxSc(i, j, k));
            const double S23 = 0.5 * ((V(i, j, k + 1) - V(i, j, k - 1)) / ds(k) / Dc + DelyW(i, j, k) + dWs * DelySc(i, j, k));
            const double lambda = Tke_Old(i, j, k) / Eps_Old(i, j, k) *
                                  std::sqrt(2.0 * (S11 * S11 + S22 * S22 + S33 * S33 +
                                                   2.0 * (S12 * S12 + S13 * S13 + S23 * S23)));
            const double l3 = lambda * lambda * lambda;
            c2e = (double)1.68f + cmiu * l3 * (1.0 - lambda / (double)4.38f) / (1.0 + (double)0.012f * l3);
            c2e = dmax(0.0, dmin(c2e, 4.0));
          }
          b0 = 1.0 + dt * c2e * Eps_Old(i, j, k) / Tke_Old(i, j, k);
        }
        if (k == Kbeg) Bc[q] = b0 - dt * (-(3.0 / 2.0 - dsigck / dsig(k)) * top(k) / (dsig(k) / 2.0 * dsigck));
        else if (k == Kend) Bc[q] = b0 - dt * (-(3.0 / 2.0 - dsigck1 / dsig(k)) * bot(k) / (dsig(k) / 2.0 * dsigck1));
        else
          Bc[q] = b0 - dt * ((top(k) - bot(k)) * beta_c / dsig(k) - (top(k) + bot(k)) / (dsigck * dsigck1));
        Rhs0[q] = Dv(i, j, k) + dt * r;
        ++q;
      }
      trig(Ac, Bc, Cc, Rhs0, Xsol, n);
      q = 0;
      for (int k = Kbeg; k <= Kend; ++k) Dv(i, j, k) = Xsol[q++];
    };
    auto rk = [&](A3& Dv, A3& Dv0, double vmin) {
      for (int i = Ibeg; i <= Iend; ++i)
        for (int j = Jbeg; j <= Jend; ++j)
          for (int k = Kbeg; k <= Kend; ++k)
            if (D(i, j) >= Dmin && Mask(i, j) == 1) {
              Dv(i, j, k) = ALPHA[istep - 1] * Dv0(i, j, k) + BETA[istep - 1] * Dv(i, j, k);
              Dv(i, j, k) = dmax(Dv(i, j, k), D(i, j) * vmin);
            }
    };
    // epsilon, then tke (whose source reads the new DEps); a column is
    // skipped only where it is both shallower than Dmin and dry
    adv_scalar_hlpa(Eps_Old, R5, 2);
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend; ++j)
        if (!(D(i, j) < Dmin && Mask(i, j) == 0)) column(i, j, 2);
    rk(DEps, DEps0, Eps_min);
    adv_scalar_hlpa(Tke_Old, R5, 1);
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend; ++j)
        if (!(D(i, j) < Dmin && Mask(i, j) == 0)) column(i, j, 1);
    rk(DTke, DTke0, Tke_min);
    // bed: wall function (src/nhwave.F:10776-10831)
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend; ++j) {
        const double dxh = DelxH(i, j), dyh = DelyH(i, j);
        const double Abot = std::sqrt(1.0 + dxh * dxh + dyh * dyh), Bbot = std::sqrt(1.0 + dxh * dxh);
        const double DUprime = (DU(i, j, Kbeg) - dxh * DW(i, j, Kbeg)) / Bbot;
        const double DVprime =
            (-(dxh * dyh * DU(i, j, Kbeg)) + (1.0 + dxh * dxh) * DV(i, j, Kbeg) - dyh * DW(i, j, Kbeg)) / Abot / Bbot;
        const double DUmag = std::sqrt(DUprime * DUprime + DVprime * DVprime);
        if (D(i, j) < Dmin || Mask(i, j) == 0) continue;
        double Tkeb, Epsb;
        if (DUmag / D(i, j) < (double)1.e-6f) {
          Tkeb = Tke_min; Epsb = Eps_min;
        } else {
          const double Dz1 = 0.5 * D(i, j) * dsig(Kbeg) / Abot;
          const double Z0 = p.zob / 30.0;
          double Cdrag;
          if (p.ibot == 1) Cdrag = p.cd0;
          else { const double t = Kappa / std::log(Dz1 / Z0); Cdrag = t * t; }
          Cdrag = dmin(Cdrag, (Cmu + CmuR + CmuVt(i, j, Kbeg)) / Dz1 / (DUmag + Small) * D(i, j));
          const double Ustar = std::sqrt(Cdrag) * DUmag / D(i, j);
          Tkeb = dmax(Ustar * Ustar / std::sqrt(cmiu), Tke_min);
          Epsb = dmax(Ustar * Ustar * Ustar / (Kappa * Dz1), Eps_min);
        }
        DTke(i, j, Kbeg) = D(i, j) * Tkeb;
        DEps(i, j, Kbeg) = D(i, j) * Epsb;
        for (int k = 1; k <= Nghost; ++k) {
          DTke(i, j, Kbeg - k) = DTke(i, j, Kbeg);
          DEps(i, j, Kbeg - k) = DEps(i, j, Kbeg);
        }
      }
    // surface: gradient condition (Derakhti et al. 2015, eq. 60)
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend; ++j) {
        if (Mask(i, j) == 0 || D(i, j) < Dmin) continue;
        for (int k = 1; k <= Nghost; ++k) {
          const double dxe = DelxEta(i, j), dye = DelyEta(i, j);
          const double Atop = std::sqrt(1.0 + dxe * dxe + dye * dye);
          const double f = (sigc(Kend + k) - sigc(Kend - k + 1)) * (D(i, j) * D(i, j)) / (Atop * Atop);
          DTke(i, j, Kend + k) = DTke(i, j, Kend - k + 1) + f * (dxe * DelxTkezL(i, j, Kend1) + dye * DelyTkezL(i, j, Kend1));
          DEps(i, j, Kend + k) = DEps(i, j, Kend - k + 1) + f * (dxe * DelxEpszL(i, j, Kend1) + dye * DelyEpszL(i, j, Kend1));
        }
      }
    // side walls: wall function on friction walls (BC = 5), then mirrors
    auto wall = [&](int ii, int jj, int kk, double Umag, double h) {
      double Tkeb, Epsb;
      if (Umag < (double)1.e-6f) {
        Tkeb = Tke_min; Epsb = Eps_min;
      } else {
        const double FricU = p.ibot == 1 ? std::sqrt(p.cd0) * Umag : Umag / (1.0 / Kappa * std::log(30.0 * h / 2.0 / p.zob));
        Tkeb = FricU * FricU / std::sqrt(cmiu);
        Epsb = FricU * FricU * FricU / (Kappa * h / 2.0);
      }
      DTke(ii, jj, kk) = D(ii, jj) * Tkeb;
      DEps(ii, jj, kk) = D(ii, jj) * Epsb;
    };
    for (int j = Jbeg; j <= Jend; ++j)
      for (int k = 1; k <= Kloc; ++k) {
        if (p.bc_x0 == 5) wall(Ibeg, j, k, std::sqrt(V(Ibeg, j, k) * V(Ibeg, j, k) + W(Ibeg, j, k) * W(Ibeg, j, k)), dx);
        for (int i = 1; i <= Nghost; ++i) {
          DTke(Ibeg - i, j, k) = DTke(Ibeg + i - 1, j, k);
          DEps(Ibeg - i, j, k) = DEps(Ibeg + i - 1, j, k);
        }
      }
    for (int j = Jbeg; j <= Jend; ++j)
      for (int k = 1; k <= Kloc; ++k) {
        if (p.bc_xn == 5) wall(Iend, j, k, std::sqrt(V(Iend, j, k) * V(Iend, j, k) + W(Iend, j, k) * W(Iend, j, k)), dx);
        for (int i = 1; i <= Nghost; ++i) {
          DTke(Iend + i, j, k) = DTke(Iend - i + 1, j, k);
          DEps(Iend + i, j, k) = DEps(Iend - i + 1, j, k);
        }
      }
    for (int i = 1; i <= Mloc; ++i)
      for (int k = 1; k <= Kloc; ++k) {
        if (p.bc_y0 == 5) wall(i, Jbeg, k, std::sqrt(U(i, Jbeg, k) * U(i, Jbeg, k) + W(i, Jbeg, k) * W(i, Jbeg, k)), dy);
        for (int j = 1; j <= Nghost; ++j) {
          DTke(i, Jbeg - j, k) = DTke(i, Jbeg + j - 1, k);
          DEps(i, Jbeg - j, k) = DEps(i, Jbeg + j - 1, k);
        }
      }
    for (int i = 1; i <= Mloc; ++i)
      for (int k = 1; k <= Kloc; ++k) {
        if (p.bc_yn == 5) wall(i, Jend, k, std::sqrt(U(i, Jend, k) * U(i, Jend, k) + W(i, Jend, k) * W(i, Jend, k)), dy);
        for (int j = 1; j <= Nghost; ++j) {
          DTke(i, Jend + j, k) = DTke(i, Jend - j + 1, k);
          DEps(i, Jend + j, k) = DEps(i, Jend - j + 1, k);
        }
      }
    // tke, epsilon and the eddy viscosity in every cell
    for (int i = 1; i <= Mloc; ++i)
      for (int j = 1; j <= Nloc; ++j)
        for (int k = 1; k <= Kloc; ++k) {
          if (D(i, j) >= Dmin && Mask(i, j) == 1) {
            Tke(i, j, k) = DTke(i, j, k) / D(i, j);
            Eps(i, j, k) = DEps(i, j, k) / D(i, j);
            if (Tke(i, j, k) < (double)1.e-6f || Eps(i, j, k) < (double)1.e-6f) CmuVt(i, j, k) = Cmut_min;
            else CmuVt(i, j, k) = cmiu * (Tke(i, j, k) * Tke(i, j, k)) / Eps(i, j, k);
          } else {
            Tke(i, j, k) = Tke_min;
            Eps(i, j, k) = Eps_min;
            DTke(i, j, k) = D(i, j) * Tke_min;
            DEps(i, j, k) = D(i, j) * Eps_min;
            CmuVt(i, j, k) = Cmut_min;
          }
        }
    for (int i = 1; i <= Mloc; ++i)
      for (int j = 1; j <= Nloc; ++j)
        for (int k = 1; k <= Nghost; ++k) {
          CmuVt(i, j, Kbeg - k) = CmuVt(i, j, Kbeg);
          CmuVt(i, j, Kend + k) = CmuVt(i, j, Kend);
        }
    // no turbulence in the wavemaker's source region (INT_, LEF_ and FOCUSED)
    if (ke_quiet_maker()) {
      for (int k = 1; k <= Kloc; ++k)
        for (int j = 1; j <= Nloc; ++j)
          for (int i = 1; i <= Mloc; ++i)
            if (xc(i) >= p.xsource_west && xc(i) <= p.xsource_east && yc(j) >= p.ysource_suth &&
                yc(j) <= p.ysource_nrth) {
              Tke(i, j, k) = Tke_min;
              Eps(i, j, k) = Eps_min;
              DTke(i, j, k) = D(i, j) * Tke_min;
              DEps(i, j, k) = D(i, j) * Eps_min;
              CmuVt(i, j, k) = Cmut_min;
            }
    }
  }
  // WaveMaker(1:3) is INT, LEF or FOC
  bool ke_quiet_maker() const {
    const int w = p.wavemaker;
    return w == NHW_WM_INT_LIN || w == NHW_WM_INT_SOL || w == NHW_WM_INT_CON || w == NHW_WM_INT_JON ||
           w == NHW_WM_INT_TMA || w == NHW_WM_INT_SPC || w == NHW_WM_INT_IRR || w == NHW_WM_LEF_LIN ||
           w == NHW_WM_LEF_SOL || w == NHW_WM_LEF_STK || w == NHW_WM_LEF_CON || w == NHW_WM_LEF_TID ||
           w == NHW_WM_LEF_JON || w == NHW_WM_LEF_TMA || w == NHW_WM_LEF_SPC || w == NHW_WM_FOCUSED;
  }

  // les_3D (src/nhwave.F:8545-8729): the Smagorinsky closure of IVTURB = 20.
  // CmuVt = (Cvs Delta)^2 sqrt(2 SijSij) with the filter width Delta =
  // (dx dy dsig D)^(1/3) in wet cells of depth above 0.02 m (others keep
  // their value); at the bed a wall function: log law of a rough wall
  // (Zob >= 0.1) or the smooth wall's friction velocity from a fixed-point
  // iteration, damped by van Driest's (1 - exp(-z+/19))^2; mirrors into the
  // ghosts; no eddy viscosity at the first column of a LEF_ maker or in an
  // INT_ maker's source region.  The reference iterates the smooth-wall law
  // until it converges; the iteration stops after kLesIter steps here.  Eps,
  // an output of the LES closure, is not formed.
  static constexpr int kLesIter = 200;
  void les_3D() {
    const double Dmin = (double)0.02f, Cvs = p.cvs;
    auto ds = [&](int k) { return sigc(k + 1) - sigc(k - 1); };
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int k = Kbeg; k <= Kend; ++k) {
          if (!(Mask9(i, j) == 1 && D(i, j) > Dmin)) continue;
          const double dUs = (U(i, j, k + 1) - U(i, j, k - 1)) / ds(k), dVs = (V(i, j, k + 1) - V(i, j, k - 1)) / ds(k);
          const double dWs = (W(i, j, k + 1) - W(i, j, k - 1)) / ds(k);
          const double S11 = (U(i + 1, j, k) - U(i - 1, j, k)) / (2.0 * dx) + dUs * DelxSc(i, j, k);
          const double S22 = (V(i, j + 1, k) - V(i, j - 1, k)) / (2.0 * dy) + dVs * DelySc(i, j, k);
          const double S33 = 1.0 / D(i, j) * (W(i, j, k + 1) - W(i, j, k - 1)) / ds(k);
          const double S12 = 0.5 * ((U(i, j + 1, k) - U(i, j - 1, k)) / (2.0 * dy) + dUs * DelySc(i, j, k) +
                                    (V(i + 1, j, k) - V(i - 1, j, k)) / (2.0 * dx) + dVs * DelxSc(i, j, k));
          const double S13 = 0.5 * (dUs / D(i, j) + (W(i + 1, j, k) - W(i - 1, j, k)) / (2.0 * dx) + dWs * DelxSc(i, j, k));
          const double S23 = 0.5 * (dVs / D(i, j) + (W(i, j + 1, k) - W(i, j - 1, k)) / (2.0 * dy) + dWs * DelySc(i, j, k));
          const double SijSij = S11 * S11 + S22 * S22 + S33 * S33 + 2.0 * (S12 * S12 + S13 * S13 + S23 * S23);
          const double Filter = std::pow(dx * dy * dsig(k) * D(i, j), (double)(1.0f / 3.0f));
          const double cf = Cvs * Filter;
          CmuVt(i, j, k) = cf * cf * std::sqrt(2.0 * SijSij);
        }
    const double kap = (double)0.41f;
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend; ++j) {
        const double Umag = std::sqrt(U(i, j, Kbeg) * U(i, j, Kbeg) + V(i, j, Kbeg) * V(i, j, Kbeg));
        if (Umag < (double)1.e-6f) {
          CmuVt(i, j, Kbeg) = Cmu;
        } else {
          const double Zdis = 0.5 * dsig(Kbeg) * D(i, j);
          double FricU;
          if (p.zob >= (double)0.1f) {
            FricU = Umag / ((double)(1.0f / 0.41f) * std::log(30.0 * Zdis / p.zob));   // 1.0/0.41 folded in default real
          } else {
            double X0 = (double)0.05f, Xn = X0;
            const double Xa = std::log(9.0 * Umag * Zdis / Cmu);
            for (int it = 0; it < kLesIter; ++it) {
              Xn = X0 + (kap - X0 * (Xa + std::log(X0))) / (1.0 + kap / X0);
              if (!(std::fabs((Xn - X0) / X0) > (double)1.e-8f && Xn > 0.0)) break;
              X0 = Xn;
            }
            FricU = Xn * Umag;
          }
          const double e = 1.0 - std::exp(-Zdis * FricU / Cmu / 19.0);
          CmuVt(i, j, Kbeg) = kap * Zdis * FricU * (e * e);
        }
        for (int k = 1; k <= Nghost; ++k) CmuVt(i, j, Kbeg - k) = CmuVt(i, j, Kbeg + k - 1);
      }
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int k = 1; k <= Nghost; ++k) CmuVt(i, j, Kend + k) = CmuVt(i, j, Kend - k + 1);
    const bool lef = (p.wavemaker >= NHW_WM_LEF_LIN && p.wavemaker <= NHW_WM_LEF_CON) || p.wavemaker == NHW_WM_LEF_TID ||
                     p.wavemaker == NHW_WM_LEF_JON || p.wavemaker == NHW_WM_LEF_TMA || p.wavemaker == NHW_WM_LEF_SPC;
    for (int j = Jbeg; j <= Jend; ++j)
      for (int k = Kbeg; k <= Kend; ++k) {
        if (lef) CmuVt(Ibeg, j, k) = Zero;   // no turbulence at the wave generation region
        for (int i = 1; i <= Nghost; ++i) CmuVt(Ibeg - i, j, k) = CmuVt(Ibeg + i - 1, j, k);
      }
    for (int j = Jbeg; j <= Jend; ++j)
      for (int k = Kbeg; k <= Kend; ++k)
        for (int i = 1; i <= Nghost; ++i) CmuVt(Iend + i, j, k) = CmuVt(Iend - i + 1, j, k);
    for (int i = Ibeg; i <= Iend; ++i)
      for (int k = Kbeg; k <= Kend; ++k)
        for (int j = 1; j <= Nghost; ++j) CmuVt(i, Jbeg - j, k) = CmuVt(i, Jbeg + j - 1, k);
    for (int i = Ibeg; i <= Iend; ++i)
      for (int k = Kbeg; k <= Kend; ++k)
        for (int j = 1; j <= Nghost; ++j) CmuVt(i, Jend + j, k) = CmuVt(i, Jend - j + 1, k);
    const int w = p.wavemaker;
    const bool int_maker = w == NHW_WM_INT_LIN || w == NHW_WM_INT_SOL || w == NHW_WM_INT_CON || w == NHW_WM_INT_JON ||
                           w == NHW_WM_INT_TMA || w == NHW_WM_INT_SPC || w == NHW_WM_INT_IRR;
    if (int_maker)   // no turbulence in the internal wavemaker region
      for (int k = 1; k <= Kloc; ++k)
        for (int j = 1; j <= Nloc; ++j)
          for (int i = 1; i <= Mloc; ++i)
            if (xc(i) >= p.xsource_west && xc(i) <= p.xsource_east && yc(j) >= p.ysource_suth &&
                yc(j) <= p.ysource_nrth)
              CmuVt(i, j, k) = Zero;
  }

  // kepsilon (src/nhwave.F:11117-11524): the 2-D k-epsilon closure of
  // IVTURB = 3.  Production from the vertical shear only, CmuVt (U_z^2 +
  // V_z^2); HLPA advection and horizontal diffusion as kepsilon_3D's; plain
  // implicit vertical diffusion; at the bed the smooth-wall law's friction
  // velocity (the fixed-point iteration of les_3D, bounded at kLesIter
  // steps; the reference's is not), mirrors elsewhere; the first six columns
  // of a LEF_ maker and an INT_ maker's source region kept at the floors.
  // The reference also stores U_z / D and V_z / D in DelzU / DelzV, which
  // the next fluxes recompute before any read.
  void kepsilon_2D(int istep) {
    const double Dmin = (double)0.01f;
    const double c1e = (double)1.44f, c2e = (double)1.92f, c3e = 0.0, cmiu = (double)0.09f;
    const double Sche = (double)1.3f, Schk = 1.0, Prod_b = 0.0;
    A3 Tke_Old = Tke, Eps_Old = Eps, Prod_s, R5;
    Prod_s.init(Mloc, Nloc, Kloc); R5.init(Mloc, Nloc, Kloc);
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int k = Kbeg; k <= Kend; ++k)
          if (D(i, j) >= Dmin && Mask(i, j) == 1) {
            const double ds = sigc(k + 1) - sigc(k - 1);
            const double uz = (U(i, j, k + 1) - U(i, j, k - 1)) / ds / D(i, j);
            const double vz = (V(i, j, k + 1) - V(i, j, k - 1)) / ds / D(i, j);
            Prod_s(i, j, k) = CmuVt(i, j, k) * (uz * uz + vz * vz);
          }
    const int n = Kend - Kbeg + 1;
    std::vector<double> Ac(n), Bc(n), Cc(n), Rhs0(n), Xsol(n);
    auto column = [&](int i, int j, int eq) {
      A3& Dv = eq == 2 ? DEps : DTke;
      const double Sch = eq == 2 ? Sche : Schk, Dc = D(i, j);
      int q = 0;
      for (int k = Kbeg; k <= Kend; ++k, ++q) {
        double r = R5(i, j, k);
        if (eq == 2) r = r + c1e * Dc * (Prod_s(i, j, k) + c3e * Prod_b) * Eps_Old(i, j, k) / Tke_Old(i, j, k);
        else r = r + Dc * (Prod_s(i, j, k) + Prod_b) - DEps(i, j, k);
        Ac[q] = k == Kbeg ? 0.0
                          : -dt / (Dc * Dc) * (0.5 * (Cmu + Cmu) + 0.5 * (CmuVt(i, j, k - 1) + CmuVt(i, j, k)) / Sch) /
                                (0.5 * dsig(k) * (dsig(k) + dsig(k - 1)));
        Cc[q] = k == Kend ? 0.0
                          : -dt / (Dc * Dc) * (0.5 * (Cmu + Cmu) + 0.5 * (CmuVt(i, j, k) + CmuVt(i, j, k + 1)) / Sch) /
                                (0.5 * dsig(k) * (dsig(k) + dsig(k + 1)));
        Bc[q] = 1.0 - Ac[q] - Cc[q];
        if (eq == 2) Bc[q] = Bc[q] + dt * c2e * Eps_Old(i, j, k) / Tke_Old(i, j, k);
        Rhs0[q] = Dv(i, j, k) + dt * r;
      }
      trig(Ac, Bc, Cc, Rhs0, Xsol, n);
      q = 0;
      for (int k = Kbeg; k <= Kend; ++k) Dv(i, j, k) = Xsol[q++];
    };
    auto rk = [&](A3& Dv, A3& Dv0, double vmin) {
      for (int i = Ibeg; i <= Iend; ++i)
        for (int j = Jbeg; j <= Jend; ++j)
          for (int k = Kbeg; k <= Kend; ++k)
            if (D(i, j) >= Dmin && Mask(i, j) == 1) {
              Dv(i, j, k) = ALPHA[istep - 1] * Dv0(i, j, k) + BETA[istep - 1] * Dv(i, j, k);
              Dv(i, j, k) = dmax(Dv(i, j, k), D(i, j) * vmin);
            }
    };
    adv_scalar_hlpa(Eps_Old, R5, 2);
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend; ++j)
        if (!(D(i, j) < Dmin && Mask(i, j) == 0)) column(i, j, 2);
    rk(DEps, DEps0, Eps_min);
    adv_scalar_hlpa(Tke_Old, R5, 1);
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend; ++j)
        if (!(D(i, j) < Dmin && Mask(i, j) == 0)) column(i, j, 1);
    rk(DTke, DTke0, Tke_min);
    const double kap = (double)0.41f;
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend; ++j) {
        const double Umag = std::sqrt(U(i, j, Kbeg) * U(i, j, Kbeg) + V(i, j, Kbeg) * V(i, j, Kbeg));
        if (Umag < (double)1.e-6f || D(i, j) < Dmin || Mask(i, j) == 0) continue;
        const double Zdis = 0.5 * dsig(Kbeg) * D(i, j);
        double X0 = (double)0.05f, Xn = X0;
        const double Xa = std::log(9.0 * Umag * Zdis / Cmu);
        for (int it = 0; it < kLesIter; ++it) {
          Xn = X0 + (kap - X0 * (Xa + std::log(X0))) / (1.0 + kap / X0);
          if (!(std::fabs((Xn - X0) / X0) > (double)1.e-8f && Xn > 0.0)) break;
          X0 = Xn;
        }
        const double FricU = Xn * Umag;
        DTke(i, j, Kbeg) = D(i, j) * (FricU * FricU / std::sqrt(cmiu));
        DEps(i, j, Kbeg) = D(i, j) * (FricU * FricU * FricU / (Kappa * Zdis));
        for (int k = 1; k <= Nghost; ++k) {
          DTke(i, j, Kbeg - k) = DTke(i, j, Kbeg + k - 1);
          DEps(i, j, Kbeg - k) = DEps(i, j, Kbeg + k - 1);
        }
      }
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int k = 1; k <= Nghost; ++k) {
          DTke(i, j, Kend + k) = DTke(i, j, Kend - k + 1);
          DEps(i, j, Kend + k) = DEps(i, j, Kend - k + 1);
        }
    const bool lef = (p.wavemaker >= NHW_WM_LEF_LIN && p.wavemaker <= NHW_WM_LEF_CON) || p.wavemaker == NHW_WM_LEF_TID ||
                     p.wavemaker == NHW_WM_LEF_JON || p.wavemaker == NHW_WM_LEF_TMA || p.wavemaker == NHW_WM_LEF_SPC;
    for (int j = Jbeg; j <= Jend; ++j)
      for (int k = Kbeg; k <= Kend; ++k) {
        if (lef)   // the first six columns (within the array)
          for (int i = Ibeg; i <= Ibeg + 5 && i <= Mloc; ++i) {
            Tke(i, j, k) = Tke_min;
            Eps(i, j, k) = Eps_min;
            DTke(i, j, k) = D(i, j) * Tke_min;
            DEps(i, j, k) = D(i, j) * Eps_min;
            CmuVt(i, j, k) = Cmut_min;
          }
        for (int i = 1; i <= Nghost; ++i) {
          DTke(Ibeg - i, j, k) = DTke(Ibeg + i - 1, j, k);
          DEps(Ibeg - i, j, k) = DEps(Ibeg + i - 1, j, k);
        }
      }
    for (int j = Jbeg; j <= Jend; ++j)
      for (int k = Kbeg; k <= Kend; ++k)
        for (int i = 1; i <= Nghost; ++i) {
          DTke(Iend + i, j, k) = DTke(Iend - i + 1, j, k);
          DEps(Iend + i, j, k) = DEps(Iend - i + 1, j, k);
        }
    for (int i = Ibeg; i <= Iend; ++i)
      for (int k = Kbeg; k <= Kend; ++k)
        for (int j = 1; j <= Nghost; ++j) {
          DTke(i, Jbeg - j, k) = DTke(i, Jbeg + j - 1, k);
          DEps(i, Jbeg - j, k) = DEps(i, Jbeg + j - 1, k);
        }
    for (int i = Ibeg; i <= Iend; ++i)
      for (int k = Kbeg; k <= Kend; ++k)
        for (int j = 1; j <= Nghost; ++j) {
          DTke(i, Jend + j, k) = DTke(i, Jend - j + 1, k);
          DEps(i, Jend + j, k) = DEps(i, Jend - j + 1, k);
        }
    for (int i = 1; i <= Mloc; ++i)
      for (int j = 1; j <= Nloc; ++j)
        for (int k = 1; k <= Kloc; ++k) {
          if (D(i, j) >= Dmin && Mask(i, j) == 1) {
            Tke(i, j, k) = DTke(i, j, k) / D(i, j);
            Eps(i, j, k) = DEps(i, j, k) / D(i, j);
            CmuVt(i, j, k) = cmiu * (Tke(i, j, k) * Tke(i, j, k)) / Eps(i, j, k);
          } else {
            Tke(i, j, k) = Tke_min;
            Eps(i, j, k) = Eps_min;
            DTke(i, j, k) = D(i, j) * Tke_min;
            DEps(i, j, k) = D(i, j) * Eps_min;
            CmuVt(i, j, k) = Cmut_min;
          }
        }
    const int w = p.wavemaker;
    if (w == NHW_WM_INT_LIN || w == NHW_WM_INT_SOL || w == NHW_WM_INT_CON || w == NHW_WM_INT_JON ||
        w == NHW_WM_INT_TMA || w == NHW_WM_INT_SPC || w == NHW_WM_INT_IRR)
      for (int k = 1; k <= Kloc; ++k)
        for (int j = 1; j <= Nloc; ++j)
          for (int i = 1; i <= Mloc; ++i)
            if (xc(i) >= p.xsource_west && xc(i) <= p.xsource_east && yc(j) >= p.ysource_suth &&
                yc(j) <= p.ysource_nrth) {
              Tke(i, j, k) = Tke_min;
              Eps(i, j, k) = Eps_min;
              DTke(i, j, k) = D(i, j) * Tke_min;
              DEps(i, j, k) = D(i, j) * Eps_min;
              CmuVt(i, j, k) = Cmut_min;
            }
  }

  // filter of les_dyn (src/nhwave.F:8412-8542): the separable [1 weit 1]
  // smoother in x (interior columns i, every j, k), y (interior i, j; every
  // k) and z (interior cells) scaled by fact, then mirrored into the ghosts
  // of the bed / surface (interior columns), the west / east sides
  // (interior rows and levels) and the south / north sides (interior
  // columns and levels); every other ghost is zero
  void les_filter(A3& In, A3& Out, double weit, double fact) {
    A3 S1, S2;
    S1.init(Mloc, Nloc, Kloc); S2.init(Mloc, Nloc, Kloc);
    Out.fill(0.0);
    for (int k = 1; k <= Kloc; ++k)
      for (int j = 1; j <= Nloc; ++j)
        for (int i = Ibeg; i <= Iend; ++i) S1(i, j, k) = In(i - 1, j, k) + weit * In(i, j, k) + In(i + 1, j, k);
    for (int k = 1; k <= Kloc; ++k)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i) S2(i, j, k) = S1(i, j - 1, k) + weit * S1(i, j, k) + S1(i, j + 1, k);
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i)
          Out(i, j, k) = fact * (S2(i, j, k - 1) + weit * S2(i, j, k) + S2(i, j, k + 1));
    les_mirror(Out, true);
  }
  // ghost mirrors of les_dyn's fields in the reference's loop order: the
  // bed, then the surface (interior columns); the west, then the east
  // sides (interior rows and levels); the south, then (if north) the north
  // side (interior columns and levels)
  void les_mirror(A3& a, bool north) {
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int k = 1; k <= Nghost; ++k) a(i, j, Kbeg - k) = a(i, j, Kbeg + k - 1);
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int k = 1; k <= Nghost; ++k) a(i, j, Kend + k) = a(i, j, Kend - k + 1);
    for (int j = Jbeg; j <= Jend; ++j)
      for (int k = Kbeg; k <= Kend; ++k)
        for (int i = 1; i <= Nghost; ++i) a(Ibeg - i, j, k) = a(Ibeg + i - 1, j, k);
    for (int j = Jbeg; j <= Jend; ++j)
      for (int k = Kbeg; k <= Kend; ++k)
        for (int i = 1; i <= Nghost; ++i) a(Iend + i, j, k) = a(Iend - i + 1, j, k);
    for (int i = Ibeg; i <= Iend; ++i)
      for (int k = Kbeg; k <= Kend; ++k)
        for (int j = 1; j <= Nghost; ++j) a(i, Jbeg - j, k) = a(i, Jbeg + j - 1, k);
    if (north)
      for (int i = Ibeg; i <= Iend; ++i)
        for (int k = Kbeg; k <= Kend; ++k)
          for (int j = 1; j <= Nghost; ++j) a(i, Jend + j, k) = a(i, Jend - j + 1, k);
  }
  // les_dyn (src/nhwave.F:7989-8410): the dynamic Smagorinsky closure of
  // IVTURB = 30 (Germano identity with Lilly's least squares).  The strain
  // rates Sij of wet interior cells deeper than 0.02 m and their ghosts
  // (the reference's north mirror copies the sixth component only, once per
  // component, and that is kept); |S| = sqrt(2 SijSij); the test-filtered
  // (weit 2, 1/64) Sij, |S|Sij, |S|, u_i u_j and u_i give Mij and Lij, the
  // coefficient -LijMij / (2 MijMij) / Delta^2 clipped to [0, 0.04] and
  // smoothed (weit 1, 1/27); CmuVt = C Delta^2 |S| in interior cells deeper
  // than 0.02 m, zero elsewhere, then the ghosts and quiet maker regions as
  // in les_3D.  |S|Sij of cells at most 0.02 m deep, which the reference
  // leaves unset, is zero here.
  void les_dyn() {
    const double Dmin = (double)0.02f;
    std::vector<A3> Sij(6);
    for (A3& a : Sij) a.init(Mloc, Nloc, Kloc);
    auto ds = [&](int k) { return sigc(k + 1) - sigc(k - 1); };
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int k = Kbeg; k <= Kend; ++k) {
          if (!(Mask(i, j) == 1 && D(i, j) > Dmin)) continue;
          const double dUs = (U(i, j, k + 1) - U(i, j, k - 1)) / ds(k), dVs = (V(i, j, k + 1) - V(i, j, k - 1)) / ds(k);
          const double dWs = (W(i, j, k + 1) - W(i, j, k - 1)) / ds(k);
          Sij[0](i, j, k) = (U(i + 1, j, k) - U(i - 1, j, k)) / (2.0 * dx) + dUs * DelxSc(i, j, k);
          Sij[1](i, j, k) = (V(i, j + 1, k) - V(i, j - 1, k)) / (2.0 * dy) + dVs * DelySc(i, j, k);
          Sij[2](i, j, k) = 1.0 / D(i, j) * (W(i, j, k + 1) - W(i, j, k - 1)) / ds(k);
          Sij[3](i, j, k) = 0.5 * ((U(i, j + 1, k) - U(i, j - 1, k)) / (2.0 * dy) + dUs * DelySc(i, j, k) +
                                   (V(i + 1, j, k) - V(i - 1, j, k)) / (2.0 * dx) + dVs * DelxSc(i, j, k));
          Sij[4](i, j, k) = 0.5 * (dVs / D(i, j) + (W(i, j + 1, k) - W(i, j - 1, k)) / (2.0 * dy) + dWs * DelySc(i, j, k));
          Sij[5](i, j, k) = 0.5 * (dUs / D(i, j) + (W(i + 1, j, k) - W(i - 1, j, k)) / (2.0 * dx) + dWs * DelxSc(i, j, k));
        }
    // the components are mirrored one by one (their loops do not mix), and
    // the reference's north loop writes the sixth component only
    for (int n = 0; n < 6; ++n) les_mirror(Sij[n], n == 5);
    A3 Sab;
    Sab.init(Mloc, Nloc, Kloc);
    std::vector<A3> SabSij(6);
    for (A3& a : SabSij) a.init(Mloc, Nloc, Kloc);
    for (int k = 1; k <= Kloc; ++k)
      for (int j = 1; j <= Nloc; ++j)
        for (int i = 1; i <= Mloc; ++i) {
          if (!(D(i, j) > Dmin)) continue;
          auto s = [&](int n) { return Sij[n](i, j, k); };
          const double a = s(0) * s(0) + s(1) * s(1) + s(2) * s(2) + 2.0 * (s(3) * s(3) + s(4) * s(4) + s(5) * s(5));
          Sab(i, j, k) = std::sqrt(2.0 * a);
          for (int n = 0; n < 6; ++n) SabSij[n](i, j, k) = Sab(i, j, k) * s(n);
        }
    const double fact1 = 1.0 / 64.0;
    std::vector<A3> FSabSij(6), FSij(6), Uij(6), FUij(6), Ui(3), FUi(3);
    A3 FSab;
    for (int n = 0; n < 6; ++n) {
      FSabSij[n].init(Mloc, Nloc, Kloc); FSij[n].init(Mloc, Nloc, Kloc);
      les_filter(SabSij[n], FSabSij[n], 2.0, fact1);
      les_filter(Sij[n], FSij[n], 2.0, fact1);
    }
    FSab.init(Mloc, Nloc, Kloc);
    les_filter(Sab, FSab, 2.0, fact1);
    for (int n = 0; n < 6; ++n) { Uij[n].init(Mloc, Nloc, Kloc); FUij[n].init(Mloc, Nloc, Kloc); }
    for (int n = 0; n < 3; ++n) { Ui[n].init(Mloc, Nloc, Kloc); FUi[n].init(Mloc, Nloc, Kloc); }
    for (size_t c = 0; c < U.v.size(); ++c) {
      const double u = U.v[c], v = V.v[c], w = W.v[c];
      Uij[0].v[c] = u * u; Uij[1].v[c] = v * v; Uij[2].v[c] = w * w;
      Uij[3].v[c] = u * v; Uij[4].v[c] = v * w; Uij[5].v[c] = u * w;
      Ui[0].v[c] = u; Ui[1].v[c] = v; Ui[2].v[c] = w;
    }
    for (int n = 0; n < 6; ++n) les_filter(Uij[n], FUij[n], 2.0, fact1);
    for (int n = 0; n < 3; ++n) les_filter(Ui[n], FUi[n], 2.0, fact1);
    A3 Smag, FW;
    Smag.init(Mloc, Nloc, Kloc); FW.init(Mloc, Nloc, Kloc);
    const double alpha2 = 4.0;
    for (int k = 1; k <= Kloc; ++k)
      for (int j = 1; j <= Nloc; ++j)
        for (int i = 1; i <= Mloc; ++i) {
          double M[6], L[6];
          for (int n = 0; n < 6; ++n) M[n] = alpha2 * FSab(i, j, k) * FSij[n](i, j, k) - FSabSij[n](i, j, k);
          auto fu = [&](int n) { return FUi[n](i, j, k); };
          L[0] = FUij[0](i, j, k) - fu(0) * fu(0);
          L[1] = FUij[1](i, j, k) - fu(1) * fu(1);
          L[2] = FUij[2](i, j, k) - fu(2) * fu(2);
          L[3] = FUij[3](i, j, k) - fu(0) * fu(1);
          L[4] = FUij[4](i, j, k) - fu(1) * fu(2);
          L[5] = FUij[5](i, j, k) - fu(2) * fu(0);
          double MM = 0.0, LM = 0.0;
          if (D(i, j) > Dmin) {
            MM = M[0] * M[0] + M[1] * M[1] + M[2] * M[2] + 2.0 * (M[3] * M[3] + M[4] * M[4] + M[5] * M[5]);
            LM = L[0] * M[0] + L[1] * M[1] + L[2] * M[2] + 2.0 * (L[3] * M[3] + L[4] * M[4] + L[5] * M[5]);
          }
          double c = 0.5 * (-LM) / (MM + (double)1.e-16f);
          FW(i, j, k) = std::pow(dx * dy * D(i, j) * dsig(k), (double)(1.0f / 3.0f));
          c = c / (FW(i, j, k) * FW(i, j, k));
          if (c < 0.0) c = 0.0;
          if (c > (double)0.04f) c = (double)0.04f;
          Smag(i, j, k) = c;
        }
    A3 FC;
    FC.init(Mloc, Nloc, Kloc);
    les_filter(Smag, FC, 1.0, (double)(1.0f / 27.0f));
    CmuVt.fill(0.0);
    for (int k = Kbeg; k <= Kend; ++k)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int i = Ibeg; i <= Iend; ++i)
          if (D(i, j) > Dmin)
            CmuVt(i, j, k) = dmax(FC(i, j, k) * (FW(i, j, k) * FW(i, j, k)) * Sab(i, j, k), 0.0);
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int k = 1; k <= Nghost; ++k) CmuVt(i, j, Kbeg - k) = CmuVt(i, j, Kbeg + k - 1);
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int k = 1; k <= Nghost; ++k) CmuVt(i, j, Kend + k) = CmuVt(i, j, Kend - k + 1);
    const bool lef = (p.wavemaker >= NHW_WM_LEF_LIN && p.wavemaker <= NHW_WM_LEF_CON) || p.wavemaker == NHW_WM_LEF_TID ||
                     p.wavemaker == NHW_WM_LEF_JON || p.wavemaker == NHW_WM_LEF_TMA || p.wavemaker == NHW_WM_LEF_SPC;
    for (int j = Jbeg; j <= Jend; ++j)
      for (int k = Kbeg; k <= Kend; ++k) {
        if (lef) CmuVt(Ibeg, j, k) = Zero;
        for (int i = 1; i <= Nghost; ++i) CmuVt(Ibeg - i, j, k) = CmuVt(Ibeg + i - 1, j, k);
      }
    for (int j = Jbeg; j <= Jend; ++j)
      for (int k = Kbeg; k <= Kend; ++k)
        for (int i = 1; i <= Nghost; ++i) CmuVt(Iend + i, j, k) = CmuVt(Iend - i + 1, j, k);
    for (int i = Ibeg; i <= Iend; ++i)
      for (int k = Kbeg; k <= Kend; ++k)
        for (int j = 1; j <= Nghost; ++j) CmuVt(i, Jbeg - j, k) = CmuVt(i, Jbeg + j - 1, k);
    for (int i = Ibeg; i <= Iend; ++i)
      for (int k = Kbeg; k <= Kend; ++k)
        for (int j = 1; j <= Nghost; ++j) CmuVt(i, Jend + j, k) = CmuVt(i, Jend - j + 1, k);
    if (ke_quiet_maker())
      for (int k = 1; k <= Kloc; ++k)
        for (int j = 1; j <= Nloc; ++j)
          for (int i = 1; i <= Mloc; ++i)
            if (xc(i) >= p.xsource_west && xc(i) <= p.xsource_east && yc(j) >= p.ysource_suth &&
                yc(j) <= p.ysource_nrth)
              CmuVt(i, j, k) = Zero;
  }

  // eval_turb (src/nhwave.F:6544-6782), called after sponge_damping.
  // Vertical: IVTURB 1 CmuVt = Cvs; 2 the subgrid model CmuVt = Cvs D
  // dsig^2 |d(U,V)/dsigma| on every level but the outermost ghosts, which
  // copy their neighbours.  Horizontal: IHTURB 1 CmuHt = Chs; 2 CmuHt = Chs
  // dx dy |S| from the horizontal strain rates, then mirrored into the
  // ghosts of the sides (interior rows) and of the bed and surface
  // (interior columns).  The reference's Strxy reads U(i,j+1,j), the row
  // index where the level belongs (:6695); the level k is used here.
  void eval_turb(int istep) {
    if (!p.viscous_flow) return;
    if (p.ivturb == 1) {
      CmuVt.fill(p.cvs);
    } else if (p.ivturb == 10) {
      kepsilon_3D(istep);
    } else if (p.ivturb == 20) {
      les_3D();
    } else if (p.ivturb == 3) {
      kepsilon_2D(istep);
    } else if (p.ivturb == 30) {
      les_dyn();
    } else {
      for (int i = 1; i <= Mloc; ++i)
        for (int j = 1; j <= Nloc; ++j) {
          for (int k = 2; k <= Kloc - 1; ++k) {
            const double DelsU = (U(i, j, k + 1) - U(i, j, k - 1)) / (sigc(k + 1) - sigc(k - 1));
            const double DelsV = (V(i, j, k + 1) - V(i, j, k - 1)) / (sigc(k + 1) - sigc(k - 1));
            CmuVt(i, j, k) = p.cvs * D(i, j) * (dsig(k) * dsig(k)) * std::sqrt(DelsU * DelsU + DelsV * DelsV);
          }
          CmuVt(i, j, 1) = CmuVt(i, j, 2);
          CmuVt(i, j, Kloc) = CmuVt(i, j, Kloc - 1);
        }
    }
    if (p.ihturb == 1) {
      CmuHt.fill(p.chs);
      return;
    }
    if (p.ihturb >= 10) {   // the 3-D model's length scales in every direction
      CmuHt = CmuVt;
      return;
    }
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int k = Kbeg; k <= Kend; ++k) {
          const double ds = sigc(k + 1) - sigc(k - 1);
          const double Strxx = (U(i + 1, j, k) - U(i - 1, j, k)) / (2.0 * dx) +
                               (U(i, j, k + 1) - U(i, j, k - 1)) / ds * DelxSc(i, j, k);
          const double Stryy = (V(i, j + 1, k) - V(i, j - 1, k)) / (2.0 * dy) +
                               (V(i, j, k + 1) - V(i, j, k - 1)) / ds * DelySc(i, j, k);
          const double Strxy = 0.5 * ((U(i, j + 1, k) - U(i, j - 1, k)) / (2.0 * dy) +
                                      (U(i, j, k + 1) - U(i, j, k - 1)) / ds * DelySc(i, j, k) +
                                      (V(i + 1, j, k) - V(i - 1, j, k)) / (2.0 * dx) +
                                      (V(i, j, k + 1) - V(i, j, k - 1)) / ds * DelxSc(i, j, k));
          CmuHt(i, j, k) = p.chs * dx * dy * std::sqrt(Strxx * Strxx + 2.0 * (Strxy * Strxy) + Stryy * Stryy);
        }
    for (int j = Jbeg; j <= Jend; ++j)
      for (int k = Kbeg; k <= Kend; ++k)
        for (int i = 1; i <= Nghost; ++i) {
          CmuHt(Ibeg - i, j, k) = CmuHt(Ibeg + i - 1, j, k);
          CmuHt(Iend + i, j, k) = CmuHt(Iend - i + 1, j, k);
        }
    for (int i = Ibeg; i <= Iend; ++i)
      for (int k = Kbeg; k <= Kend; ++k)
        for (int j = 1; j <= Nghost; ++j) {
          CmuHt(i, Jbeg - j, k) = CmuHt(i, Jbeg + j - 1, k);
          CmuHt(i, Jend + j, k) = CmuHt(i, Jend - j + 1, k);
        }
    for (int i = Ibeg; i <= Iend; ++i)
      for (int j = Jbeg; j <= Jend; ++j)
        for (int k = 1; k <= Nghost; ++k) {
          CmuHt(i, j, Kbeg - k) = CmuHt(i, j, Kbeg + k - 1);
          CmuHt(i, j, Kend + k) = CmuHt(i, j, Kend - k + 1);
        }
  }

  void sponge_damping() {
    const double Ramp = p.tramp > 0.0 ? std::tanh(TIME / p.tramp) : 1.0;
    const double Ucur = Ramp * p.cur_wave;
    for (int j = 1; j <= Nloc; ++j)
      for (int i = 1; i <= Mloc; ++i)
        if (Mask(i, j) == 1) {
          Eta(i, j) = Eta(i, j) * Sponge(i, j);
          D(i, j) = Eta(i, j) + Hc(i, j);
          for (int k = 1; k <= Kloc; ++k) {
            U(i, j, k) = (U(i, j, k) - Ucur) * Sponge(i, j) + Ucur;
            V(i, j, k) = V(i, j, k) * Sponge(i, j);
            DU(i, j, k) = D(i, j) * U(i, j, k);
            DV(i, j, k) = D(i, j) * V(i, j, k);
          }
        }
  }

  int step() {
    int st = estimate_dt();
    if (st) return status = st;
    if (p.slide_type != NHW_SLIDE_NONE) update_bathymetry();
    update_wave_bc();
    update_mask();
    update_wind();
    update_vars();
    int worst = NHW_OK;
    for (int s = 1; s <= It_Order; ++s) {
      source_terms();
      fluxes();
      int e = eval_duvw(s);
      if (e != NHW_OK && worst == NHW_OK) worst = e;
      if (p.sponge_on) sponge_damping();
      eval_turb(s);
    }
    if (worst == NHW_ERR_NAN) status = worst;
    return worst;
  }

  double mass() {
    double MassVolume = Zero;
    for (int j = Jbeg; j <= Jend; ++j)
      for (int i = Ibeg; i <= Iend; ++i) MassVolume = MassVolume + D(i, j) * dx * dy;
    return MassVolume;
  }
  // statistics (src/nhwave.F:3118-3160): MassVolume, Energy, MaxEta, MinEta,
  // MaxU, MaxV, MaxW, in the reference's loop order
  void statistics(double* out) {
    double MassVolume = Zero, Energy = Zero;
    for (int j = Jbeg; j <= Jend; ++j)
      for (int i = Ibeg; i <= Iend; ++i) {
        MassVolume = MassVolume + D(i, j) * dx * dy;
        for (int k = Kbeg; k <= Kend; ++k) {
          const double CellMass = Rho0 * dsig(k) * D(i, j) * dx * dy;
          Energy = Energy + CellMass * Grav * (D(i, j) * sigc(k) - Hc(i, j)) +
                   0.5 * CellMass * (U(i, j, k) * U(i, j, k) + V(i, j, k) * V(i, j, k) + W(i, j, k) * W(i, j, k));
        }
      }
    double MaxEta = -1e308, MinEta = 1e308, MaxU = 0.0, MaxV = 0.0, MaxW = 0.0;
    for (int j = Jbeg; j <= Jend; ++j)
      for (int i = Ibeg; i <= Iend; ++i) {
        MaxEta = std::max(MaxEta, Eta(i, j));
        MinEta = std::min(MinEta, Eta(i, j));
        for (int k = Kbeg; k <= Kend; ++k) {
          MaxU = std::max(MaxU, std::fabs(U(i, j, k)));
          MaxV = std::max(MaxV, std::fabs(V(i, j, k)));
          MaxW = std::max(MaxW, std::fabs(W(i, j, k)));
        }
      }
    out[0] = MassVolume; out[1] = Energy; out[2] = MaxEta; out[3] = MinEta;
    out[4] = MaxU; out[5] = MaxV; out[6] = MaxW;
  }

  // ------------------------------------------------------- field access
  struct FieldRef { double* d = nullptr; int32_t* i = nullptr; size_t n = 0; };
  FieldRef field(int f) {
    FieldRef r;
    auto a2 = [&](A2& a) { r.d = a.v.data(); r.n = a.v.size(); };
    auto a3 = [&](A3& a) { r.d = a.v.data(); r.n = a.v.size(); };
    auto i2 = [&](I2& a) { r.i = a.v.data(); r.n = a.v.size(); };
    switch (f) {
      case NHW_F_D: a2(D); break;            case NHW_F_D0: a2(D0); break;
      case NHW_F_ETA: a2(Eta); break;        case NHW_F_ETA0: a2(Eta0); break;
      case NHW_F_HC: a2(Hc); break;          case NHW_F_HC0: a2(Hc0); break;
      case NHW_F_DELXH: a2(DelxH); break;    case NHW_F_DELYH: a2(DelyH); break;
      case NHW_F_DELXETA: a2(DelxEta); break; case NHW_F_DELYETA: a2(DelyEta); break;
      case NHW_F_DELTH: a2(DeltH); break;    case NHW_F_DELT2H: a2(Delt2H); break;
      case NHW_F_SOURCEX: a2(SourceX); break; case NHW_F_SOURCEY: a2(SourceY); break;
      case NHW_F_SOURCEC: a2(SourceC); break; case NHW_F_SPONGE: a2(Sponge); break;
      case NHW_F_R1: a2(R1s); break;
      case NHW_F_HFX: a2(Hfx); break;        case NHW_F_HFX0: a2(Hfx0); break;
      case NHW_F_ETAXL: a2(EtaxL); break;    case NHW_F_ETAXR: a2(EtaxR); break;
      case NHW_F_HFY: a2(Hfy); break;        case NHW_F_HFY0: a2(Hfy0); break;
      case NHW_F_ETAYL: a2(EtayL); break;    case NHW_F_ETAYR: a2(EtayR); break;
      case NHW_F_MASK: i2(Mask); break;      case NHW_F_MASK_STRUCT: i2(Mask_Struct); break;
      case NHW_F_MASK9: i2(Mask9); break;
      case NHW_F_U: a3(U); break; case NHW_F_V: a3(V); break; case NHW_F_W: a3(W); break;
      case NHW_F_DU: a3(DU); break; case NHW_F_DV: a3(DV); break; case NHW_F_DW: a3(DW); break;
      case NHW_F_DU0: a3(DU0); break; case NHW_F_DV0: a3(DV0); break; case NHW_F_DW0: a3(DW0); break;
      case NHW_F_P: a3(P); break; case NHW_F_OMEGA: a3(Omega); break;
      case NHW_F_EX: a3(Ex); break; case NHW_F_FX: a3(Fx); break; case NHW_F_GX: a3(Gx); break;
      case NHW_F_HX: a3(Hx); break; case NHW_F_EY: a3(Ey); break; case NHW_F_FY: a3(Fy); break;
      case NHW_F_GY: a3(Gy); break; case NHW_F_HY: a3(Hy); break; case NHW_F_FZ: a3(Fz); break;
      case NHW_F_GZ: a3(Gz); break; case NHW_F_HZ: a3(Hz); break;
      case NHW_F_CMUVT: a3(CmuVt); break; case NHW_F_CMUHT: a3(CmuHt); break;
      case NHW_F_TKE: a3(Tke); break; case NHW_F_EPS: a3(Eps); break;
      case NHW_F_DTKE: a3(DTke); break; case NHW_F_DEPS: a3(DEps); break;
      default: break;
    }
    return r;
  }
};

}  // namespace

extern "C" {

void* orc_create(const nhw_params* p, int* status) {
  Model* m = new Model();
  int st = p ? m->create(*p) : NHW_ERR_ARG;
  if (status) *status = st;
  if (st != NHW_OK) { delete m; return nullptr; }
  return m;
}
void orc_destroy(void* o) { delete static_cast<Model*>(o); }
int orc_setup(void* o, const double* depth, const double* eta0, const double* uvw0) {
  Model* m = static_cast<Model*>(o);
  if (!m || !depth) return NHW_ERR_ARG;
  m->generate_grid();
  m->read_bathymetry(depth);
  m->initial(eta0, uvw0);
  return NHW_OK;
}
int orc_estimate_dt(void* o) { return static_cast<Model*>(o)->estimate_dt(); }
void orc_update_bathymetry(void* o) { static_cast<Model*>(o)->update_bathymetry(); }
void orc_update_mask(void* o) { static_cast<Model*>(o)->update_mask(); }
void orc_update_wave_bc(void* o) { static_cast<Model*>(o)->update_wave_bc(); }
void orc_update_vars(void* o) { Model* m = static_cast<Model*>(o); m->update_wind(); m->update_vars(); }
void orc_source_terms(void* o) { static_cast<Model*>(o)->source_terms(); }
void orc_eval_turb(void* o, int istep) { static_cast<Model*>(o)->eval_turb(istep); }
void orc_fluxes(void* o) { static_cast<Model*>(o)->fluxes(); }
int orc_eval_duvw(void* o, int istep) { return static_cast<Model*>(o)->eval_duvw(istep); }
void orc_sponge_damping(void* o) { static_cast<Model*>(o)->sponge_damping(); }
int orc_step(void* o) { return static_cast<Model*>(o)->step(); }
double orc_mass(void* o) { return static_cast<Model*>(o)->mass(); }
void orc_statistics(void* o, double* out) { static_cast<Model*>(o)->statistics(out); }
int orc_get_field(void* o, int f, void* out) {
  auto r = static_cast<Model*>(o)->field(f);
  if (!out || r.n == 0) return NHW_ERR_ARG;
  if (r.d) std::memcpy(out, r.d, r.n * sizeof(double));
  else std::memcpy(out, r.i, r.n * sizeof(int32_t));
  return NHW_OK;
}
int orc_set_field(void* o, int f, const void* in) {
  auto r = static_cast<Model*>(o)->field(f);
  if (!in || r.n == 0) return NHW_ERR_ARG;
  if (r.d) std::memcpy(r.d, in, r.n * sizeof(double));
  else std::memcpy(r.i, in, r.n * sizeof(int32_t));
  return NHW_OK;
}
void orc_get_scalars(void* o, nhw_scalars* s) {
  Model* m = static_cast<Model*>(o);
  std::memset(s, 0, sizeof(*s));
  s->time = m->TIME; s->dt = m->dt; s->dt_old = m->dt_old; s->run_step = m->RUN_STEP;
  s->last_krylov_iters = m->last_iters; s->total_krylov_iters = m->total_iters;
  s->poisson_solves = m->solves; s->last_rel_residual = m->last_relres; s->status = m->status;
}
void orc_set_time(void* o, double time, double dt, int run_step) {
  Model* m = static_cast<Model*>(o);
  m->TIME = time; m->dt = dt; m->RUN_STEP = run_step;
}
// the LEF_JON / LEF_TMA phases RanPhs (n = NumFreq), as nhw_set_wave_phases
int orc_set_wave_phases(void* o, int n, const double* phases) {
  Model* m = static_cast<Model*>(o);
  if (n != (int)m->RanPhs.size() || n == 0 || !phases) return NHW_ERR_ARG;
  for (int i = 0; i < n; ++i) m->RanPhs[i] = phases[i];
  return NHW_OK;
}
// The 2-D spectrum of LEF_SPC / INT_SPC (densities) or INT_IRR (amplitudes
// and their phases), as nhw_set_wave_spectrum takes it
int orc_set_wave_spectrum(void* o, int nf, int nd, const double* freq, const double* dire, const double* spc,
                          const double* phases) {
  Model* m = static_cast<Model*>(o);
  const int wm = m->p.wavemaker;
  if ((wm != NHW_WM_LEF_SPC && wm != NHW_WM_INT_SPC && wm != NHW_WM_INT_IRR) || nf < 2 || nd < 2 || !freq ||
      !dire || !spc)
    return NHW_ERR_ARG;
  if (wm == NHW_WM_INT_IRR && !phases) return NHW_ERR_ARG;   // irr2d.txt holds them
  if (wm != NHW_WM_LEF_SPC)   // the internal makers' direction search ends only within 90 degrees
    for (int q = 0; q < nd; ++q)
      if (!(std::fabs(dire[q]) <= 90.0)) return NHW_ERR_ARG;
  m->NumFreq_s = nf;
  m->NumDir_s = nd;
  m->Freq_s.assign(freq, freq + nf);
  m->Dire_s.assign(dire, dire + nd);
  m->Spc2d.assign(spc, spc + nf * nd);
  m->Random_Phs.assign(nf * nd, 0.0);
  for (int c = 0; c < nf * nd; ++c) m->Random_Phs[c] = phases ? phases[c] : Model::phase_of(m->p.wave_seed, c);
  return NHW_OK;
}
// the west-boundary elevation Ein_X0 (Nloc values) of the last update_wave_bc
int orc_get_inflow_eta(void* o, double* out) {
  Model* m = static_cast<Model*>(o);
  std::memcpy(out, m->Ein_X0.v.data(), m->Ein_X0.v.size() * sizeof(double));
  return (int)m->Ein_X0.v.size();
}
// grid vectors for tests: which = 0 x, 1 xc, 2 y, 3 yc, 4 sig, 5 dsig, 6 sigc
int orc_get_grid(void* o, int which, double* out) {
  Model* m = static_cast<Model*>(o);
  A1* a[] = {&m->x, &m->xc, &m->y, &m->yc, &m->sig, &m->dsig, &m->sigc};
  if (which < 0 || which > 6 || !out) return NHW_ERR_ARG;
  std::memcpy(out, a[which]->v.data(), a[which]->v.size() * sizeof(double));
  return (int)a[which]->v.size();
}
// Poisson operator access for tests: coefficient n (1..15) and Rhs
int orc_get_coef(void* o, double* coef15, double* rhs) {
  Model* m = static_cast<Model*>(o);
  if (coef15) std::memcpy(coef15, m->Coef.data(), m->Coef.size() * sizeof(double));
  if (rhs) std::memcpy(rhs, m->Rhs.data(), m->Rhs.size() * sizeof(double));
  return m->neqns;
}
void orc_generate_coef_rhs(void* o) { static_cast<Model*>(o)->generate_coef_rhs(); }
double orc_limiter(double a, double b) { return LIMITER(a, b); }
double orc_wave_number(void* o, double segma) { return static_cast<Model*>(o)->wave_dispersion(segma); }
// the AGM elliptic functions of the cnoidal boundary wave: 0 cn(u|m), 1 K(m), 2 E(m)
double orc_elliptic(int what, double u, double m) {
  return what == 0 ? cnoidal_cn(u, m) : what == 1 ? cnoidal_ck(m) : cnoidal_ce(m);
}
// cnoidal (src/waves.F:184-220): out[0..2] = wave length, trough level, m;
// returns 0, or -1 when the iteration leaves (0, 1]
int orc_cnoidal_wave(double height, double depth, double period, double* out) {
  return cnoidal(height, depth, period, out[0], out[1], out[2]) ? 0 : -1;
}

}  // extern "C"
