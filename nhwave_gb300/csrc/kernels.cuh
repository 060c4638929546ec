// kernels.cuh -- device operations of the NHWAVE time step, templated on the
// 3-D storage type T (double: plain FP64 form; float: FP32+IR form).
//
// Each operation is a functor applied to one work item (a cell, a face, or a
// water column) of one scenario; generic __global__ launchers map threads to
// work items.  Arithmetic follows the reference's evaluation order term by
// term (the FP64 instantiation is compiled without FMA contraction), so the
// FP64 form reproduces the CPU restatement of the reference exactly wherever
// no libm transcendental (cos, cosh, log, atan2) or parallel reduction is
// involved.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <type_traits>
#include "../../include/nhwave_gb300.h"
#include "cnoidal.h"
#include "components.h"
#include "state.h"

namespace nhw {

// ----------------------------------------------------------------- helpers
__device__ __forceinline__ double dmax_(double a, double b) { return a > b ? a : b; }
__device__ __forceinline__ double dmin_(double a, double b) { return a < b ? a : b; }
template <class R> __device__ __forceinline__ R rmax(R a, R b) { return a > b ? a : b; }
template <class R> __device__ __forceinline__ R rmin(R a, R b) { return a < b ? a : b; }

// van Leer LIMITER (src/nhwave.F:2889-2906)
template <class R>
__device__ __forceinline__ R limiter(R A, R B) {
  return (A * fabs(B) + fabs(A) * B) / (fabs(A) + fabs(B));
}
// limited slope of delx/y/zFun (src/nhwave.F:2060-2351): zero if |T1|+|T2| < Small
template <class R>
__device__ __forceinline__ R lim_slope(R am, R a0, R ap, R dm, R dp) {
  R t1 = (ap - a0) / dp;
  R t2 = (a0 - am) / dm;
  return (fabs(t1) + fabs(t2)) < (R)kSmall ? (R)0 : limiter(t1, t2);
}
// the same with the reciprocals of the spacings (FP32 form: products for divisions)
template <class R>
__device__ __forceinline__ R lim_slope_r(R am, R a0, R ap, R rdm, R rdp) {
  R t1 = (ap - a0) * rdp;
  R t2 = (a0 - am) * rdm;
  return (fabs(t1) + fabs(t2)) < (R)kSmall ? (R)0 : limiter(t1, t2);
}
// lim_slope over a uniform spacing d (1/d = rd): FP64 divides as the reference
// does, FP32 multiplies by the reciprocal
template <class R>
__device__ __forceinline__ R lim_slope_u(R am, R a0, R ap, R d, R rd) {
  if constexpr (sizeof(R) == 4) return lim_slope_r<R>(am, a0, ap, rd, rd);
  else return lim_slope<R>(am, a0, ap, d, d);
}
// 0.5*Grav*(eta*eta + 2*eta*h0): hydrostatic part of the momentum flux
template <class R>
__device__ __forceinline__ R hydro(R eta, R h0) {
  return (R)0.5 * (R)kGrav * (eta * eta + (R)2.0 * eta * h0);
}
template <class R>
__device__ __forceinline__ R hll_d(R sl, R sr, R fl, R fr, R d_ur_ul) {
  // HLL (src/nhwave.F:2741-2776) with UR-UL given
  if (sl >= (R)0) return fl;
  if (sr <= (R)0) return fr;
  R f = sr * fl - sl * fr + sl * sr * d_ur_ul;
  if (fabs(sr - sl) < (R)kSmall) return f / (R)kSmall;
  return f / (sr - sl);
}
template <class R>
__device__ __forceinline__ R hll(R sl, R sr, R fl, R fr, R ul, R ur) {
  return hll_d<R>(sl, sr, fl, fr, ur - ul);
}
// Contact speed of a wet/wet face for HLLC in FP32: (uL+uR)/2 + sqrt(g dL) -
// sqrt(g dR) (src/nhwave.F:2835), the difference of the two roots formed as
// g (dL - dR) / (sqrt(g dL) + sqrt(g dR)) with dL - dR in FP64.  The plain
// difference of two FP32 roots of about 1-10 m/s cancels to an absolute error
// of a few 1e-7 m/s, which the HLLC mass flux carries in full (HLL takes
// dR - dL in FP64 and never forms it).
__device__ __forceinline__ float contact_speed_f32(float uL, float uR, float pL, float pR, double dL,
                                                   double dR) {
  return 0.5f * (uL + uR) + (float)(dL - dR) * (float)kGrav / (pL + pR);
}
// HLLC (src/nhwave.F:2779-2810): uls/urs are the star states of the face
template <class R>
__device__ __forceinline__ R hllc(R sl, R sr, R ss, R fl, R fr, R ul, R uls, R ur, R urs) {
  if (sl >= (R)0) return fl;
  if (sr <= (R)0) return fr;
  if (ss >= (R)0) return fl + sl * (uls - ul);
  return fr + sr * (urs - ur);
}

__device__ __forceinline__ int mirror(int i, int b, int e) {
  return i < b ? 2 * b - 1 - i : (i > e ? 2 * e + 1 - i : i);
}

// ---------------------------------------------------------------- launchers
// In a captured step graph every kernel of the step body returns at once
// when k_dt_finalize held the step back.
template <class T>
__device__ __forceinline__ bool gated_off(const Dev<T>& S) {
  return S.graph_mode && !S.sc->step_go;
}

// work-item decoders
struct AllCols { template <class T> __device__ static int n(const Dev<T>& S) { return S.Mloc * S.Nloc; } };

template <class T, class Op>
__global__ void __launch_bounds__(256) k_allcols(Dev<T> S, Op op) {
  if (gated_off(S)) return;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= S.Mloc * S.Nloc) return;
  op(S, t % S.Mloc, t / S.Mloc);
}
template <class T, class Op>
__global__ void __launch_bounds__(256) k_incols(Dev<T> S, Op op) {
  if (gated_off(S)) return;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= S.M * S.N) return;
  op(S, S.IB + t % S.M, S.JB + t / S.M);
}
// cells over an (nx x ny x nz) box starting at (ox, oy, oz)
// (32-bit decode: a scenario's boxes hold fewer than 2^32 cells, which the
// host checks at nhw_create; 64-bit division is a long software sequence)
template <class T, class Op>
__global__ void __launch_bounds__(256) k_box(Dev<T> S, Op op, int nx, int ny, int nz, int ox, int oy, int oz) {
  if (gated_off(S)) return;
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned n = (unsigned)nx * (unsigned)ny * (unsigned)nz;
  if (t >= n) return;
  const unsigned r = t / (unsigned)nx;
  const int i = (int)(t - r * (unsigned)nx);
  const unsigned k = r / (unsigned)ny;
  const int j = (int)(r - k * (unsigned)ny);
  op(S, ox + i, oy + j, oz + (int)k);
}
// all cells of the ghosted array
template <class T, class Op>
__global__ void __launch_bounds__(256) k_allcells(Dev<T> S, Op op) {
  if (gated_off(S)) return;
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned n = (unsigned)S.Mloc * (unsigned)S.Nloc * (unsigned)S.Kloc;
  if (t >= n) return;
  const unsigned r = t / (unsigned)S.Mloc;
  const int i = (int)(t - r * (unsigned)S.Mloc);
  const unsigned k = r / (unsigned)S.Nloc;
  op(S, i, (int)(r - k * (unsigned)S.Nloc), (int)k);
}

// ------------------------------------------------------------ reductions
// Deterministic block reduction of NV doubles; the last block to finish
// combines the per-block partials in a fixed order and calls fin(S, vals).
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* sh) {
  // sh: at least NV * 32 doubles
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int q = 0; q < NV; ++q)
    for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_down_sync(0xffffffffu, v[q], o);
  __syncthreads();
  if (lane == 0)
    for (int q = 0; q < NV; ++q) sh[q * 32 + warp] = v[q];
  __syncthreads();
  if (warp == 0) {
    for (int q = 0; q < NV; ++q) {
      double x = lane < nw ? sh[q * 32 + lane] : 0.0;
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      v[q] = x;
    }
  }
}

template <int NV, class T, class Fin>
__device__ __forceinline__ void reduce_finalize(const Dev<T>& S, double (&v)[NV], int slot, Fin fin) {
  __shared__ double sh[NV * 32];
  __shared__ bool last;
  block_sum<NV>(v, sh);
  const int nb = gridDim.x;
  if (threadIdx.x == 0) {
    for (int q = 0; q < NV; ++q) S.partials[(size_t)blockIdx.x * 8 + q] = v[q];
    __threadfence();
    unsigned prev = atomicAdd(&S.sc->counter[slot], 1u);
    last = (prev == (unsigned)nb - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double acc[NV];
  for (int q = 0; q < NV; ++q) acc[q] = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
    for (int q = 0; q < NV; ++q) acc[q] += ((volatile double*)S.partials)[(size_t)b * 8 + q];
  block_sum<NV>(acc, sh);
  if (threadIdx.x == 0) {
    S.sc->counter[slot] = 0u;
    fin(S, acc);
  }
}

// =========================================================================
//   update_wave_bc: waves fed through the west boundary (BC_X0 = 3)
//   (src/nhwave.F:5514-5565; LEF_LIN src/waves.F:808-855, LEF_SOL 869-903,
//   LEF_STK 518-560, LEF_CON 92-170)
// =========================================================================
// one thread per row j (all Nloc rows for Ein/Din, interior rows for the
// velocities), evaluated at the step's new TIME
struct OpWaveBC {
  static constexpr const char* kName = "wave_bc";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int, int j, int) const {
    const double TIME = S.sc->time;
    const double hfx = S.Hfx[i2(S, S.IB, j)];
    const bool inner = j >= S.JB && j <= S.JE;
    const int Nl = S.Nloc;
    if (S.lef == 3 || S.lef == 7) {   // LEF_LIN; WAV_CUR adds the ramped current (src/waves.F:706-756)
      const double A = S.lef_amp;
      double Ucur = 0.0;
      if (S.lef == 7) Ucur = (S.tramp > 0.0 ? tanh(TIME / S.tramp) : 1.0) * S.cur_wave;
      const double phs = S.yc[j] * S.lef_sinth * S.lef_wn;
      const double arg = kPi / 2 - S.lef_segma * TIME + phs;
      const double cs = cos(arg), sn = sin(arg);
      const double E = 0.5 * A * cs;
      const double Dn = E + hfx;
      S.Ein[j] = E;
      S.Din[j] = Dn;
      if (!inner) return;
      for (int k = S.KB; k <= S.KE; ++k) {
        const double Zlev = S.sigc[k] * Dn;
        const double ch = cosh(S.lef_wn * Zlev), sh = sinh(S.lef_wn * Zlev);
        const double u = Ucur + 0.5 * A * S.lef_segma * ch / S.lef_shd * cs - S.lef_stokes * 1.0;
        S.Uin[j + Nl * k] = u * S.lef_costh;
        S.Win[j + Nl * k] = 0.5 * A * S.lef_segma * sh / S.lef_shd * sn;
        S.Vin[j + Nl * k] = u * S.lef_sinth;
      }
    } else if (S.lef == 4) {   // LEF_SOL
      const double A = S.lef_amp, Dep = S.lef_dep, Atmp = S.lef_atmp;
      const double Xc = S.lef_xstart - S.lef_cel * TIME;
      const double ch = cosh(Atmp * Xc), sh = sinh(Atmp * Xc);
      const double ch2 = ch * ch, ch3 = ch * ch2, ch4 = ch2 * ch2, ch5 = ch * ch4;
      const double E = A / ch2;
      const double Dn = E + hfx;
      S.Ein[j] = E;
      S.Din[j] = Dn;
      if (!inner) return;
      const double C2 = S.lef_c2;
      const double D2 = 2.0 * A * (Atmp * Atmp) * (2.0 * ch2 - 3.) / ch4;
      const double D1 = -2.0 * A * sh * Atmp / ch3;
      const double D3 = -8.0 * A * sh * (Atmp * Atmp * Atmp) * (ch2 - 3.) / ch5;
      for (int k = S.KB; k <= S.KE; ++k) {
        const double Zlev = S.sigc[k] * Dn;
        S.Uin[j + Nl * k] =
            C2 * E / Dep * (1.0 - 0.25 * E / Dep + Dep / 3.0 * (Dep / E) * (1.0 - 1.5 * (Zlev * Zlev) / (Dep * Dep)) * D2);
        S.Win[j + Nl * k] = -C2 * Zlev / Dep *
                            ((1.0 - 0.5 * E / Dep) * D1 +
                             (double)(1.0f / 3.0f) * (Dep * Dep) * (1.0 - 0.5 * (Zlev * Zlev) / (Dep * Dep)) * D3);
        S.Vin[j + Nl * k] = 0.0;
      }
    } else if (S.lef == 5) {   // LEF_STK: second-order Stokes wave
      const double A = S.lef_amp, Sg = S.lef_segma, wk = S.lef_wn, sh = S.lef_shd;
      const double ph = kPi / 2 - Sg * TIME;
      const double cs = cos(ph), sn = sin(ph), cs2 = cos(2. * ph), sn2 = sin(2. * ph);
      const double E = 0.5 * A * cs + S.lef_e2 * cs2;
      const double Dn = E + hfx;
      S.Ein[j] = E;
      S.Din[j] = Dn;
      if (!inner) return;
      const double sh4 = (sh * sh) * (sh * sh);
      for (int k = S.KB; k <= S.KE; ++k) {
        const double Zlev = S.sigc[k] * Dn;
        S.Uin[j + Nl * k] = 0.5 * A * Sg * cosh(wk * Zlev) / sh * cs + S.lef_u2 * cosh(2. * wk * Zlev) / sh4 * cs2;
        S.Win[j + Nl * k] = 0.5 * A * Sg * sinh(wk * Zlev) / sh * sn + S.lef_u2 * sinh(2. * wk * Zlev) / sh4 * sn2;
        S.Vin[j + Nl * k] = 0.0;
      }
    } else if (S.lef == 9) {   // LEF_TID: the S2 tide, period 43200 s (src/nhwave.F:5715-5750)
      const double E = 0.5 * S.lef_amp * cos(2.0 * kPi / 43200. * TIME - kPi / 2.0);
      S.Ein[j] = E;
      S.Din[j] = E + hfx;
      if (!inner) return;
      for (int k = S.KB; k <= S.KE; ++k) {
        S.Uin[j + Nl * k] = sqrt(kGrav / hfx) * E;
        S.Vin[j + Nl * k] = 0.0;
        S.Win[j + Nl * k] = 0.0;
      }
    } else if (S.lef == 8) {   // FOCUSED: a group of NWAVE linear components (src/waves.F:638-692)
      const int nw = S.nwave;
      const double *Ai = S.foc, *ki = S.foc + nw, *fi = S.foc + 2 * nw;
      const double tc = TIME - (double)(int)(TIME / 20.0) * 20.0;   // the group repeats every 20 s
      const double dc = S.foc_dc;
      double E = 0.0;
      for (int n = 0; n < nw; ++n) E = E + Ai[n] * cos(-ki[n] * S.foc_xb - 2. * kPi * fi[n] * (tc - S.foc_tb));
      const double Dn = E + hfx;
      S.Ein[j] = E;
      S.Din[j] = Dn;
      if (!inner) return;
      for (int k = S.KB; k <= S.KE; ++k) {
        const double Zlev = S.sigc[k] * Dn;
        double u = 0.0, w = 0.0;
        for (int n = 0; n < nw; ++n) {
          const double sg = 2. * kPi * fi[n], c = sg / ki[n];
          const double ph = -ki[n] * S.foc_xb - sg * (tc - S.foc_tb);
          const double sd = kGrav * (Ai[n] * Ai[n]) / c / dc / 2.;
          u = u + kGrav * Ai[n] * ki[n] / sg * cosh(ki[n] * Zlev) / cosh(ki[n] * (dc + E)) * cos(ph) -
              sd * (2 * ki[n] * dc) / sinh(2 * ki[n] * (dc + E)) * cosh(2 * ki[n] * Zlev) * S.foc_sd;
          w = w + kGrav * Ai[n] * ki[n] / sg * sinh(ki[n] * Zlev) / cosh(ki[n] * (dc + E)) * sin(ph);
        }
        S.Uin[j + Nl * k] = u;
        S.Win[j + Nl * k] = w;
        S.Vin[j + Nl * k] = 0.0;
      }
    } else if (S.lef == 12 || S.lef == 13) {   // LEF_JON / LEF_TMA (src/waves.F:566-623)
      const int nf = S.njon;
      const double *Wh = S.jon, *sg = S.jon + nf, *wk = S.jon + 2 * nf, *sd = S.jon + 3 * nf;
      const double *ph = S.jon + 4 * nf, *shd = S.jon + 5 * nf;
      double E = 0.0;
      for (int n = 0; n < nf; ++n) E = E + 0.5 * Wh[n] * cos(kPi / 2 - sg[n] * TIME + ph[n]);
      const double Dn = E + hfx;
      S.Ein[j] = E;
      S.Din[j] = Dn;
      if (!inner) return;
      for (int k = S.KB; k <= S.KE; ++k) {
        const double Zlev = S.sigc[k] * Dn;
        double u = 0.0, w = 0.0;
        for (int n = 0; n < nf; ++n) {
          const double arg = kPi / 2 - sg[n] * TIME + ph[n];
          u = u + 0.5 * Wh[n] * sg[n] * cosh(wk[n] * Zlev) / shd[n] * cos(arg) - sd[n] * 1.0;
          w = w + 0.5 * Wh[n] * sg[n] * sinh(wk[n] * Zlev) / shd[n] * sin(arg);
        }
        S.Uin[j + Nl * k] = u;
        S.Win[j + Nl * k] = w;
        S.Vin[j + Nl * k] = 0.0;
      }
    } else if (S.lef == 14) {   // LEF_SPC: directional components (src/waves.F:473-511)
      const int nc = S.njon;
      const double *Wh = S.jon, *sg = S.jon + nc, *wk = S.jon + 2 * nc, *sd = S.jon + 3 * nc;
      const double *ph = S.jon + 4 * nc, *shd = S.jon + 5 * nc, *sth = S.jon + 6 * nc, *cth = S.jon + 7 * nc;
      double E = 0.0;
      for (int n = 0; n < nc; ++n) {
        const double lag = S.yc[j] * sth[n] * wk[n] + ph[n];
        E = E + 0.5 * Wh[n] * cos(kPi / 2 - sg[n] * TIME + lag);
      }
      E = E * tanh(TIME / 20.0);
      const double Dn = E + hfx;
      S.Ein[j] = E;
      S.Din[j] = Dn;
      if (!inner) return;
      for (int k = S.KB; k <= S.KE; ++k) {
        const double Zlev = S.sigc[k] * Dn;
        double u = 0.0, v = 0.0, w = 0.0;
        for (int n = 0; n < nc; ++n) {
          const double arg = kPi / 2 - sg[n] * TIME + (S.yc[j] * sth[n] * wk[n] + ph[n]);
          const double a = 0.5 * Wh[n] * sg[n] * cosh(wk[n] * Zlev) / shd[n] * cos(arg) - sd[n] * 1.0;
          u = u + a * cth[n];
          w = w + 0.5 * Wh[n] * sg[n] * sinh(wk[n] * Zlev) / shd[n] * sin(arg);
          v = v + a * sth[n];
        }
        S.Uin[j + Nl * k] = u;
        S.Win[j + Nl * k] = w;
        S.Vin[j + Nl * k] = v;
      }
    } else if (S.lef == 6) {   // LEF_CON: cnoidal wave
      const double A = S.lef_amp, Dep = S.lef_dep, m = S.con_mod, ck = S.con_ck, L = S.con_len, Yt = S.con_ytr;
      const double Xcn = cnoidal_cn(S.con_x0 + 2.0 * ck * (-(TIME / S.lef_per)), m);
      const double cn2 = Xcn * Xcn;
      const double E = Yt + A * cn2;
      const double Dn = E + hfx;
      S.Ein[j] = E;
      S.Din[j] = Dn;
      if (!inner) return;
      const double Xsn = sqrt(1.0 - cn2), Xdn = sqrt(1.0 - m * (1.0 - cn2));
      const double sn2 = Xsn * Xsn, dn2 = Xdn * Xdn, DY = Dep + Yt;
      const double c0 = sqrt(kGrav * Dep);
      for (int k = S.KB; k <= S.KE; ++k) {
        const double Zlev = S.sigc[k] * Dn;
        const double Z2 = Zlev * Zlev;
        S.Uin[j + Nl * k] =
            c0 * (-5. / 4. + 3. * DY / 2.0 / Dep - (DY * DY) / 4. / (Dep * Dep) +
                  (3. * A / 2. / Dep - DY * A / 2. / (Dep * Dep)) * cn2 - (A * A) / 4. / (Dep * Dep) * (cn2 * cn2) -
                  8.0 * A * (ck * ck) / (L * L) * (Dep / 3 - Z2 / 2 / Dep) *
                      (-((m * m) * sn2 * cn2) + cn2 * dn2 - sn2 * dn2)) -
            S.lef_stokes * 1.0;
        S.Win[j + Nl * k] = c0 * Zlev * 2 * A * ck / L / Dep *
                            (1 + DY / Dep + A / Dep * cn2 +
                             32 * (ck * ck) / 3 / (L * L) * ((Dep * Dep) - Z2 / 2) *
                                 ((m * m) * sn2 - (m * m) * cn2 - dn2)) *
                            Xsn * Xcn * Xdn;
        S.Vin[j + Nl * k] = 0.0;
      }
    }
  }
};

// linear_wave_right_boundary (src/waves.F:762-803): the LEF_LIN wave given to
// the east side (BC_Xn = 3) at the step's new TIME, with the reference's
// phase and sign convention; one thread per row j
struct OpWaveBCEast {
  static constexpr const char* kName = "wave_bc_east";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int, int j, int) const {
    const double TIME = S.sc->time;
    const double hfx = S.Hfx[i2(S, S.IE + 1, j)];
    const int Nl = S.Nloc;
    const double A = S.lef_amp;
    const double phs = S.yc[j] * S.lef_sinth * S.lef_wn;
    const double arg = kPi / 2 - S.lef_segma * TIME + phs;
    const double cs = cos(arg), sn = sin(arg);
    const double E = 0.5 * A * cs;
    const double Dn = E + hfx;
    S.Ein_xn[j] = E;
    S.Din_xn[j] = Dn;
    if (j < S.JB || j > S.JE) return;
    for (int k = S.KB; k <= S.KE; ++k) {
      const double Zlev = S.sigc[k] * Dn;
      const double ch = cosh(S.lef_wn * Zlev), sh = sinh(S.lef_wn * Zlev);
      const double u = 0.5 * A * S.lef_segma * ch / S.lef_shd * cs - S.lef_stokes * 1.0;
      S.Uin_xn[j + Nl * k] = u * S.lef_costh;
      S.Win_xn[j + Nl * k] = 0.5 * A * S.lef_segma * sh / S.lef_shd * sn;
      S.Vin_xn[j + Nl * k] = u * S.lef_sinth;
    }
  }
};

// flux_left_right_boundary (src/nhwave.F:5566-5712; its sediment and
// salinity parts are outside this path), one block: the logarithmic current
// of depth-mean 0.115 m/s into the west side at eta = 0, ramped up by
// tanh(TIME/TRamp), and its volume flux FluxL, summed by one thread in the
// reference's loop order (k outer, j inner); then the east side's eta, V and
// W radiated from the last two steps and its U mixed with the outflow
// velocity FluxL/(Din_Xn dy Nglob) of this step and of the previous one.
template <class T>
__global__ void __launch_bounds__(256) k_flux_lr(Dev<T> S) {
  if (gated_off(S)) return;
  __shared__ double s_flux;
  const double TIME = S.sc->time;
  const double Ramp = S.tramp > 0.0 ? tanh(TIME / S.tramp) : 1.0;
  const int Nl = S.Nloc, nj = S.JE - S.JB + 1, nk = S.KE - S.KB + 1;
  for (int j = threadIdx.x; j < Nl; j += blockDim.x) {
    S.Ein[j] = 0.0;
    S.Din[j] = S.Ein[j] + S.Hfx[i2(S, S.IB, j)];
  }
  __syncthreads();
  const double Ufric = (double)0.115f * kKappa / (log(30. * S.Din[S.JB] / S.zob));
  for (int t = threadIdx.x; t < nj * nk; t += blockDim.x) {
    const int j = S.JB + t % nj, k = S.KB + t / nj;
    const double Zlev1 = S.sigc[k] * S.Din[j];
    S.Uin[j + Nl * k] = Ufric / kKappa * log(30. * Zlev1 / S.zob) * Ramp;
    S.Win[j + Nl * k] = 0.0;
    S.Vin[j + Nl * k] = 0.0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double FluxL = 0.0;
    for (int k = S.KB; k <= S.KE; ++k)
      for (int j = S.JB; j <= S.JE; ++j) FluxL = FluxL + S.dsig[k] * S.Din[j] * S.dy * S.Uin[j + Nl * k];
    s_flux = FluxL;
  }
  auto cg = [](double a, double b, double c) {
    const double Cg = -(a - b + kOrlSmall) / (b - c + kOrlSmall);
    return dmax_(dmin_(Cg, 1.0), 0.0);
  };
  for (int j = threadIdx.x; j < Nl; j += blockDim.x) {
    const long long e = i2(S, S.IE, j), w = i2(S, S.IE - 1, j), g = i2(S, S.IE + 1, j);
    const double Cg = cg(S.Eta0[e], S.Eta00[e], S.Eta00[w]);
    S.Ein_xn[j] = (Cg * S.Eta0[e] + (1.0 - Cg) * S.Eta0[g] + S.Eta[e]) / 2.0;
    S.Din_xn[j] = S.Hfx[g] + S.Ein_xn[j];
  }
  __syncthreads();
  const double FluxL = s_flux;
  for (int t = threadIdx.x; t < Nl * S.Kloc; t += blockDim.x) {
    const int j = t % Nl, k = t / Nl;
    const double prev = S.Uxni[t];
    S.Uxni0[t] = prev;
    if (j < S.JB || j > S.JE || k < S.KB || k > S.KE) continue;
    const double ni = FluxL / (S.Din_xn[j] * S.dy * (double)(float)S.N);
    S.Uxni[t] = ni;
    const long long e = i3(S, S.IE, j, k), w = i3(S, S.IE - 1, j, k), g = i3(S, S.IE + 1, j, k);
    double Cg = cg((double)S.U0[e], (double)S.U00[e], (double)S.U00[w]);
    const double ue = (double)S.U[e];
    S.Uin_xn[t] = (Cg * ue + prev - Cg * ni + ue) / 2.0;
    Cg = cg((double)S.V0[e], (double)S.V00[e], (double)S.V00[w]);
    S.Vin_xn[t] = (Cg * (double)S.V0[e] + (1.0 - Cg) * (double)S.V0[g] + (double)S.V[e]) / 2.0;
    Cg = cg((double)S.W0[e], (double)S.W00[e], (double)S.W00[w]);
    S.Win_xn[t] = (Cg * (double)S.W0[e] + (1.0 - Cg) * (double)S.W0[g] + (double)S.W[e]) / 2.0;
  }
}

// =========================================================================
//   2-D face states shared by flux_x/y and omega_x/y
// =========================================================================
// State of the face between cells q0 and q1 = q0 + step (x faces: step 1, y
// faces: sy): eta and D reconstructed from the eta slopes (hd = dx/2 or dy/2),
// the face bed height h0 (Hfx0 / Hfy0), with the wet/dry front fix of
// src/nhwave.F:1745-1788.  inL / inR: cell q0 / q1 is an interior cell of its
// row (x) or column (y).
struct Face2D {
  double etaL, etaR, dL, dR, h0;
  bool wrote_h0;   // the fix replaced h0 by a cell's Hc
  bool zl, zr;     // the fix zeroes the 3-D states on the left / right side
};
template <class T>
__device__ __forceinline__ void face_flags(const Dev<T>& S, long long q0, long long step, bool inL, bool inR,
                                           bool& zl, bool& zr) {
  const long long q1 = q0 + step;
  const int mL = S.Mask[q0], mR = S.Mask[q1];
  zl = inL && ((mL == 1 && mR == 0) || mL == 0);
  zr = false;
  if (inR) {
    const int mRR = S.Mask[q1 + step];
    zr = !(mR == 1 && mRR == 0) && ((mR == 1 && mL == 0) || mR == 0);
  }
}
template <class T>
__device__ __forceinline__ Face2D face_2d(const Dev<T>& S, long long q0, long long step, bool inL, bool inR,
                                          double hd, const double* Delt, const double* Hf, const double* Hf0) {
  const long long q1 = q0 + step;
  const int mL = S.Mask[q0], mR = S.Mask[q1];
  Face2D F;
  F.etaL = S.Eta[q0] + hd * Delt[q0];
  F.etaR = S.Eta[q1] - hd * Delt[q1];
  const double hf = Hf[q1];
  F.dL = dmax_(F.etaL + hf, S.min_dep);
  F.dR = dmax_(F.etaR + hf, S.min_dep);
  F.h0 = Hf0[q1];
  F.wrote_h0 = F.zl = F.zr = false;
  if (inL) {
    if (mL == 1 && mR == 0) {
      F.etaL = S.Eta[q0]; F.dL = S.D[q0]; F.h0 = S.Hc[q0]; F.wrote_h0 = true; F.zl = true;
    } else if (mL == 0) {
      F.etaL = S.Eta[q0]; F.dL = S.D[q0]; F.zl = true;
    }
  }
  if (inR) {
    const int mRR = S.Mask[q1 + step];
    if (mR == 1 && mRR == 0) {
    } else if (mR == 1 && mL == 0) {
      F.etaR = S.Eta[q1]; F.dR = S.D[q1]; F.h0 = S.Hc[q1]; F.wrote_h0 = true; F.zr = true;
    } else if (mR == 0) {
      F.etaR = S.Eta[q1]; F.dR = S.D[q1]; F.zr = true;
    }
  }
  return F;
}
// The FP32+IR form with HLL reads the 2-D face states from Dev::fxT / fyT,
// formed once per face by OpFacePrep, instead of forming them in FP64 on
// every level of the face (the FP64 pipe runs at 1/58 of the FP32 rate).
template <class R, class T>
__device__ __forceinline__ bool face_table(const Dev<T>& S) {
  if constexpr (sizeof(R) == 4) return S.fxT != nullptr && !S.hllc;
  else return false;
}
// elements of one slot of fxT / fyT: the size of a 2-D field, sy * (Nloc + 1)
template <class T>
__device__ __forceinline__ long long face_slot(const Dev<T>& S) { return (long long)S.sy * (S.Nloc + 1); }
// table slots: eta, D on each side and h0 rounded to T, then (T)(dR - dL)
struct FaceT {
  template <class T>
  __device__ __forceinline__ static void put(T* tab, long long q1, long long n2, const Face2D& F) {
    tab[q1] = (T)F.etaL; tab[n2 + q1] = (T)F.etaR; tab[2 * n2 + q1] = (T)F.dL; tab[3 * n2 + q1] = (T)F.dR;
    tab[4 * n2 + q1] = (T)F.h0; tab[5 * n2 + q1] = (T)(F.dR - F.dL);
  }
};
// one x face (f, j) and one y face (i, g) per thread over (M+1) x (N+1): the
// face states at the start of a stage (flux; writes Hfx0/Hfy0 where the fix
// replaced h0) or after it (omega; writes EtaxL/R, EtayL/R for source_terms)
struct OpFacePrep {
  static constexpr const char* kName = "face_prep";
  int omega;
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j, int) const {
    const long long n2 = face_slot(S);
    if (j <= S.JE) {   // x face f = i between cells i-1 and i
      const long long q0 = i2(S, i - 1, j);
      const Face2D F = face_2d(S, q0, 1, i - 1 >= S.IB && i - 1 <= S.IE, i >= S.IB && i <= S.IE, 0.5 * S.dx,
                               S.DelxEta, S.Hfx, S.Hfx0);
      if (omega) { S.EtaxL[q0 + 1] = F.etaL; S.EtaxR[q0 + 1] = F.etaR; }
      else if (F.wrote_h0) S.Hfx0[q0 + 1] = F.h0;
      FaceT::put(S.fxT, q0 + 1, n2, F);
    }
    if (i <= S.IE) {   // y face g = j between cells j-1 and j
      const long long q0 = i2(S, i, j - 1);
      const Face2D F = face_2d(S, q0, S.sy, j - 1 >= S.JB && j - 1 <= S.JE, j >= S.JB && j <= S.JE, 0.5 * S.dy,
                               S.DelyEta, S.Hfy, S.Hfy0);
      if (omega) { S.EtayL[q0 + S.sy] = F.etaL; S.EtayR[q0 + S.sy] = F.etaR; }
      else if (F.wrote_h0) S.Hfy0[q0 + S.sy] = F.h0;
      FaceT::put(S.fyT, q0 + S.sy, n2, F);
    }
  }
};

// =========================================================================
//                        2-D slopes of eta (delx/yFun_2D)
// =========================================================================
struct OpSlopeEta {
  static constexpr const char* kName = "slope_eta";
  // eval_duvw's call (snap = true) is followed by sigma_transform, whose
  // inputs the viscous flow keeps; the call at the start of fluxes is not
  bool snap = false;
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j) const {
    const double* E = S.Eta;
    const long long c = i2(S, i, j);
    const double rdx = 2.0 * S.i2dx, rdy = 2.0 * S.i2dy;   // 1/dx, 1/dy (FP32 form: products)
    double sx, sy;
    if (i == 0) sx = (E[c + 1] - E[c]) / S.dx;
    else if (i == S.Mloc - 1) sx = (E[c] - E[c - 1]) / S.dx;
    else if (S.Mask[c] == 0) sx = 0.0;
    else if constexpr (sizeof(T) == 4) sx = lim_slope_r<double>(E[c - 1], E[c], E[c + 1], rdx, rdx);
    else sx = lim_slope<double>(E[c - 1], E[c], E[c + 1], S.dx, S.dx);
    if (j == 0) sy = (E[c + S.sy] - E[c]) / S.dy;
    else if (j == S.Nloc - 1) sy = (E[c] - E[c - S.sy]) / S.dy;
    else if (S.Mask[c] == 0) sy = 0.0;
    else if constexpr (sizeof(T) == 4) sy = lim_slope_r<double>(E[c - S.sy], E[c], E[c + S.sy], rdy, rdy);
    else sy = lim_slope<double>(E[c - S.sy], E[c], E[c + S.sy], S.dy, S.dy);
    S.DelxEta[c] = sx;
    S.DelyEta[c] = sy;
    if (snap && S.scD) {   // viscous flow: sigma_transform's inputs, kept for the next stage's diffusion
      S.scD[c] = S.D[c];
      S.scEx[c] = sx;
      S.scEy[c] = sy;
      S.scHx[c] = S.DelxH[c];
      S.scHy[c] = S.DelyH[c];
      if (c == 0) S.sc->sig_set = 1;
    }
  }
};

// =========================================================================
//              source_terms (src/source_terms.F:30-67, 418-455)
// =========================================================================
struct OpSourceArea {
  static constexpr const char* kName = "source_area";  // one thread: Source_Area = sum over i of dx*D(i,Jbeg+1), in order
  template <class T>
  __device__ void operator()(const Dev<T>& S, int, int) const {
    double a = 0.0;
    const int jrow = S.JB + 1;
    for (int i = S.wm_i0; i <= S.wm_i1; ++i) a = a + S.dx * S.D[i2(S, i, jrow)];
    S.sc->source_area = a;
  }
};
struct OpSource {
  static constexpr const char* kName = "source_terms";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j) const {
    const long long c = i2(S, i, j);
    const double time = S.sc->time;
    const int wm = S.wavemaker;
    const bool internal = wm == NHW_WM_INT_LIN || wm == NHW_WM_INT_SOL || wm == NHW_WM_INT_CON ||
                          wm == NHW_WM_INT_JON || wm == NHW_WM_INT_TMA || wm == NHW_WM_INT_SPC ||
                          wm == NHW_WM_INT_IRR;
    if (internal && S.xc[i] >= S.wm_xw && S.xc[i] <= S.wm_xe && S.yc[j] >= S.wm_ys && S.yc[j] <= S.wm_yn) {
      const double area = S.sc->source_area;
      if (wm == NHW_WM_INT_LIN) {
        const double phs = S.yc[j] * S.wm_wnumy;
        S.SourceC[c] = S.wm_celerity * S.wm_amp / area * cos(kPi / 2 - S.wm_segma * time + phs);
      } else if (wm == NHW_WM_INT_SOL) {
        const double ch = cosh(S.wm_atmp * (S.wm_xstart - S.wm_celerity * time));
        S.SourceC[c] = 2.0 * S.wm_celerity / area * S.wm_amp / (ch * ch);
      } else if (wm == NHW_WM_INT_CON) {   // src/source_terms.F:386-395
        const double Xcn = cnoidal_cn(S.con_x0 + 2.0 * S.con_ck * (-(time / S.lef_per)), S.con_mod);
        S.SourceC[c] = 2.0 * S.wm_celerity / area * (S.con_ytr + S.wm_amp * (Xcn * Xcn));
      } else {
        // INT_JON / INT_TMA / INT_SPC / INT_IRR: the components' sum, in the
        // reference's order (frequency outer, direction inner;
        // src/source_terms.F:84-191, 207-300, 321-338); INT_IRR's eta_mean
        // is never read by the reference, so 0
        const int n = S.njon;
        const double* t = S.jon;
        const bool jon = wm == NHW_WM_INT_JON || wm == NHW_WM_INT_TMA;
        const double lag = S.dy / 2.0 + S.yc[j];
        double acc = 0.0;
        for (int q = 0; q < n; ++q) {
          const double segma = t[kIntSegma * n + q], ph = t[kJonPhase * n + q];
          const double arg = jon ? kPi / 2 - segma * time + ph
                                 : kPi / 2 - segma * time + lag * t[kIntWnumY * n + q] + ph;
          if (t[kIntKind * n + q] != 0.0)
            acc = acc + t[kIntPre * n + q] / area * (t[kIntHalfAmp * n + q] * cos(arg) + 0.0);
          else
            acc = acc + t[kIntPre * n + q] / area * cos(arg);
        }
        S.SourceC[c] = acc;
      }
    }
    const double m = (double)S.Mask[c];
    S.SourceX[c] = kGrav * 0.5 * (S.EtaxL[c + 1] + S.EtaxR[c]) * (S.Hfx0[c + 1] - S.Hfx0[c]) / S.dx * m;
    S.SourceY[c] = kGrav * 0.5 * (S.EtayL[c + S.sy] + S.EtayR[c]) * (S.Hfy0[c + S.sy] - S.Hfy0[c]) / S.dy * m;
  }
};

// =========================================================================
//    fluxes: delxyzFun + construction + wave_speed + HLL + flux_bc
//    (src/nhwave.F:1686-2351, 2354-2552, 2673-2738, 2813-2886)
// =========================================================================
// x faces: face f between cells f-1 and f, row j, level k (all interior)
struct OpFluxX {
  static constexpr const char* kName = "flux_x";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int f, int j, int k) const {
    using R = T;
    const int c0 = f - 1, c1 = f;
    const long long e0 = i3(S, c0, j, k), e1 = e0 + 1;
    const long long q0 = i2(S, c0, j), q1 = q0 + 1;
    const int mL = S.Mask[q0], mR = S.Mask[q1];
    const R hdx = S.hdxT, rdx = S.dxT, irdx = S.idxT;
    // limited x slopes of the two cells (zero in dry cells)
    auto sl = [&](const T* A, long long e, int m) -> R {
      return m == 0 ? (R)0 : lim_slope_u<R>(A[e - 1], A[e], A[e + 1], rdx, irdx);
    };
    R uL = S.U[e0] + hdx * sl(S.U, e0, mL), uR = S.U[e1] - hdx * sl(S.U, e1, mR);
    R vL = S.V[e0] + hdx * sl(S.V, e0, mL), vR = S.V[e1] - hdx * sl(S.V, e1, mR);
    R wL = S.W[e0] + hdx * sl(S.W, e0, mL), wR = S.W[e1] - hdx * sl(S.W, e1, mR);
    R duL = S.DU[e0] + hdx * sl(S.DU, e0, mL), duR = S.DU[e1] - hdx * sl(S.DU, e1, mR);
    R dvL = S.DV[e0] + hdx * sl(S.DV, e0, mL), dvR = S.DV[e1] - hdx * sl(S.DV, e1, mR);
    R dwL = S.DW[e0] + hdx * sl(S.DW, e0, mL), dwR = S.DW[e1] - hdx * sl(S.DW, e1, mR);
    // 2-D face state with the wet/dry front fix (src/nhwave.F:1745-1788)
    R reL, reR, rh0, rdL, rdR, rdd;
    double dL = 0.0, dR = 0.0, h0;   // FP64 face depths (HLLC) and bed height
    bool zl, zr;
    const bool inL = c0 >= S.IB && c0 <= S.IE, inR = c1 >= S.IB && c1 <= S.IE;
    if (face_table<R>(S)) {
      const long long n2 = face_slot(S);
      const T* ft = S.fxT + q1;
      reL = ft[0]; reR = ft[n2]; rdL = ft[2 * n2]; rdR = ft[3 * n2]; rh0 = ft[4 * n2]; rdd = ft[5 * n2];
      h0 = (double)rh0;
      face_flags(S, q0, 1, inL, inR, zl, zr);
    } else {
      const Face2D F = face_2d(S, q0, 1, inL, inR, 0.5 * S.dx, S.DelxEta, S.Hfx, S.Hfx0);
      if (F.wrote_h0 && k == S.KB) S.Hfx0[q1] = F.h0;
      dL = F.dL; dR = F.dR; h0 = F.h0; zl = F.zl; zr = F.zr;
      reL = (R)F.etaL; reR = (R)F.etaR; rh0 = (R)F.h0; rdL = (R)F.dL; rdR = (R)F.dR; rdd = (R)(F.dR - F.dL);
    }
    if (zl) uL = vL = wL = duL = dvL = dwL = (R)0;
    if (zr) uR = vR = wR = duR = dvR = dwR = (R)0;
    // physical fluxes at the faces
    const R FxL = duL * uL + hydro<R>(reL, rh0), FxR = duR * uR + hydro<R>(reR, rh0);
    const R GxL = rdL * uL * vL, GxR = rdR * uR * vR;
    const R HxL = rdL * uL * wL, HxR = rdR * uR * wR;
    // wave speeds (src/nhwave.F:2813-2849)
    R SL = (R)0, SR = (R)0, SS = (R)0;
    if (mL == 1 && mR == 1) {
      R pL = sqrt((R)kGrav * fabs(rdL)), pR = sqrt((R)kGrav * fabs(rdR));
      R pS = (R)0.5 * (pL + pR) + (R)0.25 * (uL - uR);
      R uS = (R)0.5 * (uL + uR) + pL - pR;
      SL = rmin<R>(uL - pL, uS - pS);
      SR = rmax<R>(uR + pR, uS + pS);
      SS = uS;
      if constexpr (sizeof(R) == 4) {
        if (S.hllc) SS = contact_speed_f32(uL, uR, pL, pR, dL, dR);
      }
    } else if (mL == 0 && mR == 1) {
      R pR = sqrt((R)kGrav * fabs(rdR));
      SL = uR - (R)2.0 * pR;
      SR = uR + pR;
      SS = SL;
    } else if (mL == 1 && mR == 0) {
      R pL = sqrt((R)kGrav * fabs(rdL));
      SL = uL - pL;
      SR = uL + (R)2.0 * pL;
      SS = SR;
    }
    R Ex, Fx, Gx, Hx;
    if (S.hllc) {   // HLLC (src/nhwave.F:2555-2670); the mass-flux star state in FP64
      const double sl = SL, sr = SR, ss = SS;
      const double ls = dL * (sl - (double)uL + kSmall) / (sl - ss + kSmall);
      const double rs = dR * (sr - (double)uR + kSmall) / (sr - ss + kSmall);
      Ex = (R)hllc<double>(sl, sr, ss, (double)duL, (double)duR, dL, ls, dR, rs);
      const R lsR = (R)ls, rsR = (R)rs;
      Fx = hllc<R>(SL, SR, SS, FxL, FxR, duL, lsR * SS, duR, rsR * SS);
      Gx = hllc<R>(SL, SR, SS, GxL, GxR, dvL, lsR * vL, dvR, rsR * vR);
      Hx = hllc<R>(SL, SR, SS, HxL, HxR, dwL, lsR * wL, dwR, rsR * wR);
    } else {
      Ex = hll_d<R>(SL, SR, duL, duR, rdd);
      Fx = hll<R>(SL, SR, FxL, FxR, duL, duR);
      Gx = hll<R>(SL, SR, GxL, GxR, dvL, dvR);
      Hx = hll<R>(SL, SR, HxL, HxR, dwL, dwR);
    }
    // flux_bc: walls, then dry cells (src/nhwave.F:2366-2434, 2508-2549)
    if (f == S.IB) {
      if (S.bc_x0 == 3) {   // inflow (src/nhwave.F:2381-2387)
        const double dn = S.Din[j], un = S.Uin[j + S.Nloc * k];
        const double vn = S.Vin[j + S.Nloc * k], wn = S.Win[j + S.Nloc * k], en = S.Ein[j];
        Ex = (R)(dn * un);
        Fx = (R)(dn * un * un + 0.5 * kGrav * (en * en + 2.0 * en * h0));
        Gx = (R)(dn * un * vn);
        Hx = (R)(dn * un * wn);
      } else {
        Ex = (R)0; Fx = hydro<R>(reR, rh0); Gx = (R)0; Hx = (R)0;
      }
    }
    // east wall; an open (Orlanski) east face keeps its Riemann fluxes
    if (f == S.IE + 1 && S.bc_xn == 3) {   // inflow/outflow (src/nhwave.F:2411-2416)
      const double dn = S.Din_xn[j], un = S.Uin_xn[j + S.Nloc * k];
      const double vn = S.Vin_xn[j + S.Nloc * k], wn = S.Win_xn[j + S.Nloc * k], en = S.Ein_xn[j];
      Ex = (R)(dn * un);
      Fx = (R)(dn * un * un + 0.5 * kGrav * (en * en + 2.0 * en * h0));
      Gx = (R)(dn * un * vn);
      Hx = (R)(dn * un * wn);
    } else if (f == S.IE + 1 && S.bc_xn != 6) {
      Ex = (R)0; Fx = hydro<R>(reL, rh0); Gx = (R)0; Hx = (R)0;
    }
    if (mR == 0) {
      Ex = (R)0; Gx = (R)0; Hx = (R)0;
      Fx = (f == S.IB) ? (R)0 : hydro<R>(reL, rh0) * (R)mL;
    } else if (mL == 0) {
      Ex = (R)0; Gx = (R)0; Hx = (R)0;
      Fx = (c0 == S.IE) ? (R)0 : hydro<R>(reR, rh0) * (R)mR;
    }
    const long long o = i3(S, f, j, k);
    S.Ex[o] = Ex; S.Fx[o] = Fx; S.Gx[o] = Gx; S.Hx[o] = Hx;
  }
};

// y faces: face g between cells g-1 and g in column i
struct OpFluxY {
  static constexpr const char* kName = "flux_y";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int g, int k) const {
    using R = T;
    const int c0 = g - 1, c1 = g;
    const long long sy = S.sy;
    const long long e0 = i3(S, i, c0, k), e1 = e0 + sy;
    const long long q0 = i2(S, i, c0), q1 = q0 + sy;
    const int mL = S.Mask[q0], mR = S.Mask[q1];
    const R hdy = S.hdyT, rdy = S.dyT, irdy = S.idyT;
    auto sl = [&](const T* A, long long e, int m) -> R {
      return m == 0 ? (R)0 : lim_slope_u<R>(A[e - sy], A[e], A[e + sy], rdy, irdy);
    };
    R uL = S.U[e0] + hdy * sl(S.U, e0, mL), uR = S.U[e1] - hdy * sl(S.U, e1, mR);
    R vL = S.V[e0] + hdy * sl(S.V, e0, mL), vR = S.V[e1] - hdy * sl(S.V, e1, mR);
    R wL = S.W[e0] + hdy * sl(S.W, e0, mL), wR = S.W[e1] - hdy * sl(S.W, e1, mR);
    R duL = S.DU[e0] + hdy * sl(S.DU, e0, mL), duR = S.DU[e1] - hdy * sl(S.DU, e1, mR);
    R dvL = S.DV[e0] + hdy * sl(S.DV, e0, mL), dvR = S.DV[e1] - hdy * sl(S.DV, e1, mR);
    R dwL = S.DW[e0] + hdy * sl(S.DW, e0, mL), dwR = S.DW[e1] - hdy * sl(S.DW, e1, mR);
    R reL, reR, rh0, rdL, rdR, rdd;
    double dL = 0.0, dR = 0.0;   // FP64 face depths (HLLC)
    bool zl, zr;
    const bool inL = c0 >= S.JB && c0 <= S.JE, inR = c1 >= S.JB && c1 <= S.JE;
    if (face_table<R>(S)) {
      const long long n2 = face_slot(S);
      const T* ft = S.fyT + q1;
      reL = ft[0]; reR = ft[n2]; rdL = ft[2 * n2]; rdR = ft[3 * n2]; rh0 = ft[4 * n2]; rdd = ft[5 * n2];
      face_flags(S, q0, sy, inL, inR, zl, zr);
    } else {
      const Face2D F = face_2d(S, q0, sy, inL, inR, 0.5 * S.dy, S.DelyEta, S.Hfy, S.Hfy0);
      if (F.wrote_h0 && k == S.KB) S.Hfy0[q1] = F.h0;
      dL = F.dL; dR = F.dR; zl = F.zl; zr = F.zr;
      reL = (R)F.etaL; reR = (R)F.etaR; rh0 = (R)F.h0; rdL = (R)F.dL; rdR = (R)F.dR; rdd = (R)(F.dR - F.dL);
    }
    if (zl) uL = vL = wL = duL = dvL = dwL = (R)0;
    if (zr) uR = vR = wR = duR = dvR = dwR = (R)0;
    const R FyL = rdL * uL * vL, FyR = rdR * uR * vR;
    const R GyL = dvL * vL + hydro<R>(reL, rh0), GyR = dvR * vR + hydro<R>(reR, rh0);
    const R HyL = rdL * vL * wL, HyR = rdR * vR * wR;
    R SL = (R)0, SR = (R)0, SS = (R)0;
    if (mL == 1 && mR == 1) {
      R pL = sqrt((R)kGrav * fabs(rdL)), pR = sqrt((R)kGrav * fabs(rdR));
      R pS = (R)0.5 * (pL + pR) + (R)0.25 * (vL - vR);
      R uS = (R)0.5 * (vL + vR) + pL - pR;
      SL = rmin<R>(vL - pL, uS - pS);
      SR = rmax<R>(vR + pR, uS + pS);
      SS = uS;
      if constexpr (sizeof(R) == 4) {
        if (S.hllc) SS = contact_speed_f32(vL, vR, pL, pR, dL, dR);
      }
    } else if (mL == 0 && mR == 1) {
      R pR = sqrt((R)kGrav * fabs(rdR));
      SL = vR - (R)2.0 * pR;
      SR = vR + pR;
      SS = SL;
    } else if (mL == 1 && mR == 0) {
      R pL = sqrt((R)kGrav * fabs(rdL));
      SL = vL - pL;
      SR = vL + (R)2.0 * pL;
      SS = SR;
    }
    R Ey, Fy, Gy, Hy;
    if (S.hllc) {   // HLLC (src/nhwave.F:2555-2670); the mass-flux star state in FP64
      const double sl = SL, sr = SR, ss = SS;
      const double ls = dL * (sl - (double)vL + kSmall) / (sl - ss + kSmall);
      const double rs = dR * (sr - (double)vR + kSmall) / (sr - ss + kSmall);
      Ey = (R)hllc<double>(sl, sr, ss, (double)dvL, (double)dvR, dL, ls, dR, rs);
      const R lsR = (R)ls, rsR = (R)rs;
      Fy = hllc<R>(SL, SR, SS, FyL, FyR, duL, lsR * uL, duR, rsR * uR);
      Gy = hllc<R>(SL, SR, SS, GyL, GyR, dvL, lsR * SS, dvR, rsR * SS);
      Hy = hllc<R>(SL, SR, SS, HyL, HyR, dwL, lsR * wL, dwR, rsR * wR);
    } else {
      Ey = hll_d<R>(SL, SR, dvL, dvR, rdd);
      Fy = hll<R>(SL, SR, FyL, FyR, duL, duR);
      Gy = hll<R>(SL, SR, GyL, GyR, dvL, dvR);
      Hy = hll<R>(SL, SR, HyL, HyR, dwL, dwR);
    }
    if (g == S.JB) { Ey = (R)0; Fy = (R)0; Gy = hydro<R>(reR, rh0); Hy = (R)0; }
    if (g == S.JE + 1) { Ey = (R)0; Fy = (R)0; Gy = hydro<R>(reL, rh0); Hy = (R)0; }
    if (mR == 0) {
      Ey = (R)0; Fy = (R)0; Hy = (R)0;
      Gy = (g == S.JB) ? (R)0 : hydro<R>(reL, rh0) * (R)mL;
    } else if (mL == 0) {
      Ey = (R)0; Fy = (R)0; Hy = (R)0;
      Gy = (c0 == S.JE) ? (R)0 : hydro<R>(reR, rh0) * (R)mR;
    }
    const long long o = i3(S, i, g, k);
    S.Ey[o] = Ey; S.Fy[o] = Fy; S.Gy[o] = Gy; S.Hy[o] = Hy;
  }
};

// z faces k in [KB, KE+1] of an interior column (src/nhwave.F:1998-2023, 2719-2730)
struct OpFluxZ {
  static constexpr const char* kName = "flux_z";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j, int k) const {
    using R = T;
    const long long o = i3(S, i, j, k);
    if (k == S.KB || k == S.KE + 1) { S.Fz[o] = (R)0; S.Gz[o] = (R)0; S.Hz[o] = (R)0; return; }
    const long long sz = S.sz;
    const T* dsc = S.lvT + S.Kloc;       // sigc_k - sigc_k-1
    const T* hds = S.lvT + 2 * S.Kloc;   // dsig_k / 2
    const R dm = dsc[k - 1], d0 = dsc[k], dp = dsc[k + 1];
    const R hm = hds[k - 1], h0 = hds[k];
    auto face = [&](const T* A, R& L, R& Rr) {
      const R am = A[o - 2 * sz], a0 = A[o - sz], a1 = A[o], a2 = A[o + sz];
      L = a0 + hm * lim_slope<R>(am, a0, a1, dm, d0);
      Rr = a1 - h0 * lim_slope<R>(a0, a1, a2, d0, dp);
    };
    R uL, uR, vL, vR, wL, wR;
    face(S.U, uL, uR); face(S.V, vL, vR); face(S.W, wL, wR);
    const R om = S.Omega[o], ao = fabs(om);
    S.Fz[o] = (R)0.5 * (om * (uL + uR) - ao * (uR - uL));
    S.Gz[o] = (R)0.5 * (om * (vL + vR) - ao * (vR - vL));
    S.Hz[o] = (R)0.5 * (om * (wL + wR) - ao * (wR - wL));
  }
};

// =========================================================================
//   eval_duvw, explicit part: R1, D, R2-R4, DU/DV/DW (src/nhwave.F:611-1182)
// =========================================================================
struct OpExplicit {
  static constexpr const char* kName = "stage_explicit";
  int istep;
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j) const {
    using R = T;
    const long long c = i2(S, i, j);
    const double dt = S.sc->dt;
    double r1 = 0.0;
    if (S.Mask[c] != 0) {
      for (int k = S.KB; k <= S.KE; ++k) {
        const long long o = i3(S, i, j, k);
        const double dEx = (double)S.Ex[o + 1] - (double)S.Ex[o];
        const double dEy = (double)S.Ey[o + S.sy] - (double)S.Ey[o];
        r1 = r1 - 1.0 / S.dx * dEx * S.dsig[k] - 1.0 / S.dy * dEy * S.dsig[k];
      }
      r1 = r1 + S.D[c] * S.SourceC[c];
      S.D[c] = S.alpha[istep] * S.D0[c] + S.beta[istep] * (S.D[c] + dt * r1);
      const R rdx = S.idxT, rdy = S.idyT, rdt = (R)dt, fc = (R)S.fcor;
      const R sx = (R)S.SourceX[c], syy = (R)S.SourceY[c];
      for (int k = S.KB; k <= S.KE; ++k) {
        const long long o = i3(S, i, j, k);
        const R rds = S.lvT[k];   // (R)(1.0 / dsig_k)
        const R du = S.DU[o], dv = S.DV[o], dw = S.DW[o];
        R R2 = -rdx * (S.Fx[o + 1] - S.Fx[o]) - rdy * (S.Fy[o + S.sy] - S.Fy[o]) -
               rds * (S.Fz[o + S.sz] - S.Fz[o]) + fc * dv + sx;
        R R3 = -rdx * (S.Gx[o + 1] - S.Gx[o]) - rdy * (S.Gy[o + S.sy] - S.Gy[o]) -
               rds * (S.Gz[o + S.sz] - S.Gz[o]) - fc * du + syy;
        R R4 = -rdx * (S.Hx[o + 1] - S.Hx[o]) - rdy * (S.Hy[o + S.sy] - S.Hy[o]) -
               rds * (S.Hz[o + S.sz] - S.Hz[o]);
        if (S.Dxx) {   // viscous terms of diffusion (src/nhwave.F:642-679)
          R2 = R2 + S.Dxx[o] + S.Dxy[o];
          R3 = R3 + S.Dyx[o] + S.Dyy[o];
          R4 = R4 + S.Dzx[o] + S.Dzy[o];
        }
        // viscous flow: DU + dt R2 is the right-hand side of OpVertVisc
        S.DU[o] = du + rdt * R2;
        S.DV[o] = dv + rdt * R3;
        S.DW[o] = dw + rdt * R4;
      }
    } else {
      for (int k = S.KB; k <= S.KE; ++k) {
        const long long o = i3(S, i, j, k);
        S.DU[o] = (R)0; S.DV[o] = (R)0; S.DW[o] = (R)0;
      }
    }
    S.R1[c] = r1;
    S.D[c] = dmax_(S.D[c], S.min_dep);
  }
};

// D ghosts (wl_bc, walls) and Eta = D - Hc over the whole ghosted array
struct OpWlBcEta {
  static constexpr const char* kName = "wl_bc_eta";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j) const {
    const long long c = i2(S, i, j);
    const int mi = mirror(i, S.IB, S.IE), mj = mirror(j, S.JB, S.JE);
    if (i <= S.IB && S.bc_x0 == 3 && S.lef == 9)
      // tide (src/nhwave.F:5145-5148): D = Din in the ghosts and the first
      // interior column; ghost rows copy their mirrored row's value
      S.D[c] = S.Din[mj];
    else if (i < S.IB && S.bc_x0 == 3)   // inflow (src/nhwave.F:5148-5157); corners copy their row's value
      S.D[c] = 2.0 * S.Din[mj] - S.D[i2(S, mi, mj)];
    else if (i > S.IE && (S.bc_xn == 6 || S.bc_xn == 3)) {
      // Orlanski radiation (src/nhwave.F:5182-5206, the same for the open and
      // the inflow/outflow east side) from the last two steps' eta; corner
      // rows copy their mirrored row's value, as the y pass does
      const long long a = i2(S, i - 1, mj), b = i2(S, i - 2, mj), g = i2(S, i, mj);
      double Cg = -(S.Eta0[a] - S.Eta00[a] + kOrlSmall) / (S.Eta00[a] - S.Eta00[b] + kOrlSmall);
      Cg = dmax_(dmin_(Cg, 1.0), 0.0);
      const double eta = Cg * S.Eta0[a] + (1.0 - Cg) * S.Eta0[g];
      S.D[c] = S.Hc[g] + eta;
    } else if (mi != i || mj != j)
      S.D[c] = S.D[i2(S, mi, mj)];
    S.Eta[c] = S.D[c] - S.Hc[c];
  }
};

// =========================================================================
//              get_UVW + vel_bc (src/nhwave.F:1651-1683, 4416-5117)
// =========================================================================
struct OpGetUVW {
  static constexpr const char* kName = "get_uvw";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j, int k) const {
    const long long o = i3(S, i, j, k);
    const T d = (T)S.D[i2(S, i, j)];
    S.U[o] = S.DU[o] / d;
    S.V[o] = S.DV[o] / d;
    S.W[o] = S.DW[o] / d;
  }
};

// vel_bc, part A: lateral ghosts (walls) and the surface/bed face states of
// every interior column after the kinematic conditions (KBC_surface/bottom).
struct OpVelBcA {
  static constexpr const char* kName = "vel_bc_a";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j) const {
    // interior columns: surface and bed face states (the lateral ghost cells
    // are filled per cell by OpVelBcLat)
    const long long c = i2(S, i, j);
    {
      const long long sz = S.sz;
      // arithmetic of the face states: FP64 in the FP64 form, FP32 in FP32+IR
      using R = typename std::conditional<sizeof(T) == 4, float, double>::type;
      auto zface = [&](const T* A, double& top, double& bot) {
        // top: UzL(Kend1) = U(Kend) + 0.5 dsig(Kend) DelzU(Kend)
        const int kt = S.KE, kb = S.KB;
        const long long ot = i3(S, i, j, kt), ob = i3(S, i, j, kb);
        R s_t = lim_slope<R>((R)A[ot - sz], (R)A[ot], (R)A[ot + sz], (R)(S.sigc[kt] - S.sigc[kt - 1]),
                             (R)(S.sigc[kt + 1] - S.sigc[kt]));
        R s_b = lim_slope<R>((R)A[ob - sz], (R)A[ob], (R)A[ob + sz], (R)(S.sigc[kb] - S.sigc[kb - 1]),
                             (R)(S.sigc[kb + 1] - S.sigc[kb]));
        top = (double)((R)A[ot] + (R)0.5 * (R)S.dsig[kt] * s_t);
        bot = (double)((R)A[ob] - (R)0.5 * (R)S.dsig[kb] * s_b);
      };
      double uL, uR, vL, vR, wL, wR;
      zface(S.U, uL, uR); zface(S.V, vL, vR); zface(S.W, wL, wR);
      const double dt = S.sc->dt;
      wL = (S.Eta[c] - S.Eta0[c]) / dt + S.DelxEta[c] * uL + S.DelyEta[c] * vL;
      wR = -S.DeltH[c] - S.DelxH[c] * uR - S.DelyH[c] * vR;
      S.zUL[c] = uL; S.zVL[c] = vL; S.zWL[c] = wL;
      S.zUR[c] = uR; S.zVR[c] = vR; S.zWR[c] = wR;
    }
  }
};
// lateral ghost cells of U, V, W, DU, DV, DW (src/nhwave.F:4416-4621): one
// thread per (ghost column or ghost row, level); corner columns stay untouched
// Wall friction factor of a BC = 5 side (src/nhwave.F:4486-4493): h the
// spacing across the wall, a and b the first interior cell's tangential
// velocities; Cmu + CmuHt of the cell e (CmuHt = 0 on the inviscid path)
template <class T>
__device__ __forceinline__ double wall_phi(const Dev<T>& S, double h, double a, double b, long long e) {
  double Cdrag = S.cd0;
  if (S.ibot != 1) {
    const double lg = 1. / kKappa * log(30.0 * h / 2.0 / S.zob);
    Cdrag = 1. / (lg * lg);
  }
  const double cmh = S.CmuHt ? (double)S.CmuHt[e] : 0.0;
  const double Phi = h * Cdrag * sqrt(a * a + b * b) / (S.v_cmu + cmh);
  return dmin_(Phi, 2.0);
}
struct OpVelBcLat {
  static constexpr const char* kName = "vel_bc_lat";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j, int k) const {
    const bool ii = (i >= S.IB && i <= S.IE), jj = (j >= S.JB && j <= S.JE);
    if (ii == jj) return;
    const long long o = i3(S, i, j, k);
    if (jj && i < S.IB && S.bc_x0 == 3) {  // inflow ghosts (src/nhwave.F:4468-4476)
      const int src = mirror(i, S.IB, S.IE);
      const long long q = i3(S, src, j, k);
      const double dn = S.Din[j];
      const double un = S.Uin[j + S.Nloc * k], vn = S.Vin[j + S.Nloc * k], wn = S.Win[j + S.Nloc * k];
      S.U[o] = (T)(2.0 * un - (double)S.U[q]);
      S.V[o] = (T)(2.0 * vn - (double)S.V[q]);
      S.W[o] = (T)(2.0 * wn - (double)S.W[q]);
      S.DU[o] = (T)(2.0 * dn * un - (double)S.DU[q]);
      S.DV[o] = (T)(2.0 * dn * vn - (double)S.DV[q]);
      S.DW[o] = (T)(2.0 * dn * wn - (double)S.DW[q]);
    } else if (jj && i > S.IE && S.bc_xn == 3) {  // inflow/outflow (src/nhwave.F:4547-4572)
      // U(Iend+1) = Cg U(Iend) + Uin_Xni0 - Cg Uin_Xni and U(Iend+2) = Cg U(Iend+1)
      // + (1 - Cg) U(Iend+2), U(Iend+2) as it was before this call: the second
      // ghost's thread forms the first ghost's new value itself
      auto cgf = [&](const T* X0, const T* X00, int ii) -> double {
        const long long a = i3(S, ii - 1, j, k), b = i3(S, ii - 2, j, k);
        const double Cg = -((double)X0[a] - (double)X00[a] + kOrlSmall) / ((double)X00[a] - (double)X00[b] + kOrlSmall);
        return dmax_(dmin_(Cg, 1.0), 0.0);
      };
      const int jk = j + S.Nloc * k;
      const double c1 = cgf(S.U0, S.U00, S.IE + 1);
      double u = c1 * (double)S.U[i3(S, S.IE, j, k)] + S.Uxni0[jk] - c1 * S.Uxni[jk];
      if (i == S.IE + 2) {
        const T u1 = (T)u;
        const double c2 = cgf(S.U0, S.U00, i);
        u = c2 * (double)u1 + (1.0 - c2) * (double)S.U[o];
      }
      const long long a = i3(S, i - 1, j, k);
      double Cg = cgf(S.V0, S.V00, i);
      const double v = Cg * (double)S.V0[a] + (1.0 - Cg) * (double)S.V0[o];
      Cg = cgf(S.W0, S.W00, i);
      const double w = Cg * (double)S.W0[a] + (1.0 - Cg) * (double)S.W0[o];
      const long long q = i3(S, mirror(i, S.IB, S.IE), j, k);
      const double dn = S.Din_xn[j];
      const double un = S.Uin_xn[jk], vn = S.Vin_xn[jk], wn = S.Win_xn[jk];
      S.U[o] = (T)u; S.V[o] = (T)v; S.W[o] = (T)w;
      S.DU[o] = (T)(2.0 * dn * un - (double)S.DU[q]);
      S.DV[o] = (T)(2.0 * dn * vn - (double)S.DV[q]);
      S.DW[o] = (T)(2.0 * dn * wn - (double)S.DW[q]);
    } else if (jj && i > S.IE && S.bc_xn == 6) {  // Orlanski radiation (src/nhwave.F:4599-4621)
      const long long a = i3(S, i - 1, j, k), b = i3(S, i - 2, j, k);
      auto orl = [&](const T* X0, const T* X00) -> double {
        double Cg = -((double)X0[a] - (double)X00[a] + kOrlSmall) / ((double)X00[a] - (double)X00[b] + kOrlSmall);
        Cg = dmax_(dmin_(Cg, 1.0), 0.0);
        return Cg * (double)X0[a] + (1.0 - Cg) * (double)X0[o];
      };
      const T u = (T)orl(S.U0, S.U00), v = (T)orl(S.V0, S.V00), w = (T)orl(S.W0, S.W00);
      const double d = S.D[i2(S, i, j)];
      S.U[o] = u; S.V[o] = v; S.W[o] = w;
      S.DU[o] = (T)(d * (double)u); S.DV[o] = (T)(d * (double)v); S.DW[o] = (T)(d * (double)w);
    } else if (jj && (i < S.IB ? S.bc_x0 : S.bc_xn) == 5) {  // wall friction (src/nhwave.F:4486-4500, 4583-4598)
      const bool west = i < S.IB;
      const int g = west ? S.IB - i : i - S.IE;   // ghost offset 1, 2
      const long long q = i3(S, mirror(i, S.IB, S.IE), j, k), e = i3(S, west ? S.IB : S.IE, j, k);
      const double Phi = wall_phi(S, S.dx, (double)S.V[e], (double)S.W[e], e);
      const double d = S.D[i2(S, g - 1, j)];   // the reference's D(i,j) with i the ghost offset
      const T u = -S.U[q], v = (T)((1.0 - Phi) * (double)S.V[q]), w = (T)((1.0 - Phi) * (double)S.W[q]);
      S.U[o] = u; S.V[o] = v; S.W[o] = w;
      S.DU[o] = (T)(d * (double)u); S.DV[o] = (T)(d * (double)v); S.DW[o] = (T)(d * (double)w);
    } else if (!jj && (j < S.JB ? S.bc_y0 : S.bc_yn) == 5) {  // wall friction (src/nhwave.F:4676-4691, 4737-4752)
      const bool south = j < S.JB;
      const int g = south ? S.JB - j : j - S.JE;
      const long long q = i3(S, i, mirror(j, S.JB, S.JE), k), e = i3(S, i, south ? S.JB : S.JE, k);
      const double Phi = wall_phi(S, S.dy, (double)S.U[e], (double)S.W[e], e);
      const double d = S.D[i2(S, i, g - 1)];   // D(i,j) with j the ghost offset
      const T u = (T)((1.0 - Phi) * (double)S.U[q]), v = -S.V[q], w = (T)((1.0 - Phi) * (double)S.W[q]);
      S.U[o] = u; S.V[o] = v; S.W[o] = w;
      S.DU[o] = (T)(d * (double)u); S.DV[o] = (T)(d * (double)v); S.DW[o] = (T)(d * (double)w);
    } else if (jj) {  // west/east ghost columns of interior rows
      const int src = mirror(i, S.IB, S.IE);
      const T s = (T)((i < S.IB ? S.bc_x0 : S.bc_xn) == 1 ? 1 : -1);
      const long long q = i3(S, src, j, k);
      S.U[o] = -S.U[q]; S.V[o] = s * S.V[q]; S.W[o] = s * S.W[q];
      S.DU[o] = -S.DU[q]; S.DV[o] = s * S.DV[q]; S.DW[o] = s * S.DW[q];
    } else {  // south/north ghost rows of interior columns
      const int src = mirror(j, S.JB, S.JE);
      const T s = (T)((j < S.JB ? S.bc_y0 : S.bc_yn) == 1 ? 1 : -1);
      const long long q = i3(S, i, src, k);
      S.U[o] = s * S.U[q]; S.V[o] = -S.V[q]; S.W[o] = s * S.W[q];
      S.DU[o] = s * S.DU[q]; S.DV[o] = -S.DV[q]; S.DW[o] = s * S.DW[q];
    }
  }
};
struct OpVelBcB {
  static constexpr const char* kName = "vel_bc_b";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j) const {
    const long long c = i2(S, i, j);
    auto zl = [&](const double* a, int x, int y) -> double {
      return (x >= S.IB && x <= S.IE && y >= S.JB && y <= S.JE) ? a[i2(S, x, y)] : 0.0;
    };
    const bool wet = S.Mask[c] != 0;
    // arithmetic of the surface stress ghosts: FP64 in the FP64 form, FP32 in FP32+IR
    using R = typename std::conditional<sizeof(T) == 4, float, double>::type;
    auto dx_ = [&](const double* a) -> R {
      return wet ? lim_slope<R>((R)zl(a, i - 1, j), (R)a[c], (R)zl(a, i + 1, j), S.dxT, S.dxT) : (R)0;
    };
    auto dy_ = [&](const double* a) -> R {
      return wet ? lim_slope<R>((R)zl(a, i, j - 1), (R)a[c], (R)zl(a, i, j + 1), S.dyT, S.dyT) : (R)0;
    };
    const R DelxUzL = dx_(S.zUL), DelxVzL = dx_(S.zVL), DelxWzL = dx_(S.zWL);
    const R DelyUzL = dy_(S.zUL), DelyVzL = dy_(S.zVL), DelyWzL = dy_(S.zWL);
    const R dxe = (R)S.DelxEta[c], dye = (R)S.DelyEta[c], Dij = (R)S.D[c];
    const R Atop = sqrt((R)1.0 + dxe * dxe + dye * dye);
    const R Fext_Wind1 = (R)1.0 / Atop * (((R)1 - dxe * dxe) * (R)S.Wsx[c] - dxe * dye * (R)S.Wsy[c]);
    const R Fext_Wind2 = (R)1.0 / Atop * (((R)1 - dye * dye) * (R)S.Wsy[c] - dxe * dye * (R)S.Wsx[c]);
    const R MinDepBC = (R)(double)0.01f;
    const R WzLt = (R)S.zWL[c], WzRb = (R)S.zWR[c], UzLt = (R)S.zUL[c], VzLt = (R)S.zVL[c];
    const int KB = S.KB, KE = S.KE;
    // Small + 0.5 (Cmu + CmuR + CmuVt) at the surface level and the one above;
    // Cmu + CmuR + CmuVt at the bed level (CmuR = 0; CmuVt = 0 inviscid)
    const double vtK = S.CmuVt ? (double)S.CmuVt[i3(S, i, j, KE)] : 0.0;
    const double vtK1 = S.CmuVt ? (double)S.CmuVt[i3(S, i, j, KE + 1)] : 0.0;
    const double vtB = S.CmuVt ? (double)S.CmuVt[i3(S, i, j, KB)] : 0.0;
    const R vtop = (R)(S.CmuVt ? kSmall + 0.5 * (S.v_cmu + 0.0 + vtK + S.v_cmu + 0.0 + vtK1) : S.visc_top);
    // bed stress (src/nhwave.F:4806-4847) for BC_Z0 = 2 (no slip) and 5 (friction)
    const R dxh = (R)S.DelxH[c], dyh = (R)S.DelyH[c];
    const R Abot = sqrt((R)1.0 + dxh * dxh + dyh * dyh), Bbot = sqrt((R)1.0 + dxh * dxh);
    const R nub = (R)(S.v_cmu + 0.0 + vtB);
    R Fext_Bot1 = (R)0, Fext_Bot2 = (R)0;
    R DelxUzR = (R)0, DelxVzR = (R)0, DelxWzR = (R)0, DelyUzR = (R)0, DelyVzR = (R)0, DelyWzR = (R)0;
    if (S.bc_z0 != 1) {
      DelxUzR = dx_(S.zUR); DelxVzR = dx_(S.zVR); DelxWzR = dx_(S.zWR);
      DelyUzR = dy_(S.zUR); DelyVzR = dy_(S.zVR); DelyWzR = dy_(S.zWR);
      const long long ok = i3(S, i, j, KB);
      const R du0 = (R)S.DU[ok], dv0 = (R)S.DV[ok], dw0 = (R)S.DW[ok];
      const R DUprime = (du0 - dxh * dw0) / Bbot;
      // "DU(i,j,Kbeg)* +(1.0+DelxH**2)*DV(i,j,Kbeg)" in the reference multiplies
      // the two terms, so on a flat bed DVprime is 0
      const R DVprime = (-(dxh * dyh * du0 * (((R)1.0 + dxh * dxh) * dv0)) - dyh * dw0) / Abot / Bbot;
      const R DUmag = sqrt(DUprime * DUprime + DVprime * DVprime);
      const R Dz1 = (R)0.5 * Dij * (R)S.dsig[KB] / Abot;
      R Cdrag = (R)S.cd0;
      if (S.ibot != 1) {
        const R lg = (R)kKappa / log(Dz1 / (R)(S.zob / 30.0));
        Cdrag = lg * lg;
      }
      Cdrag = rmin<R>(Cdrag, nub / Dz1 / (DUmag + (R)kSmall) * Dij);
      R TauBot1 = (R)0, TauBot2 = (R)0;
      if (S.bc_z0 == 2) {
        TauBot1 = DUprime / Dij / Dz1 * nub;
        TauBot2 = DVprime / Dij / Dz1 * nub;
      } else {
        TauBot1 = Cdrag * DUprime * DUmag / (Dij * Dij);
        TauBot2 = Cdrag * DVprime * DUmag / (Dij * Dij);
      }
      Fext_Bot1 = Bbot * TauBot1;
      Fext_Bot2 = (dxh * dyh * TauBot1 + Abot * TauBot2) / Bbot;
    }
    const R vbot = (R)(kSmall + S.v_cmu + 0.0 + vtB);
    const R UzRb = (R)S.zUR[c], VzRb = (R)S.zVR[c];
    for (int k = 1; k <= NG; ++k) {
      const long long ob = i3(S, i, j, KB - k), oi = i3(S, i, j, KB + k - 1);
      const long long ot = i3(S, i, j, KE + k), os = i3(S, i, j, KE - k + 1);
      S.DW[ob] = (T)((R)2.0 * Dij * WzRb - (R)S.DW[oi]);
      if (S.bc_z0 == 1) {
        S.DU[ob] = S.DU[oi];
        S.DV[ob] = S.DV[oi];
      } else {   // stress ghosts (src/nhwave.F:4869-4903)
        const R dsb = (R)(S.sigc[KB + k - 1] - S.sigc[KB - k]);
        const R DUi = (R)S.DU[oi], DVi = (R)S.DV[oi], DWi = (R)S.DW[oi];
        R du = DUi - dsb * (Fext_Bot1 * (Dij * Dij / Abot / vbot) + dxh * (DWi - Dij * WzRb) / (dsb / (R)2.0) +
                            Dij * Dij / (Abot * Abot) *
                                (-(R)2.0 * dxh * DelxUzR - ((R)1.0 - dxh * dxh) * DelxWzR -
                                 dyh * (DelyUzR + DelxVzR - dxh * DelyWzR)));
        const R DUbot_old = (R)2.0 * Dij * UzRb - DUi;
        if (DUbot_old > (R)0) du = rmin<R>((R)3.0 * DUbot_old, rmax<R>((R)-1.0 * DUbot_old, du));
        else if (DUbot_old < (R)0) du = rmax<R>((R)3.0 * DUbot_old, rmin<R>((R)-1.0 * DUbot_old, du));
        if (Dij < MinDepBC) du = DUi;
        R dv = DVi - dsb * (Fext_Bot2 * (Dij * Dij / Abot / vbot) + dyh * (DWi - Dij * WzRb) / (dsb / (R)2.0) +
                            Dij * Dij / (Abot * Abot) *
                                (-(R)2.0 * dyh * DelyVzR - ((R)1.0 - dyh * dyh) * DelyWzR -
                                 dxh * (DelxVzR + DelyUzR - dyh * DelxWzR)));
        const R DVbot_old = (R)2.0 * Dij * VzRb - DVi;
        if (DVbot_old > (R)0) dv = rmin<R>((R)3.0 * DVbot_old, rmax<R>((R)-1.0 * DVbot_old, dv));
        else if (DVbot_old < (R)0) dv = rmax<R>((R)3.0 * DVbot_old, rmin<R>((R)-1.0 * DVbot_old, dv));
        if (Dij < MinDepBC) dv = DVi;
        S.DU[ob] = (T)du;
        S.DV[ob] = (T)dv;
      }
      const R dsg = (R)(S.sigc[KE + k] - S.sigc[KE - k + 1]);
      const R DWs = (R)S.DW[os], DUs = (R)S.DU[os], DVs = (R)S.DV[os];
      S.DW[ot] = (T)((R)2.0 * Dij * WzLt - DWs);
      R du = DUs + dsg * (Fext_Wind1 * (Dij * Dij / Atop / vtop) -
                          dxe * (Dij * WzLt - DWs) / (dsg / (R)2.0) +
                          Dij * Dij / (Atop * Atop) *
                              (+(R)2.0 * dxe * DelxUzL - ((R)1.0 - dxe * dxe) * DelxWzL +
                               dye * (DelyUzL + DelxVzL + dxe * DelyWzL)));
      const R DUtop_old = (R)2.0 * Dij * UzLt - DUs;
      if (DUtop_old > (R)0) du = rmin<R>((R)3.0 * DUtop_old, rmax<R>((R)-1.0 * DUtop_old, du));
      else if (DUtop_old < (R)0) du = rmax<R>((R)3.0 * DUtop_old, rmin<R>((R)-1.0 * DUtop_old, du));
      if (Dij < MinDepBC) du = DUs;
      R dv = DVs + dsg * (Fext_Wind2 * (Dij * Dij / Atop / vtop) -
                          dye * (Dij * WzLt - DWs) / (dsg / (R)2.0) +
                          Dij * Dij / (Atop * Atop) *
                              (+(R)2.0 * dye * DelyVzL - ((R)1.0 - dye * dye) * DelyWzL +
                               dxe * (DelxVzL + DelyUzL + dye * DelxWzL)));
      const R DVtop_old = (R)2.0 * Dij * VzLt - DVs;
      if (DVtop_old > (R)0) dv = rmin<R>((R)3.0 * DVtop_old, rmax<R>((R)-1.0 * DVtop_old, dv));
      else if (DVtop_old < (R)0) dv = rmax<R>((R)3.0 * DVtop_old, rmin<R>((R)-1.0 * DVtop_old, dv));
      if (Dij < MinDepBC) dv = DVs;
      S.DU[ot] = (T)du;
      S.DV[ot] = (T)dv;
      const T d = (T)Dij;
      S.U[ob] = S.DU[ob] / d; S.V[ob] = S.DV[ob] / d; S.W[ob] = S.DW[ob] / d;
      S.U[ot] = S.DU[ot] / d; S.V[ot] = S.DV[ot] / d; S.W[ot] = S.DW[ot] / d;
    }
  }
};

// =========================================================================
//   viscous flow with constant viscosities (IVTURB = IHTURB = 1)
// =========================================================================
// diffusion (src/nhwave.F:6785-7141): the explicit viscous terms of R2-R4,
// one thread per interior cell, from the stage's starting DU/DV/DW and the
// sigma slopes of the last sigma_transform (zero before the first one).
// Cmu = Visc; CmuHt per cell (Cmut_min until eval_turb).  Each bracket
// keeps the reference's evaluation order (bit-exact in the FP64 form).
struct OpDiffusion {
  static constexpr const char* kName = "diffusion";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j, int k) const {
    using R = T;
    const long long c = i2(S, i, j), o = i3(S, i, j, k);
    if (S.Mask[c] == 0) {
      S.Dxx[o] = (T)0; S.Dxy[o] = (T)0; S.Dyx[o] = (T)0; S.Dyy[o] = (T)0; S.Dzx[o] = (T)0; S.Dzy[o] = (T)0;
      return;
    }
    const bool set = S.sc->sig_set != 0;
    // DelxSc / DelySc at level kk (sigc) and DelxSl / DelySl at face kk (sig)
    auto slope = [&](const double* lev, const double* H, const double* E, int ii, int jj, int kk) -> R {
      if (!set) return (R)0;
      const long long q = i2(S, ii, jj);
      return (R)((1.0 - lev[kk]) / S.scD[q] * H[q] - lev[kk] / S.scD[q] * E[q]);
    };
    auto Scx = [&](int ii, int jj, int kk) { return slope(S.sigc, S.scHx, S.scEx, ii, jj, kk); };
    auto Scy = [&](int ii, int jj, int kk) { return slope(S.sigc, S.scHy, S.scEy, ii, jj, kk); };
    const T* DU = S.DU;
    const T* DV = S.DV;
    const T* DW = S.DW;
    auto F = [&](const T* a, int ii, int jj, int kk) -> R { return a[i3(S, ii, jj, kk)]; };
    const R dx = (R)S.dx, dy = (R)S.dy;
    const R cmu = (R)S.v_cmu, sch = (R)S.v_schmidt;
    // CmuHt of a cell; face viscosity between two cells; cell viscosity
    auto H = [&](int ii, int jj, int kk) -> R { return (R)S.CmuHt[i3(S, ii, jj, kk)]; };
    auto nuF = [&](R ha, R hb) -> R { return (R)0.5 * (cmu + cmu) + (R)0.5 * (ha + hb) / sch; };
    auto nuC = [&](int ii, int jj, int kk) -> R { return cmu + H(ii, jj, kk) / sch; };
    const R h0 = H(i, j, k);
    const R nuE = nuF(H(i + 1, j, k), h0), nuW = nuF(h0, H(i - 1, j, k));
    const R nuN = nuF(H(i, j + 1, k), h0), nuS = nuF(h0, H(i, j - 1, k));
    const R cE = nuC(i + 1, j, k), cW = nuC(i - 1, j, k), cN = nuC(i, j + 1, k), cS = nuC(i, j - 1, k);
    const R cD = nuC(i, j, k - 1), c0 = nuC(i, j, k), cU = nuC(i, j, k + 1);
    const double* dsg = S.dsig;
    const double L1top = dsg[k + 1] / (dsg[k] + dsg[k + 1]), L2top = dsg[k] / (dsg[k] + dsg[k + 1]);
    const double L1bot = dsg[k] / (dsg[k] + dsg[k - 1]), L2bot = dsg[k - 1] / (dsg[k] + dsg[k - 1]);
    const double ck = (dsg[k] + dsg[k + 1]) / 2.0, ck1 = (dsg[k - 1] + dsg[k]) / 2.0;
    const R ac = (R)(-ck / (ck + ck1) / ck1), bc = (R)((ck - ck1) / (ck * ck1)), gc = (R)(ck1 / (ck + ck1) / ck);
    const R nuH_top = ((R)L1top * cmu + (R)L2top * cmu) + ((R)L1top * h0 + (R)L2top * H(i, j, k + 1)) / sch;
    const R nuH_bot = ((R)L1bot * cmu + (R)L2bot * cmu) + ((R)L1bot * H(i, j, k - 1) + (R)L2bot * h0) / sch;
    const R Dc = (R)S.D[c], dsk = (R)dsg[k], rck = (R)ck, rck1 = (R)ck1;
    auto s3 = [&](const T* a, bool y, int ii, int jj) -> R {   // a F(k-1) Sc(k-1) + b .. + c ..
      auto sc = [&](int kk) { return y ? Scy(ii, jj, kk) : Scx(ii, jj, kk); };
      return ac * F(a, ii, jj, k - 1) * sc(k - 1) + bc * F(a, ii, jj, k) * sc(k) + gc * F(a, ii, jj, k + 1) * sc(k + 1);
    };
    auto s3x = [&](R lead, int ii, int jj) -> R {   // lead + a (Sx DV + Sy DU)(k-1) + ..
      return lead + ac * (Scx(ii, jj, k - 1) * F(DV, ii, jj, k - 1) + Scy(ii, jj, k - 1) * F(DU, ii, jj, k - 1)) +
             bc * (Scx(ii, jj, k) * F(DV, ii, jj, k) + Scy(ii, jj, k) * F(DU, ii, jj, k)) +
             gc * (Scx(ii, jj, k + 1) * F(DV, ii, jj, k + 1) + Scy(ii, jj, k + 1) * F(DU, ii, jj, k + 1));
    };
    auto s3w = [&](bool y, const T* a, int ii, int jj) -> R {   // a (W Sc + F/D)(k-1) + ..
      auto sc = [&](int kk) { return y ? Scy(ii, jj, kk) : Scx(ii, jj, kk); };
      return ac * (F(DW, ii, jj, k - 1) * sc(k - 1) + F(a, ii, jj, k - 1) / Dc) +
             bc * (F(DW, ii, jj, k) * sc(k) + F(a, ii, jj, k) / Dc) +
             gc * (F(DW, ii, jj, k + 1) * sc(k + 1) + F(a, ii, jj, k + 1) / Dc);
    };
    auto vco = [&](bool y, R& cA, R& cB, R& cC) {   // coefficients of d/dsigma[nu Sl d/dsigma]
      const R st = slope(S.sig, y ? S.scHy : S.scHx, y ? S.scEy : S.scEx, i, j, k + 1);
      const R sb = slope(S.sig, y ? S.scHy : S.scHx, y ? S.scEy : S.scEx, i, j, k);
      const R Pq = nuH_top * st - nuH_bot * sb, Sq = nuH_top * st + nuH_bot * sb;
      cA = Pq * ac / dsk + Sq / rck1 / (rck + rck1);
      cB = Pq * bc / dsk - Sq / rck1 / rck;
      cC = Pq * gc / dsk + Sq / rck / (rck + rck1);
    };
    R xA, xB, xC, yA, yB, yC;
    vco(false, xA, xB, xC);
    vco(true, yA, yB, yC);
    auto mixed = [&](int kk) -> R {   // d/dy DU + d/dx DV at level kk
      return (F(DU, i, j + 1, kk) - F(DU, i, j - 1, kk)) / (R)2.0 / dy +
             (F(DV, i + 1, j, kk) - F(DV, i - 1, j, kk)) / (R)2.0 / dx;
    };
    const R two = (R)2.0;
    S.Dxx[o] =
        (two * nuE * (F(DU, i + 1, j, k) - F(DU, i, j, k)) / dx - two * nuW * (F(DU, i, j, k) - F(DU, i - 1, j, k)) / dx) / dx +
        (two * cE * s3(DU, false, i + 1, j) - two * cW * s3(DU, false, i - 1, j)) / two / dx +
        (ac * two * cD * Scx(i, j, k - 1) * (F(DU, i + 1, j, k - 1) - F(DU, i - 1, j, k - 1)) / two / dx +
         bc * two * c0 * Scx(i, j, k) * (F(DU, i + 1, j, k) - F(DU, i - 1, j, k)) / two / dx +
         gc * two * cU * Scx(i, j, k + 1) * (F(DU, i + 1, j, k + 1) - F(DU, i - 1, j, k + 1)) / two / dx);
    S.Dxy[o] =
        (nuN * (F(DU, i, j + 1, k) - F(DU, i, j, k)) / dy - nuS * (F(DU, i, j, k) - F(DU, i, j - 1, k)) / dy) / dy +
        (cN * s3x((F(DV, i + 1, j + 1, k) - F(DV, i - 1, j + 1, k)) / two / dx, i, j + 1) -
         cS * s3x((F(DV, i + 1, j - 1, k) - F(DV, i - 1, j - 1, k)) / two / dx, i, j - 1)) / two / dy +
        (ac * cD * Scy(i, j, k - 1) * mixed(k - 1) + bc * c0 * Scy(i, j, k) * mixed(k) +
         gc * cU * Scy(i, j, k + 1) * mixed(k + 1)) +
        (yA * Scx(i, j, k - 1) * F(DV, i, j, k - 1) + yB * Scx(i, j, k) * F(DV, i, j, k) +
         yC * Scx(i, j, k + 1) * F(DV, i, j, k + 1));
    S.Dyx[o] =
        (nuE * (F(DV, i + 1, j, k) - F(DV, i, j, k)) / dx - nuW * (F(DV, i, j, k) - F(DV, i - 1, j, k)) / dx) / dx +
        (cE * s3x((F(DU, i + 1, j + 1, k) - F(DU, i + 1, j - 1, k)) / two / dy, i + 1, j) -
         cW * s3x((F(DU, i - 1, j + 1, k) - F(DU, i - 1, j - 1, k)) / two / dy, i - 1, j)) / two / dx +
        (ac * cD * Scx(i, j, k - 1) * mixed(k - 1) + bc * c0 * Scx(i, j, k) * mixed(k) +
         gc * cU * Scx(i, j, k + 1) * mixed(k + 1)) +
        (xA * Scy(i, j, k - 1) * F(DU, i, j, k - 1) + xB * Scy(i, j, k) * F(DU, i, j, k) +
         xC * Scy(i, j, k + 1) * F(DU, i, j, k + 1));
    S.Dyy[o] =
        (two * nuN * (F(DV, i, j + 1, k) - F(DV, i, j, k)) / dy - two * nuS * (F(DV, i, j, k) - F(DV, i, j - 1, k)) / dy) / dy +
        (two * cN * s3(DV, true, i, j + 1) - two * cS * s3(DV, true, i, j - 1)) / two / dy +
        (ac * two * cD * Scy(i, j, k - 1) * (F(DV, i, j + 1, k - 1) - F(DV, i, j - 1, k - 1)) / two / dy +
         bc * two * c0 * Scy(i, j, k) * (F(DV, i, j + 1, k) - F(DV, i, j - 1, k)) / two / dy +
         gc * two * cU * Scy(i, j, k + 1) * (F(DV, i, j + 1, k + 1) - F(DV, i, j - 1, k + 1)) / two / dy);
    S.Dzx[o] =
        (nuE * (F(DW, i + 1, j, k) - F(DW, i, j, k)) / dx - nuW * (F(DW, i, j, k) - F(DW, i - 1, j, k)) / dx) / dx +
        (cE * s3w(false, DU, i + 1, j) - cW * s3w(false, DU, i - 1, j)) / two / dx +
        (ac * cD * Scx(i, j, k - 1) * (F(DW, i + 1, j, k - 1) - F(DW, i - 1, j, k - 1)) / two / dx +
         bc * c0 * Scx(i, j, k) * (F(DW, i + 1, j, k) - F(DW, i - 1, j, k)) / two / dx +
         gc * cU * Scx(i, j, k + 1) * (F(DW, i + 1, j, k + 1) - F(DW, i - 1, j, k + 1)) / two / dx) +
        (xA * F(DU, i, j, k - 1) / Dc + xB * F(DU, i, j, k) / Dc + xC * F(DU, i, j, k + 1) / Dc);
    S.Dzy[o] =
        (nuN * (F(DW, i, j + 1, k) - F(DW, i, j, k)) / dy - nuS * (F(DW, i, j, k) - F(DW, i, j - 1, k)) / dy) / dy +
        (cN * s3w(true, DV, i, j + 1) - cS * s3w(true, DV, i, j - 1)) / two / dy +
        (ac * cD * Scy(i, j, k - 1) * (F(DW, i, j + 1, k - 1) - F(DW, i, j - 1, k - 1)) / two / dy +
         bc * c0 * Scy(i, j, k) * (F(DW, i, j + 1, k) - F(DW, i, j - 1, k)) / two / dy +
         gc * cU * Scy(i, j, k + 1) * (F(DW, i, j + 1, k + 1) - F(DW, i, j - 1, k + 1)) / two / dy) +
        (yA * F(DV, i, j, k - 1) / Dc + yB * F(DV, i, j, k) / Dc + yC * F(DV, i, j, k + 1) / Dc);
  }
};

// eval_turb (src/nhwave.F:6544-6782), after sponge_damping.  Vertical
// (every column, ghosts included): IVTURB 1 CmuVt = Cvs; IVTURB 2 the
// subgrid model CmuVt = Cvs D dsig^2 |d(U,V)/dsigma| on the levels 2 ..
// Kloc-1 (1-based), the outermost ghost levels copying their neighbours.
// IHTURB 1 fills CmuHt = Chs here and IHTURB >= 10 copies CmuVt, after the
// vertical model (k-epsilon's kernels run first); IHTURB 2 is OpTurbH +
// OpTurbHGhost.
// Products in the reference's order, in FP64 (bit-exact in the FP64 form).
struct OpTurbV {
  static constexpr const char* kName = "eval_turb_v";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j) const {
    const long long q = i2(S, i, j);
    T* cv = S.CmuVt + q;
    if (S.ivturb == 1) {
      for (int k = 0; k < S.Kloc; ++k) cv[S.sz * k] = (T)S.v_cvs;
    } else if (S.ivturb == 2) {
      const double Dq = S.D[q];
      for (int k = 1; k <= S.Kloc - 2; ++k) {
        const long long a = q + S.sz * (k + 1), b = q + S.sz * (k - 1);
        const double ds = S.sigc[k + 1] - S.sigc[k - 1];
        const double dU = ((double)S.U[a] - (double)S.U[b]) / ds;
        const double dV = ((double)S.V[a] - (double)S.V[b]) / ds;
        cv[S.sz * k] = (T)(S.v_cvs * Dq * (S.dsig[k] * S.dsig[k]) * sqrt(dU * dU + dV * dV));
      }
      cv[0] = cv[S.sz];
      cv[S.sz * (S.Kloc - 1)] = cv[S.sz * (S.Kloc - 2)];
    }   // IVTURB = 10 and 20: the k-epsilon / LES kernels set CmuVt before this one
    // no turbulence in an INT_ maker's source region (LES), or in an INT_,
    // LEF_ or FOCUSED maker's (dynamic LES)
    if (((S.ivturb == 20 && S.les_int) || (S.ivturb == 30 && S.ke_quiet)) && S.xc[i] >= S.wm_xw &&
        S.xc[i] <= S.wm_xe && S.yc[j] >= S.wm_ys && S.yc[j] <= S.wm_yn)
      for (int k = 0; k < S.Kloc; ++k) cv[S.sz * k] = (T)0;
    if (S.ihturb == 1)
      for (int k = 0; k < S.Kloc; ++k) S.CmuHt[q + S.sz * k] = (T)S.v_chs;
    else if (S.ihturb >= 10)   // the 3-D model's length scales in every direction
      for (int k = 0; k < S.Kloc; ++k) S.CmuHt[q + S.sz * k] = cv[S.sz * k];
  }
};
// IHTURB 2, interior cells: CmuHt = Chs dx dy sqrt(Sxx^2 + 2 Sxy^2 + Syy^2)
// with the horizontal strain rates in sigma coordinates; DelxSc / DelySc
// are the slopes of the last sigma_transform (zero before the first one).
// The reference's Strxy reads U(i,j+1,j), the row index in place of the
// level (src/nhwave.F:6695); the level k is read here.
struct OpTurbH {
  static constexpr const char* kName = "eval_turb_h";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j, int k) const {
    const long long q = i2(S, i, j), o = i3(S, i, j, k);
    auto U = [&](long long x) { return (double)S.U[x]; };
    auto V = [&](long long x) { return (double)S.V[x]; };
    double sx = 0.0, sy = 0.0;
    if (S.sc->sig_set) {
      sx = (1.0 - S.sigc[k]) / S.scD[q] * S.scHx[q] - S.sigc[k] / S.scD[q] * S.scEx[q];
      sy = (1.0 - S.sigc[k]) / S.scD[q] * S.scHy[q] - S.sigc[k] / S.scD[q] * S.scEy[q];
    }
    const double ds = S.sigc[k + 1] - S.sigc[k - 1];
    const long long up = o + S.sz, dn = o - S.sz;
    const double Sxx = (U(o + 1) - U(o - 1)) / (2.0 * S.dx) + (U(up) - U(dn)) / ds * sx;
    const double Syy = (V(o + S.sy) - V(o - S.sy)) / (2.0 * S.dy) + (V(up) - V(dn)) / ds * sy;
    const double Sxy = 0.5 * ((U(o + S.sy) - U(o - S.sy)) / (2.0 * S.dy) + (U(up) - U(dn)) / ds * sy +
                              (V(o + 1) - V(o - 1)) / (2.0 * S.dx) + (V(up) - V(dn)) / ds * sx);
    S.CmuHt[o] = (T)(S.v_chs * S.dx * S.dy * sqrt(Sxx * Sxx + 2.0 * (Sxy * Sxy) + Syy * Syy));
  }
};
// IHTURB 2, ghosts: CmuHt mirrored across the west/east sides (interior
// rows and levels), the south/north sides (interior columns i, levels) and
// the bed/surface (interior columns).  One thread per line, its NG ghosts
// in the reference's order, so a grid narrower than NG reads what the same
// line wrote before, as the reference does.  Lines t of the x sides, then
// of the y sides, then of the vertical.
struct OpTurbHGhost {
  static constexpr const char* kName = "eval_turb_ghost";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int t, int, int) const {
    T* c = S.CmuHt;
    const long long nx = (long long)S.N * S.K, ny = (long long)S.M * S.K;
    long long base, step;
    int lo, hi;
    if (t < nx) {
      base = i3(S, 0, S.JB + (int)(t % S.N), S.KB + (int)(t / S.N)); step = 1; lo = S.IB; hi = S.IE;
    } else if (t < nx + ny) {
      const long long u = t - nx;
      base = i3(S, S.IB + (int)(u % S.M), 0, S.KB + (int)(u / S.M)); step = S.sy; lo = S.JB; hi = S.JE;
    } else {
      const long long u = t - nx - ny;
      base = i3(S, S.IB + (int)(u % S.M), S.JB + (int)(u / S.M), 0); step = S.sz; lo = S.KB; hi = S.KE;
    }
    for (int g = 1; g <= NG; ++g) {
      c[base + step * (lo - g)] = c[base + step * (lo + g - 1)];
      c[base + step * (hi + g)] = c[base + step * (hi - g + 1)];
    }
  }
};

// =========================================================================
//   k-epsilon closure, IVTURB = 10 (kepsilon_3D, src/nhwave.F:10030-11114)
// =========================================================================
// Barotropic flow: Rho = Rho0 (src/initialize.F:2561), so the buoyancy
// production is zero.  Everything is evaluated in FP64 in the reference's
// order (bit-exact in the FP64 form).  The reference leaves alpha_c,
// beta_c, gamma_c of the interior vertical coefficients unset; the three-
// point weights of the momentum equations (src/nhwave.F:6826-6828) stand in.
constexpr double kTkeMin = (double)1.e-9f, kEpsMin = (double)1.e-9f;

// limited horizontal slopes (delxFun_3D / delyFun_3D) of U and V as
// get_Omega leaves them (uv = 1, before sponge_damping), or of W as fluxes
// leaves them (uv = 0), at the interior cells the production reads
struct OpKeSlopes {
  static constexpr const char* kName = "ke_slopes";
  int uv;
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j, int k) const {
    const long long q = i2(S, i, j), o = i3(S, i, j, k);
    const bool dry = S.Mask[q] == 0;
    auto sx = [&](const T* a) -> T {
      return dry ? (T)0 : (T)lim_slope<double>((double)a[o - 1], (double)a[o], (double)a[o + 1], S.dx, S.dx);
    };
    auto sy = [&](const T* a) -> T {
      return dry ? (T)0 : (T)lim_slope<double>((double)a[o - S.sy], (double)a[o], (double)a[o + S.sy], S.dy, S.dy);
    };
    if (uv) {
      S.keDxU[o] = sx(S.U); S.keDyU[o] = sy(S.U);
      S.keDxV[o] = sx(S.V); S.keDyV[o] = sy(S.V);
    } else {
      S.keDxW[o] = sx(S.W); S.keDyW[o] = sy(S.W);
    }
  }
};

// surface face values of tke and epsilon (construct_3D_z over the limited
// vertical slope, interior columns; zero elsewhere), floored at Tke_min /
// Eps_min (src/nhwave.F:10321-10334); every column
struct OpKeTop {
  static constexpr const char* kName = "ke_surface_values";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j) const {
    const long long q = i2(S, i, j);
    double tk = 0.0, ep = 0.0;
    if (i >= S.IB && i <= S.IE && j >= S.JB && j <= S.JE) {
      const int K = S.KE;
      auto top = [&](const T* a) {
        const double am = (double)a[i3(S, i, j, K - 1)], a0 = (double)a[i3(S, i, j, K)], ap = (double)a[i3(S, i, j, K + 1)];
        const double t1 = (ap - a0) / (S.sigc[K + 1] - S.sigc[K]);
        const double t2 = (a0 - am) / (S.sigc[K] - S.sigc[K - 1]);
        const double dz = (fabs(t1) + fabs(t2)) < kSmall ? 0.0 : limiter(t1, t2);
        return a0 + 0.5 * S.dsig[K] * dz;
      };
      tk = top(S.Tke);
      ep = top(S.Eps);
    }
    S.keTopK[q] = dmax_(tk, kTkeMin);
    S.keTopE[q] = dmax_(ep, kEpsMin);
  }
};

// HLPA face value (src/nhwave.F:7809-7847)
__device__ __forceinline__ double ke_hlpa(double Uw, double Fww, double Fw, double Fp, double Fe) {
  double h = 0.0;
  if (Uw >= 0.0) {
    const double a = fabs(Fp - 2.0 * Fw + Fww) < fabs(Fp - Fww) ? 1.0 : 0.0;
    h = fabs(Fp - Fww) <= (double)1.e-16f ? Fw : Fw + a * (Fp - Fw) * (Fw - Fww) / (Fp - Fww);
  }
  if (Uw < 0.0) {
    const double a = fabs(Fw - 2.0 * Fp + Fe) < fabs(Fw - Fe) ? 1.0 : 0.0;
    h = fabs(Fw - Fe) <= (double)1.e-16f ? Fp : Fp + a * (Fw - Fp) * (Fp - Fe) / (Fw - Fe);
  }
  return h;
}

// adv_scalar_hlpa with flux_scalar_bc (src/nhwave.F:7604-7806, 7850-7986) at
// one interior cell: minus the divergence of the HLPA fluxes of Phi by Ex,
// Ey and Omega (the boundary scalar of a BC_X0 = 3 side is zero; faces of
// dry cells carry none) plus the horizontal diffusion with Cmu + CmuHt /
// SchtH; zero in a dry cell
template <class T>
__device__ double ke_r5(const Dev<T>& S, int i, int j, int k, const T* Phi, double SchtH) {
  if (S.Mask[i2(S, i, j)] == 0) return 0.0;
  auto scx = [&](int f) -> double {
    if ((f <= S.IE && S.Mask[i2(S, f, j)] == 0) || (f - 1 >= S.IB && S.Mask[i2(S, f - 1, j)] == 0)) return 0.0;
    if (f == S.IE + 1) return 0.0;
    const long long o = i3(S, f, j, k);
    const double u = (double)S.Ex[o];
    if (f == S.IB) {
      if (S.bc_x0 == 1 || S.bc_x0 == 2 || S.bc_x0 == 5) return 0.0;
      if (S.bc_x0 == 3) return u * 0.0;
    }
    return u * ke_hlpa(u, (double)Phi[o - 2], (double)Phi[o - 1], (double)Phi[o], (double)Phi[o + 1]);
  };
  auto scy = [&](int f) -> double {
    if ((f <= S.JE && S.Mask[i2(S, i, f)] == 0) || (f - 1 >= S.JB && S.Mask[i2(S, i, f - 1)] == 0)) return 0.0;
    if (f == S.JB && (S.bc_y0 == 1 || S.bc_y0 == 2 || S.bc_y0 == 5)) return 0.0;
    if (f == S.JE + 1 && (S.bc_yn == 1 || S.bc_yn == 2 || S.bc_yn == 5)) return 0.0;
    const long long o = i3(S, i, f, k);
    const long long y = S.sy;
    const double v = (double)S.Ey[o];
    return v * ke_hlpa(v, (double)Phi[o - 2 * y], (double)Phi[o - y], (double)Phi[o], (double)Phi[o + y]);
  };
  auto scz = [&](int f) -> double {
    if (f == S.KB || f == S.KE + 1) return 0.0;
    const long long o = i3(S, i, j, f);
    const long long z = S.sz;
    const double w = (double)S.Omega[o];
    return w * ke_hlpa(w, (double)Phi[o - 2 * z], (double)Phi[o - z], (double)Phi[o], (double)Phi[o + z]);
  };
  const double cmu = S.v_cmu;
  auto nu = [&](double ha, double hb) { return 0.5 * (cmu + cmu) + 0.5 * (ha + hb) / SchtH; };
  auto H = [&](int ii, int jj) { return (double)S.CmuHt[i3(S, ii, jj, k)]; };
  auto Dq = [&](int ii, int jj) { return S.D[i2(S, ii, jj)]; };
  auto Ph = [&](int ii, int jj) { return (double)Phi[i3(S, ii, jj, k)]; };
  const double Sdx = 0.5 *
                     (nu(H(i + 1, j), H(i, j)) * (Dq(i + 1, j) + Dq(i, j)) * (Ph(i + 1, j) - Ph(i, j)) -
                      nu(H(i, j), H(i - 1, j)) * (Dq(i, j) + Dq(i - 1, j)) * (Ph(i, j) - Ph(i - 1, j))) /
                     (S.dx * S.dx);
  const double Sdy = 0.5 *
                     (nu(H(i, j + 1), H(i, j)) * (Dq(i, j + 1) + Dq(i, j)) * (Ph(i, j + 1) - Ph(i, j)) -
                      nu(H(i, j), H(i, j - 1)) * (Dq(i, j) + Dq(i, j - 1)) * (Ph(i, j) - Ph(i, j - 1))) /
                     (S.dy * S.dy);
  return -(1.0 / S.dx * (scx(i + 1) - scx(i))) - 1.0 / S.dy * (scy(j + 1) - scy(j)) -
         1.0 / S.dsig[k] * (scz(k + 1) - scz(k)) + Sdx + Sdy;
}

// shear production of the nonlinear model (ke_model = 2, src/nhwave.F:
// 10139-10274): Reynolds stresses from the velocity gradient G, contracted
// with G per PRODTYPE (1 vertical shear of U, V; 2 vertical shear; else 3-D)
__device__ inline double ke_production(const double (&G)[3][3], double tk, double ep, int prod_type) {
  const double c23 = (double)(2.0f / 3.0f), c13 = (double)(1.0f / 3.0f);
  double smax = 0.0;
  for (int n = 0; n < 3; ++n)
    if (fabs(G[n][n]) > smax) smax = fabs(G[n][n]);
  smax = smax * tk / ep;
  const double c_d = c23 * (1.0 / ((double)7.4f + 2.0 * smax));
  double dmx = 0.0;
  for (int n = 0; n < 3; ++n)
    for (int m = 0; m < 3; ++m)
      if (fabs(G[n][m]) > dmx) dmx = fabs(G[n][m]);
  dmx = dmx * tk / ep;
  const double c_1 = 1.0 / ((double)185.2f + 3.0 * (dmx * dmx));
  const double c_2 = -(1.0 / (58.5 + 2.0 * (dmx * dmx)));
  const double c_3 = 1.0 / ((double)370.4f + 3.0 * (dmx * dmx));
  const double tk2 = tk * tk, tk3 = tk * tk * tk, ep2 = ep * ep;
  const int n1 = prod_type == 1 ? 2 : 3, m0 = (prod_type == 1 || prod_type == 2) ? 2 : 0;
  double P = 0.0;
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
      if (n < n1 && m >= m0) P = P + r * G[n][m];
    }
  return P;
}

// one interior column of kepsilon_3D: production, the epsilon equation
// (HLPA advection, horizontal diffusion, source, implicit vertical
// diffusion with the bed and surface terms), its SSP-RK combination and
// floor, the same for tke (whose source reads the new DEps), then the bed
// wall function and the surface gradient condition (src/nhwave.F:10100-
// 10858).  The column's own snapshot gives DelxSc / DelySc / DelxSl /
// DelySl; neighbours are read only through Tke, Eps, CmuHt, D, U, V, W, Ex,
// Ey, Omega, Mask and the surface values, which no thread writes here.
struct OpKeColumn {
  static constexpr const char* kName = "kepsilon_column";
  static constexpr int kMaxK = 64;   // Kglob <= 64 (nhw_create)
  int istep;                         // 0-based stage
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j) const {
    const long long q = i2(S, i, j);
    const double Dc = S.D[q];
    const int mk = S.Mask[q];
    const double Dmin = S.ke_dmin, dt = S.sc->dt, cmu = S.v_cmu, cmuR = 0.0;
    const bool rng = S.ke_rng != 0;
    const double c1e = rng ? (double)1.42f : (double)1.44f;
    double c2e = rng ? 0.0 : (double)1.92f;
    const double c3e = 0.0, Prod_b = 0.0;
    const double cmiu = rng ? (double)0.085f : (double)0.09f;
    const double Sche = rng ? (double)0.72f : (double)1.3f, Schk = rng ? (double)0.72f : 1.0;
    const int KB = S.KB, KE = S.KE, n = KE - KB + 1;
    const double* sigc = S.sigc;
    const double* sig = S.sig;
    const double* dsig = S.dsig;
    const bool set = S.sc->sig_set != 0;
    auto slope = [&](const double* lev, bool y, int kk) -> double {
      if (!set) return 0.0;
      return (1.0 - lev[kk]) / S.scD[q] * (y ? S.scHy[q] : S.scHx[q]) - lev[kk] / S.scD[q] * (y ? S.scEy[q] : S.scEx[q]);
    };
    auto Scx = [&](int kk) { return slope(sigc, false, kk); };
    auto Scy = [&](int kk) { return slope(sigc, true, kk); };
    auto Slx = [&](int kk) { return slope(sig, false, kk); };
    auto Sly = [&](int kk) { return slope(sig, true, kk); };
    auto at = [&](const T* a, int kk) -> double { return (double)a[i3(S, i, j, kk)]; };
    auto ds = [&](int kk) { return sigc[kk + 1] - sigc[kk - 1]; };
    const double dxh = S.DelxH[q], dyh = S.DelyH[q], dxe = S.DelxEta[q], dye = S.DelyEta[q];
    // production (zero in shallow or dry columns; no negative production at the surface)
    double prod[kMaxK];
    for (int k = KB; k <= KE; ++k) {
      double P = 0.0;
      if (Dc >= Dmin && mk == 1) {
        double G[3][3];
        const double dU = at(S.U, k + 1) - at(S.U, k - 1), dV = at(S.V, k + 1) - at(S.V, k - 1);
        const double dW = at(S.W, k + 1) - at(S.W, k - 1);
        G[0][0] = at(S.keDxU, k) + dU / ds(k) * Scx(k);
        G[0][1] = at(S.keDyU, k) + dU / ds(k) * Scy(k);
        G[0][2] = 1.0 / Dc * dU / ds(k);
        G[1][0] = at(S.keDxV, k) + dV / ds(k) * Scx(k);
        G[1][1] = at(S.keDyV, k) + dV / ds(k) * Scy(k);
        G[1][2] = 1.0 / Dc * dV / ds(k);
        G[2][0] = at(S.keDxW, k) + dW / ds(k) * Scx(k);
        G[2][1] = at(S.keDyW, k) + dW / ds(k) * Scy(k);
        G[2][2] = 1.0 / Dc * dW / ds(k);
        P = ke_production(G, at(S.Tke, k), at(S.Eps, k), S.ke_prod);
        if (k == KE && P < 0.0) P = 0.0;
      }
      prod[k - KB] = P;
    }
    double A[kMaxK], B[kMaxK], C[kMaxK], X[kMaxK];
    // one equation: eq = 2 epsilon, 1 tke
    auto column = [&](int eq) {
      const T* Old = eq == 2 ? S.Eps : S.Tke;
      T* Dv = eq == 2 ? S.DEps : S.DTke;
      const double zL = eq == 2 ? S.keTopE[q] : S.keTopK[q];
      const double Sch = eq == 2 ? Sche : Schk;
      const double DxD = (dxh + dxe) / Dc, DyD = (dyh + dye) / Dc;
      for (int k = KB; k <= KE; ++k) {
        const int m = k - KB;
        const double L1top = dsig[k + 1] / (dsig[k] + dsig[k + 1]), L2top = dsig[k] / (dsig[k] + dsig[k + 1]);
        const double L1bot = dsig[k] / (dsig[k] + dsig[k - 1]), L2bot = dsig[k - 1] / (dsig[k] + dsig[k - 1]);
        const double dsigck = (dsig[k] + dsig[k + 1]) / 2.0, dsigck1 = (dsig[k - 1] + dsig[k]) / 2.0;
        const double alpha_c = -dsigck / (dsigck + dsigck1) / dsigck1;
        const double beta_c = (dsigck - dsigck1) / (dsigck * dsigck1);
        const double gamma_c = dsigck1 / (dsigck + dsigck1) / dsigck;
        const double nuV_top = (L1top * cmu + L2top * cmu) + (L1top * cmuR + L2top * cmuR) +
                               (L1top * at(S.CmuVt, k) + L2top * at(S.CmuVt, k + 1)) / Sch;
        const double nuH_top = (L1top * cmu + L2top * cmu) + (L1top * cmuR + L2top * cmuR) +
                               (L1top * at(S.CmuHt, k) + L2top * at(S.CmuHt, k + 1)) / Sch;
        const double nuV_bot = (L1bot * cmu + L2bot * cmu) + (L1bot * cmuR + L2bot * cmuR) +
                               (L1bot * at(S.CmuVt, k - 1) + L2bot * at(S.CmuVt, k)) / Sch;
        const double nuH_bot = (L1bot * cmu + L2bot * cmu) + (L1bot * cmuR + L2bot * cmuR) +
                               (L1bot * at(S.CmuHt, k - 1) + L2bot * at(S.CmuHt, k)) / Sch;
        double r = ke_r5(S, i, j, k, Old, Sch);
        if (eq == 2) r = r + c1e * Dc * (prod[m] + c3e * Prod_b) * at(S.Eps, k) / at(S.Tke, k);
        else r = r + Dc * (prod[m] + Prod_b) - at(S.DEps, k);
        if (k == KB) {
          r = r - (-(nuH_bot * (dxh * DxD + dyh * DyD) * at(Old, k))) / dsig[k] +
              (dsig[k] - dsigck) / (dsig[k] * dsig[k] / 2.0 * (dsigck + dsig[k] / 2.0)) *
                  (nuH_top * (Slx(k + 1) * dxh + Sly(k + 1) * dyh) + nuV_top / Dc) * at(Old, k);
        } else if (k == KE) {
          r = r + ((nuH_top * (dxe * dxe + dye * dye) + nuV_top) / (Dc * Dc) * (at(Old, k + 1) - at(Old, k)) * Dc / dsigck -
                   nuH_top * (-(dxe * DxD) - dye * DyD) * zL) /
                      dsig[k] +
              (dsig[k] - dsigck1) / (dsig[k] * dsig[k] / 2.0 * (dsigck1 + dsig[k] / 2.0)) *
                  (nuH_bot * (-(Slx(k) * dxe) - Sly(k) * dye) + nuV_bot / Dc) * zL;
        }
        auto top = [&](int kk) { return nuH_top * (Slx(k + 1) * Scx(kk) + Sly(k + 1) * Scy(kk)) + nuV_top / (Dc * Dc); };
        auto bot = [&](int kk) { return nuH_bot * (Slx(k) * Scx(kk) + Sly(k) * Scy(kk)) + nuV_bot / (Dc * Dc); };
        if (k == KB) A[m] = 0.0;
        else if (k == KE) A[m] = -dt * (3.0 / 2.0 * bot(k - 1) / (dsigck1 * (dsigck1 + dsig[k] / 2.0)));
        else
          A[m] = -dt * ((top(k - 1) - bot(k - 1)) * alpha_c / dsig[k] +
                        (top(k - 1) + bot(k - 1)) / (dsigck1 * (dsigck1 + dsigck)));
        if (k == KB) C[m] = -dt * (3.0 / 2.0 * top(k + 1) / (dsigck * (dsigck + dsig[k] / 2.0)));
        else if (k == KE) C[m] = 0.0;
        else
          C[m] = -dt * ((top(k + 1) - bot(k + 1)) * gamma_c / dsig[k] +
                        (top(k + 1) + bot(k + 1)) / (dsigck * (dsigck1 + dsigck)));
        double b0 = 1.0;
        if (eq == 2) {
          if (rng) {   // c2e of Yakhot et al. (1992) from the strain rate
            const double dUs = (at(S.U, k + 1) - at(S.U, k - 1)) / ds(k), dVs = (at(S.V, k + 1) - at(S.V, k - 1)) / ds(k);
            const double dWs = (at(S.W, k + 1) - at(S.W, k - 1)) / ds(k);
            const double S11 = at(S.keDxU, k) + dUs * Scx(k);
            const double S22 = at(S.keDyV, k) + dVs * Scy(k);
            const double S33 = 1.0 / Dc * (at(S.W, k + 1) - at(S.W, k - 1)) / ds(k);
            const double S12 = 0.5 * (at(S.keDyU, k) + dUs * Scy(k) + at(S.keDxV, k) + dVs * Scx(k));
            const double S13 = 0.5 * ((at(S.U, k + 1) - at(S.U, k - 1)) / ds(k) / Dc + at(S.keDxW, k) + dWs * Scx(k));
            const double S23 = 0.5 * ((at(S.V, k + 1) - at(S.V, k - 1)) / ds(k) / Dc + at(S.keDyW, k) + dWs * Scy(k));
            const double lambda = at(S.Tke, k) / at(S.Eps, k) *
                                  sqrt(2.0 * (S11 * S11 + S22 * S22 + S33 * S33 + 2.0 * (S12 * S12 + S13 * S13 + S23 * S23)));
            const double l3 = lambda * lambda * lambda;
            c2e = (double)1.68f + cmiu * l3 * (1.0 - lambda / (double)4.38f) / (1.0 + (double)0.012f * l3);
            c2e = dmax_(0.0, dmin_(c2e, 4.0));
          }
          b0 = 1.0 + dt * c2e * at(S.Eps, k) / at(S.Tke, k);
        }
        if (k == KB) B[m] = b0 - dt * (-(3.0 / 2.0 - dsigck / dsig[k]) * top(k) / (dsig[k] / 2.0 * dsigck));
        else if (k == KE) B[m] = b0 - dt * (-(3.0 / 2.0 - dsigck1 / dsig[k]) * bot(k) / (dsig[k] / 2.0 * dsigck1));
        else B[m] = b0 - dt * ((top(k) - bot(k)) * beta_c / dsig[k] - (top(k) + bot(k)) / (dsigck * dsigck1));
        X[m] = at(Dv, k) + dt * r;
      }
      // trig (src/nhwave.F:13182-13224): elimination in place, then back substitution
      for (int m = 1; m < n; ++m) {
        const double coeff = A[m] / B[m - 1];
        B[m] = B[m] - coeff * C[m - 1];
        X[m] = X[m] - coeff * X[m - 1];
      }
      X[n - 1] = X[n - 1] / B[n - 1];
      for (int m = n - 2; m >= 0; --m) X[m] = (X[m] - C[m] * X[m + 1]) / B[m];
      for (int k = KB; k <= KE; ++k) Dv[i3(S, i, j, k)] = (T)X[k - KB];
    };
    auto rk = [&](T* Dv, const T* Dv0, double vmin) {
      if (!(Dc >= Dmin && mk == 1)) return;
      const double al = S.alpha[istep], be = S.beta[istep];
      for (int k = KB; k <= KE; ++k) {
        const long long o = i3(S, i, j, k);
        const double v = al * (double)Dv0[o] + be * (double)Dv[o];
        Dv[o] = (T)dmax_(v, Dc * vmin);
      }
    };
    const bool solve = !(Dc < Dmin && mk == 0);
    if (solve) column(2);
    rk(S.DEps, S.DEps0, kEpsMin);
    if (solve) column(1);
    rk(S.DTke, S.DTke0, kTkeMin);
    // bed: wall function (src/nhwave.F:10776-10831)
    if (!(Dc < Dmin || mk == 0)) {
      const long long ob = i3(S, i, j, KB);
      const double Abot = sqrt(1.0 + dxh * dxh + dyh * dyh), Bbot = sqrt(1.0 + dxh * dxh);
      const double du = (double)S.DU[ob], dv = (double)S.DV[ob], dw = (double)S.DW[ob];
      const double DUprime = (du - dxh * dw) / Bbot;
      const double DVprime = (-(dxh * dyh * du) + (1.0 + dxh * dxh) * dv - dyh * dw) / Abot / Bbot;
      const double DUmag = sqrt(DUprime * DUprime + DVprime * DVprime);
      double Tkeb = kTkeMin, Epsb = kEpsMin;
      if (!(DUmag / Dc < (double)1.e-6f)) {
        const double Dz1 = 0.5 * Dc * dsig[KB] / Abot;
        double Cdrag;
        if (S.ibot == 1) Cdrag = S.cd0;
        else {
          const double t = kKappa / log(Dz1 / (S.zob / 30.0));
          Cdrag = t * t;
        }
        Cdrag = dmin_(Cdrag, (cmu + cmuR + at(S.CmuVt, KB)) / Dz1 / (DUmag + kSmall) * Dc);
        const double Ustar = sqrt(Cdrag) * DUmag / Dc;
        Tkeb = dmax_(Ustar * Ustar / sqrt(cmiu), kTkeMin);
        Epsb = dmax_(Ustar * Ustar * Ustar / (kKappa * Dz1), kEpsMin);
      }
      const T tb = (T)(Dc * Tkeb), eb = (T)(Dc * Epsb);
      for (int k = 0; k <= NG; ++k) {
        S.DTke[ob - S.sz * k] = tb;
        S.DEps[ob - S.sz * k] = eb;
      }
    }
    // surface: gradient condition (Derakhti et al. 2015, eq. 60) with the
    // limited slopes of the surface values
    if (!(mk == 0 || Dc < Dmin)) {
      auto tsl = [&](const double* top, bool y) {
        const long long st = y ? S.sy : 1;
        const double h = y ? S.dy : S.dx;
        return lim_slope<double>(top[q - st], top[q], top[q + st], h, h);
      };
      const double gK = dxe * tsl(S.keTopK, false) + dye * tsl(S.keTopK, true);
      const double gE = dxe * tsl(S.keTopE, false) + dye * tsl(S.keTopE, true);
      const double Atop = sqrt(1.0 + dxe * dxe + dye * dye);
      for (int k = 1; k <= NG; ++k) {
        const double f = (sigc[KE + k] - sigc[KE - k + 1]) * (Dc * Dc) / (Atop * Atop);
        S.DTke[i3(S, i, j, KE + k)] = (T)(at(S.DTke, KE - k + 1) + f * gK);
        S.DEps[i3(S, i, j, KE + k)] = (T)(at(S.DEps, KE - k + 1) + f * gE);
      }
    }
  }
};

// wall function of a friction wall (BC = 5) at one cell (src/nhwave.F:
// 10870-11023): u* from the drag coefficient (Ibot 1) or the log law at
// half a cell width h/2 (Ibot 2)
template <class T>
__device__ inline void ke_wall(const Dev<T>& S, int i, int j, int k, double Umag, double h) {
  const double cmiu = S.ke_rng ? (double)0.085f : (double)0.09f;
  double Tkeb = kTkeMin, Epsb = kEpsMin;
  if (!(Umag < (double)1.e-6f)) {
    const double FricU = S.ibot == 1 ? sqrt(S.cd0) * Umag : Umag / (1.0 / kKappa * log(30.0 * h / 2.0 / S.zob));
    Tkeb = FricU * FricU / sqrt(cmiu);
    Epsb = FricU * FricU * FricU / (kKappa * h / 2.0);
  }
  const double Dq = S.D[i2(S, i, j)];
  S.DTke[i3(S, i, j, k)] = (T)(Dq * Tkeb);
  S.DEps[i3(S, i, j, k)] = (T)(Dq * Epsb);
}
// west and east sides: one thread per interior row and level (every level)
struct OpKeSidesX {
  static constexpr const char* kName = "ke_sides_x";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int t, int, int) const {
    const int j = S.JB + t % S.N, k = t / S.N;
    auto speed = [&](int i) {
      const long long o = i3(S, i, j, k);
      return sqrt((double)S.V[o] * (double)S.V[o] + (double)S.W[o] * (double)S.W[o]);
    };
    auto mirror = [&](int lo, int sgn) {   // DTke(lo - sgn g) = DTke(lo + sgn (g - 1))
      for (int g = 1; g <= NG; ++g) {
        const long long d = i3(S, lo - sgn * g, j, k), s = i3(S, lo + sgn * (g - 1), j, k);
        S.DTke[d] = S.DTke[s];
        S.DEps[d] = S.DEps[s];
      }
    };
    if (S.bc_x0 == 5) ke_wall(S, S.IB, j, k, speed(S.IB), S.dx);
    mirror(S.IB, 1);
    if (S.bc_xn == 5) ke_wall(S, S.IE, j, k, speed(S.IE), S.dx);
    mirror(S.IE, -1);
  }
};
// south and north sides: one thread per column i (ghosts included) and level
struct OpKeSidesY {
  static constexpr const char* kName = "ke_sides_y";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int t, int, int) const {
    const int i = t % S.Mloc, k = t / S.Mloc;
    auto speed = [&](int j) {
      const long long o = i3(S, i, j, k);
      return sqrt((double)S.U[o] * (double)S.U[o] + (double)S.W[o] * (double)S.W[o]);
    };
    auto mirror = [&](int lo, int sgn) {
      for (int g = 1; g <= NG; ++g) {
        const long long d = i3(S, i, lo - sgn * g, k), s = i3(S, i, lo + sgn * (g - 1), k);
        S.DTke[d] = S.DTke[s];
        S.DEps[d] = S.DEps[s];
      }
    };
    if (S.bc_y0 == 5) ke_wall(S, i, S.JB, k, speed(S.JB), S.dy);
    mirror(S.JB, 1);
    if (S.bc_yn == 5) ke_wall(S, i, S.JE, k, speed(S.JE), S.dy);
    mirror(S.JE, -1);
  }
};
// tke, epsilon and CmuVt = cmiu k^2 / eps in every cell (Cmut_min where k or
// eps is below 1e-6, and in shallow or dry columns, which are reset to the
// floors); CmuVt's ghost levels copy the outermost interior ones; the
// source region of an INT_, LEF_ or FOCUSED maker is reset too
// (src/nhwave.F:11039-11100)
struct OpKeFinal {
  static constexpr const char* kName = "ke_update";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j) const {
    const long long q = i2(S, i, j);
    const double Dq = S.D[q];
    const double cmiu = S.ke_rng ? (double)0.085f : (double)0.09f;
    const bool wet = Dq >= S.ke_dmin && S.Mask[q] == 1;
    const bool quiet = S.ke_quiet && S.xc[i] >= S.wm_xw && S.xc[i] <= S.wm_xe && S.yc[j] >= S.wm_ys && S.yc[j] <= S.wm_yn;
    for (int k = 0; k < S.Kloc; ++k) {
      const long long o = q + S.sz * k;
      if (wet) {
        const T tk = (T)((double)S.DTke[o] / Dq), ep = (T)((double)S.DEps[o] / Dq);
        S.Tke[o] = tk;
        S.Eps[o] = ep;
        const double a = (double)tk, b = (double)ep;
        S.CmuVt[o] = (a < (double)1.e-6f || b < (double)1.e-6f) ? (T)S.v_cmut0 : (T)(cmiu * (a * a) / b);
      } else {
        S.Tke[o] = (T)kTkeMin;
        S.Eps[o] = (T)kEpsMin;
        S.DTke[o] = (T)(Dq * kTkeMin);
        S.DEps[o] = (T)(Dq * kEpsMin);
        S.CmuVt[o] = (T)S.v_cmut0;
      }
    }
    for (int g = 1; g <= NG; ++g) {
      S.CmuVt[q + S.sz * (S.KB - g)] = S.CmuVt[q + S.sz * S.KB];
      S.CmuVt[q + S.sz * (S.KE + g)] = S.CmuVt[q + S.sz * S.KE];
    }
    if (quiet)
      for (int k = 0; k < S.Kloc; ++k) {
        const long long o = q + S.sz * k;
        S.Tke[o] = (T)kTkeMin;
        S.Eps[o] = (T)kEpsMin;
        S.DTke[o] = (T)(Dq * kTkeMin);
        S.DEps[o] = (T)(Dq * kEpsMin);
        S.CmuVt[o] = (T)S.v_cmut0;
      }
  }
};

// =========================================================================
//   Smagorinsky LES closure, IVTURB = 20 (les_3D, src/nhwave.F:8545-8729)
// =========================================================================
// CmuVt = (Cvs Delta)^2 sqrt(2 SijSij), Delta = (dx dy dsig D)^(1/3), in wet
// cells deeper than 0.02 m (others keep their value); the bed's wall
// function; mirrors; no eddy viscosity at the first column of a LEF_ maker
// or (in OpTurbV) in an INT_ maker's source region.  pow, log and exp are
// CUDA's, whose last bit may differ from the host libm's.  The smooth-wall
// iteration stops after kLesIter steps (the reference iterates until it
// converges).
constexpr int kLesIter = 200;
struct OpLesCell {
  static constexpr const char* kName = "les_cells";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j, int k) const {
    const long long q = i2(S, i, j), o = i3(S, i, j, k);
    const double Dq = S.D[q];
    if (!(S.Mask9[q] == 1 && Dq > (double)0.02f)) return;
    double sx = 0.0, sy = 0.0;   // DelxSc, DelySc of the last sigma_transform
    if (S.sc->sig_set) {
      sx = (1.0 - S.sigc[k]) / S.scD[q] * S.scHx[q] - S.sigc[k] / S.scD[q] * S.scEx[q];
      sy = (1.0 - S.sigc[k]) / S.scD[q] * S.scHy[q] - S.sigc[k] / S.scD[q] * S.scEy[q];
    }
    auto U = [&](long long x) { return (double)S.U[x]; };
    auto V = [&](long long x) { return (double)S.V[x]; };
    auto W = [&](long long x) { return (double)S.W[x]; };
    const long long up = o + S.sz, dn = o - S.sz, e = o + 1, w = o - 1, n = o + S.sy, s = o - S.sy;
    const double ds = S.sigc[k + 1] - S.sigc[k - 1];
    const double dUs = (U(up) - U(dn)) / ds, dVs = (V(up) - V(dn)) / ds, dWs = (W(up) - W(dn)) / ds;
    const double S11 = (U(e) - U(w)) / (2.0 * S.dx) + dUs * sx;
    const double S22 = (V(n) - V(s)) / (2.0 * S.dy) + dVs * sy;
    const double S33 = 1.0 / Dq * (W(up) - W(dn)) / ds;
    const double S12 = 0.5 * ((U(n) - U(s)) / (2.0 * S.dy) + dUs * sy + (V(e) - V(w)) / (2.0 * S.dx) + dVs * sx);
    const double S13 = 0.5 * (dUs / Dq + (W(e) - W(w)) / (2.0 * S.dx) + dWs * sx);
    const double S23 = 0.5 * (dVs / Dq + (W(n) - W(s)) / (2.0 * S.dy) + dWs * sy);
    const double SijSij = S11 * S11 + S22 * S22 + S33 * S33 + 2.0 * (S12 * S12 + S13 * S13 + S23 * S23);
    const double Filter = pow(S.dx * S.dy * S.dsig[k] * Dq, (double)(1.0f / 3.0f));
    const double cf = S.v_cvs * Filter;
    S.CmuVt[o] = (T)(cf * cf * sqrt(2.0 * SijSij));
  }
};
// the bed's wall function and the bed / surface ghosts of one interior column
struct OpLesColumn {
  static constexpr const char* kName = "les_bed";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j) const {
    const long long q = i2(S, i, j), ob = i3(S, i, j, S.KB);
    const double kap = (double)0.41f, cmu = S.v_cmu;
    const double u = (double)S.U[ob], v = (double)S.V[ob];
    const double Umag = sqrt(u * u + v * v);
    double cb;
    if (Umag < (double)1.e-6f) {
      cb = cmu;
    } else {
      const double Zdis = 0.5 * S.dsig[S.KB] * S.D[q];
      double FricU;
      if (S.zob >= (double)0.1f) {
        FricU = Umag / ((double)(1.0f / 0.41f) * log(30.0 * Zdis / S.zob));
      } else {
        double X0 = (double)0.05f, Xn = X0;
        const double Xa = log(9.0 * Umag * Zdis / cmu);
        for (int it = 0; it < kLesIter; ++it) {
          Xn = X0 + (kap - X0 * (Xa + log(X0))) / (1.0 + kap / X0);
          if (!(fabs((Xn - X0) / X0) > (double)1.e-8f && Xn > 0.0)) break;
          X0 = Xn;
        }
        FricU = Xn * Umag;
      }
      const double e = 1.0 - exp(-Zdis * FricU / cmu / 19.0);
      cb = kap * Zdis * FricU * (e * e);
    }
    T* c = S.CmuVt;
    c[ob] = (T)cb;
    for (int g = 1; g <= NG; ++g) {
      c[ob - S.sz * g] = c[ob + S.sz * (g - 1)];
      c[i3(S, i, j, S.KE + g)] = c[i3(S, i, j, S.KE - g + 1)];
    }
  }
};
// the side mirrors: y = 0 the west and east sides (interior rows and
// levels; the west first zeroes the first column of a LEF_ maker), y = 1
// the south and north sides (interior columns and levels), launched after,
// as the reference's loops run
struct OpLesSides {
  static constexpr const char* kName = "les_sides";
  int y;
  template <class T>
  __device__ void operator()(const Dev<T>& S, int t, int, int) const {
    T* c = S.CmuVt;
    if (!y) {
      const int j = S.JB + t % S.N, k = S.KB + t / S.N;
      if (S.les_lef) c[i3(S, S.IB, j, k)] = (T)0;
      for (int g = 1; g <= NG; ++g) c[i3(S, S.IB - g, j, k)] = c[i3(S, S.IB + g - 1, j, k)];
      for (int g = 1; g <= NG; ++g) c[i3(S, S.IE + g, j, k)] = c[i3(S, S.IE - g + 1, j, k)];
    } else {
      const int i = S.IB + t % S.M, k = S.KB + t / S.M;
      for (int g = 1; g <= NG; ++g) c[i3(S, i, S.JB - g, k)] = c[i3(S, i, S.JB + g - 1, k)];
      for (int g = 1; g <= NG; ++g) c[i3(S, i, S.JE + g, k)] = c[i3(S, i, S.JE - g + 1, k)];
    }
  }
};

// =========================================================================
//   2-D k-epsilon closure, IVTURB = 3 (kepsilon, src/nhwave.F:11117-11524)
// =========================================================================
// Production from the vertical shear, CmuVt (U_z^2 + V_z^2); the HLPA
// residual of kepsilon_3D; plain implicit vertical diffusion; the bed's
// smooth-wall friction velocity (the bounded iteration of les_3D); mirrors;
// the floors in the first six columns of a LEF_ maker and in an INT_ maker's
// source region.  Shallow means D < 0.01 m here.
constexpr double kKe2Dmin = (double)0.01f;
struct OpKe2Column {
  static constexpr const char* kName = "kepsilon2d_column";
  static constexpr int kMaxK = 64;   // Kglob <= 64 (nhw_create)
  int istep;                         // 0-based stage
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j) const {
    const long long q = i2(S, i, j);
    const double Dc = S.D[q], Dmin = kKe2Dmin, dt = S.sc->dt, cmu = S.v_cmu;
    const int mk = S.Mask[q];
    const double c1e = (double)1.44f, c2e = (double)1.92f, c3e = 0.0, cmiu = (double)0.09f;
    const double Sche = (double)1.3f, Schk = 1.0, Prod_b = 0.0;
    const bool rng = S.ke_rng != 0;   // adv_scalar_hlpa's Schmidt numbers follow RNG
    const int KB = S.KB, KE = S.KE, n = KE - KB + 1;
    const double* dsig = S.dsig;
    auto at = [&](const T* a, int kk) -> double { return (double)a[i3(S, i, j, kk)]; };
    double prod[kMaxK];
    for (int k = KB; k <= KE; ++k) {
      double P = 0.0;
      if (Dc >= Dmin && mk == 1) {
        const double ds = S.sigc[k + 1] - S.sigc[k - 1];
        const double uz = (at(S.U, k + 1) - at(S.U, k - 1)) / ds / Dc;
        const double vz = (at(S.V, k + 1) - at(S.V, k - 1)) / ds / Dc;
        P = at(S.CmuVt, k) * (uz * uz + vz * vz);
      }
      prod[k - KB] = P;
    }
    double A[kMaxK], B[kMaxK], C[kMaxK], X[kMaxK];
    auto column = [&](int eq) {
      const T* Old = eq == 2 ? S.Eps : S.Tke;
      T* Dv = eq == 2 ? S.DEps : S.DTke;
      const double Sch = eq == 2 ? Sche : Schk;
      const double SchtH = rng ? (double)0.72f : (eq == 2 ? (double)1.3f : 1.0);
      for (int k = KB; k <= KE; ++k) {
        const int m = k - KB;
        double r = ke_r5(S, i, j, k, Old, SchtH);
        if (eq == 2) r = r + c1e * Dc * (prod[m] + c3e * Prod_b) * at(S.Eps, k) / at(S.Tke, k);
        else r = r + Dc * (prod[m] + Prod_b) - at(S.DEps, k);
        A[m] = k == KB ? 0.0
                       : -dt / (Dc * Dc) * (0.5 * (cmu + cmu) + 0.5 * (at(S.CmuVt, k - 1) + at(S.CmuVt, k)) / Sch) /
                             (0.5 * dsig[k] * (dsig[k] + dsig[k - 1]));
        C[m] = k == KE ? 0.0
                       : -dt / (Dc * Dc) * (0.5 * (cmu + cmu) + 0.5 * (at(S.CmuVt, k) + at(S.CmuVt, k + 1)) / Sch) /
                             (0.5 * dsig[k] * (dsig[k] + dsig[k + 1]));
        B[m] = 1.0 - A[m] - C[m];
        if (eq == 2) B[m] = B[m] + dt * c2e * at(S.Eps, k) / at(S.Tke, k);
        X[m] = at(Dv, k) + dt * r;
      }
      for (int m = 1; m < n; ++m) {   // trig (src/nhwave.F:13182-13224)
        const double coeff = A[m] / B[m - 1];
        B[m] = B[m] - coeff * C[m - 1];
        X[m] = X[m] - coeff * X[m - 1];
      }
      X[n - 1] = X[n - 1] / B[n - 1];
      for (int m = n - 2; m >= 0; --m) X[m] = (X[m] - C[m] * X[m + 1]) / B[m];
      for (int k = KB; k <= KE; ++k) Dv[i3(S, i, j, k)] = (T)X[k - KB];
    };
    auto rk = [&](T* Dv, const T* Dv0, double vmin) {
      if (!(Dc >= Dmin && mk == 1)) return;
      const double al = S.alpha[istep], be = S.beta[istep];
      for (int k = KB; k <= KE; ++k) {
        const long long o = i3(S, i, j, k);
        const double v = al * (double)Dv0[o] + be * (double)Dv[o];
        Dv[o] = (T)dmax_(v, Dc * vmin);
      }
    };
    const bool solve = !(Dc < Dmin && mk == 0);
    if (solve) column(2);
    rk(S.DEps, S.DEps0, kEpsMin);
    if (solve) column(1);
    rk(S.DTke, S.DTke0, kTkeMin);
    // bed: smooth-wall law (columns with a bed velocity, deep enough and wet)
    const double ub = at(S.U, KB), vb = at(S.V, KB);
    const double Umag = sqrt(ub * ub + vb * vb);
    if (!(Umag < (double)1.e-6f || Dc < Dmin || mk == 0)) {
      const double kap = (double)0.41f;
      const double Zdis = 0.5 * dsig[KB] * Dc;
      double X0 = (double)0.05f, Xn = X0;
      const double Xa = log(9.0 * Umag * Zdis / cmu);
      for (int it = 0; it < kLesIter; ++it) {
        Xn = X0 + (kap - X0 * (Xa + log(X0))) / (1.0 + kap / X0);
        if (!(fabs((Xn - X0) / X0) > (double)1.e-8f && Xn > 0.0)) break;
        X0 = Xn;
      }
      const double FricU = Xn * Umag;
      const long long ob = i3(S, i, j, KB);
      S.DTke[ob] = (T)(Dc * (FricU * FricU / sqrt(cmiu)));
      S.DEps[ob] = (T)(Dc * (FricU * FricU * FricU / (kKappa * Zdis)));
      for (int g = 1; g <= NG; ++g) {
        S.DTke[ob - S.sz * g] = S.DTke[ob + S.sz * (g - 1)];
        S.DEps[ob - S.sz * g] = S.DEps[ob + S.sz * (g - 1)];
      }
    }
    for (int g = 1; g <= NG; ++g) {   // surface
      const long long d = i3(S, i, j, KE + g), s = i3(S, i, j, KE - g + 1);
      S.DTke[d] = S.DTke[s];
      S.DEps[d] = S.DEps[s];
    }
  }
};
// sides: y = 0 west (after the floors in the first six columns of a LEF_
// maker) and east, one thread per interior row and level; y = 1 south and
// north, one thread per interior column and level, launched after
struct OpKe2Sides {
  static constexpr const char* kName = "kepsilon2d_sides";
  int y;
  template <class T>
  __device__ void operator()(const Dev<T>& S, int t, int, int) const {
    auto mir = [&](long long d, long long s) {
      S.DTke[d] = S.DTke[s];
      S.DEps[d] = S.DEps[s];
    };
    if (!y) {
      const int j = S.JB + t % S.N, k = S.KB + t / S.N;
      if (S.les_lef)
        for (int i = S.IB; i <= S.IB + 5 && i < S.Mloc; ++i) {
          const long long o = i3(S, i, j, k);
          const double Dq = S.D[i2(S, i, j)];
          S.Tke[o] = (T)kTkeMin;
          S.Eps[o] = (T)kEpsMin;
          S.DTke[o] = (T)(Dq * kTkeMin);
          S.DEps[o] = (T)(Dq * kEpsMin);
          S.CmuVt[o] = (T)S.v_cmut0;
        }
      for (int g = 1; g <= NG; ++g) mir(i3(S, S.IB - g, j, k), i3(S, S.IB + g - 1, j, k));
      for (int g = 1; g <= NG; ++g) mir(i3(S, S.IE + g, j, k), i3(S, S.IE - g + 1, j, k));
    } else {
      const int i = S.IB + t % S.M, k = S.KB + t / S.M;
      for (int g = 1; g <= NG; ++g) mir(i3(S, i, S.JB - g, k), i3(S, i, S.JB + g - 1, k));
      for (int g = 1; g <= NG; ++g) mir(i3(S, i, S.JE + g, k), i3(S, i, S.JE - g + 1, k));
    }
  }
};
// tke, epsilon and CmuVt = cmiu k^2 / eps in every cell (the floors in
// shallow or dry columns), then an INT_ maker's source region at the floors
struct OpKe2Final {
  static constexpr const char* kName = "kepsilon2d_update";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j) const {
    const long long q = i2(S, i, j);
    const double Dq = S.D[q], cmiu = (double)0.09f;
    const bool wet = Dq >= kKe2Dmin && S.Mask[q] == 1;
    const bool quiet = S.les_int && S.xc[i] >= S.wm_xw && S.xc[i] <= S.wm_xe && S.yc[j] >= S.wm_ys && S.yc[j] <= S.wm_yn;
    for (int k = 0; k < S.Kloc; ++k) {
      const long long o = q + S.sz * k;
      if (wet && !quiet) {
        const T tk = (T)((double)S.DTke[o] / Dq), ep = (T)((double)S.DEps[o] / Dq);
        S.Tke[o] = tk;
        S.Eps[o] = ep;
        S.CmuVt[o] = (T)(cmiu * ((double)tk * (double)tk) / (double)ep);
      } else {
        S.Tke[o] = (T)kTkeMin;
        S.Eps[o] = (T)kEpsMin;
        S.DTke[o] = (T)(Dq * kTkeMin);
        S.DEps[o] = (T)(Dq * kEpsMin);
        S.CmuVt[o] = (T)S.v_cmut0;
      }
    }
  }
};

// =========================================================================
//   dynamic Smagorinsky LES, IVTURB = 30 (les_dyn, src/nhwave.F:7989-8542)
// =========================================================================
// Scratch fields of n3 cells each, from S.ld: 0-5 Sij (S11 S22 S33 S12 S23
// S13), 6 |S| = sqrt(2 SijSij), 7-12 the test-filtered |S|Sij, 13-18
// filtered Sij, 19 filtered |S|, 20-25 filtered u_i u_j (uu vv ww uv vw uw),
// 26-28 filtered u_i, 29 the clipped coefficient, 30 its smoothed value.
// Every kernel writes every cell it owns (zero where the reference leaves
// zero); ghosts then follow the reference's mirror loops.
constexpr double kLdDmin = (double)0.02f;
template <class T>
__device__ __forceinline__ T* ldf(const Dev<T>& S, int f) { return S.ld + S.ld_n * f; }
template <class T>
__device__ __forceinline__ bool ld_interior(const Dev<T>& S, int i, int j, int k) {
  return i >= S.IB && i <= S.IE && j >= S.JB && j <= S.JE && k >= S.KB && k <= S.KE;
}
// the strain rates of wet interior cells deeper than 0.02 m (zero elsewhere)
struct OpLdStrain {
  static constexpr const char* kName = "lesdyn_strain";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j, int k) const {
    const long long q = i2(S, i, j), o = i3(S, i, j, k);
    double s[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    const double Dq = S.D[q];
    if (ld_interior(S, i, j, k) && S.Mask[q] == 1 && Dq > kLdDmin) {
      double sx = 0.0, sy = 0.0;
      if (S.sc->sig_set) {
        sx = (1.0 - S.sigc[k]) / S.scD[q] * S.scHx[q] - S.sigc[k] / S.scD[q] * S.scEx[q];
        sy = (1.0 - S.sigc[k]) / S.scD[q] * S.scHy[q] - S.sigc[k] / S.scD[q] * S.scEy[q];
      }
      auto U = [&](long long x) { return (double)S.U[x]; };
      auto V = [&](long long x) { return (double)S.V[x]; };
      auto W = [&](long long x) { return (double)S.W[x]; };
      const long long up = o + S.sz, dn = o - S.sz, e = o + 1, w = o - 1, n = o + S.sy, so = o - S.sy;
      const double ds = S.sigc[k + 1] - S.sigc[k - 1];
      const double dUs = (U(up) - U(dn)) / ds, dVs = (V(up) - V(dn)) / ds, dWs = (W(up) - W(dn)) / ds;
      s[0] = (U(e) - U(w)) / (2.0 * S.dx) + dUs * sx;
      s[1] = (V(n) - V(so)) / (2.0 * S.dy) + dVs * sy;
      s[2] = 1.0 / Dq * (W(up) - W(dn)) / ds;
      s[3] = 0.5 * ((U(n) - U(so)) / (2.0 * S.dy) + dUs * sy + (V(e) - V(w)) / (2.0 * S.dx) + dVs * sx);
      s[4] = 0.5 * (dVs / Dq + (W(n) - W(so)) / (2.0 * S.dy) + dWs * sy);
      s[5] = 0.5 * (dUs / Dq + (W(e) - W(w)) / (2.0 * S.dx) + dWs * sx);
    }
    for (int c = 0; c < 6; ++c) ldf(S, c)[o] = (T)s[c];
  }
};
// ghost mirrors of scratch fields [f0, f1) (f0 < 0: CmuVt) along one group
// of lines: grp 0 the bed then the surface of an interior column, 1 the
// west then the east side of an interior row and level, 2 the south then
// (north_all, or the last field alone) the north side of an interior column
// and level -- each line in the reference's order
struct OpLdMirror {
  static constexpr const char* kName = "lesdyn_mirror";
  int grp, f0, f1, north_all;
  template <class T>
  __device__ void operator()(const Dev<T>& S, int t, int, int) const {
    const int fa = f0 < 0 ? 0 : f0, fb = f0 < 0 ? 1 : f1;
    for (int f = fa; f < fb; ++f) {
      T* a = f0 < 0 ? S.CmuVt : ldf(S, f);
      if (grp == 0) {
        const int i = S.IB + t % S.M, j = S.JB + t / S.M;
        for (int g = 1; g <= NG; ++g) a[i3(S, i, j, S.KB - g)] = a[i3(S, i, j, S.KB + g - 1)];
        for (int g = 1; g <= NG; ++g) a[i3(S, i, j, S.KE + g)] = a[i3(S, i, j, S.KE - g + 1)];
      } else if (grp == 1) {
        const int j = S.JB + t % S.N, k = S.KB + t / S.N;
        for (int g = 1; g <= NG; ++g) a[i3(S, S.IB - g, j, k)] = a[i3(S, S.IB + g - 1, j, k)];
        for (int g = 1; g <= NG; ++g) a[i3(S, S.IE + g, j, k)] = a[i3(S, S.IE - g + 1, j, k)];
      } else {
        const int i = S.IB + t % S.M, k = S.KB + t / S.M;
        for (int g = 1; g <= NG; ++g) a[i3(S, i, S.JB - g, k)] = a[i3(S, i, S.JB + g - 1, k)];
        if (north_all || f == fb - 1)
          for (int g = 1; g <= NG; ++g) a[i3(S, i, S.JE + g, k)] = a[i3(S, i, S.JE - g + 1, k)];
      }
    }
  }
};
// |S| in every cell deeper than 0.02 m (zero elsewhere)
struct OpLdSab {
  static constexpr const char* kName = "lesdyn_sab";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j, int k) const {
    const long long o = i3(S, i, j, k);
    double v = 0.0;
    if (S.D[i2(S, i, j)] > kLdDmin) {
      double s[6];
      for (int c = 0; c < 6; ++c) s[c] = (double)ldf(S, c)[o];
      const double a = s[0] * s[0] + s[1] * s[1] + s[2] * s[2] + 2.0 * (s[3] * s[3] + s[4] * s[4] + s[5] * s[5]);
      v = sqrt(2.0 * a);
    }
    ldf(S, 6)[o] = (T)v;
  }
};
// the separable [1 w 1] filter of src/nhwave.F:8412-8452 at an interior
// cell, in the reference's order: x sums, then y, then z, times fact
template <class F>
__device__ __forceinline__ double ld_filter_at(F P, int i, int j, int k, double w, double fact) {
  auto s1 = [&](int jj, int kk) { return P(i - 1, jj, kk) + w * P(i, jj, kk) + P(i + 1, jj, kk); };
  auto s2 = [&](int kk) { return s1(j - 1, kk) + w * s1(j, kk) + s1(j + 1, kk); };
  return fact * (s2(k - 1) + w * s2(k) + s2(k + 1));
}
// the 22 test-filtered fields (weit 2, fact 1/64) at interior cells, zero
// elsewhere; |S|Sij is zero where D <= 0.02 m
struct OpLdFilter {
  static constexpr const char* kName = "lesdyn_filter";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j, int k) const {
    const long long o = i3(S, i, j, k);
    if (!ld_interior(S, i, j, k)) {
      for (int f = 7; f <= 28; ++f) ldf(S, f)[o] = (T)0;
      return;
    }
    const double fact = 1.0 / 64.0;
    for (int f = 7; f <= 28; ++f) {
      auto P = [&](int ii, int jj, int kk) -> double {
        const long long x = i3(S, ii, jj, kk);
        if (f <= 12) return S.D[i2(S, ii, jj)] > kLdDmin ? (double)ldf(S, 6)[x] * (double)ldf(S, f - 7)[x] : 0.0;
        if (f <= 18) return (double)ldf(S, f - 13)[x];
        if (f == 19) return (double)ldf(S, 6)[x];
        const double u = (double)S.U[x], v = (double)S.V[x], ww = (double)S.W[x];
        switch (f) {
          case 20: return u * u;
          case 21: return v * v;
          case 22: return ww * ww;
          case 23: return u * v;
          case 24: return v * ww;
          case 25: return u * ww;
          case 26: return u;
          case 27: return v;
          default: return ww;
        }
      };
      ldf(S, f)[o] = (T)ld_filter_at(P, i, j, k, 2.0, fact);
    }
  }
};
// the coefficient -LijMij / (2 MijMij) / Delta^2, clipped to [0, 0.04], in
// every cell (Delta = (dx dy D dsig)^(1/3))
struct OpLdCoef {
  static constexpr const char* kName = "lesdyn_coef";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j, int k) const {
    const long long o = i3(S, i, j, k);
    const double Dq = S.D[i2(S, i, j)];
    auto F = [&](int f) { return (double)ldf(S, f)[o]; };
    double M[6], L[6];
    for (int n = 0; n < 6; ++n) M[n] = 4.0 * F(19) * F(13 + n) - F(7 + n);
    L[0] = F(20) - F(26) * F(26);
    L[1] = F(21) - F(27) * F(27);
    L[2] = F(22) - F(28) * F(28);
    L[3] = F(23) - F(26) * F(27);
    L[4] = F(24) - F(27) * F(28);
    L[5] = F(25) - F(28) * F(26);
    double MM = 0.0, LM = 0.0;
    if (Dq > kLdDmin) {
      MM = M[0] * M[0] + M[1] * M[1] + M[2] * M[2] + 2.0 * (M[3] * M[3] + M[4] * M[4] + M[5] * M[5]);
      LM = L[0] * M[0] + L[1] * M[1] + L[2] * M[2] + 2.0 * (L[3] * M[3] + L[4] * M[4] + L[5] * M[5]);
    }
    double c = 0.5 * (-LM) / (MM + (double)1.e-16f);
    const double FW = pow(S.dx * S.dy * Dq * S.dsig[k], (double)(1.0f / 3.0f));
    c = c / (FW * FW);
    if (c < 0.0) c = 0.0;
    if (c > (double)0.04f) c = (double)0.04f;
    ldf(S, 29)[o] = (T)c;
  }
};
// the coefficient smoothed (weit 1, fact 1/27) at interior cells, zero elsewhere
struct OpLdSmooth {
  static constexpr const char* kName = "lesdyn_smooth";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j, int k) const {
    const long long o = i3(S, i, j, k);
    if (!ld_interior(S, i, j, k)) {
      ldf(S, 30)[o] = (T)0;
      return;
    }
    auto P = [&](int ii, int jj, int kk) -> double { return (double)ldf(S, 29)[i3(S, ii, jj, kk)]; };
    ldf(S, 30)[o] = (T)ld_filter_at(P, i, j, k, 1.0, (double)(1.0f / 27.0f));
  }
};
// CmuVt = max(C Delta^2 |S|, 0) in interior cells deeper than 0.02 m, zero elsewhere
struct OpLdVisc {
  static constexpr const char* kName = "lesdyn_visc";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j, int k) const {
    const long long o = i3(S, i, j, k);
    const double Dq = S.D[i2(S, i, j)];
    double v = 0.0;
    if (ld_interior(S, i, j, k) && Dq > kLdDmin) {
      const double FW = pow(S.dx * S.dy * Dq * S.dsig[k], (double)(1.0f / 3.0f));
      v = dmax_((double)ldf(S, 30)[o] * (FW * FW) * (double)ldf(S, 6)[o], 0.0);
    }
    S.CmuVt[o] = (T)v;
  }
};

// Implicit vertical viscous step of eval_duvw (src/nhwave.F:690-822 DU,
// 850-1010 DV, 1012-1182 DW), one thread per wet interior column,
// after the new D, Eta and eta slopes: DU/DV/DW hold the explicit update
// DU + dt R2 on entry.  The tridiagonal systems are solved by trig's
// elimination (src/nhwave.F:13182-13224) in FP64, with the eliminated
// right-hand side kept in place (in T); the coefficients depend on the level
// only, so they are recomputed rather than stored.
struct OpVertVisc {
  static constexpr const char* kName = "vertical_viscous";
  static constexpr int kMaxK = 64;   // Kglob <= 64 (nhw_create)
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j) const {
    const long long c = i2(S, i, j);
    if (S.Mask[c] == 0) return;
    const int KB = S.KB, KE = S.KE, n = KE - KB + 1;
    const double dt = S.sc->dt, Dc = S.D[c];
    // CmuVt of level k and the face viscosity between levels k1 and k2
    auto vt = [&](int k) { return (double)S.CmuVt[i3(S, i, j, k)]; };
    auto nuz = [&](int k1, int k2) { return 0.5 * (S.v_cmu + S.v_cmu) + 0.5 * (vt(k1) + vt(k2)) / S.v_schmidt; };
    const double* dsg = S.dsig;
    auto A = [&](int k) {
      return k == KB ? 0.0 : -dt / (Dc * Dc) * nuz(k - 1, k) / (0.5 * dsg[k] * (dsg[k] + dsg[k - 1]));
    };
    auto C = [&](int k) {
      return k == KE ? 0.0 : -dt / (Dc * Dc) * nuz(k, k + 1) / (0.5 * dsg[k] * (dsg[k] + dsg[k + 1]));
    };
    const double Wbot = -S.DeltH[c] - (double)S.U[i3(S, i, j, KB)] * S.DelxH[c] - (double)S.V[i3(S, i, j, KB)] * S.DelyH[c];
    const double Wtop = (S.Eta[c] - S.Eta0[c]) / dt + (double)S.U[i3(S, i, j, KE)] * S.DelxEta[c] +
                        (double)S.V[i3(S, i, j, KE)] * S.DelyEta[c];
    double bp[kMaxK];   // eliminated diagonal; the eliminated right-hand side goes in place
    for (int which = 0; which < 3; ++which) {
      T* Fv = which == 0 ? S.DU : which == 1 ? S.DV : S.DW;
      auto coefs = [&](int k, double& b, double& r) {
        const double f = (double)Fv[i3(S, i, j, k)];
        if (which < 2) {
          if (k == KB && S.bc_z0 == 2)   // no-slip bed
            b = 1.0 - C(k) + dt / (Dc * Dc) * (S.v_cmu + 0.0 + vt(k) / S.v_schmidt) / (0.5 * dsg[k] * dsg[k]);
          else
            b = 1.0 - A(k) - C(k);
          if (k == KB && S.bc_z0 == 5) {   // friction law: bed stress in the first right-hand side
            const double Dz1 = 0.5 * Dc * dsg[KB];
            double Cdrag = S.cd0;
            if (S.ibot != 1) {
              const double lg = 1. / kKappa * log(30.0 * Dz1 / S.zob);
              Cdrag = 1. / (lg * lg);
            }
            const double u = (double)S.U[i3(S, i, j, k)], v = (double)S.V[i3(S, i, j, k)];
            const double Ustar2 = Cdrag * sqrt(u * u + v * v) * (which == 0 ? u : v);
            r = f - dt * Ustar2 / dsg[k];
          } else if (k == KE) {
            r = f + dt * (which == 0 ? S.Wsx[c] : S.Wsy[c]) / dsg[k];
          } else {
            r = f;
          }
        } else if (k == KB) {
          const double q = 0.25 * dsg[k] * (dsg[k] + dsg[k - 1]);
          b = 1.0 - C(k) + dt / (Dc * Dc) * nuz(k - 1, k) / q;
          r = f + dt / Dc * nuz(k - 1, k) / q * Wbot;
        } else if (k == KE) {
          const double q = 0.25 * dsg[k] * (dsg[k] + dsg[k + 1]);
          b = 1.0 - A(k) + dt / (Dc * Dc) * nuz(k, k + 1) / q;
          r = f + dt / Dc * nuz(k, k + 1) / q * Wtop;
        } else {
          b = 1.0 - A(k) - C(k);
          r = f;
        }
      };
      double rprev;
      coefs(KB, bp[0], rprev);
      Fv[i3(S, i, j, KB)] = (T)rprev;
      for (int q = 1; q < n; ++q) {
        double b, r;
        coefs(KB + q, b, r);
        const double coeff = A(KB + q) / bp[q - 1];
        bp[q] = b - coeff * C(KB + q - 1);
        rprev = r - coeff * rprev;
        Fv[i3(S, i, j, KB + q)] = (T)rprev;
      }
      double x = rprev / bp[n - 1];
      Fv[i3(S, i, j, KE)] = (T)x;
      for (int q = n - 2; q >= 0; --q) {
        x = ((double)Fv[i3(S, i, j, KB + q)] - C(KB + q) * x) / bp[q];
        Fv[i3(S, i, j, KB + q)] = (T)x;
      }
    }
  }
};

// initial: DU = D*U*Mask over all cells (src/initialize.F:3160-3170)
struct OpInitDU {
  static constexpr const char* kName = "init_du";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j, int k) const {
    const long long c = i2(S, i, j), o = i3(S, i, j, k);
    const double d = S.D[c], m = (double)S.Mask[c];
    S.DU[o] = (T)((double)(T)(d * (double)S.U[o]) * m);
    S.DV[o] = (T)((double)(T)(d * (double)S.V[o]) * m);
    S.DW[o] = (T)((double)(T)(d * (double)S.W[o]) * m);
    // viscous flow: the seeding viscosity Cmut_min, after vel_bc, which so
    // saw CmuVt = 0, and k-epsilon's seeds (src/initialize.F:3155, 3172-3195)
    if (S.CmuVt) S.CmuVt[o] = S.CmuHt[o] = (T)S.v_cmut0;
    if (S.Tke) {
      S.Tke[o] = (T)kTkeMin;
      S.Eps[o] = (T)kEpsMin;
      S.DTke[o] = (T)(d * kTkeMin * m);
      S.DEps[o] = (T)(d * kEpsMin * m);
      S.DTke0[o] = (T)0;
      S.DEps0[o] = (T)0;
    }
  }
};

// =========================================================================
//      Poisson: generate_coef_rhs (src/pressure.F:475-840), FP64
// =========================================================================
// per-column factors of the sigma transformation, used by the Poisson
// assembly and the projection: DelxS(k) = (1-sig_k) DelxH/D - sig_k DelxEta/D
struct OpColFactors {
  static constexpr const char* kName = "col_factors";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j) const {
    const long long q = i2(S, i, j);
    const double inv = 1.0 / S.D[q];
    S.cf_invD[q] = inv;
    S.cf_hx[q] = S.DelxH[q] * inv;
    S.cf_ex[q] = S.DelxEta[q] * inv;
    S.cf_hy[q] = S.DelyH[q] * inv;
    S.cf_ey[q] = S.DelyEta[q] * inv;
  }
};

struct OpPoissonCoef {
  static constexpr const char* kName = "poisson_coef";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j, int k) const {
    const int ic = ic_of(S, i, j, k);
    const long long sy = S.sy, sz = S.sz;
    auto inside = [&](int x, int y) { return x >= S.IB && x <= S.IE && y >= S.JB && y <= S.JE; };
    const double sgk = S.sig[k], omk = 1. - sgk;
    // DelxS/DelyS at level sig(k) of interior columns, zero outside (src/pressure.F:494-505)
    auto dxs = [&](int x, int y) -> double {
      if (!inside(x, y)) return 0.0;
      const long long q = i2(S, x, y);
      return omk * S.cf_hx[q] - sgk * S.cf_ex[q];
    };
    auto dys = [&](int x, int y) -> double {
      if (!inside(x, y)) return 0.0;
      const long long q = i2(S, x, y);
      return omk * S.cf_hy[q] - sgk * S.cf_ey[q];
    };
    const long long q = i2(S, i, j);
    const double DelxS = dxs(i, j), DelyS = dys(i, j), DelzS = S.cf_invD[q];
    const double A1 = DelxS * DelxS + DelyS * DelyS + DelzS * DelzS;
    const double lx = S.lv_x[k], ly = S.lv_y[k], ih = S.lv_h[k];
    // Rhs (src/pressure.F:521-525); Uf/Vf: linear interpolation to sig(k) (src/nhwave.F:1346-1355)
    const double dsk = S.dsig[k], dskm = S.dsig[k - 1];
    const double fint = S.lv_fint[k];   // dsk / (dsk + dskm)
    const long long o = i3(S, i, j, k);
    auto uf = [&](const T* A, long long e) -> double {
      return (1.0 - fint) * (double)A[e] + fint * (double)A[e - sz];
    };
    const double i2dx = S.i2dx, i2dy = S.i2dy;
    double rhs = -((uf(S.U, o + 1) - uf(S.U, o - 1)) * i2dx + ((double)S.U[o] - (double)S.U[o - sz]) * ih * DelxS +
                   (uf(S.V, o + sy) - uf(S.V, o - sy)) * i2dy + ((double)S.V[o] - (double)S.V[o - sz]) * ih * DelyS +
                   ((double)S.W[o] - (double)S.W[o - sz]) * ih * DelzS - S.SourceC[q]) *
                 S.sc->rho_dt;
    double C[NCOEF + 1];
    const double cxx = S.cxx, cyy = S.cyy;
    C[1] = -2. * cxx - 2. * cyy + A1 * S.lv_up[k] + A1 * S.lv_dn[k];
    C[2] = cxx;
    C[3] = cyy;
    C[4] = (dys(i, j - 1) + DelyS) * ly;
    C[5] = (dxs(i - 1, j) + DelxS) * lx;
    C[6] = -A1 * S.lv_up[k];
    C[7] = -(dxs(i + 1, j) + DelxS) * lx;
    C[8] = -(dys(i, j + 1) + DelyS) * ly;
    C[9] = cxx;
    C[10] = cyy;
    C[11] = -C[8];
    C[12] = -C[7];
    C[13] = -A1 * S.lv_dn[k];
    C[14] = -C[5];
    C[15] = -C[4];
    // boundary folds in the reference's order (src/pressure.F:649-814)
    if (i == S.IB) { C[1] = C[1] + C[9]; C[6] = C[6] + C[5]; C[13] = C[13] + C[14]; C[9] = C[5] = C[14] = 0.0; }
    if (i == S.IE) { C[1] = C[1] + C[2]; C[6] = C[6] + C[7]; C[13] = C[13] + C[12]; C[2] = C[7] = C[12] = 0.0; }
    if (j == S.JB) { C[1] = C[1] + C[10]; C[6] = C[6] + C[4]; C[13] = C[13] + C[15]; C[10] = C[4] = C[15] = 0.0; }
    if (j == S.JE) { C[1] = C[1] + C[3]; C[6] = C[6] + C[8]; C[13] = C[13] + C[11]; C[3] = C[8] = C[11] = 0.0; }
    if (k == S.KB) {
      if (S.slide) {
        const double* D = S.D;
        const double* H2 = S.Delt2H;
        rhs = rhs + kRho0 * (dsk + dskm) *
                        (C[13] * D[q] * H2[q] + C[12] * D[q + 1] * H2[q + 1] + C[11] * D[q + sy] * H2[q + sy] +
                         C[14] * D[q - 1] * H2[q - 1] + C[15] * D[q - sy] * H2[q - sy]);
      }
      C[6] = C[6] + C[13]; C[7] = C[7] + C[12]; C[8] = C[8] + C[11]; C[5] = C[5] + C[14]; C[4] = C[4] + C[15];
      C[13] = C[12] = C[11] = C[14] = C[15] = 0.0;
    }
    // compact form: C1, C6, C13 after every fold; the k+1 cross terms before
    // the top row's zeroing (their negatives are the k-1 terms of this cell)
    const size_t n = (size_t)S.neq;
    double* o7 = S.coef64 + ic;
    o7[3 * n] = C[4]; o7[4 * n] = C[5]; o7[5 * n] = C[7]; o7[6 * n] = C[8];
    if (k == S.KE) { C[4] = C[5] = C[6] = C[7] = C[8] = 0.0; }
    o7[0] = C[1]; o7[n] = C[6]; o7[2 * n] = C[13];
    S.rhs64[ic] = rhs;
  }
};

// copy of the FP64 operator into the inner precision (FP32 form only)
struct OpCoefToT {
  static constexpr const char* kName = "coef_to_inner";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j, int k) const {
    const int ic = ic_of(S, i, j, k);
    const size_t n = (size_t)S.neq;
    for (int m = 0; m < 7; ++m) S.coefT[m * n + ic] = (T)S.coef64[m * n + ic];
  }
};

// vertical-line preconditioner factors: tridiagonal (C13, C1, C6) per column
struct OpLineFactor {
  static constexpr const char* kName = "line_factor";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j) const {
    const size_t n = (size_t)S.neq, mn = (size_t)S.M * S.N;
    const size_t base = (size_t)(i - S.IB) + (size_t)S.M * (j - S.JB);
    // in the storage type: FP64 as before, FP32 in the FP32+IR form (the
    // factors are stored in FP32 there anyway)
    T cpm = (T)0;
    for (int k = 0; k < S.K; ++k) {
      const size_t ic = base + mn * k;
      const T a = k > 0 ? (T)S.coef64[2 * n + ic] : (T)0;
      const T b = (T)S.coef64[ic];
      const T c = k < S.K - 1 ? (T)S.coef64[n + ic] : (T)0;
      const T den = b - a * cpm;
      const T inv = (T)1 / den;
      cpm = c * inv;
      S.lcp[ic] = cpm;
      S.linv[ic] = inv;
      if (S.sp0) {   // colour-split copy for the level-0 half-sweeps (layout in mg.cuh, MGL::sp)
        const int ii = i - S.IB, jj = j - S.JB, Mh = (S.M + 1) >> 1;
        const size_t nmh = (size_t)Mh * S.N, cs = nmh * S.K;
        T* e = S.sp0 + (size_t)((ii + jj) & 1) * cs + nmh * k + (size_t)Mh * jj + (ii >> 1);
        e[0] = (T)a;
        e[2 * cs] = (T)inv;
        e[4 * cs] = (T)cpm;
        e[6 * cs] = (T)S.coef64[3 * n + ic];
        e[8 * cs] = (T)S.coef64[4 * n + ic];
        e[10 * cs] = (T)S.coef64[5 * n + ic];
        e[12 * cs] = (T)S.coef64[6 * n + ic];
      }
    }
  }
};

// P interior <- FP64 solution; lateral P ghosts (src/pressure.F:185-239)
struct OpPFromX {
  static constexpr const char* kName = "p_from_x";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j, int k) const {
    const int ic = ic_of(S, i, j, k);
    if (S.sc->zero_x) S.xsol64[ic] = 0.0;   // b = 0: HYPRE returns x = 0
    S.P[i3(S, i, j, k)] = S.xsol64[ic];
  }
};
struct OpXFromP {
  static constexpr const char* kName = "x_from_p";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j, int k) const {
    S.xsol64[ic_of(S, i, j, k)] = S.P[i3(S, i, j, k)];
  }
};
struct OpPGhost {
  static constexpr const char* kName = "p_ghost";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j) const {
    const bool ii = (i >= S.IB && i <= S.IE), jj = (j >= S.JB && j <= S.JE);
    if (ii == jj) return;  // interior or corner
    const int si = mirror(i, S.IB, S.IE), sj = mirror(j, S.JB, S.JE);
    for (int k = S.KB; k <= S.KE; ++k) S.P[i3(S, i, j, k)] = S.P[i3(S, si, sj, k)];
  }
};

// projection_corrector (src/nhwave.F:487-536)
struct OpProjection {
  static constexpr const char* kName = "projection";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j, int k) const {
    const long long q = i2(S, i, j);
    if (S.Mask[q] == 0) return;
    const long long o = i3(S, i, j, k), sy = S.sy, sz = S.sz;
    const double* P = S.P;
    const double i2dx = S.i2dx, i2dy = S.i2dy;
    const double DelxP = 0.5 * ((P[o + 1] - P[o - 1]) * i2dx + (P[o + 1 + sz] - P[o - 1 + sz]) * i2dx);
    const double DelyP = 0.5 * ((P[o + sy] - P[o - sy]) * i2dy + (P[o + sy + sz] - P[o - sy + sz]) * i2dy);
    const double DelzP = (P[o + sz] - P[o]) * S.lv_ds[k];
    const double sc = S.sigc[k], omc = 1.0 - sc;
    const double DelxSc = omc * S.cf_hx[q] - sc * S.cf_ex[q];
    const double DelySc = omc * S.cf_hy[q] - sc * S.cf_ey[q];
    const double g = S.sc->dt_rho, f = S.D[q] * g;   // dt / Rho0
    S.DU[o] = (T)((double)S.DU[o] - f * (DelxP + DelzP * DelxSc));
    S.DV[o] = (T)((double)S.DV[o] - f * (DelyP + DelzP * DelySc));
    S.DW[o] = (T)((double)S.DW[o] - g * DelzP);
  }
};
// The same in the FP32+IR form: the pressure differences in FP64 (P is FP64),
// each rounded once, and the rest in FP32
struct OpProjection32 {
  static constexpr const char* kName = "projection";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j, int k) const {
    const long long q = i2(S, i, j);
    if (S.Mask[q] == 0) return;
    const long long o = i3(S, i, j, k), sy = S.sy, sz = S.sz;
    const double* P = S.P;
    const T hx = (T)S.i2dx, hy = (T)S.i2dy;
    const T dx0 = (T)(P[o + 1] - P[o - 1]), dx1 = (T)(P[o + 1 + sz] - P[o - 1 + sz]);
    const T dy0 = (T)(P[o + sy] - P[o - sy]), dy1 = (T)(P[o + sy + sz] - P[o - sy + sz]);
    const T DelxP = (T)0.5 * (dx0 * hx + dx1 * hx), DelyP = (T)0.5 * (dy0 * hy + dy1 * hy);
    const T DelzP = (T)(P[o + sz] - P[o]) * S.lvT[k];
    const T sc = (T)S.sigc[k], omc = (T)1 - sc;
    const T DelxSc = omc * (T)S.cf_hx[q] - sc * (T)S.cf_ex[q];
    const T DelySc = omc * (T)S.cf_hy[q] - sc * (T)S.cf_ey[q];
    const T g = (T)S.sc->dt_rho, f = (T)S.D[q] * g;
    S.DU[o] = S.DU[o] - f * (DelxP + DelzP * DelxSc);
    S.DV[o] = S.DV[o] - f * (DelyP + DelzP * DelySc);
    S.DW[o] = S.DW[o] - g * DelzP;
  }
};

// SSP-RK combination, mask and Froude cap (src/nhwave.F:1227-1261)
struct OpSSP {
  static constexpr const char* kName = "ssp_combine";
  int istep;
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j, int k) const {
    using R = T;
    const long long q = i2(S, i, j), o = i3(S, i, j, k);
    const R al = (R)S.alpha[istep], be = (R)S.beta[istep];
    R du = al * S.DU0[o] + be * S.DU[o];
    R dv = al * S.DV0[o] + be * S.DV[o];
    R dw = al * S.DW0[o] + be * S.DW[o];
    const int m = S.Mask[q];
    if (m == 0) { du = (R)0; dv = (R)0; dw = (R)0; }
    if (S.froude_on && m > 0) {
      const double Dq = S.D[q];
      bool over;
      double FroudeU = 0.0;
      if constexpr (sizeof(R) == 4) {   // FP32+IR form: the test in FP32, the cap itself in FP64
        const R rD = (R)Dq;
        over = sqrt(du * du + dv * dv + dw * dw) > sqrt((R)kGrav * rD) * (R)S.froude_cap * rD;
        if (over) FroudeU = sqrt(kGrav * Dq) * S.froude_cap * Dq;
      } else {
        FroudeU = sqrt(kGrav * Dq) * S.froude_cap * Dq;
        const double a = (double)du, b = (double)dv, cc = (double)dw;
        over = sqrt(a * a + b * b + cc * cc) > FroudeU;
      }
      if (over) {
        const double ang = atan2((double)dv, (double)du);
        du = (R)(FroudeU * cos(ang));
        dv = (R)(FroudeU * sin(ang));
        dw = (R)0;
      }
    }
    S.DU[o] = du; S.DV[o] = dv; S.DW[o] = dw;
  }
};

// =========================================================================
//               get_Omega (src/nhwave.F:1411-1648)
// =========================================================================
struct OpOmegaX {
  static constexpr const char* kName = "omega_x";  // Ex on x faces from the new state; EtaxL/EtaxR kept for source_terms
  template <class T>
  __device__ void operator()(const Dev<T>& S, int f, int j, int k) const {
    using R = T;
    const int c0 = f - 1, c1 = f;
    const long long e0 = i3(S, c0, j, k), e1 = e0 + 1;
    const long long q0 = i2(S, c0, j), q1 = q0 + 1;
    const int mL = S.Mask[q0], mR = S.Mask[q1];
    const R hdx = S.hdxT, rdx = S.dxT, irdx = S.idxT;
    auto sl = [&](const T* A, long long e, int m) -> R {
      return m == 0 ? (R)0 : lim_slope_u<R>(A[e - 1], A[e], A[e + 1], rdx, irdx);
    };
    const R uL = S.U[e0] + hdx * sl(S.U, e0, mL), uR = S.U[e1] - hdx * sl(S.U, e1, mR);
    R duL = S.DU[e0] + hdx * sl(S.DU, e0, mL), duR = S.DU[e1] - hdx * sl(S.DU, e1, mR);
    R rdL, rdR, rdd;
    bool zl, zr;
    const bool inL = c0 >= S.IB && c0 <= S.IE, inR = c1 >= S.IB && c1 <= S.IE;
    if (face_table<R>(S)) {
      const long long n2 = face_slot(S);
      const T* ft = S.fxT + q1;
      rdL = ft[2 * n2]; rdR = ft[3 * n2]; rdd = ft[5 * n2];
      face_flags(S, q0, 1, inL, inR, zl, zr);
    } else {
      const Face2D F = face_2d(S, q0, 1, inL, inR, 0.5 * S.dx, S.DelxEta, S.Hfx, S.Hfx0);
      if (k == S.KB) { S.EtaxL[q1] = F.etaL; S.EtaxR[q1] = F.etaR; }
      rdL = (R)F.dL; rdR = (R)F.dR; rdd = (R)(F.dR - F.dL); zl = F.zl; zr = F.zr;
    }
    if (zl) duL = (R)0;
    if (zr) duR = (R)0;
    R SL = (R)0, SR = (R)0;
    if (mL == 1 && mR == 1) {
      R pL = sqrt((R)kGrav * fabs(rdL)), pR = sqrt((R)kGrav * fabs(rdR));
      R pS = (R)0.5 * (pL + pR) + (R)0.25 * (uL - uR);
      R uS = (R)0.5 * (uL + uR) + pL - pR;
      SL = rmin<R>(uL - pL, uS - pS);
      SR = rmax<R>(uR + pR, uS + pS);
    } else if (mL == 0 && mR == 1) {
      R pR = sqrt((R)kGrav * fabs(rdR));
      SL = uR - (R)2.0 * pR;
      SR = uR + pR;
    } else if (mL == 1 && mR == 0) {
      R pL = sqrt((R)kGrav * fabs(rdL));
      SL = uL - pL;
      SR = uL + (R)2.0 * pL;
    }
    R Ex = hll_d<R>(SL, SR, duL, duR, rdd);
    if (f == S.IB || (f == S.IE + 1 && S.bc_xn != 6)) Ex = (R)0;
    if (f == S.IB && S.bc_x0 == 3) Ex = (R)(S.Din[j] * S.Uin[j + S.Nloc * k]);   // src/nhwave.F:1564-1566
    if (f == S.IE + 1 && S.bc_xn == 3) Ex = (R)(S.Din_xn[j] * S.Uin_xn[j + S.Nloc * k]);   // :1580-1581
    S.Ex[i3(S, f, j, k)] = Ex;
  }
};
struct OpOmegaY {
  static constexpr const char* kName = "omega_y";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int g, int k) const {
    using R = T;
    const int c0 = g - 1, c1 = g;
    const long long sy = S.sy;
    const long long e0 = i3(S, i, c0, k), e1 = e0 + sy;
    const long long q0 = i2(S, i, c0), q1 = q0 + sy;
    const int mL = S.Mask[q0], mR = S.Mask[q1];
    const R hdy = S.hdyT, rdy = S.dyT, irdy = S.idyT;
    auto sl = [&](const T* A, long long e, int m) -> R {
      return m == 0 ? (R)0 : lim_slope_u<R>(A[e - sy], A[e], A[e + sy], rdy, irdy);
    };
    const R vL = S.V[e0] + hdy * sl(S.V, e0, mL), vR = S.V[e1] - hdy * sl(S.V, e1, mR);
    R dvL = S.DV[e0] + hdy * sl(S.DV, e0, mL), dvR = S.DV[e1] - hdy * sl(S.DV, e1, mR);
    R rdL, rdR, rdd;
    bool zl, zr;
    const bool inL = c0 >= S.JB && c0 <= S.JE, inR = c1 >= S.JB && c1 <= S.JE;
    if (face_table<R>(S)) {
      const long long n2 = face_slot(S);
      const T* ft = S.fyT + q1;
      rdL = ft[2 * n2]; rdR = ft[3 * n2]; rdd = ft[5 * n2];
      face_flags(S, q0, sy, inL, inR, zl, zr);
    } else {
      const Face2D F = face_2d(S, q0, sy, inL, inR, 0.5 * S.dy, S.DelyEta, S.Hfy, S.Hfy0);
      if (k == S.KB) { S.EtayL[q1] = F.etaL; S.EtayR[q1] = F.etaR; }
      rdL = (R)F.dL; rdR = (R)F.dR; rdd = (R)(F.dR - F.dL); zl = F.zl; zr = F.zr;
    }
    if (zl) dvL = (R)0;
    if (zr) dvR = (R)0;
    R SL = (R)0, SR = (R)0;
    if (mL == 1 && mR == 1) {
      R pL = sqrt((R)kGrav * fabs(rdL)), pR = sqrt((R)kGrav * fabs(rdR));
      R pS = (R)0.5 * (pL + pR) + (R)0.25 * (vL - vR);
      R uS = (R)0.5 * (vL + vR) + pL - pR;
      SL = rmin<R>(vL - pL, uS - pS);
      SR = rmax<R>(vR + pR, uS + pS);
    } else if (mL == 0 && mR == 1) {
      R pR = sqrt((R)kGrav * fabs(rdR));
      SL = vR - (R)2.0 * pR;
      SR = vR + pR;
    } else if (mL == 1 && mR == 0) {
      R pL = sqrt((R)kGrav * fabs(rdL));
      SL = vL - pL;
      SR = vL + (R)2.0 * pL;
    }
    R Ey = hll_d<R>(SL, SR, dvL, dvR, rdd);
    if (g == S.JB || g == S.JE + 1) Ey = (R)0;
    S.Ey[i3(S, i, g, k)] = Ey;
  }
};
// Omega column scan (src/nhwave.F:1617-1628)
struct OpOmegaScan {
  static constexpr const char* kName = "omega_scan";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j) const {
    const long long q = i2(S, i, j);
    const bool wet = S.Mask[q] != 0;
    const double r1 = S.R1[q];
    const double rdx = 2.0 * S.i2dx, rdy = 2.0 * S.i2dy;   // 1/dx, 1/dy
    double om = 0.0;
    S.Omega[i3(S, i, j, S.KB)] = (T)0;
    for (int k = S.KB + 1; k <= S.KE + 1; ++k) {
      const long long o = i3(S, i, j, k - 1);
      const double dEx = (double)S.Ex[o + 1] - (double)S.Ex[o];
      const double dEy = (double)S.Ey[o + S.sy] - (double)S.Ey[o];
      double v;
      if constexpr (sizeof(T) == 4) v = om - S.dsig[k - 1] * (r1 + dEx * rdx + dEy * rdy);   // FP32 form: products
      else v = om - S.dsig[k - 1] * (r1 + dEx / S.dx + dEy / S.dy);
      if (!wet) v = 0.0;
      S.Omega[i3(S, i, j, k)] = (T)v;
      om = (double)(T)v;
    }
  }
};

// sponge_damping over every wet cell of the ghosted array (src/nhwave.F:6463-6502)
struct OpSponge {
  static constexpr const char* kName = "sponge";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j) const {
    const long long c = i2(S, i, j);
    if (S.Mask[c] != 1) return;
    const double time = S.sc->time;
    const double Ramp = S.tramp > 0.0 ? tanh(time / S.tramp) : 1.0;
    const double Ucur = Ramp * S.cur_wave;
    const double sp = S.Sponge[c];
    S.Eta[c] = S.Eta[c] * sp;
    S.D[c] = S.Eta[c] + S.Hc[c];
    const double d = S.D[c];
    if constexpr (sizeof(T) == 4) {   // FP32 form: the 3-D part in FP32
      const T rsp = (T)sp, ruc = (T)Ucur, rd = (T)d;
      for (int k = 0; k < S.Kloc; ++k) {
        const long long o = i3(S, i, j, k);
        const T u = (S.U[o] - ruc) * rsp + ruc, v = S.V[o] * rsp;
        S.U[o] = u;
        S.V[o] = v;
        S.DU[o] = rd * u;
        S.DV[o] = rd * v;
      }
    } else {
      for (int k = 0; k < S.Kloc; ++k) {
        const long long o = i3(S, i, j, k);
        const double u = ((double)S.U[o] - Ucur) * sp + Ucur;
        const double v = (double)S.V[o] * sp;
        S.U[o] = (T)u;
        S.V[o] = (T)v;
        S.DU[o] = (T)(d * (double)(T)u);
        S.DV[o] = (T)(d * (double)(T)v);
      }
    }
  }
};

// =========================================================================
//                 estimate_dt (src/nhwave.F:3694-3874)
// =========================================================================
template <class T>
__global__ void __launch_bounds__(256) k_dt_min(Dev<T> S) {
  // One thread per water column.  D, hence sqrt(g D), is the column's, and
  // division is monotonic in the denominator, so the smallest dx/tmp1 of a
  // column is dx over its largest tmp1 -- the same value, bit for bit, with
  // two divisions and one square root per column instead of per cell.  The
  // vertical candidate dsig(k) D / max(|W|, Small) keeps one division per
  // cell.  A candidate replaces m only if it is smaller, as the reference's
  // `if(dxonu<tmp2) tmp2=dxonu` (src/nhwave.F:3730-3746): a NaN candidate
  // leaves m unchanged (tmp1 = max(NaN, Small) is Small, whose quotient is
  // never the minimum).  Viscous flow: the limit dx^2 / (|CmuHt| + 1e-16)
  // over the interior (src/nhwave.F:3812-3832) is, by the same monotonicity,
  // the one of the largest |CmuHt|, gathered as its bit pattern + 1 (0: no
  // finite value; NaN cells never give the minimum and are skipped).
  __shared__ double sh[8];
  __shared__ unsigned long long shh[8];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double m = kLarge;
  unsigned long long hb = 0ull;
  if (t < S.M * S.N && S.CmuHt) {
    const int i = S.IB + t % S.M, j = S.JB + t / S.M;
    for (int k = S.KB; k <= S.KE; ++k) {
      const double a = fabs((double)S.CmuHt[i3(S, i, j, k)]);
      if (a == a) {
        const unsigned long long b = (unsigned long long)__double_as_longlong(a) + 1ull;
        if (b > hb) hb = b;
      }
    }
  }
  if (t < S.M * S.N) {
    const int i = S.IB + t % S.M, j = S.JB + t / S.M;
    const long long q = i2(S, i, j);
    const double Dq = S.D[q];
    const double c = sqrt(kGrav * Dq);
    double ux = kSmall, vy = kSmall;
    for (int k = S.KB; k <= S.KE; ++k) {
      const long long o = i3(S, i, j, k);
      ux = dmax_(ux, dmax_(fabs((double)S.U[o]) + c, kSmall));
      vy = dmax_(vy, dmax_(fabs((double)S.V[o]) + c, kSmall));
      const double x = S.dsig[k] * Dq / dmax_(fabs((double)S.W[o]), kSmall);
      if (x < m) m = x;
    }
    double x = S.dx / ux;
    if (x < m) m = x;
    x = S.dy / vy;
    if (x < m) m = x;
  }
  for (int o = 16; o > 0; o >>= 1) {
    m = dmin_(m, __shfl_down_sync(0xffffffffu, m, o));
    const unsigned long long b = __shfl_down_sync(0xffffffffu, hb, o);
    if (b > hb) hb = b;
  }
  if ((threadIdx.x & 31) == 0) { sh[threadIdx.x >> 5] = m; shh[threadIdx.x >> 5] = hb; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      m = dmin_(m, sh[w]);
      if (shh[w] > hb) hb = shh[w];
    }
    atomicMin(&S.sc->dtmin_bits, (unsigned long long)__double_as_longlong(m));
    if (hb) atomicMax(&S.sc->htmax_bits, hb);
  }
}
template <class T>
__global__ void k_dt_finalize(Dev<T> S, int gated) {
  DevScal* sc = S.sc;
  const double tmp2 = __longlong_as_double((long long)sc->dtmin_bits);
  sc->dtmin_bits = (unsigned long long)__double_as_longlong(kLarge);
  const unsigned long long hb = sc->htmax_bits;
  sc->htmax_bits = 0ull;
  // A dt below DT_MIN stops the run for good (src/nhwave.F:3840-3850 stops
  // the program).  The gated form also holds the step back once the run is
  // over (the main loop's TIME < TOTAL_TIME and RUN_STEP < SIM_STEPS test,
  // src/nhwave.F:119) or the previous step's pressure solve went non-finite.
  bool go = sc->status != 5;
  if (go && gated)
    go = sc->time < S.total_time && sc->run_step < S.sim_steps && sc->step_status != 7;
  if (go) {
    sc->dt_old = sc->dt;
    const double dt_growth = (double)1.05f * sc->dt_old;
    const double dt_courant = S.cfl * tmp2;
    // limit of the explicit viscous terms (src/nhwave.F:3812-3832), from
    // the largest finite |CmuHt| that k_dt_min found
    double dt_viscous = kLarge;
    if (S.viscous) {
      double t2 = kLarge;
      if (hb) {
        const double ch = __longlong_as_double((long long)(hb - 1ull)) + (double)1.e-16f;
        const double ax = S.dx * S.dx / ch, ay = S.dy * S.dy / ch;
        if (ax < t2) t2 = ax;
        if (ay < t2) t2 = ay;
      }
      dt_viscous = S.v_number * t2;
    }
    const double dt = dmin_(dmin_(dmin_(dt_growth, dt_courant), dt_viscous), S.dt_max);
    sc->dt = dt;
    sc->rho_dt = kRho0 / dt;
    sc->dt_rho = dt / kRho0;
    if (dt < S.dt_min) {
      sc->status = 5;
      if (5 > sc->worst) sc->worst = 5;
      go = false;
    } else {
      sc->time = sc->time + dt;
      sc->run_step = sc->run_step + 1;
      sc->step_status = 0;
      sc->bar_count = 0u;   // grid barrier of this step's persistent solves
      sc->bar_err = 0;
    }
  }
  sc->step_go = go ? 1 : 0;
  if (S.graph_mode && S.h_go) cudaGraphSetConditional(S.h_go, go ? 1u : 0u);
}

// =========================================================================
//            update_bathymetry, RIGID_3D (src/nhwave.F:5755-6071)
// =========================================================================
struct OpSlideA {
  static constexpr const char* kName = "slide_a";  // Ho = Hc everywhere; new Hc in the interior
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j) const {
    const long long c = i2(S, i, j);
    S.Ho[c] = S.Hc[c];
    if (i < S.IB || i > S.IE || j < S.JB || j > S.JE) return;
    const double time = S.sc->time;
    const double st = S.sl_s0 * log(cosh(time / S.sl_t0)) * S.sl_cosslope;
    const double x0 = S.sl_x0 + st * S.sl_cosa, y0 = S.sl_y0 + st * S.sl_sina;
    const double xt = (S.xc[i] - x0) * S.sl_cosa + (S.yc[j] - y0) * S.sl_sina;
    const double yt = -((S.xc[i] - x0) * S.sl_sina) + (S.yc[j] - y0) * S.sl_cosa;
    const double zt = S.sl_T / (1 - S.sl_e) * (1.0 / cosh(S.sl_kb * xt) / cosh(S.sl_kw * yt) - S.sl_e);
    S.Hc[c] = S.Hc0[c] - dmax_(0.0, zt);
  }
};
struct OpSlideB {
  static constexpr const char* kName = "slide_b";  // Hc ghosts (phi_2D_coll)
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j) const {
    const int mi = mirror(i, S.IB, S.IE), mj = mirror(j, S.JB, S.JE);
    if (mi != i || mj != j) S.Hc[i2(S, i, j)] = S.Hc[i2(S, mi, mj)];
  }
};
struct OpSlideC {
  static constexpr const char* kName = "slide_c";  // face depths, slopes, dH/dt (src/nhwave.F:6026-6069); grid (Mloc+1) x (Nloc+1)
  template <class T>
  __device__ double hcx(const Dev<T>& S, int i, int j) const {
    // Hc(i,j) with the Fortran column-major continuation past the last row/column
    if (i == S.Mloc) { i = 0; ++j; }
    if (j >= S.Nloc) return 0.0;
    return S.Hc[i2(S, i, j)];
  }
  template <class T>
  __device__ double hfx(const Dev<T>& S, int i, int j) const {  // i in [0, Mloc], j < Nloc
    if (i == 0) i = 1;
    if (i == S.Mloc) i = S.Mloc - 1;
    return 0.5 * (S.Hc[i2(S, i, j)] + hcx(S, i + 1, j));
  }
  template <class T>
  __device__ double hfy(const Dev<T>& S, int i, int j) const {  // j in [0, Nloc], i < Mloc
    if (j == 0) j = 1;
    if (j == S.Nloc) j = S.Nloc - 1;
    return 0.5 * (S.Hc[i2(S, i, j)] + hcx(S, i, j + 1));
  }
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j, int) const {
    const long long c = i2(S, i, j);
    if (j < S.Nloc) { const double h = hfx(S, i, j); S.Hfx[c] = h; S.Hfx0[c] = h; }
    if (i < S.Mloc) { const double h = hfy(S, i, j); S.Hfy[c] = h; S.Hfy0[c] = h; }
    if (i < S.Mloc && j < S.Nloc) {
      S.DelxH[c] = (hfx(S, i + 1, j) - hfx(S, i, j)) / S.dx;
      S.DelyH[c] = (hfy(S, i, j + 1) - hfy(S, i, j)) / S.dy;
      const double dt = S.sc->dt;
      const double old = S.DeltH[c];
      const double nw = (S.Hc[c] - S.Ho[c]) / dt;
      S.DeltHo[c] = old;
      S.DeltH[c] = nw;
      if (S.sc->run_step > 2) S.Delt2H[c] = (nw - old) / dt;
    }
  }
};

// =========================================================================
//                 update_mask (src/nhwave.F:5403-5456)
// =========================================================================
struct OpMaskA {
  static constexpr const char* kName = "mask_a";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j) const {
    const long long c = i2(S, i, j);
    int m = S.Mask[c];
    if (i >= S.IB && i <= S.IE && j >= S.JB && j <= S.JE && S.Mask_Struct[c] != 0) {
      const double thr = (double)1.e-6f, md = S.min_dep;
      const double* E = S.Eta;
      const double* D = S.D;
      const int* Mk = S.Mask;
      if (Mk[c] == 0) {
        const long long nb[4] = {c - 1, c + 1, c - S.sy, c + S.sy};
        for (int q = 0; q < 4; ++q)
          if (Mk[nb[q]] == 1 && E[nb[q]] > E[c] && D[nb[q]] - md > thr) m = 1;
      } else if (fabs(D[c] - md) <= thr) {
        m = 0;
        // the neighbours read E/D only under a D > MinDep + 1e-6 test, which a
        // cell that dries fails before and after this write
        const double e = md - S.Hc[c];
        S.Eta[c] = e;
        S.D[c] = e + S.Hc[c];
      }
    }
    S.MaskT[c] = m;
  }
};
struct OpMaskB {
  static constexpr const char* kName = "mask_b";
  template <class T>
  __device__ void operator()(const Dev<T>& S, int i, int j) const {
    const long long c = i2(S, i, j);
    const int* Mt = S.MaskT;
    S.Mask[c] = Mt[c] * S.Mask_Struct[c];
    if (i >= S.IB && i <= S.IE && j >= S.JB && j <= S.JE) {
      auto m = [&](long long x) { return Mt[x] * S.Mask_Struct[x]; };
      const long long sy = S.sy;
      S.Mask9[c] = m(c) * m(c - 1) * m(c + 1) * m(c + 1 + sy) * m(c + sy) * m(c - 1 + sy) * m(c + 1 - sy) *
                   m(c - sy) * m(c - 1 - sy);
    }
  }
};

// =========================================================================
//                             diagnostics
// =========================================================================
// statistics (src/nhwave.F:3118-3160), per interior column: MassVolume's
// D dx dy; Energy's sum over the column's levels, in k order, of
// CellMass (g (D sigc_k - Hc) + (U^2 + V^2 + W^2) / 2) with
// CellMass = Rho0 dsig_k D dx dy; eta; the largest |U|, |V|, |W|.  Slots of a
// block's partial (stride 8 in S.partials): sums 0-1, maxima 2-6 (slot 3
// holds -eta, so that MinEta is minus its maximum).  k_stats_final combines
// the partials in block order.
constexpr int kStatN = 7;
template <class T>
__global__ void __launch_bounds__(256) k_stats(Dev<T> S) {
  __shared__ double sh[kStatN][256];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double v[kStatN] = {0.0, 0.0, -1.0e308, -1.0e308, 0.0, 0.0, 0.0};
  if (t < S.M * S.N) {
    const int i = S.IB + t % S.M, j = S.JB + t / S.M;
    const long long q = i2(S, i, j);
    const double D = S.D[q], hc = S.Hc[q];
    v[0] = D * S.dx * S.dy;
    double e = 0.0;
    for (int k = S.KB; k <= S.KE; ++k) {
      const long long o = i3(S, i, j, k);
      const double cm = kRho0 * S.dsig[k] * D * S.dx * S.dy;
      const double u = (double)S.U[o], w1 = (double)S.V[o], w2 = (double)S.W[o];
      e = e + cm * kGrav * (D * S.sigc[k] - hc) + 0.5 * cm * (u * u + w1 * w1 + w2 * w2);
      v[4] = dmax_(v[4], fabs(u));
      v[5] = dmax_(v[5], fabs(w1));
      v[6] = dmax_(v[6], fabs(w2));
    }
    v[1] = e;
    v[2] = S.Eta[q];
    v[3] = -S.Eta[q];
  }
  for (int m = 0; m < kStatN; ++m) sh[m][threadIdx.x] = v[m];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int m = 0; m < kStatN; ++m)
        sh[m][threadIdx.x] = m < 2 ? sh[m][threadIdx.x] + sh[m][threadIdx.x + w]
                                   : dmax_(sh[m][threadIdx.x], sh[m][threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int m = 0; m < kStatN; ++m) S.partials[(size_t)blockIdx.x * 8 + m] = sh[m][0];
}
template <class T>
__global__ void __launch_bounds__(256) k_stats_final(Dev<T> S, int nb, double* out) {
  __shared__ double sh[kStatN][256];
  double v[kStatN] = {0.0, 0.0, -1.0e308, -1.0e308, 0.0, 0.0, 0.0};
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
    for (int m = 0; m < kStatN; ++m) {
      const double x = S.partials[(size_t)b * 8 + m];
      v[m] = m < 2 ? v[m] + x : dmax_(v[m], x);
    }
  for (int m = 0; m < kStatN; ++m) sh[m][threadIdx.x] = v[m];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int m = 0; m < kStatN; ++m)
        sh[m][threadIdx.x] = m < 2 ? sh[m][threadIdx.x] + sh[m][threadIdx.x + w]
                                   : dmax_(sh[m][threadIdx.x], sh[m][threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    for (int m = 0; m < kStatN; ++m) out[m] = sh[m][0];
    out[3] = -out[3];
  }
}

template <class T>
__global__ void k_mass(Dev<T> S, double* out) {
  // MassVolume = sum over interior (j outer, i inner) of D*dx*dy, FP64, in order
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double m = 0.0;
  for (int j = S.JB; j <= S.JE; ++j)
    for (int i = S.IB; i <= S.IE; ++i) m = m + S.D[i2(S, i, j)] * S.dx * S.dy;
  *out = m;
}

}  // namespace nhw
