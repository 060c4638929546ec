// setup_host.cpp -- host-side set-up of one scenario: generate_grid
// (src/initialize.F:1647-1729), read_bathymetry (src/initialize.F:1734-2175,
// CELL_CENTER / CELL_GRID and the RIGID_3D slide), update_wind for a constant
// wind (src/nhwave.F:5333-5400), calculate_sponge (src/nhwave.F:6405-6460) and
// the non-optional parts of initial (src/initialize.F:2502-3408) up to the
// vel_bc call, which runs on the device.  Built with -ffp-contract=off so the
// arithmetic is the reference's, operation for operation.
#include "setup_host.h"

#include <cmath>
#include <cstring>

#include "cnoidal.h"

namespace nhw {
namespace {
const double kPiH = (double)3.141592653f;
const double kGravH = (double)9.81f;
inline double dmx(double a, double b) { return a > b ? a : b; }
inline double dmn(double a, double b) { return a < b ? a : b; }
bool cnoidal_params(double H, double d, double T, double& L, double& x2, double& m, double* c = nullptr);
bool cnoidal_start(double Ytrough, double A, double m, double& Xstart);
}  // namespace

int check_params(const nhw_params& p) {
  if (p.Mglob < 1 || p.Nglob < 1 || p.Kglob < 1) return NHW_ERR_ARG;
  if (!(p.dx > 0) || !(p.dy > 0) || !(p.cfl > 0) || !(p.dt_ini > 0)) return NHW_ERR_ARG;
  if (p.Kglob > 64) return NHW_ERR_UNSUPPORTED;
  // the ghosted face arrays index cells with 32-bit integers (and neq, the
  // unknowns of the Poisson system, is an int)
  if ((long long)(p.Mglob + 5) * (p.Nglob + 5) * (p.Kglob + 5) >= (1LL << 31)) return NHW_ERR_UNSUPPORTED;
  // BAROTROPIC = F adds baropg_z's baroclinic pressure gradient (src/nhwave.F:
  // 573, 13038-13179).  Without salinity, temperature, sediment or bubbles the
  // density stays Rho0 (src/initialize.F:2561), Rho - Rho0 is zero, and so are
  // DRhoX and DRhoY (signed zeros, which leave R2 and R3 unchanged): the flag
  // runs the same path.
  // viscous flow: IVTURB 1 constant, 2 subgrid, 3 the 2-D and 10 the 3-D
  // k-epsilon model, 20 the Smagorinsky and 30 the dynamic LES; IHTURB 1, 2
  // or >= 10 (CmuHt = CmuVt)
  if (p.viscous_flow &&
      !(p.ivturb == 1 || p.ivturb == 2 || p.ivturb == 3 || p.ivturb == 10 || p.ivturb == 20 || p.ivturb == 30))
    return NHW_ERR_UNSUPPORTED;
  if (p.viscous_flow && !(p.ihturb == 1 || p.ihturb == 2 || p.ihturb >= 10)) return NHW_ERR_UNSUPPORTED;
  if (p.viscous_flow && (!(p.schmidt != 0.0) || !(p.viscous_number > 0.0))) return NHW_ERR_ARG;
  // lateral sides: 1 free slip, 2 no slip, 5 wall friction; BC_Xn = 6 Orlanski
  for (int b : {p.bc_y0, p.bc_yn})
    if (b != 1 && b != 2 && b != 5) return NHW_ERR_UNSUPPORTED;
  // east side: BC_Xn = 3 only with RIG_LIN or FLUX_LR, which feed it
  const bool east_in = p.wavemaker == NHW_WM_RIG_LIN || p.wavemaker == NHW_WM_FLUX_LR;
  if (p.bc_xn != 1 && p.bc_xn != 2 && p.bc_xn != 5 && p.bc_xn != 6 && !(p.bc_xn == 3 && east_in))
    return NHW_ERR_UNSUPPORTED;
  const bool lef = (p.wavemaker >= NHW_WM_LEF_LIN && p.wavemaker <= NHW_WM_LEF_TID) ||
                   p.wavemaker == NHW_WM_FLUX_LR || p.wavemaker == NHW_WM_LEF_JON ||
                   p.wavemaker == NHW_WM_LEF_TMA || p.wavemaker == NHW_WM_LEF_SPC;
  // west inflow (BC_X0 = 3) only with a wave or current fed through it
  if (!(p.bc_x0 == 1 || p.bc_x0 == 2 || p.bc_x0 == 5 || (p.bc_x0 == 3 && lef))) return NHW_ERR_UNSUPPORTED;
  if (p.wavemaker == NHW_WM_FLUX_LR && !(p.zob > 0.0)) return NHW_ERR_ARG;   // log-profile inflow
  // bed: 1 free slip, 2 no slip, 5 friction law with Ibot 1 (Cd0) or 2 (Zob)
  if (p.bc_z0 != 1 && p.bc_z0 != 2 && p.bc_z0 != 5) return NHW_ERR_UNSUPPORTED;
  const bool fric = p.bc_z0 == 5 || p.bc_x0 == 5 || p.bc_xn == 5 || p.bc_y0 == 5 || p.bc_yn == 5;
  if (fric && p.ibot != 1 && p.ibot != 2) return NHW_ERR_UNSUPPORTED;
  if (fric && p.ibot == 2 && !(p.zob > 0.0)) return NHW_ERR_ARG;
  if (p.wavemaker < 0 || p.wavemaker > NHW_WM_INT_IRR) return NHW_ERR_UNSUPPORTED;
  if (p.krylov_kernel < 0 || p.krylov_kernel > 2) return NHW_ERR_ARG;
  if (p.slide_type < 0 || p.slide_type > 1) return NHW_ERR_UNSUPPORTED;
  if (p.precision != NHW_FP64 && p.precision != NHW_FP32_IR) return NHW_ERR_ARG;
  if (p.time_order < 1 || p.time_order > 3) return NHW_ERR_ARG;
  const bool spectral = p.wavemaker == NHW_WM_LEF_JON || p.wavemaker == NHW_WM_LEF_TMA ||
                        p.wavemaker == NHW_WM_LEF_SPC || p.wavemaker == NHW_WM_INT_JON ||
                        p.wavemaker == NHW_WM_INT_TMA || p.wavemaker == NHW_WM_INT_SPC ||
                        p.wavemaker == NHW_WM_INT_IRR;
  if (p.wavemaker && p.wavemaker != NHW_WM_FOCUSED && p.wavemaker != NHW_WM_FLUX_LR && !spectral &&
      !(p.per_wave > 0 && p.dep_wave > 0))
    return NHW_ERR_ARG;
  // FOCUSED: at least two components (the frequency spacing divides by
  // NWAVE - 1), at most the reference's 12000
  if (p.wavemaker == NHW_WM_FOCUSED &&
      (p.nwave < 2 || p.nwave > 12000 || !(p.f_center > 0) || !(p.depth_comp > 0) ||
       (p.component_amp_type == 1 && !(p.k_center > 0))))
    return NHW_ERR_ARG;
  if (spectral && !(p.dep_wave > 0)) return NHW_ERR_ARG;
  if (p.wavemaker == NHW_WM_LEF_JON || p.wavemaker == NHW_WM_LEF_TMA || p.wavemaker == NHW_WM_INT_JON ||
      p.wavemaker == NHW_WM_INT_TMA) {   // src/initialize.F:880-941
    if (!(p.hm0 > 0) || !(p.tp > 0) || !(p.freq_min > 0) || !(p.freq_max > p.freq_min) || p.numfreq < 1 ||
        p.numfreq > 500 || !(p.dep_wave > 0))
      return NHW_ERR_ARG;
  }
  if (p.wavemaker == NHW_WM_LEF_CON || p.wavemaker == NHW_WM_INT_CON) {   // the cnoidal parameter and start phase must exist
    double L = 0, Yt = 0, m = 0, Xstart = 0;
    if (!(p.amp_wave > 0) || !cnoidal_params(p.amp_wave, p.dep_wave, p.per_wave, L, Yt, m) ||
        !cnoidal_start(Yt, p.amp_wave, m, Xstart))
      return NHW_ERR_ARG;
  }
  return NHW_OK;
}

namespace {
// cnoidal (src/waves.F:184-220): Newton iteration for the elliptic parameter
// m of a cnoidal wave of height H in depth d with period T, then its length
// L, trough level x2 and (c) celerity.  Returns false when m leaves (0, 1].
bool cnoidal_params(double H, double d, double T, double& L, double& x2, double& m, double* c) {
  m = 0.99999999;
  for (int n = 1;; ++n) {
    if (!(m > 0.0 && m <= 1.0)) return false;
    const double ck = cnoidal_ck(m), ce = cnoidal_ce(m);
    const double xa = m * d + 2.0 * H - m * H - 3.0 * H * ce / ck -
                      16.0 * (d * d * d) * (m * m) * (ck * ck) / 3.0 / kGravH / H / (T * T);
    if (std::fabs(xa) <= (double)1.0e-8f || n > 1000) break;
    const double xb = d - H + 3.0 * H / 2.0 / m / (1.0 - m) / (ck * ck) *
                                  ((1.0 - m) * (ck * ck) + ce * ce - 2.0 * (1.0 - m) * ck * ce) -
                      16.0 * (d * d * d) * m * ck / 3.0 / kGravH / (1.0 - m) / H / (T * T) *
                          ((1.0 - m) * ck + ce);
    m = m - xa / xb;
  }
  if (!(m > 0.0 && m <= 1.0)) return false;
  const double ck = cnoidal_ck(m), ce = cnoidal_ce(m);
  L = 4.0 * ck * d * std::sqrt(m * d / H / 3.0);
  const double xtemp = -m + 2.0 - 3.0 * ce / ck;
  if (c) *c = std::sqrt(kGravH * d * (1.0 + H / d / m * xtemp));
  x2 = H / m * (1.0 - m - ce / ck);
  return std::isfinite(L) && std::isfinite(x2);
}

// Start phase of the cnoidal boundary wave (src/waves.F:106-130): bisection
// for the phase in [0, 1] where the elevation crosses zero, to 1e-6.
bool cnoidal_start(double Ytrough, double A, double m, double& Xstart) {
  const double ck = cnoidal_ck(m);
  double Zup = 1.0, Zlow = 0.0, Zmid = (Zup + Zlow) / 2.0;
  for (int nn = 1;; ++nn) {
    const double cn = cnoidal_cn(Zmid * 0.5 * ck, m);
    const double Zero1 = Ytrough + A * (cn * cn);
    if (std::fabs(Zero1) <= (double)1.0e-6f) break;
    if (nn > 1000) return false;   // the reference stops the run here
    if (Zero1 < 0.0) Zup = Zmid; else Zlow = Zmid;
    Zmid = (Zup + Zlow) / 2.0;
  }
  Xstart = Zmid;
  return true;
}
}  // namespace

double wave_number(double Segma, double Dep) {
  double Wn = (Segma * Segma) / (kGravH * std::pow(std::tanh(Segma * Segma * Dep / kGravH), 0.5));
  double error = 100.;
  int guard = 0;
  while (error >= (double)1.0e-8f && guard++ < 200) {
    const double Fk = Segma * Segma - kGravH * Wn * std::tanh(Wn * Dep);
    const double ch = std::cosh(Wn * Dep);
    const double Fkdif = -(kGravH * (std::tanh(Wn * Dep) + (Wn * Dep) / (ch * ch)));
    const double Wn_new = Wn - Fk / Fkdif;
    error = std::fabs((Wn - Wn_new) / Wn);
    Wn = Wn_new;
  }
  return Wn;
}

double wave_phase(int32_t seed, int i) {
  // SplitMix64, element i + 1 of the stream that starts at the seed
  uint64_t z = (uint64_t)(uint32_t)seed + (uint64_t)(i + 1) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (double)(z >> 11) * 0x1.0p-53 * 2.0 * kPiH;
}

namespace {
// JONSWAP (TMA with `tma`) spectrum at NumFreq band centres, scaled to
// m0 = Hm0^2/16 (src/initialize.F:893-941), then the boundary routine's
// per-component constants (src/waves.F:580-593).  The reference's boundary
// routine calls wave_dispersion with three arguments where it takes two
// (src/waves.F:585), so its wave number is undefined; the wave number here is
// wave_dispersion's of each component, as the spectral routine computes it
// (src/waves.F:395).
// The JONSWAP (TMA) spectrum of src/initialize.F:893-941: NumFreq band
// centres and their densities scaled to m0 = Hm0^2/16.
void jonswap_spectrum(const nhw_params& p, bool tma, std::vector<double>& Freq, std::vector<double>& Spc) {
  const int nf = p.numfreq;
  const double Dep = p.dep_wave;
  const double gam = (double)3.3f, sa = (double)0.07f, sb = (double)0.09f;
  const double Freq_Peak = 1.0 / p.tp;
  const double DFreq = (p.freq_max - p.freq_min) / nf;
  Freq.assign(nf, 0.0);
  Spc.assign(nf, 0.0);
  for (int i = 1; i <= nf; ++i) {
    const double F = p.freq_min + 0.5 * DFreq + (i - 1) * DFreq;
    Freq[i - 1] = F;
    const double Per = 1.0 / F, Segma = 2.0 * kPiH / Per;
    const double Celerity = std::sqrt(kGravH * Dep), Wave_Length = Celerity * Per;
    double k = 2.0 * kPiH / Wave_Length;
    for (int it = 0;; ++it) {
      const double th = std::tanh(k * Dep);
      const double Fk = kGravH * k * th - Segma * Segma;
      if (std::fabs(Fk) <= (double)1.0e-8f || it > 1000) break;
      const double Fkdif = kGravH * k * Dep * (1.0 - th * th) + kGravH * th;
      k = k - Fk / Fkdif;
    }
    const double r = Freq_Peak / F, f5 = (F * F) * (F * F) * F, s2 = F < Freq_Peak ? sa * sa : sb * sb;
    double S = (kGravH * kGravH) / f5 * std::exp(-1.25 * ((r * r) * (r * r))) *
               std::pow(gam, std::exp(-0.5 * ((F / Freq_Peak - 1.0) * (F / Freq_Peak - 1.0)) / s2));
    if (tma) {
      const double th = std::tanh(k * Dep);
      S = S * (th * th) / (1.0 + 2 * k * Dep / std::sinh(2. * k * Dep));
    }
    Spc[i - 1] = S;
  }
  double SumInt = 0.0;
  for (int i = 0; i < nf; ++i) SumInt = SumInt + Spc[i] * DFreq;
  const double A_Jon = (p.hm0 * p.hm0) / 16.0 / SumInt;
  for (int i = 0; i < nf; ++i) Spc[i] = Spc[i] * A_Jon;
}

// LEF_JON / LEF_TMA: the boundary routine's per-component constants
// (src/waves.F:580-593).  The reference's boundary routine calls
// wave_dispersion with three arguments where it takes two (src/waves.F:585),
// so its wave number is undefined; the wave number here is wave_dispersion's
// of each component, as the spectral routine computes it (src/waves.F:395).
void jonswap_components(const nhw_params& p, bool tma, std::vector<double>& out) {
  const int nf = p.numfreq;
  const double Dep = p.dep_wave;
  std::vector<double> Freq, Spc;
  jonswap_spectrum(p, tma, Freq, Spc);
  out.assign((size_t)kJonSlots * nf, 0.0);
  const double dfreq = (p.freq_max - p.freq_min) / (double)(float)nf;
  for (int i = 0; i < nf; ++i) {
    const double S = Spc[i];
    const double Per = 1.0 / Freq[i], Segma = 2.0 * kPiH / Per;
    const double k = wave_number(Segma, Dep), Wave_Length = 2.0 * kPiH / k;
    const double Wh = 2.0 * std::sqrt(2.0 * S * dfreq);
    out[0 * nf + i] = Wh;
    out[1 * nf + i] = 2.0 * kPiH * Freq[i];   // the per-step loops' Segma = 2 pi Freq
    out[2 * nf + i] = k;
    out[3 * nf + i] = kGravH * (Wh * Wh) / (Wave_Length / Per) / Dep / 8.0;
    out[kJonPhase * nf + i] = wave_phase(p.wave_seed, i);
    out[5 * nf + i] = std::sinh(k * Dep);
    out[6 * nf + i] = 0.0;
    out[7 * nf + i] = 1.0;
  }
}

// INT_JON / INT_TMA (src/source_terms.F:305-340): per component, in the
// internal makers' layout (setup_host.h), Celerity * Amp_Wave with
// Amp_Wave = 2 sqrt(2 Jon_Spc DFreq), Segma = 2 pi / Per_Wave and the phase.
void internal_jonswap_components(const nhw_params& p, bool tma, std::vector<double>& out) {
  const int nf = p.numfreq;
  std::vector<double> Freq, Spc;
  jonswap_spectrum(p, tma, Freq, Spc);
  out.assign((size_t)kJonSlots * nf, 0.0);
  const double DFreq = (p.freq_max - p.freq_min) / (double)(float)nf;
  for (int i = 0; i < nf; ++i) {
    const double Per = 1.0 / Freq[i], Segma = 2.0 * kPiH / Per;
    const double k = wave_number(Segma, p.dep_wave), Wave_Length = 2.0 * kPiH / k;
    const double Celerity = Wave_Length / Per;
    const double Amp = 2.0 * std::sqrt(2.0 * Spc[i] * DFreq);
    out[kIntPre * nf + i] = Celerity * Amp;
    out[kIntSegma * nf + i] = Segma;
    out[kJonPhase * nf + i] = wave_phase(p.wave_seed, i);
  }
}
}  // namespace

bool spectrum_components(const nhw_params& p, int numfreq, int numdir, const double* freq, const double* dire,
                         const double* spc2d, const double* phases, std::vector<double>& out) {
  if (numfreq < 2 || numdir < 2 || (long long)numfreq * numdir > 12000 || !freq || !dire || !spc2d) return false;
  const int nc = numfreq * numdir;
  const double Dep = p.dep_wave;
  out.assign((size_t)kJonSlots * nc, 0.0);
  for (int nfq = 1; nfq <= numfreq; ++nfq)
    for (int nd = 1; nd <= numdir; ++nd) {
      const int c = (nd - 1) + numdir * (nfq - 1);
      const double Per = 1.0 / freq[nfq - 1], Segma = 2.0 * kPiH / Per;
      const double k = wave_number(Segma, Dep), Wave_Length = 2.0 * kPiH / k;
      const double Angle = dire[nd - 1] * kPiH / 180.;
      double dfreq = nfq == 1 ? freq[1] - freq[0]
                     : nfq == numfreq ? freq[numfreq - 1] - freq[numfreq - 2]
                                      : 0.5 * (freq[nfq] - freq[nfq - 2]);
      dfreq = std::fabs(dfreq);
      double ddir = nd == 1 ? dire[1] - dire[0]
                    : nd == numdir ? dire[numdir - 1] - dire[numdir - 2]
                                   : 0.5 * (dire[nd] - dire[nd - 2]);
      ddir = std::fabs(ddir);
      const double Wh = 2.0 * std::sqrt(2.0 * spc2d[c] * dfreq * ddir);
      if (!(Wh == Wh) || !(k > 0)) return false;
      out[0 * nc + c] = Wh;
      out[1 * nc + c] = 2.0 * kPiH * freq[nfq - 1];
      out[2 * nc + c] = k;
      out[3 * nc + c] = kGravH * (Wh * Wh) / (Wave_Length / Per) / Dep / 8.0;
      out[kJonPhase * nc + c] = phases ? phases[c] : wave_phase(p.wave_seed, c);
      out[5 * nc + c] = std::sinh(k * Dep);
      out[6 * nc + c] = std::sin(Angle);
      out[7 * nc + c] = std::cos(Angle);
    }
  return true;
}

bool snap_direction(double Angle, double k, int Nglob, double dy, bool irr, double& out) {
  const double small = (double)1.0e-16f;
  const double width = Nglob * dy;
  const int kSnapMax = 10000000;   // the reference's loop has no bound; |Angle| <= 90 deg ends it
  if (!(k > 0.0)) return false;
  if (Angle > 0.0) {
    double tmp3 = 0.0;
    int nk = 0;
    while (tmp3 < Angle) {
      if (++nk > kSnapMax) return false;
      const double tmp2 = nk * 2.0 * kPiH / width;
      tmp3 = tmp2 >= k ? 0.5 * kPiH - small : std::asin(tmp2 / k);
    }
    const double tmp4 = std::asin((nk - 1) * 2.0 * kPiH / width / k);
    out = std::fabs(tmp4 - Angle) < std::fabs(Angle - tmp3) ? tmp4 : tmp3;
  } else if (Angle < 0.0 || !irr) {
    // (INT_SPC takes this branch for a zero direction too, and keeps zero;
    // both makers compare with the positive arcsine here)
    double tmp3 = 0.0;
    int nk = 0;
    while (tmp3 > Angle) {
      if (++nk > kSnapMax) return false;
      const double tmp2 = nk * 2.0 * kPiH / width;
      tmp3 = tmp2 >= k ? -0.5 * kPiH + small : -std::asin(tmp2 / k);
    }
    const double tmp4 = std::asin((nk - 1) * 2.0 * kPiH / width / k);
    out = std::fabs(tmp4 - Angle) < std::fabs(Angle - tmp3) ? tmp4 : tmp3;
  } else {
    out = 0.0;
  }
  return true;
}

bool internal_spectrum_components(const nhw_params& p, int numfreq, int numdir, const double* freq,
                                  const double* dire, const double* spc2d, const double* phases,
                                  std::vector<double>& out) {
  const bool irr = p.wavemaker == NHW_WM_INT_IRR;
  if (numfreq < 2 || numdir < 2 || (long long)numfreq * numdir > 12000 || !freq || !dire || !spc2d) return false;
  if (irr && !phases) return false;   // irr2d.txt holds them
  const int nc = numfreq * numdir;
  out.assign((size_t)kJonSlots * nc, 0.0);
  for (int nfq = 1; nfq <= numfreq; ++nfq)
    for (int nd = 1; nd <= numdir; ++nd) {
      const int c = (nd - 1) + numdir * (nfq - 1);
      const double Per = 1.0 / freq[nfq - 1], Segma = 2.0 * kPiH / Per;
      const double k = wave_number(Segma, p.dep_wave), Wave_Length = 2.0 * kPiH / k;
      const double Celerity = Wave_Length / Per;
      double Angle = 0.0;
      if (!snap_direction(dire[nd - 1] * kPiH / 180., k, p.Nglob, p.dy, irr, Angle)) return false;
      double Amp;
      if (irr) {
        Amp = 2.0 * spc2d[c];
      } else {
        double dfreq = nfq == 1 ? freq[1] - freq[0]
                       : nfq == numfreq ? freq[numfreq - 1] - freq[numfreq - 2]
                                        : 0.5 * (freq[nfq] - freq[nfq - 2]);
        dfreq = std::fabs(dfreq);
        double ddir = nd == 1 ? dire[1] - dire[0]
                      : nd == numdir ? dire[numdir - 1] - dire[numdir - 2]
                                     : 0.5 * (dire[nd] - dire[nd - 2]);
        ddir = std::fabs(ddir);
        Amp = 2.0 * std::sqrt(2.0 * spc2d[c] * ddir * dfreq);
      }
      if (!(Amp == Amp) || !std::isfinite(Celerity)) return false;
      if (irr && nfq == 1) {   // 2 Celerity / Source_Area (Amp_Wave/2 cos(..) + eta_mean)
        out[kIntPre * nc + c] = 2 * Celerity;
        out[kIntHalfAmp * nc + c] = Amp / 2;
        out[kIntKind * nc + c] = 1.0;
      } else {
        out[kIntPre * nc + c] = Celerity * Amp;
      }
      out[kIntSegma * nc + c] = Segma;
      out[kIntWnumY * nc + c] = k * std::sin(Angle);
      out[kJonPhase * nc + c] = phases ? phases[c] : wave_phase(p.wave_seed, c);
    }
  return true;
}

int host_setup(const nhw_params& p, const double* depth, const double* eta0, const double* uvw0,
               HostInit& h) {
  const int M = p.Mglob, N = p.Nglob, K = p.Kglob;
  const int Ml = M + 4, Nl = N + 4, Kl = K + 4, Ml1 = Ml + 1, Nl1 = Nl + 1, Kl1 = Kl + 1;
  h.Mloc = Ml; h.Nloc = Nl; h.Kloc = Kl;
  // Fortran 1-based accessors
  auto a2 = [&](std::vector<double>& v, int n1, int i, int j) -> double& { return v[(size_t)(i - 1) + (size_t)n1 * (j - 1)]; };
  auto m2 = [&](std::vector<int32_t>& v, int i, int j) -> int32_t& { return v[(size_t)(i - 1) + (size_t)Ml * (j - 1)]; };
  const size_t c2 = (size_t)Ml * Nl;
  h.x.assign(Ml1, 0.0); h.xc.assign(Ml, 0.0); h.y.assign(Nl1, 0.0); h.yc.assign(Nl, 0.0);
  h.sig.assign(Kl1, 0.0); h.dsig.assign(Kl, 0.0); h.sigc.assign(Kl, 0.0);
  for (auto* v : {&h.Hc, &h.Hc0, &h.DelxH, &h.DelyH, &h.Eta, &h.D, &h.Sponge, &h.Wsx, &h.Wsy}) v->assign(c2, 0.0);
  h.Hfx.assign((size_t)Ml1 * Nl, 0.0); h.Hfy.assign((size_t)Ml * Nl1, 0.0);
  h.Mask.assign(c2, 0); h.Mask_Struct.assign(c2, 0); h.Mask9.assign(c2, 0);
  const size_t c3 = c2 * Kl;
  h.U.assign(c3, 0.0); h.V.assign(c3, 0.0); h.W.assign(c3, 0.0);
  const int Ib = 3, Ie = Ml - 2, Jb = 3, Je = Nl - 2, Kb = 3, Ke = Kl - 2;
  const double dx = p.dx, dy = p.dy;
  // ---- generate_grid
  auto X = [&](int i) -> double& { return h.x[i - 1]; };
  auto XC = [&](int i) -> double& { return h.xc[i - 1]; };
  auto Y = [&](int j) -> double& { return h.y[j - 1]; };
  auto YC = [&](int j) -> double& { return h.yc[j - 1]; };
  X(Ib) = 0.0;
  for (int i = Ib + 1; i <= Ml1; ++i) { X(i) = X(i - 1) + dx; XC(i - 1) = X(i - 1) + 0.5 * dx; }
  for (int i = Ib - 1; i >= Ib - 2; --i) { X(i) = X(i + 1) - dx; XC(i) = X(i + 1) - 0.5 * dx; }
  Y(Jb) = 0.0;
  for (int j = Jb + 1; j <= Nl1; ++j) { Y(j) = Y(j - 1) + dy; YC(j - 1) = Y(j - 1) + 0.5 * dy; }
  for (int j = Jb - 1; j >= Jb - 2; --j) { Y(j) = Y(j + 1) - dy; YC(j) = Y(j + 1) - 0.5 * dy; }
  auto DS = [&](int k) -> double& { return h.dsig[k - 1]; };
  auto SG = [&](int k) -> double& { return h.sig[k - 1]; };
  auto SC = [&](int k) -> double& { return h.sigc[k - 1]; };
  if (p.ivgrd == 2) {
    DS(Kb) = (p.grd_r - 1.0) / (std::pow(p.grd_r, (double)(float)K) - 1.0);
    for (int k = Kb + 1; k <= Ke; ++k) DS(k) = DS(k - 1) * p.grd_r;
    for (int k = 1; k <= 2; ++k) DS(Kb - k) = DS(Kb + k - 1);
    for (int k = 1; k <= 2; ++k) DS(Ke + k) = DS(Ke - k + 1);
  } else {
    const double d = (double)(1.0f / (float)K);
    for (int k = 1; k <= Kl; ++k) DS(k) = d;
  }
  SG(Kb) = 0.0;
  for (int k = Kb + 1; k <= Kl1; ++k) { SG(k) = SG(k - 1) + DS(k - 1); SC(k - 1) = SG(k - 1) + 0.5 * DS(k - 1); }
  for (int k = Kb - 1; k >= 1; --k) { SG(k) = SG(k + 1) - DS(k); SC(k) = SG(k + 1) - 0.5 * DS(k); }
  // ---- read_bathymetry
  auto HC = [&](int i, int j) -> double& { return a2(h.Hc, Ml, i, j); };
  if (p.depth_type == NHW_DEPTH_CELL_GRID) {
    auto HG = [&](int i, int j) { return depth[(size_t)(i - 1) + (size_t)(M + 1) * (j - 1)]; };
    auto Mp = [&](int i, int j) { return HG(i, j) < -1000.0 ? 0 : 1; };
    for (int j = Jb; j <= Je; ++j)
      for (int i = Ib; i <= Ie; ++i) {
        const int ig = i - 2, jg = j - 2;
        const int ms = Mp(ig, jg) + Mp(ig + 1, jg) + Mp(ig, jg + 1) + Mp(ig + 1, jg + 1);
        const double num = HG(ig, jg) * Mp(ig, jg) + HG(ig + 1, jg) * Mp(ig + 1, jg) +
                           HG(ig, jg + 1) * Mp(ig, jg + 1) + HG(ig + 1, jg + 1) * Mp(ig + 1, jg + 1);
        HC(i, j) = num / (double)((float)ms + 1.e-16f);
      }
  } else {
    for (int j = Jb; j <= Je; ++j)
      for (int i = Ib; i <= Ie; ++i) HC(i, j) = depth[(size_t)(i - 3) + (size_t)M * (j - 3)];
  }
  auto coll = [&](std::vector<double>& v) {  // phi_2D_coll
    for (int j = Jb; j <= Je; ++j)
      for (int i = 1; i <= 2; ++i) { a2(v, Ml, i, j) = a2(v, Ml, Ib + 2 - i, j); a2(v, Ml, Ie + i, j) = a2(v, Ml, Ie - i + 1, j); }
    for (int i = 1; i <= Ml; ++i)
      for (int j = 1; j <= 2; ++j) { a2(v, Ml, i, j) = a2(v, Ml, i, Jb + 2 - j); a2(v, Ml, i, Je + j) = a2(v, Ml, i, Je - j + 1); }
  };
  coll(h.Hc);
  h.Hc0 = h.Hc;
  if (p.slide_type == NHW_SLIDE_RIGID_3D) {
    const double e = (double)0.717f;
    const double alpha0 = p.slide_angle * kPiH / 180.;
    const double kb = 2.0 * std::acosh(1.0 / e) / p.slide_l;
    const double kw = 2.0 * std::acosh(1.0 / e) / p.slide_w;
    for (int j = Jb; j <= Je; ++j)
      for (int i = Ib; i <= Ie; ++i) {
        const double xt = (XC(i) - p.slide_x0) * std::cos(alpha0) + (YC(j) - p.slide_y0) * std::sin(alpha0);
        const double yt = -((XC(i) - p.slide_x0) * std::sin(alpha0)) + (YC(j) - p.slide_y0) * std::cos(alpha0);
        const double zt = p.slide_t / (1 - e) * (1.0 / std::cosh(kb * xt) / std::cosh(kw * yt) - e);
        HC(i, j) = a2(h.Hc0, Ml, i, j) - dmx(0.0, zt);
      }
  }
  for (int j = 1; j <= Nl; ++j)
    for (int i = 1; i <= Ml; ++i) m2(h.Mask_Struct, i, j) = 1;
  for (int j = Jb; j <= Je; ++j)
    for (int i = Ib; i <= Ie; ++i)
      if (HC(i, j) < -1000.0) m2(h.Mask_Struct, i, j) = 0;
  for (int j = 1; j <= Nl; ++j) {
    for (int i = 2; i <= Ml; ++i) a2(h.Hfx, Ml1, i, j) = 0.5 * (HC(i - 1, j) + HC(i, j));
    a2(h.Hfx, Ml1, 1, j) = HC(1, j);
    a2(h.Hfx, Ml1, Ml1, j) = HC(Ml, j);
  }
  h.Hfx0 = h.Hfx;
  for (int i = 1; i <= Ml; ++i) {
    for (int j = 2; j <= Nl; ++j) a2(h.Hfy, Ml, i, j) = 0.5 * (HC(i, j - 1) + HC(i, j));
    a2(h.Hfy, Ml, i, 1) = HC(i, 1);
    a2(h.Hfy, Ml, i, Nl1) = HC(i, Nl);
  }
  h.Hfy0 = h.Hfy;
  for (int j = 1; j <= Nl; ++j)
    for (int i = 1; i <= Ml; ++i) {
      a2(h.DelxH, Ml, i, j) = (a2(h.Hfx, Ml1, i + 1, j) - a2(h.Hfx, Ml1, i, j)) / dx;
      a2(h.DelyH, Ml, i, j) = (a2(h.Hfy, Ml, i, j + 1) - a2(h.Hfy, Ml, i, j)) / dy;
    }
  // ---- initial
  auto ETA = [&](int i, int j) -> double& { return a2(h.Eta, Ml, i, j); };
  if (eta0 || uvw0) {
    const size_t g2 = (size_t)M * N, g3 = g2 * K;
    for (int j = Jb; j <= Je; ++j)
      for (int i = Ib; i <= Ie; ++i) {
        const size_t g = (size_t)(i - 3) + (size_t)M * (j - 3);
        if (eta0) ETA(i, j) = eta0[g];
        if (uvw0)
          for (int k = Kb; k <= Ke; ++k) {
            const size_t gk = g + g2 * (k - 3);
            const size_t o = (size_t)(i - 1) + (size_t)Ml * ((j - 1) + (size_t)Nl * (k - 1));
            h.U[o] = uvw0[gk];
            h.V[o] = uvw0[gk + g3];
            h.W[o] = uvw0[gk + 2 * g3];
          }
      }
  }
  for (int j = 1; j <= Nl; ++j)
    for (int i = 1; i <= Ml; ++i) {
      if ((ETA(i, j) + HC(i, j)) <= p.min_dep) { m2(h.Mask, i, j) = 0; ETA(i, j) = p.min_dep - HC(i, j); }
      else m2(h.Mask, i, j) = 1;
    }
  for (int j = 1; j <= Nl; ++j)
    for (int i = 1; i <= Ml; ++i) m2(h.Mask, i, j) = m2(h.Mask, i, j) * m2(h.Mask_Struct, i, j);
  coll(h.Eta);
  for (int j = Jb; j <= Je; ++j)
    for (int i = Ib; i <= Ie; ++i)
      m2(h.Mask9, i, j) = m2(h.Mask, i, j) * m2(h.Mask, i - 1, j) * m2(h.Mask, i + 1, j) * m2(h.Mask, i + 1, j + 1) *
                          m2(h.Mask, i, j + 1) * m2(h.Mask, i - 1, j + 1) * m2(h.Mask, i + 1, j - 1) *
                          m2(h.Mask, i, j - 1) * m2(h.Mask, i - 1, j - 1);
  for (int j = 1; j <= Nl; ++j)
    for (int i = 1; i <= Ml; ++i) a2(h.D, Ml, i, j) = dmx(HC(i, j) + ETA(i, j), p.min_dep);
  // update_wind, Iws = 1: constant in time
  {
    const double Cdsmin = (double)(1.e-3f * (0.61f + 0.063f * 6.0f));
    const double Cdsmax = (double)(1.e-3f * (0.61f + 0.063f * 50.0f));
    const double WdU = p.wind_u, WdV = p.wind_v;
    const double Wds = std::sqrt(WdU * WdU + WdV * WdV);
    double Cds = (double)1.e-3f * ((double)0.61f + (double)0.063f * Wds);
    Cds = dmn(dmx(Cds, Cdsmin), Cdsmax);
    for (int j = Jb; j <= Je; ++j)
      for (int i = Ib; i <= Ie; ++i) {
        a2(h.Wsx, Ml, i, j) = (double)0.001293f * Cds * WdU * Wds;
        a2(h.Wsy, Ml, i, j) = (double)0.001293f * Cds * WdV * Wds;
      }
  }
  // SSP-RK coefficients (default-real divisions)
  if (p.time_order == 3) {
    h.it_order = 3;
    h.alpha[0] = 0.0; h.alpha[1] = (double)(3.0f / 4.0f); h.alpha[2] = (double)(1.0f / 3.0f);
    h.beta[0] = 1.0; h.beta[1] = (double)(1.0f / 4.0f); h.beta[2] = (double)(2.0f / 3.0f);
  } else if (p.time_order == 2) {
    h.it_order = 2;
    h.alpha[0] = 0.0; h.alpha[1] = (double)(1.0f / 2.0f);
    h.beta[0] = 1.0; h.beta[1] = (double)(1.0f / 2.0f);
  } else {
    h.it_order = 1; h.alpha[0] = 0.0; h.beta[0] = 1.0;
  }
  // sponge
  for (auto& s : h.Sponge) s = 1.0;
  if (p.sponge_on) {
    auto SP = [&](int i, int j) -> double& { return a2(h.Sponge, Ml, i, j); };
    auto f = [&](double t) { return std::sqrt(1.0 - dmn(t * t, 1.0)); };
    if (p.sponge_west_width > 0.0)
      for (int j = 1; j <= Nl; ++j)
        for (int i = 1; i <= Ml; ++i)
          if (XC(i) <= p.sponge_west_width) SP(i, j) = f((XC(i) - p.sponge_west_width) / p.sponge_west_width);
    if (p.sponge_east_width > 0.0)
      for (int j = 1; j <= Nl; ++j)
        for (int i = 1; i <= Ml; ++i)
          if (XC(i) >= M * dx - p.sponge_east_width)
            SP(i, j) = f((XC(i) - (M * dx - p.sponge_east_width)) / p.sponge_east_width);
    if (p.sponge_south_width > 0.0)
      for (int j = 1; j <= Nl; ++j)
        for (int i = 1; i <= Ml; ++i)
          if (YC(j) <= p.sponge_south_width) SP(i, j) = f((YC(j) - p.sponge_south_width) / p.sponge_south_width);
    if (p.sponge_north_width > 0.0)
      for (int j = 1; j <= Nl; ++j)
        for (int i = 1; i <= Ml; ++i)
          if (YC(j) >= N * dy - p.sponge_north_width)
            SP(i, j) = f((YC(j) - (N * dy - p.sponge_north_width)) / p.sponge_north_width);
  }
  // wavemaker constants (src/source_terms.F:30-45, 418-424)
  if (p.wavemaker == NHW_WM_INT_LIN) {
    h.wm_segma = 2.0 * kPiH / p.per_wave;
    const double wn = wave_number(h.wm_segma, p.dep_wave);
    const double wl = 2.0 * kPiH / wn;
    h.wm_celerity = wl / p.per_wave;
    h.wm_wnumy = wn * std::sin(p.theta_wave * kPiH / 180.);
  } else if (p.wavemaker == NHW_WM_INT_SOL) {
    const double A = p.amp_wave, Dep = p.dep_wave;
    h.wm_celerity = std::sqrt(kGravH * Dep * (1.0 + A / Dep));
    h.wm_atmp = std::sqrt((double)0.75f * A / (Dep * Dep * Dep));
    h.wm_xstart = 4.0 * Dep / std::sqrt(A / Dep);
  } else if (p.wavemaker == NHW_WM_LEF_LIN || p.wavemaker == NHW_WM_WAV_CUR ||
             p.wavemaker == NHW_WM_RIG_LIN) {   // src/waves.F:720-730, 774-784, 820-829
    h.lef_segma = 2.0 * kPiH / p.per_wave;
    h.lef_wn = wave_number(h.lef_segma, p.dep_wave);
    const double wl = 2.0 * kPiH / h.lef_wn;
    h.lef_stokes = kGravH * (p.amp_wave * p.amp_wave) / (wl / p.per_wave) / p.dep_wave / 8.0;
    const double th = p.theta_wave * kPiH / 180.;
    h.lef_sinth = std::sin(th);
    h.lef_costh = std::cos(th);
    h.lef_shd = std::sinh(h.lef_wn * p.dep_wave);
  } else if (p.wavemaker == NHW_WM_LEF_SOL) {   // src/waves.F:879-886
    const double A = p.amp_wave, Dep = p.dep_wave;
    h.lef_cel = std::sqrt(kGravH * Dep * (1.0 + A / Dep));
    h.lef_atmp = std::sqrt((double)0.75f * A / (Dep * Dep * Dep));
    h.lef_xstart = 4.0 * Dep / std::sqrt(A / Dep);
    h.lef_c2 = std::sqrt(kGravH * Dep);
  } else if (p.wavemaker == NHW_WM_LEF_STK) {   // src/waves.F:531-540
    const double A = p.amp_wave;
    h.lef_segma = 2.0 * kPiH / p.per_wave;
    h.lef_wn = wave_number(h.lef_segma, p.dep_wave);
    const double wk = h.lef_wn, Dep = p.dep_wave;
    h.lef_shd = std::sinh(wk * Dep);
    const double sh = h.lef_shd;
    // second-order elevation and velocity amplitudes, in the reference's
    // left-to-right order up to the trigonometric factor of the step
    h.lef_e2 = (A * A) * wk / 16. * std::cosh(wk * Dep) / (sh * sh * sh) * (2.0 + std::cosh(2. * wk * Dep));
    h.lef_u2 = (double)(3.f / 16.f) * (A * A) * h.lef_segma * wk;
  } else if (p.wavemaker == NHW_WM_FOCUSED) {   // components (src/initialize.F:742-781)
    const int nw = p.nwave;
    const double dc = p.depth_comp;
    h.foc.assign(3 * (size_t)nw, 0.0);
    for (int n = 1; n <= nw; ++n) {
      const double fi = p.f_center - 0.5 * p.normalized_delta_f * p.f_center +
                        (n - 1.0) * p.normalized_delta_f * p.f_center / (nw - 1.0);
      const double period = 1.0 / fi;
      // wave number by Newton's method from the shallow-water guess, to |F| <= 1e-6
      const double sq = 2.0 * kPiH / period, segmasqr = sq * sq;
      const double ctmp = std::sqrt(kGravH * dc), xltmp = ctmp * period;
      double xxk = 2.0 * kPiH / xltmp;
      for (int it = 0;; ++it) {
        const double Fk = kGravH * xxk * std::tanh(xxk * dc) - segmasqr;
        if (std::fabs(Fk) <= (double)1.0e-6f || it > 1000) break;
        const double th = std::tanh(xxk * dc);
        const double Fkdif = kGravH * xxk * dc * (1.0 - th * th) + kGravH * std::tanh(xxk * dc);
        xxk = xxk - Fk / Fkdif;
      }
      h.foc[n - 1] = p.component_amp_type == 1 ? p.slope_group / nw / p.k_center : p.slope_group / nw / xxk;
      h.foc[nw + n - 1] = xxk;
      h.foc[2 * nw + n - 1] = fi;
    }
  } else if (p.wavemaker == NHW_WM_LEF_JON || p.wavemaker == NHW_WM_LEF_TMA) {
    jonswap_components(p, p.wavemaker == NHW_WM_LEF_TMA, h.jon);
  } else if (p.wavemaker == NHW_WM_INT_JON || p.wavemaker == NHW_WM_INT_TMA) {
    internal_jonswap_components(p, p.wavemaker == NHW_WM_INT_TMA, h.jon);
  } else if (p.wavemaker == NHW_WM_LEF_CON || p.wavemaker == NHW_WM_INT_CON) {
    // src/waves.F:100-140; src/source_terms.F:343-385 (the same start phase)
    const double A = p.amp_wave, Dep = p.dep_wave;
    double L = 0, Yt = 0, m = 0, Xstart = 0, cel = 0;
    if (!cnoidal_params(A, Dep, p.per_wave, L, Yt, m, &cel)) return NHW_ERR_ARG;
    h.wm_celerity = cel;
    if (!cnoidal_start(Yt, A, m, Xstart)) return NHW_ERR_ARG;
    double a[kCnMax], c[kCnMax];
    if (!(std::fabs(c[cn_agm(m, a, c)]) < kCnEps)) return NHW_ERR_ARG;   // sequence must fit kCnMax
    h.con_mod = m;
    h.con_len = L;
    h.con_ytr = Yt;
    h.con_ck = cnoidal_ck(m);
    h.con_x0 = Xstart * 0.5 * h.con_ck;
    h.lef_stokes = kGravH * (A * A) / (L / p.per_wave) / Dep / 8.0;
  }
  return NHW_OK;
}

}  // namespace nhw
