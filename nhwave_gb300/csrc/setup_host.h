// setup_host.h -- host-side scenario set-up (the work of generate_grid,
// read_bathymetry and initial), producing Fortran-layout arrays to upload.
#pragma once
#include <cstdint>
#include <vector>
#include "../../include/nhwave_gb300.h"
#include "components.h"

namespace nhw {

struct HostInit {
  int Mloc = 0, Nloc = 0, Kloc = 0;
  std::vector<double> x, xc, y, yc, sig, dsig, sigc;                 // 1-D grid
  std::vector<double> Hc, Hc0, DelxH, DelyH, Eta, D, Sponge, Wsx, Wsy; // (Mloc,Nloc)
  std::vector<double> Hfx, Hfx0;                                      // (Mloc+1,Nloc)
  std::vector<double> Hfy, Hfy0;                                      // (Mloc,Nloc+1)
  std::vector<int32_t> Mask, Mask_Struct, Mask9;                      // (Mloc,Nloc)
  std::vector<double> U, V, W;                                        // (Mloc,Nloc,Kloc)
  double alpha[3] = {0, 0, 0}, beta[3] = {0, 0, 0};
  int it_order = 1;
  // host-computed wavemaker constants
  double wm_segma = 0, wm_celerity = 0, wm_wnumy = 0, wm_atmp = 0, wm_xstart = 0;
  // LEF_* boundary waves (src/waves.F:92-170, 518-560, 808-903)
  double lef_segma = 0, lef_wn = 0, lef_shd = 0, lef_stokes = 0, lef_sinth = 0, lef_costh = 0;
  double lef_cel = 0, lef_atmp = 0, lef_xstart = 0, lef_c2 = 0;
  double lef_e2 = 0, lef_u2 = 0;                          // LEF_STK second-order amplitudes
  double con_mod = 0, con_len = 0, con_ytr = 0, con_ck = 0, con_x0 = 0;   // LEF_CON
  std::vector<double> foc;   // FOCUSED: Amp_i [nwave], k_i [nwave], f_i [nwave]
  // LEF_JON / LEF_TMA components, slot-major [8][NumFreq]: wave height Wh,
  // angular frequency 2 pi f, wave number, Stokes drift, phase, sinh(k h),
  // sin and cos of the direction (0 and 1 here; LEF_SPC fills them)
  std::vector<double> jon;
};

// Validate parameters against the path's scope; NHW_OK or an error code.
int check_params(const nhw_params& p);
// Build the initial state.  depth/eta0/uvw0 follow nhw_setup's contract.
int host_setup(const nhw_params& p, const double* depth, const double* eta0, const double* uvw0,
               HostInit& out);
// Wave number of linear dispersion by Newton iteration (src/waves.F:61-91).
double wave_number(double segma, double dep);
// Phase i (radians, [0, 2 pi)) of the irregular boundary waves' stream `seed`.
double wave_phase(int32_t seed, int i);

// LEF_SPC components from a 2-D spectrum (src/waves.F:388-465), slot-major
// [8][numfreq * numdir], component (nfreq, ndir) at ndir + numdir * nfreq;
// phases == nullptr: the stream of p.wave_seed.  False on a bad spectrum.
bool spectrum_components(const nhw_params& p, int numfreq, int numdir, const double* freq, const double* dire,
                         const double* spc2d, const double* phases, std::vector<double>& out);
// INT_SPC / INT_IRR components (src/source_terms.F:71-300) in the internal
// makers' layout, component (nfreq, ndir) at ndir + numdir * nfreq; each
// direction snapped as the reference does (snap_direction).  INT_IRR takes
// amplitudes and needs the phases.  False on a bad spectrum.
bool internal_spectrum_components(const nhw_params& p, int numfreq, int numdir, const double* freq,
                                  const double* dire, const double* spc2d, const double* phases,
                                  std::vector<double>& out);
// A component direction (radians) snapped to the nearest one whose
// cross-channel wave number nk 2 pi / (Nglob dy) the channel repeats
// (src/source_terms.F:94-136; INT_IRR's form, irr, keeps a zero direction,
// :203-247).  False when the search does not end (|Angle| > 90 degrees).
bool snap_direction(double Angle, double k, int Nglob, double dy, bool irr, double& out);

}  // namespace nhw
