// capi.cu -- the C-ABI of include/nhwave_gb300.h over the device solvers.
#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

#include "ensemble.cuh"

struct nhw_handle {
  nhw::SolverBase* s = nullptr;
  nhw_params p{};
};
struct nhw_ensemble {
  nhw::EnsembleBase* e = nullptr;
  int device = 0;
};

namespace nhw {
namespace {
std::mutex g_err_mu;
std::string g_err;
thread_local std::string t_err_copy;
}  // namespace
void set_last_error(const std::string& s) {
  std::lock_guard<std::mutex> g(g_err_mu);
  g_err = s;
}
}  // namespace nhw

using nhw::SolverBase;

#define NHW_GUARD(h)                              \
  if (!(h) || !(h)->s) return NHW_ERR_ARG;        \
  if (!(h)->s->is_setup()) return NHW_ERR_STATE;  \
  { int b_ = (h)->s->bind(); if (b_) return b_; }
#define NHW_BIND(h)                               \
  if (!(h) || !(h)->s) return NHW_ERR_ARG;        \
  { int b_ = (h)->s->bind(); if (b_) return b_; }

extern "C" {

int nhw_create(const nhw_params* params, nhw_handle** out) {
  if (!params || !out) return NHW_ERR_ARG;
  *out = nullptr;
  int st = NHW_OK;
  SolverBase* s = params->precision == NHW_FP32_IR ? nhw::make_solver_fp32(*params, &st)
                                                   : nhw::make_solver_fp64(*params, &st);
  if (!s) return st ? st : NHW_ERR_NOMEM;
  nhw_handle* h = new nhw_handle();
  h->s = s;
  h->p = *params;
  *out = h;
  return NHW_OK;
}

int nhw_device_bytes(const nhw_params* params, int64_t* bytes) {
  if (!params || !bytes) return NHW_ERR_ARG;
  size_t b = 0;
  const int rc = params->precision == NHW_FP32_IR ? nhw::device_bytes_fp32(*params, &b)
                                                  : nhw::device_bytes_fp64(*params, &b);
  *bytes = (int64_t)b;
  return rc;
}

int nhw_destroy(nhw_handle* h) {
  if (!h) return NHW_ERR_ARG;
  if (h->s) h->s->bind();
  delete h->s;
  delete h;
  return NHW_OK;
}

int nhw_setup(nhw_handle* h, const double* depth, const double* eta0, const double* uvw0) {
  if (!depth) return NHW_ERR_ARG;
  NHW_BIND(h);
  return h->s->setup(depth, eta0, uvw0);
}

int nhw_get_field(nhw_handle* h, int field, void* host) {
  NHW_BIND(h);
  return h->s->get_field(field, host);
}
int nhw_set_field(nhw_handle* h, int field, const void* host) {
  NHW_BIND(h);
  return h->s->set_field(field, host);
}
int nhw_field_shape(const nhw_handle* h, int field, int32_t dims[3], int32_t* elem_bytes) {
  if (!h || !h->s || !dims || !elem_bytes) return NHW_ERR_ARG;
  int d[3], eb;
  int rc = h->s->field_shape(field, d, &eb);
  if (rc) return rc;
  dims[0] = d[0]; dims[1] = d[1]; dims[2] = d[2];
  *elem_bytes = eb;
  return NHW_OK;
}
int nhw_get_scalars(nhw_handle* h, nhw_scalars* out) {
  if (!out) return NHW_ERR_ARG;
  NHW_BIND(h);
  return h->s->get_scalars(out);
}
int nhw_set_time(nhw_handle* h, double time, double dt, int32_t run_step) {
  NHW_BIND(h);
  return h->s->set_time(time, dt, run_step);
}

int nhw_set_wave_phases(nhw_handle* h, int32_t n, const double* phases) {
  NHW_GUARD(h);
  return h->s->set_wave_phases(n, phases);
}

int nhw_set_wave_spectrum(nhw_handle* h, int32_t numfreq, int32_t numdir, const double* freq,
                          const double* dire, const double* spc2d, const double* phases) {
  NHW_BIND(h);
  return h->s->set_wave_spectrum(numfreq, numdir, freq, dire, spc2d, phases);
}

int nhw_estimate_dt(nhw_handle* h) { NHW_GUARD(h); return h->s->estimate_dt(); }
int nhw_update_bathymetry(nhw_handle* h) { NHW_GUARD(h); int rc = h->s->update_bathymetry(); return rc ? rc : h->s->sync(); }
int nhw_update_wave_bc(nhw_handle* h) { NHW_GUARD(h); int rc = h->s->update_wave_bc(); return rc ? rc : h->s->sync(); }
int nhw_update_mask(nhw_handle* h) { NHW_GUARD(h); int rc = h->s->update_mask(); return rc ? rc : h->s->sync(); }
int nhw_update_vars(nhw_handle* h) { NHW_GUARD(h); int rc = h->s->update_vars(); return rc ? rc : h->s->sync(); }
int nhw_source_terms(nhw_handle* h) { NHW_GUARD(h); int rc = h->s->source_terms(); return rc ? rc : h->s->sync(); }
int nhw_fluxes(nhw_handle* h) { NHW_GUARD(h); int rc = h->s->fluxes(); return rc ? rc : h->s->sync(); }
int nhw_eval_duvw(nhw_handle* h, int32_t istep) {
  NHW_GUARD(h);
  int rc = h->s->eval_duvw(istep);
  int rs = h->s->sync();
  return rs ? rs : rc;
}
int nhw_sponge_damping(nhw_handle* h) { NHW_GUARD(h); int rc = h->s->sponge_damping(); return rc ? rc : h->s->sync(); }
int nhw_eval_turb(nhw_handle* h, int32_t istep) {
  NHW_GUARD(h);
  int rc = h->s->eval_turb(istep);
  return rc ? rc : h->s->sync();
}

int nhw_step(nhw_handle* h, double* time, double* dt, int32_t* run_step) {
  NHW_GUARD(h);
  int rc = h->s->step();
  if (rc == NHW_ERR_CUDA) return rc;
  if (time || dt || run_step) {
    nhw_scalars sc;
    int r2 = h->s->get_scalars(&sc);
    if (r2) return r2;
    if (time) *time = sc.time;
    if (dt) *dt = sc.dt;
    if (run_step) *run_step = sc.run_step;
  }
  return rc;
}

int nhw_run(nhw_handle* h, int32_t nsteps, int32_t* steps_done) {
  NHW_GUARD(h);
  int done = 0;
  const int rc = nsteps > 0 ? h->s->run(nsteps, &done) : NHW_OK;
  if (steps_done) *steps_done = done;
  return rc;
}

int nhw_ensemble_create(nhw_handle* const* members, int32_t n, const nhw_ensemble_opts* opts,
                        nhw_ensemble** out) {
  if (!members || n < 1 || !out) return NHW_ERR_ARG;
  *out = nullptr;
  std::vector<SolverBase*> ss;
  for (int i = 0; i < n; ++i) {
    if (!members[i] || !members[i]->s) return NHW_ERR_ARG;
    if (!members[i]->s->is_setup()) return NHW_ERR_STATE;
    for (int j = 0; j < i; ++j)
      if (members[j] == members[i]) return NHW_ERR_ARG;
    ss.push_back(members[i]->s);
  }
  int rc = members[0]->s->bind();
  if (rc) return rc;
  int st = NHW_OK;
  nhw::EnsembleBase* e = members[0]->p.precision == NHW_FP32_IR
                             ? nhw::make_ensemble_fp32(ss.data(), n, opts, &st)
                             : nhw::make_ensemble_fp64(ss.data(), n, opts, &st);
  if (!e) return st ? st : NHW_ERR_NOMEM;
  *out = new nhw_ensemble{e, members[0]->p.device};
  return NHW_OK;
}
#define NHW_ENS(e)                                            \
  if (!(e) || !(e)->e) return NHW_ERR_ARG;                    \
  {                                                           \
    const cudaError_t de_ = cudaSetDevice((e)->device);      \
    if (de_ != cudaSuccess) return NHW_ERR_CUDA;              \
  }
int nhw_ensemble_step(nhw_ensemble* e, int32_t nsteps) {
  NHW_ENS(e);
  if (nsteps < 0) return NHW_ERR_ARG;
  return e->e->step(nsteps);
}
int nhw_ensemble_run_timed(nhw_ensemble* e, int32_t nsteps, double* device_ms) {
  NHW_ENS(e);
  if (nsteps < 1 || !device_ms) return NHW_ERR_ARG;
  return e->e->run_timed(nsteps, device_ms);
}
int nhw_ensemble_tune(nhw_ensemble* e, int32_t steps_per_trial, nhw_ensemble_opts* chosen) {
  NHW_ENS(e);
  return e->e->tune(steps_per_trial, chosen);
}
int nhw_ensemble_get_info(nhw_ensemble* e, nhw_ensemble_info* out) {
  NHW_ENS(e);
  if (!out) return NHW_ERR_ARG;
  return e->e->info(out);
}
int nhw_ensemble_destroy(nhw_ensemble* e) {
  if (!e) return NHW_ERR_ARG;
  cudaSetDevice(e->device);
  delete e->e;
  delete e;
  return NHW_OK;
}

int nhw_checkpoint_bytes(nhw_handle* h, int64_t* bytes) {
  NHW_GUARD(h);
  if (!bytes) return NHW_ERR_ARG;
  size_t b = 0;
  const int rc = h->s->checkpoint_bytes(&b);
  *bytes = (int64_t)b;
  return rc;
}
int nhw_save_state(nhw_handle* h, void* host, int64_t bytes) {
  NHW_GUARD(h);
  if (bytes < 0) return NHW_ERR_ARG;
  return h->s->save_state(host, (size_t)bytes);
}
int nhw_load_state(nhw_handle* h, const void* host, int64_t bytes) {
  NHW_GUARD(h);
  if (bytes < 0) return NHW_ERR_ARG;
  return h->s->load_state(host, (size_t)bytes);
}

int nhw_mass(nhw_handle* h, double* mass) {
  NHW_GUARD(h);
  if (!mass) return NHW_ERR_ARG;
  return h->s->mass(mass);
}
int nhw_statistics(nhw_handle* h, nhw_stats* out) {
  NHW_GUARD(h);
  if (!out) return NHW_ERR_ARG;
  double v[7];
  const int rc = h->s->statistics(v);
  if (rc) return rc;
  out->mass_volume = v[0]; out->energy = v[1]; out->max_eta = v[2]; out->min_eta = v[3];
  out->max_u = v[4]; out->max_v = v[5]; out->max_w = v[6];
  return NHW_OK;
}
int nhw_synchronize(nhw_handle* h) {
  NHW_BIND(h);
  return h->s->sync();
}

int nhw_run_timed(nhw_handle* h, int32_t nsteps, double* device_ms) {
  NHW_GUARD(h);
  if (!device_ms || nsteps < 0) return NHW_ERR_ARG;
  return h->s->run_timed(nsteps, device_ms);
}
int nhw_profile(nhw_handle* h, int32_t on) {
  NHW_BIND(h);
  return h->s->profile(on);
}
int nhw_profile_report(nhw_handle* h, char* buf, int32_t buflen) {
  NHW_BIND(h);
  return h->s->profile_report(buf, buflen);
}
int nhw_time_smoother(nhw_handle* h, int32_t reps, int64_t flush_bytes, double* us_per_launch) {
  NHW_GUARD(h);
  if (!us_per_launch) return NHW_ERR_ARG;
  return h->s->time_smoother(reps, (long long)flush_bytes, us_per_launch);
}

int nhw_abi_sizes(int32_t* params_bytes, int32_t* scalars_bytes) {
  if (!params_bytes || !scalars_bytes) return NHW_ERR_ARG;
  *params_bytes = (int32_t)sizeof(nhw_params);
  *scalars_bytes = (int32_t)sizeof(nhw_scalars);
  return NHW_OK;
}

const char* nhw_status_string(int status) {
  switch (status) {
    case NHW_OK: return "ok";
    case NHW_ERR_ARG: return "bad argument";
    case NHW_ERR_UNSUPPORTED: return "option outside the GPU path";
    case NHW_ERR_CUDA: return "CUDA error";
    case NHW_ERR_NOMEM: return "device allocation failed";
    case NHW_ERR_DT_MIN: return "time step too small (dt < DT_MIN)";
    case NHW_ERR_KRYLOV_NOCONV: return "Poisson solve did not reach TOL within ITMAX";
    case NHW_ERR_NAN: return "non-finite Poisson residual";
    case NHW_ERR_TIMEOUT: return "bounded device wait timed out";
    case NHW_ERR_STATE: return "call out of order";
    case NHW_ERR_CAPACITY: return "capacity exhausted";
    case NHW_ERR_NOT_FOUND: return "unknown id";
    default: return "unknown status";
  }
}
const char* nhw_last_error(void) {
  std::lock_guard<std::mutex> g(nhw::g_err_mu);
  nhw::t_err_copy = nhw::g_err;
  return nhw::t_err_copy.c_str();
}

}  // extern "C"
