// ensemble.cuh -- many scenarios advanced together.
//
// One ensemble step is one CUDA graph launch.  The graph holds, for every
// member scenario, its step as kernels on a branch of its own, the branches
// running concurrently.  Per RK stage the branches join for the pressure
// solve: the solves of all members run as the groups of one persistent
// cooperative launch (psolve.cuh) -- or a few such launches ("waves") when the
// members need more blocks than the GPU holds at once -- and then fork again.
// Every member kernel is gated by its own k_dt_finalize, so a member whose run
// is over (TIME >= TOTAL_TIME or RUN_STEP >= SIM_STEPS) or that stopped at
// DT_MIN costs a few empty launches and nothing else.
//
// A member's blocks (its group size) depend only on its own size and the
// tuning options, never on the other members: a member's results are the same
// bits alone and in any mix.
//
// Tuning: the solver form, blocks per group (cells per block), block height
// and coarse-level sweeps are chosen by timing candidate settings on real
// ensemble steps (Ensemble::tune).
#pragma once
#include "solver.cuh"

namespace nhw {

class EnsembleBase {
 public:
  virtual ~EnsembleBase() {}
  virtual int step(int nsteps) = 0;
  virtual int run_timed(int nsteps, double* ms) = 0;
  virtual int tune(int steps_per_trial, nhw_ensemble_opts* chosen) = 0;
  virtual int info(nhw_ensemble_info* out) = 0;
};

template <class T>
class Ensemble final : public EnsembleBase {
 public:
  std::vector<Solver<T>*> m;
  nhw_ensemble_opts opts{};
  cudaStream_t st0 = nullptr;
  std::vector<cudaStream_t> br;
  std::vector<cudaEvent_t> ev;
  cudaEvent_t ev_fork = nullptr, ev0 = nullptr, ev1 = nullptr;
  cudaGraphExec_t exec = nullptr;
  PsGroup<T>* d_groups = nullptr;
  struct Wave { int g0, ng, blocks; size_t smem; };
  std::vector<Wave> waves;
  long long kernels = 0;
  int max_blocks = 0, device = 0, order = 3, non_hydro = 1;
  size_t smem_max = 0;
  cudaError_t lerr = cudaSuccess;
  // kernel launches: per graph launch outside loops, and per refinement sweep
  // and per BiCGSTAB iteration of each member's own solver loops
  long long per_launch = 0;
  std::vector<long long> per_sweep, per_iter;
  std::vector<int64_t> acc_ir, acc_it;
  long long launches = 0;

  ~Ensemble() override {
    cudaSetDevice(device);
    if (st0) cudaStreamSynchronize(st0);
    if (exec) cudaGraphExecDestroy(exec);
    for (auto s : br) cudaStreamDestroy(s);
    for (auto e : ev) cudaEventDestroy(e);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (d_groups) cudaFree(d_groups);
    if (st0) cudaStreamDestroy(st0);
  }

  static void defaults(nhw_ensemble_opts* o) {
    if (o->cells_per_block <= 0) o->cells_per_block = 16384;
    if (o->block_rows != 8 && o->block_rows != 16) o->block_rows = kPsBYEnsemble;
    if (o->coarse_sweeps <= 0) o->coarse_sweeps = 2;
    if (o->solver != 1) o->solver = 0;
  }

  int create(const std::vector<Solver<T>*>& members, const nhw_ensemble_opts* o) {
    m = members;
    if (o) opts = *o;
    defaults(&opts);
    device = m[0]->params().device;
    order = m[0]->order();
    non_hydro = m[0]->dev().non_hydro;
    for (auto* s : m) {
      if (!s->is_setup()) return NHW_ERR_STATE;
      if (s->params().device != device || s->order() != order || s->dev().non_hydro != non_hydro) {
        set_last_error("ensemble members must share device, TIME_ORDER and NON_HYDRO");
        return NHW_ERR_ARG;
      }
      if (non_hydro && !s->persistent_capable()) {
        set_last_error("ensemble members need the multigrid preconditioner (precond = 0)");
        return NHW_ERR_UNSUPPORTED;
      }
      smem_max = std::max(smem_max, sizeof(T) * 4 * 32 * (size_t)s->dev().K);
    }
    NHW_CU(cudaSetDevice(device));
    NHW_CU(cudaStreamCreateWithFlags(&st0, cudaStreamNonBlocking));
    br.resize(m.size());
    ev.resize(m.size());
    for (size_t i = 0; i < m.size(); ++i) {
      NHW_CU(cudaStreamCreateWithFlags(&br[i], cudaStreamNonBlocking));
      NHW_CU(cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming));
    }
    NHW_CU(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
    NHW_CU(cudaEventCreate(&ev0));
    NHW_CU(cudaEventCreate(&ev1));
    NHW_CU(cudaMalloc((void**)&d_groups, sizeof(PsGroup<T>) * m.size()));
    for (auto* s : m) NHW_CU(cudaStreamSynchronize(s->st));
    return build();
  }

  template <int BY>
  int occupancy() {
    NHW_CU(cudaFuncSetAttribute(k_psolve<T, BY>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max));
    int nsm = 0, per_sm = 0;
    NHW_CU(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device));
    NHW_CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_psolve<T, BY>, 32 * BY, smem_max));
    max_blocks = per_sm * nsm;
    if (max_blocks < 1) {
      set_last_error("ensemble: the persistent solve does not fit on a multiprocessor");
      return NHW_ERR_CUDA;
    }
    return NHW_OK;
  }

  template <int BY>
  void launch_solves() {
    for (const Wave& w : waves) {
      cudaLaunchConfig_t cfg{};
      cfg.gridDim = dim3((unsigned)w.blocks);
      cfg.blockDim = dim3(32, BY);
      cfg.dynamicSmemBytes = w.smem;
      cfg.stream = st0;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeCooperative;
      at[0].val.cooperative = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      const cudaError_t e = cudaLaunchKernelEx(&cfg, k_psolve<T, BY>, (const PsGroup<T>*)(d_groups + w.g0), w.ng, 1);
      if (e != cudaSuccess && lerr == cudaSuccess) lerr = e;
      ++kernels;
    }
  }

  // group sizes, waves, the table, then the captured graph of one step
  int build() {
    NHW_CU(cudaSetDevice(device));
    if (exec) { cudaGraphExecDestroy(exec); exec = nullptr; }
    int rc = opts.block_rows == 16 ? occupancy<16>() : occupancy<8>();
    if (rc) return rc;
    const int cap = std::min(max_blocks, kPsMaxBlocks);
    std::vector<PsGroup<T>> groups(m.size());
    waves.clear();
    Wave cur{0, 0, 0, 0};
    for (size_t i = 0; i < m.size(); ++i) {
      const long long n = m[i]->dev().neq;
      const int nb = (int)std::max(1LL, std::min<long long>(cap, (n + opts.cells_per_block - 1) / opts.cells_per_block));
      if (cur.blocks + nb > max_blocks) {
        waves.push_back(cur);
        cur = Wave{(int)i, 0, 0, 0};
      }
      groups[i] = m[i]->make_group(nb, cur.blocks, opts.coarse_sweeps);
      cur.ng += 1;
      cur.blocks += nb;
      cur.smem = std::max(cur.smem, sizeof(T) * 4 * 32 * (size_t)m[i]->dev().K);
    }
    waves.push_back(cur);
    NHW_CU(cudaMemcpyAsync(d_groups, groups.data(), sizeof(PsGroup<T>) * m.size(), cudaMemcpyHostToDevice, st0));
    NHW_CU(cudaStreamSynchronize(st0));
    // ---- capture
    kernels = 0;
    lerr = cudaSuccess;
    cudaGraph_t g = nullptr, root = nullptr;
    for (auto* s : m) s->ens_reset_counts();
    NHW_CU(cudaStreamBeginCapture(st0, cudaStreamCaptureModeThreadLocal));
    {
      cudaStreamCaptureStatus cs;
      unsigned long long id = 0;
      const cudaError_t e = cudaStreamGetCaptureInfo(st0, &cs, &id, &root, nullptr, nullptr, nullptr);
      if (e != cudaSuccess) lerr = e;
    }
    auto fork = [&] {
      cudaEventRecord(ev_fork, st0);
      for (auto s : br) cudaStreamWaitEvent(s, ev_fork, 0);
    };
    auto join = [&] {
      for (size_t i = 0; i < m.size(); ++i) {
        cudaEventRecord(ev[i], br[i]);
        cudaStreamWaitEvent(st0, ev[i], 0);
      }
    };
    int err = NHW_OK;
    auto member = [&](size_t i, auto fn) {
      const long long l0 = m[i]->launches;
      int r = m[i]->ens_begin(br[i], root, opts.coarse_sweeps);
      if (!r) fn(m[i]);
      const int r2 = m[i]->ens_end();
      m[i]->launches = l0;
      if (!r) r = r2;
      if (r && !err) err = r;
    };
    const bool groups_solve = non_hydro && opts.solver == 1;
    fork();
    for (size_t i = 0; i < m.size(); ++i)
      member(i, [&](Solver<T>* s) {
        s->ens_prefix();
        s->ens_stage_head(0);
      });
    for (int st = 0; st < order; ++st) {
      if (groups_solve) {
        // each member's coarse operators (formed on its side stream) before the solves
        for (size_t i = 0; i < m.size(); ++i) member(i, [&](Solver<T>* s) { s->ens_join_mg(); });
        join();
        if (opts.block_rows == 16) launch_solves<16>();
        else launch_solves<8>();
        fork();
      }
      for (size_t i = 0; i < m.size(); ++i)
        member(i, [&](Solver<T>* s) {
          if (non_hydro && !groups_solve) s->ens_solve();
          s->ens_stage_tail(st);
          if (st + 1 < order) s->ens_stage_head(st + 1);
        });
    }
    join();
    per_launch = kernels;   // the persistent solves
    per_sweep.assign(m.size(), 0);
    per_iter.assign(m.size(), 0);
    for (size_t i = 0; i < m.size(); ++i) {
      const long long ns = std::max(1, m[i]->cap_solves);
      per_launch += m[i]->cap_counts[3] + m[i]->cap_counts[0];
      per_sweep[i] = m[i]->cap_counts[1] / ns;
      per_iter[i] = m[i]->cap_counts[2] / ns;
    }
    kernels = per_launch;
    cudaError_t ce = cudaStreamEndCapture(st0, &g);
    if (ce == cudaSuccess && lerr != cudaSuccess) ce = lerr;
    if (ce != cudaSuccess || err) {
      if (g) cudaGraphDestroy(g);
      if (ce != cudaSuccess) set_last_error(std::string("ensemble capture: ") + cudaGetErrorString(ce));
      return err ? err : NHW_ERR_CUDA;
    }
    const cudaError_t ie = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
      set_last_error(std::string("ensemble graph instantiate: ") + cudaGetErrorString(ie));
      exec = nullptr;
      return NHW_ERR_CUDA;
    }
    return NHW_OK;
  }

  // worst member status after a batch of steps (DT_MIN or a non-finite solve)
  // pull every member's scalars; remember the loop counters for accounting
  int snapshot() {
    NHW_CU(cudaStreamSynchronize(st0));
    acc_ir.resize(m.size());
    acc_it.resize(m.size());
    for (size_t i = 0; i < m.size(); ++i) {
      const int rc = m[i]->pull();
      if (rc) return rc;
      acc_ir[i] = m[i]->scal().total_ir;
      acc_it[i] = m[i]->scal().total_it;
    }
    return NHW_OK;
  }
  int collect(int nlaunch) {
    NHW_CU(cudaStreamSynchronize(st0));
    int worst = NHW_OK;
    launches += per_launch * nlaunch;
    for (size_t ii = 0; ii < m.size(); ++ii) {
      auto* s = m[ii];
      int rc = s->pull();
      if (rc) return rc;
      const DevScal& sc = s->scal();
      if (ii < acc_ir.size()) {
        launches += per_sweep[ii] * (sc.total_ir - acc_ir[ii]) + per_iter[ii] * (sc.total_it - acc_it[ii]);
        acc_ir[ii] = sc.total_ir;
        acc_it[ii] = sc.total_it;
      }
      if (sc.status == NHW_ERR_DT_MIN) worst = std::max(worst, (int)NHW_ERR_DT_MIN);
      if (sc.bar_err) worst = std::max(worst, (int)NHW_ERR_TIMEOUT);
      if (sc.step_status == NHW_ERR_NAN) worst = std::max(worst, (int)NHW_ERR_NAN);
    }
    return worst;
  }

  int step(int nsteps) override {
    NHW_CU(cudaSetDevice(device));
    int rc = snapshot();
    if (rc) return rc;
    for (int q = 0; q < nsteps; ++q) NHW_CU(cudaGraphLaunch(exec, st0));
    return collect(nsteps);
  }

  int run_timed(int nsteps, double* ms) override {
    NHW_CU(cudaSetDevice(device));
    int rc = snapshot();
    if (rc) return rc;
    NHW_CU(cudaEventRecord(ev0, st0));
    for (int q = 0; q < nsteps; ++q) NHW_CU(cudaGraphLaunch(exec, st0));
    NHW_CU(cudaEventRecord(ev1, st0));
    NHW_CU(cudaEventSynchronize(ev1));
    float f = 0.f;
    NHW_CU(cudaEventElapsedTime(&f, ev0, ev1));
    *ms = (double)f;
    return collect(nsteps);
  }

  // Autotuner: times every candidate setting on real ensemble steps (the
  // members advance) and keeps the fastest.
  int tune(int steps_per_trial, nhw_ensemble_opts* chosen) override {
    if (steps_per_trial < 1) steps_per_trial = 1;
    std::vector<nhw_ensemble_opts> cand;
    for (int w : {2, 4, 6}) {
      nhw_ensemble_opts o{};
      o.solver = 0;
      o.coarse_sweeps = w;
      cand.push_back(o);
      if (!non_hydro) break;
      for (int c : {4096, 16384, 65536})
        for (int r : {8, 16}) {
          nhw_ensemble_opts q{};
          q.solver = 1;
          q.cells_per_block = c;
          q.block_rows = r;
          q.coarse_sweeps = w;
          cand.push_back(q);
        }
    }
    nhw_ensemble_opts best = opts;
    double best_ms = 1e300;
    for (auto o : cand) {
      defaults(&o);
      opts = o;
      int rc = build();
      if (rc) return rc;
      double ms = 0.0;
      rc = run_timed(steps_per_trial, &ms);
      if (rc) return rc;
      if (ms < best_ms) {
        best_ms = ms;
        best = opts;
      }
    }
    opts = best;
    if (chosen) *chosen = best;
    return build();
  }

  int info(nhw_ensemble_info* out) override {
    std::memset(out, 0, sizeof(*out));
    out->members = (int32_t)m.size();
    out->kernels_per_step = per_launch;
    out->kernels_launched = launches;
    out->solve_launches_per_stage = (int32_t)waves.size();
    int blocks = 0;
    for (const Wave& w : waves) blocks = std::max(blocks, w.blocks);
    out->blocks_per_launch = blocks;
    out->max_resident_blocks = max_blocks;
    out->opts = opts;
    long long cells = 0;
    for (auto* s : m) cells += s->dev().neq;
    out->cells = cells;
    return NHW_OK;
  }
};

EnsembleBase* make_ensemble_fp64(SolverBase* const* members, int n, const nhw_ensemble_opts* o, int* status);
EnsembleBase* make_ensemble_fp32(SolverBase* const* members, int n, const nhw_ensemble_opts* o, int* status);

template <class T>
EnsembleBase* make_ensemble_t(SolverBase* const* members, int n, const nhw_ensemble_opts* o, int* status) {
  std::vector<Solver<T>*> ms;
  for (int i = 0; i < n; ++i) {
    auto* s = dynamic_cast<Solver<T>*>(members[i]);
    if (!s) {
      set_last_error("ensemble members must all use the same precision");
      *status = NHW_ERR_ARG;
      return nullptr;
    }
    ms.push_back(s);
  }
  auto* e = new Ensemble<T>();
  const int rc = e->create(ms, o);
  *status = rc;
  if (rc) {
    delete e;
    return nullptr;
  }
  return e;
}

}  // namespace nhw
