// psolve.cuh -- one whole pressure solve as one persistent kernel.
//
// The solve of poisson_solver (src/pressure.F:63-245; HYPRE GMRES+SMG in the
// parallel build, :260-462) is, here, FP64 iterative refinement around a
// right-preconditioned BiCGSTAB whose preconditioner is the multigrid V-cycle
// of mg.cuh.  Launched phase by phase that is about 57 kernels per BiCGSTAB
// iteration, most of them a few microseconds of work on coarse levels, so the
// solve is bound by launch and tail latency.  Here one cooperative launch runs
// all of it: the blocks of a group (one scenario) sweep each phase in a
// block-strided loop and meet at a grid barrier between phases.  Several
// groups -- several scenarios -- can share one launch, each with its own
// barrier and its own blocks.
//
// Barrier: arrival counter and generation word in the scenario's DevScal,
// polled with a bounded spin; a block that gives up sets bar_err, after which
// every barrier of that group returns at once and every loop still ends
// (inner iterations are capped by ITMAX, refinement sweeps by max_ir), and
// the host reports NHW_ERR_TIMEOUT.  The cooperative launch guarantees that
// all blocks are resident, so the spin limit is a safety net only.
//
// Memory visibility: data written by other blocks between barriers is read
// with plain loads (no __restrict__, no read-only cache path); the barrier's
// __threadfence on both sides orders it.
//
// Dot products: each block reduces its cells, writes one partial per value
// (double-buffered, so a block that runs ahead cannot overwrite a partial
// another block still reads), and after the barrier every block sums the
// partials in the same fixed order -- every block gets bit-identical totals
// and takes identical decisions, with no second barrier.
#pragma once
#include "mg.cuh"

namespace nhw {

constexpr int kPsBY = 16;                          // block = 32 x kPsBY threads (one scenario)
constexpr int kPsBYEnsemble = 8;                   // 32 x 8 when many scenarios share a launch
constexpr int kPsMaxLevels = 16;
constexpr int kPsMaxBlocks = 1024;                 // blocks of one group at most
constexpr long long kPsSpinLimit = 1ll << 20;      // about a second of polling (L2 round trip + 64 ns sleep)

template <class T>
struct PsGroup {
  Dev<T> S;
  MGL<T> L[kPsMaxLevels];   // L[0] is the fine level (its b and x are set per V-cycle)
  int nl;                   // levels 0..nl-1 are swept by all blocks of the group
  int ntot;                 // levels nl..ntot-1 run inside the group's first block
  T w;                      // coarse-correction weight
  int coarse_sweeps;
  int b0, nb;               // the group's blocks: [b0, b0 + nb)
  int bar_nb;               // arrivals a barrier waits for (nb; more only in the timeout test)
  double* part;             // [2][nb][4] partial sums
};

// ------------------------------------------------------------------ barrier
__device__ __forceinline__ void ps_sync(DevScal* sc, int nb) {
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    volatile int* verr = &sc->bar_err;
    if (*verr == 0) {
      volatile unsigned* vgen = &sc->bar_gen;
      const unsigned g = *vgen;
      __threadfence();
      if (atomicAdd(&sc->bar_count, 1u) == (unsigned)nb - 1) {
        atomicExch(&sc->bar_count, 0u);
        __threadfence();
        atomicAdd(&sc->bar_gen, 1u);
      } else {
        long long spins = 0;
        while (*vgen == g) {
          if (++spins > kPsSpinLimit) {
            atomicExch(&sc->bar_err, 1);
            break;
          }
          __nanosleep(64);
        }
      }
    }
    __threadfence();
  }
  __syncthreads();
}

// Block sum of NV doubles, then the group-wide total of every value in every
// block (fixed order).  `rid` selects the partial buffer and advances.
template <int NV, class T>
__device__ __forceinline__ void ps_reduce(const PsGroup<T>& G, int lb, int& rid, double (&v)[NV],
                                          double (&tot)[NV]) {
  __shared__ double s_w[NV][32];
  __shared__ double s_t[NV];
  const int tid = threadIdx.x + 32 * threadIdx.y, lane = tid & 31, warp = tid >> 5, nw = blockDim.y;
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    double x = v[q];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) s_w[q][warp] = x;
  }
  __syncthreads();
  double* part = G.part + (size_t)(rid & 1) * G.nb * 4;
  if (tid < NV) {
    double x = 0.0;
    for (int w = 0; w < nw; ++w) x += s_w[tid][w];
    part[(size_t)lb * 4 + tid] = x;
  }
  ps_sync(G.S.sc, G.bar_nb);
  if (warp == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      double x = 0.0;
      for (int b = lane; b < G.nb; b += 32) x += ((volatile double*)part)[(size_t)b * 4 + q];
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if (lane == 0) s_t[q] = x;
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NV; ++q) tot[q] = s_t[q];
  __syncthreads();
  ++rid;
}

// --------------------------------------------- operator pieces (plain loads)
template <class T>
__device__ __forceinline__ T ps_xval(const T* x, const Prolong<T>& P, int ic) {
  if (!P.xc) return x[ic];
  return x[ic] + P.w * P.coarse(ic);
}

// off-column part of (A x): everything but C1, C6, C13
template <class T>
__device__ __forceinline__ T ps_off_column(const MGL<T>& L, const T* x, const Prolong<T>& P, int ic, int ii, int jj,
                                           int kk) {
  const int M = L.M, MN = L.M * L.N, n = L.n;
  const bool im = ii > 0, ip = ii < L.M - 1, jm = jj > 0, jp = jj < L.N - 1, km = kk > 0, kp = kk < L.K - 1;
  T s = (T)0;
  if (ip) s += cx_p(L, ic) * ps_xval(x, P, ic + 1);
  if (im) s += cx_m(L, ic) * ps_xval(x, P, ic - 1);
  if (jp) s += cy_p(L, ic) * ps_xval(x, P, ic + M);
  if (jm) s += cy_m(L, ic) * ps_xval(x, P, ic - M);
  const T c4 = L.coef[3 * n + ic], c5 = L.coef[4 * n + ic], c7 = L.coef[5 * n + ic], c8 = L.coef[6 * n + ic];
  if (kp) {
    const int u = ic + MN;
    if (ip) s += c7 * ps_xval(x, P, u + 1);
    if (im) s += c5 * ps_xval(x, P, u - 1);
    if (jp) s += c8 * ps_xval(x, P, u + M);
    if (jm) s += c4 * ps_xval(x, P, u - M);
  }
  if (km) {
    const int d = ic - MN;
    if (ip) s -= c7 * ps_xval(x, P, d + 1);
    if (im) s -= c5 * ps_xval(x, P, d - 1);
    if (jp) s -= c8 * ps_xval(x, P, d + M);
    if (jm) s -= c4 * ps_xval(x, P, d - M);
  }
  return s;
}

template <class T>
__device__ __forceinline__ T ps_apply(const MGL<T>& L, const T* x, int ic, int ii, int jj, int kk) {
  const Prolong<T> none{nullptr, (T)0, 1, 1, 1, 1, 1, 1};
  const int MN = L.M * L.N;
  T s = L.coef[ic] * x[ic] + ps_off_column(L, x, none, ic, ii, jj, kk);
  if (kk < L.K - 1) s += L.coef[L.n + ic] * x[ic + MN];
  if (kk > 0) s += L.coef[2 * L.n + ic] * x[ic - MN];
  return s;
}

// compact-operator product (A x)_ic of krylov.cuh, plain loads of x
template <class C, class V>
__device__ __forceinline__ V ps_spmv(const C* cf, const V* x, size_t n, int ic, int ii, int jj, int kk, int M, int N,
                                     int K, V cxx, V cyy) {
  const int MN = M * N;
  const bool im = ii > 0, ip = ii < M - 1, jm = jj > 0, jp = jj < N - 1, km = kk > 0, kp = kk < K - 1;
  V s = (V)cf[ic] * x[ic];
  V h = (V)0;
  if (ip) h += x[ic + 1];
  if (im) h += x[ic - 1];
  s += cxx * h;
  h = (V)0;
  if (jp) h += x[ic + M];
  if (jm) h += x[ic - M];
  s += cyy * h;
  const V c4 = (V)cf[3 * n + ic], c5 = (V)cf[4 * n + ic], c7 = (V)cf[5 * n + ic], c8 = (V)cf[6 * n + ic];
  if (kp) {
    const int u = ic + MN;
    s += (V)cf[n + ic] * x[u];
    if (ip) s += c7 * x[u + 1];
    if (im) s += c5 * x[u - 1];
    if (jp) s += c8 * x[u + M];
    if (jm) s += c4 * x[u - M];
  }
  if (km) {
    const int d = ic - MN;
    s += (V)cf[2 * n + ic] * x[d];
    if (ip) s -= c7 * x[d + 1];
    if (im) s -= c5 * x[d - 1];
    if (jp) s -= c8 * x[d + M];
    if (jm) s -= c4 * x[d - M];
  }
  return s;
}

// ------------------------------------------- right-hand sides of the fine level
template <class T>
struct PsPlainB {   // b as stored
  const T* b;
  __device__ __forceinline__ T operator()(int ic) const { return b[ic]; }
};
template <class T>
struct PsInP {      // p = r + beta (p - omega v) (p = r on the first pass), stored as it is formed
  T* p;
  const T* r;
  const T* v;
  T beta, omega;
  int first;
  __device__ __forceinline__ T operator()(int ic) const {
    const T val = first ? r[ic] : r[ic] + beta * (p[ic] - omega * v[ic]);
    p[ic] = val;
    return val;
  }
};
template <class T>
struct PsInS {      // s = r - alpha v, stored as it is formed
  T* s;
  const T* r;
  const T* v;
  T alpha;
  __device__ __forceinline__ T operator()(int ic) const {
    const T val = r[ic] - alpha * v[ic];
    s[ic] = val;
    return val;
  }
};

// ----------------------------------------------------- multigrid phases
// Red-black line Gauss-Seidel half-sweep over the columns of one colour, in
// units of 32 columns: the block forms the line right-hand sides of a unit in
// shared memory (lanes along the columns, warps along the levels), then warp
// 0 runs the Thomas sweeps.  `in` yields the right-hand side; `P` applies a
// pending coarse correction to neighbour values.  Units first, first + step,
// ... go to this block.  sh holds 4 x [K][32] values.
template <class T, class In>
__device__ void ps_sweep(const MGL<T>& L, int color, bool zero_x, In in, const Prolong<T>& P, T* sh, int first,
                         int step) {
  const int K = L.K, M = L.M, MN = L.M * L.N, n = L.n;
  T* s_rhs = sh;
  T* s_a = sh + K * 32;
  T* s_inv = sh + 2 * K * 32;
  T* s_cp = sh + 3 * K * 32;
  const int tx = threadIdx.x, ty = threadIdx.y, by = blockDim.y;
  const int ncol_row0 = (M + 1 - color) / 2, ncol_row1 = (M + color) / 2, pair = ncol_row0 + ncol_row1;
  const int ncols = pair * ((L.N + 1) / 2);
  const int nunits = (ncols + 31) / 32;
  for (int u = first; u < nunits; u += step) {
    const int t = u * 32 + tx;
    const int jp2 = t / pair, rem = t - jp2 * pair;
    int jj, ii;
    if (rem < ncol_row0) { jj = 2 * jp2; ii = 2 * rem + color; }
    else { jj = 2 * jp2 + 1; ii = 2 * (rem - ncol_row0) + (1 - color); }
    const bool valid = t < ncols && jj < L.N && ii < M;
    const int col = ii + M * jj;
    for (int k = ty; k < K; k += by) {
      T rhs = (T)0, a = (T)0, inv = (T)0, cp = (T)0;
      if (valid) {
        const int ic = col + MN * k;
        const T off = zero_x ? (T)0 : ps_off_column(L, L.x, P, ic, ii, jj, k);
        rhs = in(ic) - off;
        a = k > 0 ? L.coef[2 * n + ic] : (T)0;
        inv = L.linv[ic];
        cp = L.lcp[ic];
      }
      s_rhs[k * 32 + tx] = rhs;
      s_a[k * 32 + tx] = a;
      s_inv[k * 32 + tx] = inv;
      s_cp[k * 32 + tx] = cp;
    }
    __syncthreads();
    if (ty == 0 && valid) {
      T prev = (T)0;
      for (int k = 0; k < K; ++k) {
        prev = (s_rhs[k * 32 + tx] - s_a[k * 32 + tx] * prev) * s_inv[k * 32 + tx];
        s_rhs[k * 32 + tx] = prev;
      }
      T z = prev;
      L.x[col + MN * (K - 1)] = z;
      for (int k = K - 2; k >= 0; --k) {
        z = s_rhs[k * 32 + tx] - s_cp[k * 32 + tx] * z;
        L.x[col + MN * k] = z;
      }
    }
    __syncthreads();
  }
}

// b_c = P^T (b_f - A_f x_f), x_c = 0 over coarse cells first..n step `step`
template <class T>
__device__ void ps_restrict(const MGL<T>& F, const MGL<T>& C, int first, int step) {
  for (int ic = first; ic < C.n; ic += step) {
    int I, J, k;
    decode(ic, C.M, C.N, I, J, k);
    T acc = (T)0;
    for (int b = 0; b < F.ry; ++b) {
      const int j = J * F.ry + b;
      if (j >= F.N) break;
      for (int a = 0; a < F.rx; ++a) {
        const int i = I * F.rx + a;
        if (i >= F.M) break;
        const int f = i + F.M * (j + F.N * k);
        acc += F.b[f] - ps_apply(F, F.x, f, i, j, k);
      }
    }
    C.b[ic] = acc;
    C.x[ic] = (T)0;
  }
}

// V-cycle over levels lo..hi-1 inside one block
template <class T>
__device__ void ps_cta_cycle(const MGL<T>* Ls, int lo, int hi, T w, int coarse_sweeps, T* sh) {
  const Prolong<T> none{nullptr, (T)0, 1, 1, 1, 1, 1, 1};
  const int tid = threadIdx.x + blockDim.x * threadIdx.y, nt = blockDim.x * blockDim.y;
  for (int l = lo; l < hi - 1; ++l) {
    ps_sweep(Ls[l], 0, true, PsPlainB<T>{Ls[l].b}, none, sh, 0, 1);
    ps_sweep(Ls[l], 1, false, PsPlainB<T>{Ls[l].b}, none, sh, 0, 1);
    ps_restrict(Ls[l], Ls[l + 1], tid, nt);
    __syncthreads();
  }
  const MGL<T>& cl = Ls[hi - 1];
  for (int s = 0; s < coarse_sweeps; ++s) {
    ps_sweep(cl, 0, s == 0, PsPlainB<T>{cl.b}, none, sh, 0, 1);
    ps_sweep(cl, 1, false, PsPlainB<T>{cl.b}, none, sh, 0, 1);
  }
  for (int l = hi - 2; l >= lo; --l) {
    const MGL<T>& F = Ls[l];
    const MGL<T>& C = Ls[l + 1];
    const Prolong<T> pr = prolong_from(F, C, w);
    ps_sweep(F, 1, false, PsPlainB<T>{F.b}, pr, sh, 0, 1);
    ps_sweep(F, 0, false, PsPlainB<T>{F.b}, none, sh, 0, 1);
  }
}

// x ~= A^-1 b by one V-cycle; the fine level's b is formed (and stored) by
// `in0` during the first two half-sweeps.  Ls[0] carries the fine level's b/x.
template <class T, class In>
__device__ void ps_vcycle(const PsGroup<T>& G, const MGL<T>* Ls, In in0, T* sh, int lb) {
  const Prolong<T> none{nullptr, (T)0, 1, 1, 1, 1, 1, 1};
  const int tid = threadIdx.x + 32 * threadIdx.y, nt = 32 * blockDim.y;
  DevScal* sc = G.S.sc;
  if (G.nl == 0) {   // the whole hierarchy fits one block: form b first
    for (int ic = lb * nt + tid; ic < Ls[0].n; ic += G.nb * nt) (void)in0(ic);
    ps_sync(sc, G.bar_nb);
    if (lb == 0) ps_cta_cycle(Ls, 0, G.ntot, G.w, G.coarse_sweeps, sh);
    ps_sync(sc, G.bar_nb);
    return;
  }
  for (int l = 0; l < G.nl; ++l) {
    const MGL<T>& Lv = Ls[l];
    if (l == 0) {
      ps_sweep(Lv, 0, true, in0, none, sh, lb, G.nb);
      ps_sync(sc, G.bar_nb);
      ps_sweep(Lv, 1, false, in0, none, sh, lb, G.nb);
    } else {
      ps_sweep(Lv, 0, true, PsPlainB<T>{Lv.b}, none, sh, lb, G.nb);
      ps_sync(sc, G.bar_nb);
      ps_sweep(Lv, 1, false, PsPlainB<T>{Lv.b}, none, sh, lb, G.nb);
    }
    ps_sync(sc, G.bar_nb);
    ps_restrict(Lv, Ls[l + 1], lb * nt + tid, G.nb * nt);
    ps_sync(sc, G.bar_nb);
  }
  if (lb == 0) ps_cta_cycle(Ls, G.nl, G.ntot, G.w, G.coarse_sweeps, sh);
  ps_sync(sc, G.bar_nb);
  for (int l = G.nl - 1; l >= 0; --l) {
    const MGL<T>& F = Ls[l];
    const MGL<T>& C = Ls[l + 1];
    const Prolong<T> pr = prolong_from(F, C, G.w);
    ps_sweep(F, 1, false, PsPlainB<T>{F.b}, pr, sh, lb, G.nb);
    ps_sync(sc, G.bar_nb);
    ps_sweep(F, 0, false, PsPlainB<T>{F.b}, none, sh, lb, G.nb);
    ps_sync(sc, G.bar_nb);
  }
}

// ------------------------------------------------------------ the solve
// Decisions follow the refinement and BiCGSTAB tests of k_res64, k_bicg_init
// and k_bicg_xr (krylov.cuh) exactly; the group's first block reports them
// in DevScal for the host.
// `gated` (a kernel captured into a step graph): a group whose scenario's
// step was held back by k_dt_finalize returns at once -- every block of the
// group reads the same flag, so no block is left waiting at a barrier.
template <class T, int BY>
__global__ void __launch_bounds__(32 * BY, BY >= 16 ? 1 : 2) k_psolve(const PsGroup<T>* groups, int ngroups,
                                                                     int gated) {
  extern __shared__ unsigned char smem_raw[];
  using A = typename Acc<T>::type;
  int gi = 0;
  while (gi + 1 < ngroups && (int)blockIdx.x >= groups[gi + 1].b0) ++gi;
  const PsGroup<T>& G = groups[gi];
  const int lb = (int)blockIdx.x - G.b0;
  const Dev<T>& S = G.S;
  DevScal* sc = S.sc;
  if (gated && !sc->step_go) return;
  const int tid = threadIdx.x + 32 * threadIdx.y;
  const bool reporter = lb == 0 && tid == 0;
  T* sh = reinterpret_cast<T*>(smem_raw);   // 4 x [K][32] line-sweep values
  const int n = S.neq, M = S.M, N = S.N, K = S.K;
  const int c0 = lb * 32 * BY + tid, cstep = G.nb * 32 * BY;
  const T cxxT = (T)S.cxx, cyyT = (T)S.cyy;
  // per-block copy of the level table so that the fine level's b/x can be swapped
  __shared__ MGL<T> Ls[kPsMaxLevels];
  for (int l = tid; l < G.ntot; l += 32 * BY) Ls[l] = G.L[l];
  __syncthreads();

  int rid = 0;
  int ir_count = 0, inner_total = 0, pstat = 0, conv = 0;
  if (reporter) {
    sc->solves = sc->solves + 1;
    sc->zero_x = 0;
  }
  while (true) {
    // ---- FP64 residual r64 = b - A64 x64; inner start r = r0 = (T) r64, x = 0
    double v3[3] = {0.0, 0.0, 0.0};
    A rho_acc = (A)0;
    for (int ic = c0; ic < n; ic += cstep) {
      int ii, jj, kk;
      decode(ic, M, N, ii, jj, kk);
      const double b = S.rhs64[ic];
      const double r = b - ps_spmv<double, double>(S.coef64, S.xsol64, (size_t)n, ic, ii, jj, kk, M, N, K, S.cxx,
                                                   S.cyy);
      S.res64[ic] = r;
      const T rt = (T)r;
      S.kr0[ic] = rt;
      S.kr[ic] = rt;
      S.kx[ic] = (T)0;
      v3[0] += r * r;
      v3[1] += b * b;
      rho_acc += (A)rt * (A)rt;
    }
    v3[2] = (double)rho_acc;
    double t3[3];
    ps_reduce<3>(G, lb, rid, v3, t3);
    const double bnorm = sqrt(t3[1]);
    const double rel = bnorm > 0.0 ? sqrt(t3[0]) / bnorm : 0.0;
    int go = 0, st = 0;
    double tol_in = 0.0;
    int itmax_in = 0;
    if (conv == 5 || !(rel == rel)) st = kStNaN;
    else if (bnorm == 0.0) { if (reporter) sc->zero_x = 1; }
    else if (rel <= S.tol) {}
    else if (ir_count >= S.max_ir || inner_total >= S.itmax) st = kStKrylovNoconv;
    else {
      tol_in = 0.5 * S.tol / rel;
      if (tol_in < S.tol_floor) tol_in = S.tol_floor;
      itmax_in = S.itmax - inner_total;
      ++ir_count;
      go = 1;
    }
    if (reporter) {
      sc->bnorm = bnorm;
      sc->relres64 = rel;
      if (go) sc->total_ir = sc->total_ir + 1;
    }
    if (!go) {
      pstat = st;
      break;
    }
    // ---- BiCGSTAB from c = 0
    double rho = t3[2];
    const double red0 = sqrt(rho);
    double alpha = 1.0, omega = 1.0, beta = 0.0;
    int it = 0;
    conv = (rho == 0.0) ? 1 : 0;
    int first = 1;
    while (conv == 0) {
      // ph = M^-1 p
      if (tid == 0) {
        Ls[0].b = S.kp;
        Ls[0].x = S.kph;
      }
      __syncthreads();
      ps_vcycle(G, Ls, PsInP<T>{S.kp, S.kr, S.kv, (T)beta, (T)omega, first}, sh, lb);
      first = 0;
      // v = A ph; alpha = rho / (r0, v)
      A a1 = (A)0;
      for (int ic = c0; ic < n; ic += cstep) {
        int ii, jj, kk;
        decode(ic, M, N, ii, jj, kk);
        const T y = ps_spmv<T, T>(S.coefT, S.kph, (size_t)n, ic, ii, jj, kk, M, N, K, cxxT, cyyT);
        S.kv[ic] = y;
        a1 += (A)S.kr0[ic] * (A)y;
      }
      double v1[1] = {(double)a1}, t1[1];
      ps_reduce<1>(G, lb, rid, v1, t1);
      if (t1[0] == 0.0 || !(t1[0] == t1[0])) { conv = 2; break; }
      alpha = rho / t1[0];
      // sh = M^-1 s
      if (tid == 0) {
        Ls[0].b = S.ks;
        Ls[0].x = S.ksh;
      }
      __syncthreads();
      ps_vcycle(G, Ls, PsInS<T>{S.ks, S.kr, S.kv, (T)alpha}, sh, lb);
      // t = A sh; omega = (t, s) / (t, t)
      A a2[2] = {(A)0, (A)0};
      for (int ic = c0; ic < n; ic += cstep) {
        int ii, jj, kk;
        decode(ic, M, N, ii, jj, kk);
        const T y = ps_spmv<T, T>(S.coefT, S.ksh, (size_t)n, ic, ii, jj, kk, M, N, K, cxxT, cyyT);
        S.kt[ic] = y;
        a2[0] += (A)y * (A)S.ks[ic];
        a2[1] += (A)y * (A)y;
      }
      double v2[2] = {(double)a2[0], (double)a2[1]}, t2[2];
      ps_reduce<2>(G, lb, rid, v2, t2);
      omega = t2[1] > 0.0 ? t2[0] / t2[1] : 0.0;
      // x += alpha ph + omega sh; r = s - omega t
      const T aT = (T)alpha, oT = (T)omega;
      A a3[2] = {(A)0, (A)0};
      for (int ic = c0; ic < n; ic += cstep) {
        S.kx[ic] = S.kx[ic] + aT * S.kph[ic] + oT * S.ksh[ic];
        const T r = S.ks[ic] - oT * S.kt[ic];
        S.kr[ic] = r;
        a3[0] += (A)S.kr0[ic] * (A)r;
        a3[1] += (A)r * (A)r;
      }
      double v4[2] = {(double)a3[0], (double)a3[1]}, t4[2];
      ps_reduce<2>(G, lb, rid, v4, t4);
      ++it;
      ++inner_total;
      const double rel_in = red0 > 0.0 ? sqrt(t4[1]) / red0 : 0.0;
      if (!(rel_in == rel_in)) conv = 5;
      else if (rel_in <= tol_in) conv = 1;
      else if (it >= itmax_in) conv = 4;
      else if (t4[0] == 0.0 || omega == 0.0) conv = 2;
      else {
        beta = (t4[0] / rho) * (alpha / omega);
        rho = t4[0];
      }
      if (reporter) {
        sc->total_it = sc->total_it + 1;
        sc->relres = rel_in;
      }
    }
    if (reporter) {
      sc->it = it;
      sc->conv = conv;
      sc->rho = rho;
      sc->alpha = alpha;
      sc->omega = omega;
      sc->beta = beta;
    }
    // x64 += c
    for (int ic = c0; ic < n; ic += cstep) S.xsol64[ic] = S.xsol64[ic] + (double)S.kx[ic];
    ps_sync(sc, G.bar_nb);
  }
  if (reporter) {
    if (sc->bar_err) pstat = kStTimeout;
    sc->ir_count = ir_count;
    sc->inner_total = inner_total;
    sc->pstat = pstat;
    sc->ir_go = 0;
    if (pstat) {
      if (sc->step_status == 0) sc->step_status = pstat;
      if (pstat > sc->worst) sc->worst = pstat;
    }
  }
}

}  // namespace nhw

