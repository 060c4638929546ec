// krylov.cuh -- device Poisson solver: right-preconditioned BiCGSTAB with a
// vertical-line (tridiagonal per water column) preconditioner, inside an FP64
// iterative-refinement loop.  Replaces NSPCG (src/nspcg.f, serial build) and
// HYPRE Struct GMRES+SMG (src/pressure.F:260-462, parallel build); the stopping
// test is HYPRE's relative residual ||b - A x||_2 <= TOL ||b||_2, evaluated on
// the FP64 operator, and the initial guess is the previous P
// (src/pressure.F:104-113, 386-397).
//
// Operator storage.  After the boundary folds of generate_coef_rhs
// (src/pressure.F:649-814) the 15 diagonals of a cell are fully described by
// seven numbers: C1, C6, C13 and the k+1 cross terms C4, C5, C7, C8 (stored
// before the top row's zeroing); the in-level neighbours are -1/dx^2 and
// -1/dy^2, and the k-1 cross terms are exact negatives of the k+1 ones
// (C15 = -C4, C14 = -C5, C12 = -C7, C11 = -C8), a relation every fold
// preserves.  Neighbours outside the domain are skipped, which realises the
// folds' zero coefficients.  Layout [7][neq], compact interior order
// ic = i + M*(j + N*k); slot order C1, C6, C13, C4, C5, C7, C8.
//
// Every iteration kernel returns at once when the solve has stopped
// (sc->conv != 0), so iterations can be queued without host round trips.  Dot
// products are deterministic block reductions finished by the last block.
#pragma once
#include "kernels.cuh"

namespace nhw {

constexpr int NCOMPACT = 7;
constexpr int kCPT = 8;    // cells per thread in the reducing kernels (fewer blocks to combine)
constexpr int KREG = 32;   // columns up to this height are held in registers

template <class T>
struct Acc { using type = double; };
template <>
struct Acc<float> { using type = float; };

// y_ic = (A x)_ic on the compact operator
template <class C, class V>
__device__ __forceinline__ V spmv_c(const C* __restrict__ cf, const V* __restrict__ x, size_t n, int ic, int ii,
                                    int jj, int kk, int M, int N, int K, V cxx, V cyy) {
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

// y = A x walked up a water column: thread t takes column t % (M N) and the
// levels [k0, k1) of chunk t / (M N) (chunks of kc levels).  x at the
// column and its four horizontal neighbours is loaded once per level and kept
// in registers for the levels above and below, so a level costs five loads of
// x instead of the fifteen of spmv_c; each level's sum is formed in spmv_c's
// order, so y is the same bit for bit.  f(ic, y) takes each result.
// The BiCGSTAB matvecs of the FP32+IR form walk columns (C2: 30.9 -> 23.6 us
// for v = A ph); in FP64 the walk's registers (58-80) cost more than the
// reloads it saves, so the FP64 operator keeps one cell per thread.
template <class T>
constexpr bool kColumnWalk = sizeof(T) == 4;

template <class V>
struct Xcol {
  V c, e, w, nn, s;
};
template <class C, class V, class F>
__device__ __forceinline__ void spmv_column(const C* __restrict__ cf, const V* __restrict__ x, size_t n, int t,
                                            int kc, int M, int N, int K, V cxx, V cyy, F f) {
  const int MN = M * N;
  const int col = t % MN, chunk = t / MN;
  const int ii = col % M, jj = col / M;
  const int k0 = chunk * kc, k1 = min(K, k0 + kc);
  if (k0 >= K) return;
  const bool im = ii > 0, ip = ii < M - 1, jm = jj > 0, jp = jj < N - 1;
  auto load = [&](int k) {
    const int ic = col + MN * k;
    Xcol<V> r;
    r.c = x[ic];
    r.e = ip ? x[ic + 1] : (V)0;
    r.w = im ? x[ic - 1] : (V)0;
    r.nn = jp ? x[ic + M] : (V)0;
    r.s = jm ? x[ic - M] : (V)0;
    return r;
  };
  Xcol<V> lo{}, mid = load(k0), hi{};
  if (k0 > 0) lo = load(k0 - 1);
#pragma unroll 2
  for (int k = k0; k < k1; ++k) {
    const int ic = col + MN * k;
    const bool kp = k < K - 1, km = k > 0;
    if (kp) hi = load(k + 1);
    V s = (V)cf[ic] * mid.c;
    V h = (V)0;
    if (ip) h += mid.e;
    if (im) h += mid.w;
    s += cxx * h;
    h = (V)0;
    if (jp) h += mid.nn;
    if (jm) h += mid.s;
    s += cyy * h;
    const V c4 = (V)cf[3 * n + ic], c5 = (V)cf[4 * n + ic], c7 = (V)cf[5 * n + ic], c8 = (V)cf[6 * n + ic];
    if (kp) {
      s += (V)cf[n + ic] * hi.c;
      if (ip) s += c7 * hi.e;
      if (im) s += c5 * hi.w;
      if (jp) s += c8 * hi.nn;
      if (jm) s += c4 * hi.s;
    }
    if (km) {
      s += (V)cf[2 * n + ic] * lo.c;
      if (ip) s -= c7 * lo.e;
      if (im) s -= c5 * lo.w;
      if (jp) s -= c8 * lo.nn;
      if (jm) s -= c4 * lo.s;
    }
    f(ic, s);
    lo = mid;
    mid = hi;
  }
}

// block-wide sum of NV accumulators (A = float or double), result in lane 0 of warp 0
template <int NV, class A>
__device__ __forceinline__ void block_sum_t(A (&v)[NV], double (&out)[NV]) {
  __shared__ double sh[NV * 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int q = 0; q < NV; ++q)
    for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_down_sync(0xffffffffu, v[q], o);
  __syncthreads();
  if (lane == 0)
    for (int q = 0; q < NV; ++q) sh[q * 32 + warp] = (double)v[q];
  __syncthreads();
  if (warp == 0) {
    for (int q = 0; q < NV; ++q) {
      double x = lane < nw ? sh[q * 32 + lane] : 0.0;
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      out[q] = x;
    }
  }
}

// partials + last-block finalisation (fixed order); `part` holds `stride`
// doubles per block
template <int NV, class T, class Fin>
__device__ __forceinline__ void finish_reduce_at(const Dev<T>& S, double* part, int stride, double (&v)[NV],
                                                 Fin fin) {
  __shared__ bool last;
  __shared__ double sh2[NV * 32];
  const int nb = gridDim.x;
  if (threadIdx.x == 0) {
    for (int q = 0; q < NV; ++q) part[(size_t)blockIdx.x * stride + q] = v[q];
    __threadfence();
    const unsigned prev = atomicAdd(&S.sc->counter[0], 1u);
    last = (prev == (unsigned)nb - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double acc[NV];
  for (int q = 0; q < NV; ++q) acc[q] = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
    for (int q = 0; q < NV; ++q) acc[q] += ((volatile double*)part)[(size_t)b * stride + q];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  for (int q = 0; q < NV; ++q)
    for (int o = 16; o > 0; o >>= 1) acc[q] += __shfl_down_sync(0xffffffffu, acc[q], o);
  if (lane == 0)
    for (int q = 0; q < NV; ++q) sh2[q * 32 + warp] = acc[q];
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot[NV];
    for (int q = 0; q < NV; ++q) {
      tot[q] = 0.0;
      for (int w = 0; w < nw; ++w) tot[q] += sh2[q * 32 + w];
    }
    S.sc->counter[0] = 0u;
    fin(S, tot);
  }
}
template <int NV, class T, class Fin>
__device__ __forceinline__ void finish_reduce(const Dev<T>& S, double (&v)[NV], Fin fin) {
  finish_reduce_at<NV>(S, S.partials, 8, v, fin);
}

__device__ __forceinline__ void decode(int ic, int M, int N, int& ii, int& jj, int& kk) {
  ii = ic % M;
  const int r = ic / M;
  jj = r % N;
  kk = r / N;
}

// ------------------------------------------------------------------ FP64 residual
// Sets the condition of a conditional graph node from the finalising thread;
// eagerly launched kernels (graph_mode 0) leave handles alone.
template <class T>
__device__ __forceinline__ void set_cond(const Dev<T>& S, unsigned long long h, bool v) {
  if (S.graph_mode && h) cudaGraphSetConditional(h, v ? 1u : 0u);
}

// Status codes of the C interface that the device writes.
constexpr int kStKrylovNoconv = 6, kStNaN = 7, kStTimeout = 8;

// r64 = b - A64 x64; inner right-hand side rT = (T) r64; ||r64||, ||b||.
// The last block then makes the refinement decision of the outer loop (the
// HYPRE stopping test ||r||/||b|| <= TOL, src/pressure.F:225-258 calls the
// solver with TOL and ITMAX): stop on convergence, on b = 0 (the solution is
// then x = 0), on a non-finite residual or an inner breakdown flagged as NaN,
// or when ITMAX inner iterations or the sweep cap are used up; otherwise it
// sets the next inner tolerance and iteration budget.  kFirst opens a solve.
template <class T, bool kFirst>
__global__ void __launch_bounds__(256) k_res64(Dev<T> S) {
  // a step held back by k_dt_finalize: the loop conditions keep their
  // launch default (0), so no sweep runs
  if (gated_off(S)) return;
  const int M = S.M, N = S.N, K = S.K;
  const size_t n = (size_t)S.neq;
  double v[2] = {0.0, 0.0};
#pragma unroll
  for (int q = 0; q < kCPT; ++q) {
    const int ic = (blockIdx.x * kCPT + q) * blockDim.x + threadIdx.x;
    if (ic < S.neq) {
      int ii, jj, kk;
      decode(ic, M, N, ii, jj, kk);
      const double b = S.rhs64[ic];
      const double r = b - spmv_c<double, double>(S.coef64, S.xsol64, n, ic, ii, jj, kk, M, N, K, S.cxx, S.cyy);
      S.res64[ic] = r;
      S.kr0[ic] = (T)r;
      v[0] += r * r;
      v[1] += b * b;
    }
  }
  double out[2];
  block_sum_t<2, double>(v, out);
  finish_reduce<2>(S, out, [] __device__(const Dev<T>& S2, double* a) {
    DevScal* sc = S2.sc;
    if (kFirst) {
      sc->ir_count = 0;
      sc->inner_total = 0;
      sc->pstat = 0;
      sc->zero_x = 0;
      sc->conv = 0;
      sc->solves = sc->solves + 1;
    }
    sc->bnorm = sqrt(a[1]);
    const double rel = sc->bnorm > 0.0 ? sqrt(a[0]) / sc->bnorm : 0.0;
    sc->relres64 = rel;
    int go = 0, st = 0;
    if (sc->conv == 5 || !(rel == rel)) st = kStNaN;
    else if (sc->bnorm == 0.0) sc->zero_x = 1;
    else if (rel <= S2.tol) {}
    else if (sc->ir_count >= S2.max_ir || sc->inner_total >= S2.itmax) st = kStKrylovNoconv;
    else {
      double tol_in = 0.5 * S2.tol / rel;
      if (tol_in < S2.tol_floor) tol_in = S2.tol_floor;
      sc->tol_in = tol_in;
      sc->itmax_in = S2.itmax - sc->inner_total;
      sc->ir_count = sc->ir_count + 1;
      sc->total_ir = sc->total_ir + 1;
      go = 1;
    }
    if (st) {
      sc->pstat = st;
      if (sc->step_status == 0) sc->step_status = st;
      if (st > sc->worst) sc->worst = st;
    }
    sc->ir_go = go;
    set_cond(S2, S2.h_ir, go != 0);
  });
}

// start of an inner solve from c = 0: r = r0 = rT, p = v = 0, rho = (r, r)
// (tolerance and iteration budget come from the preceding k_res64)
template <class T>
__global__ void __launch_bounds__(256) k_bicg_init(Dev<T> S) {
  using A = typename Acc<T>::type;
  A v[1] = {(A)0};
#pragma unroll
  for (int q = 0; q < kCPT; ++q) {
    const int t = (blockIdx.x * kCPT + q) * blockDim.x + threadIdx.x;
    if (t < S.neq) {
      const T r = S.kr0[t];
      S.kr[t] = r;
      S.kx[t] = (T)0;
      S.kp[t] = (T)0;
      S.kv[t] = (T)0;
      v[0] += (A)r * (A)r;
    }
  }
  double out[1];
  block_sum_t<1, A>(v, out);
  finish_reduce<1>(S, out, [] __device__(const Dev<T>& S2, double* a) {
    DevScal* sc = S2.sc;
    sc->rho = a[0];
    sc->red[0] = sqrt(a[0]);
    sc->alpha = 1.0;
    sc->omega = 1.0;
    sc->beta = 0.0;
    sc->it = 0;
    sc->relres = 1.0;
    sc->conv = (a[0] == 0.0) ? 1 : 0;
    set_cond(S2, S2.h_inner, sc->conv == 0);
  });
}

// Thomas sweeps of one column held in registers: dp forward then back-substitution.
// `in(k)` yields the right-hand side of level k; the result is written to out.
template <class T, class In>
__device__ __forceinline__ void line_solve_reg(const Dev<T>& S, size_t col, In in, T* __restrict__ out) {
  const size_t mn = (size_t)S.M * S.N, n = (size_t)S.neq;
  const T* __restrict__ a = S.coefT + 2 * n;   // C13: coupling to k-1
  const int K = S.K;
  if (K <= KREG) {
    T dp[KREG];
    T prev = (T)0;
#pragma unroll
    for (int k = 0; k < KREG; ++k) {
      if (k < K) {
        const size_t ic = col + mn * k;
        const T am = k > 0 ? a[ic] : (T)0;
        prev = (in(k) - am * prev) * S.linv[ic];
        dp[k] = prev;
      }
    }
    T z = (T)0;
#pragma unroll
    for (int k = KREG - 1; k >= 0; --k) {
      if (k < K) {
        const size_t ic = col + mn * k;
        z = (k == K - 1) ? dp[k] : dp[k] - S.lcp[ic] * z;
        out[ic] = z;
      }
    }
  } else {
    T prev = (T)0;
    for (int k = 0; k < K; ++k) {
      const size_t ic = col + mn * k;
      const T am = k > 0 ? a[ic] : (T)0;
      prev = (in(k) - am * prev) * S.linv[ic];
      out[ic] = prev;
    }
    T z = out[col + mn * (K - 1)];
    for (int k = K - 2; k >= 0; --k) {
      const size_t ic = col + mn * k;
      z = out[ic] - S.lcp[ic] * z;
      out[ic] = z;
    }
  }
}

// p = r + beta (p - omega v); ph = M^-1 p  (one column per thread)
template <class T>
__global__ void __launch_bounds__(128) k_bicg_p(Dev<T> S) {
  if (S.sc->conv) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= S.M * S.N) return;
  const T beta = (T)S.sc->beta, omega = (T)S.sc->omega;
  const size_t mn = (size_t)S.M * S.N, col = (size_t)t;
  const T* __restrict__ r = S.kr;
  const T* __restrict__ v = S.kv;
  T* __restrict__ p = S.kp;
  line_solve_reg<T>(S, col, [&](int k) {
    const size_t ic = col + mn * k;
    const T pk = r[ic] + beta * (p[ic] - omega * v[ic]);
    p[ic] = pk;
    return pk;
  }, S.kph);
}

// s = r - alpha v; sh = M^-1 s
template <class T>
__global__ void __launch_bounds__(128) k_bicg_s(Dev<T> S) {
  if (S.sc->conv) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= S.M * S.N) return;
  const T alpha = (T)S.sc->alpha;
  const size_t mn = (size_t)S.M * S.N, col = (size_t)t;
  const T* __restrict__ r = S.kr;
  const T* __restrict__ v = S.kv;
  T* __restrict__ s = S.ks;
  line_solve_reg<T>(S, col, [&](int k) {
    const size_t ic = col + mn * k;
    const T sk = r[ic] - alpha * v[ic];
    s[ic] = sk;
    return sk;
  }, S.ksh);
}

// v = A ph; alpha = rho / (r0, v)
template <class T>
__global__ void __launch_bounds__(256) k_bicg_v(Dev<T> S) {
  if (S.sc->conv) return;
  using A = typename Acc<T>::type;
  A v[1] = {(A)0};
  const T* __restrict__ ph = S.kph;
  const T* __restrict__ r0 = S.kr0;
  T* __restrict__ vv = S.kv;
  if constexpr (kColumnWalk<T>) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < S.M * S.N * S.col_chunks)
      spmv_column<T, T>(S.coefT, ph, (size_t)S.neq, t, S.col_kc, S.M, S.N, S.K, (T)S.cxx, (T)S.cyy,
                        [&](int ic, T y) {
                          vv[ic] = y;
                          v[0] += (A)r0[ic] * (A)y;
                        });
  } else {
#pragma unroll
    for (int q = 0; q < kCPT; ++q) {
      const int ic = (blockIdx.x * kCPT + q) * blockDim.x + threadIdx.x;
      if (ic < S.neq) {
        int ii, jj, kk;
        decode(ic, S.M, S.N, ii, jj, kk);
        const T y = spmv_c<T, T>(S.coefT, ph, (size_t)S.neq, ic, ii, jj, kk, S.M, S.N, S.K, (T)S.cxx, (T)S.cyy);
        vv[ic] = y;
        v[0] += (A)r0[ic] * (A)y;
      }
    }
  }
  double out[1];
  block_sum_t<1, A>(v, out);
  finish_reduce<1>(S, out, [] __device__(const Dev<T>& S2, double* a) {
    DevScal* sc = S2.sc;
    if (a[0] == 0.0 || !(a[0] == a[0])) { sc->conv = 2; return; }
    sc->alpha = sc->rho / a[0];
  });
}

// t = A sh; omega = (t, s) / (t, t)
template <class T>
__global__ void __launch_bounds__(256) k_bicg_t(Dev<T> S) {
  if (S.sc->conv) return;
  using A = typename Acc<T>::type;
  A v[2] = {(A)0, (A)0};
  const T* __restrict__ sh = S.ksh;
  const T* __restrict__ ss = S.ks;
  T* __restrict__ tt = S.kt;
  if constexpr (kColumnWalk<T>) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < S.M * S.N * S.col_chunks)
      spmv_column<T, T>(S.coefT, sh, (size_t)S.neq, t, S.col_kc, S.M, S.N, S.K, (T)S.cxx, (T)S.cyy,
                        [&](int ic, T y) {
                          tt[ic] = y;
                          v[0] += (A)y * (A)ss[ic];
                          v[1] += (A)y * (A)y;
                        });
  } else {
#pragma unroll
    for (int q = 0; q < kCPT; ++q) {
      const int ic = (blockIdx.x * kCPT + q) * blockDim.x + threadIdx.x;
      if (ic < S.neq) {
        int ii, jj, kk;
        decode(ic, S.M, S.N, ii, jj, kk);
        const T y = spmv_c<T, T>(S.coefT, sh, (size_t)S.neq, ic, ii, jj, kk, S.M, S.N, S.K, (T)S.cxx, (T)S.cyy);
        tt[ic] = y;
        v[0] += (A)y * (A)ss[ic];
        v[1] += (A)y * (A)y;
      }
    }
  }
  double out[2];
  block_sum_t<2, A>(v, out);
  finish_reduce<2>(S, out, [] __device__(const Dev<T>& S2, double* a) {
    DevScal* sc = S2.sc;
    sc->omega = a[1] > 0.0 ? a[0] / a[1] : 0.0;
  });
}

// x += alpha ph + omega sh; r = s - omega t; convergence test.  Ends the
// iteration loop of a captured graph: every path leaves the loop condition
// set, and `it` grows by one per pass, so the loop stops by itmax_in.
template <class T>
__global__ void __launch_bounds__(256) k_bicg_xr(Dev<T> S) {
  if (S.sc->conv) {   // stopped earlier in this pass (breakdown in k_bicg_v)
    if (blockIdx.x == 0 && threadIdx.x == 0) set_cond(S, S.h_inner, false);
    return;
  }
  using A = typename Acc<T>::type;
  const T alpha = (T)S.sc->alpha, omega = (T)S.sc->omega;
  A v[2] = {(A)0, (A)0};
  T* __restrict__ x = S.kx;
  T* __restrict__ rr = S.kr;
  const T* __restrict__ ph = S.kph;
  const T* __restrict__ sh = S.ksh;
  const T* __restrict__ ss = S.ks;
  const T* __restrict__ tt = S.kt;
  const T* __restrict__ r0 = S.kr0;
#pragma unroll
  for (int q = 0; q < kCPT; ++q) {
    const int t = (blockIdx.x * kCPT + q) * blockDim.x + threadIdx.x;
    if (t < S.neq) {
      x[t] = x[t] + alpha * ph[t] + omega * sh[t];
      const T r = ss[t] - omega * tt[t];
      rr[t] = r;
      v[0] += (A)r0[t] * (A)r;
      v[1] += (A)r * (A)r;
    }
  }
  double out[2];
  block_sum_t<2, A>(v, out);
  finish_reduce<2>(S, out, [] __device__(const Dev<T>& S2, double* a) {
    DevScal* sc = S2.sc;
    const double tol_in = sc->tol_in;
    const int itmax_in = sc->itmax_in;
    sc->it = sc->it + 1;
    sc->total_it = sc->total_it + 1;
    sc->inner_total = sc->inner_total + 1;
    const double rel = sc->red[0] > 0.0 ? sqrt(a[1]) / sc->red[0] : 0.0;
    sc->relres = rel;
    int conv = 0;
    if (!(rel == rel)) conv = 5;
    else if (rel <= tol_in) conv = 1;
    else if (sc->it >= itmax_in) conv = 4;
    else if (a[0] == 0.0 || sc->omega == 0.0) conv = 2;
    else {
      sc->beta = (a[0] / sc->rho) * (sc->alpha / sc->omega);
      sc->rho = a[0];
    }
    sc->conv = conv;
    set_cond(S2, S2.h_inner, conv == 0);
  });
}

// x64 += c
template <class T>
__global__ void __launch_bounds__(256) k_xupd(Dev<T> S) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < S.neq) S.xsol64[t] = S.xsol64[t] + (double)S.kx[t];
}

// ------------------------------------------------------------------ GMRES
// Right-preconditioned GMRES: one cycle of at most kGmMax iterations per
// refinement sweep, so the sweeps of k_res64 are its restarts.  It is the
// method of the reference's parallel build, HYPRE StructGMRES preconditioned
// by one SMG cycle (src/pressure.F:399-423); the preconditioner here is the
// V-cycle of mg.cuh.  Iteration j:
//   z_j = M^-1 v_j          the V-cycle, whose first half-sweeps form
//                           v_j = w / ||w|| (MgInV) and store it;
//   w = A z_j, h_ij = (w, v_i), i <= j                      k_gm_arnoldi;
//   w -= sum_i h_ij v_i, h_j+1,j = ||w||                     k_gm_orth
//     (classical Gram-Schmidt; its last block rotates column j of H with the
//     Givens rotations so far, updates the residual norm |g_j+1| and decides
//     the loop, and at the end solves R y = g);
// after the loop k_gm_xupd adds sum_i y_i z_i to the FP64 solution.  One
// iteration is one preconditioner application (BiCGSTAB takes two).
constexpr int kGmMax = 16;
constexpr int kGmM1 = kGmMax + 1;
// FP64 state in Dev::gm: H column-major (h_ij at j * kGmM1 + i), cosines,
// sines, g, y
constexpr int kGmH = 0, kGmCs = kGmM1 * kGmMax, kGmSn = kGmCs + kGmMax, kGmG = kGmSn + kGmMax,
              kGmY = kGmG + kGmM1, kGmSize = kGmY + kGmMax;
// T copies in Dev::gmT: column j of H, y, 1/||w||
constexpr int kGmTH = 0, kGmTY = kGmMax, kGmTInv = 2 * kGmMax, kGmTSize = 2 * kGmMax + 1;

// start of a cycle from c = 0: w = r0 (the inner right-hand side), beta = ||w||
template <class T>
__global__ void __launch_bounds__(256) k_gm_init(Dev<T> S) {
  using A = typename Acc<T>::type;
  A v[1] = {(A)0};
#pragma unroll
  for (int q = 0; q < kCPT; ++q) {
    const int t = (blockIdx.x * kCPT + q) * blockDim.x + threadIdx.x;
    if (t < S.neq) {
      const T r = S.kr0[t];
      S.kt[t] = r;
      v[0] += (A)r * (A)r;
    }
  }
  double out[1];
  block_sum_t<1, A>(v, out);
  finish_reduce<1>(S, out, [] __device__(const Dev<T>& S2, double* a) {
    DevScal* sc = S2.sc;
    double* gm = S2.gm;
    const double beta = sqrt(a[0]);
    sc->red[0] = beta;
    sc->it = 0;
    sc->relres = 1.0;
    for (int i = 0; i < kGmM1; ++i) gm[kGmG + i] = 0.0;
    gm[kGmG] = beta;
    sc->gm_inv = beta > 0.0 ? 1.0 / beta : 0.0;
    S2.gmT[kGmTInv] = (T)sc->gm_inv;
    sc->conv = !(beta == beta) ? 5 : (beta == 0.0 ? 1 : 0);
    set_cond(S2, S2.h_inner, sc->conv == 0);
  });
}

// w = A z_j (z_j = the V-cycle's output in kph, kept as column j of Z);
// h_ij = (w, v_i) for i <= j
template <class T>
__global__ void __launch_bounds__(256) k_gm_arnoldi(Dev<T> S) {
  if (S.sc->conv) return;
  using A = typename Acc<T>::type;
  const int j = S.sc->it;
  const size_t n = (size_t)S.neq;
  const T* __restrict__ z = S.kph;
  T* __restrict__ zj = S.gmZ + (size_t)j * n;
  A v[kGmMax];
#pragma unroll
  for (int i = 0; i < kGmMax; ++i) v[i] = (A)0;
  for (int q = 0; q < kCPT; ++q) {
    const int ic = (blockIdx.x * kCPT + q) * blockDim.x + threadIdx.x;
    if (ic < S.neq) {
      int ii, jj, kk;
      decode(ic, S.M, S.N, ii, jj, kk);
      const T y = spmv_c<T, T>(S.coefT, z, n, ic, ii, jj, kk, S.M, S.N, S.K, (T)S.cxx, (T)S.cyy);
      S.kt[ic] = y;
      zj[ic] = z[ic];
#pragma unroll
      for (int i = 0; i < kGmMax; ++i)
        if (i <= j) v[i] += (A)y * (A)S.gmV[(size_t)i * n + ic];
    }
  }
  double out[kGmMax];
  block_sum_t<kGmMax, A>(v, out);
  finish_reduce_at<kGmMax>(S, S.gm_part, kGmMax, out, [] __device__(const Dev<T>& S2, double* a) {
    const int j2 = S2.sc->it;
    for (int i = 0; i <= j2; ++i) {
      S2.gm[kGmH + j2 * kGmM1 + i] = a[i];
      S2.gmT[kGmTH + i] = (T)a[i];
    }
  });
}

// w -= sum_i h_ij v_i; ||w||; rotations, residual estimate, loop decision
template <class T>
__global__ void __launch_bounds__(256) k_gm_orth(Dev<T> S) {
  if (S.sc->conv) {
    if (blockIdx.x == 0 && threadIdx.x == 0) set_cond(S, S.h_inner, false);
    return;
  }
  using A = typename Acc<T>::type;
  const int j = S.sc->it;
  const size_t n = (size_t)S.neq;
  T h[kGmMax];
#pragma unroll
  for (int i = 0; i < kGmMax; ++i) h[i] = i <= j ? S.gmT[kGmTH + i] : (T)0;
  A v[1] = {(A)0};
  for (int q = 0; q < kCPT; ++q) {
    const int ic = (blockIdx.x * kCPT + q) * blockDim.x + threadIdx.x;
    if (ic < S.neq) {
      T w = S.kt[ic];
#pragma unroll
      for (int i = 0; i < kGmMax; ++i)
        if (i <= j) w -= h[i] * S.gmV[(size_t)i * n + ic];
      S.kt[ic] = w;
      v[0] += (A)w * (A)w;
    }
  }
  double out[1];
  block_sum_t<1, A>(v, out);
  finish_reduce<1>(S, out, [] __device__(const Dev<T>& S2, double* a) {
    DevScal* sc = S2.sc;
    double* gm = S2.gm;
    const int j2 = sc->it;
    const double hn = sqrt(a[0]);
    double* Hj = gm + kGmH + j2 * kGmM1;
    Hj[j2 + 1] = hn;
    for (int i = 0; i < j2; ++i) {   // earlier rotations on column j
      const double c = gm[kGmCs + i], s = gm[kGmSn + i];
      const double t0 = c * Hj[i] + s * Hj[i + 1];
      Hj[i + 1] = -s * Hj[i] + c * Hj[i + 1];
      Hj[i] = t0;
    }
    const double a0 = Hj[j2], b0 = Hj[j2 + 1], rr = sqrt(a0 * a0 + b0 * b0);
    const double c = rr > 0.0 ? a0 / rr : 1.0, s = rr > 0.0 ? b0 / rr : 0.0;
    gm[kGmCs + j2] = c;
    gm[kGmSn + j2] = s;
    Hj[j2] = rr;
    Hj[j2 + 1] = 0.0;
    const double gj = gm[kGmG + j2];
    gm[kGmG + j2] = c * gj;
    gm[kGmG + j2 + 1] = -s * gj;
    sc->it = j2 + 1;
    sc->total_it = sc->total_it + 1;
    sc->inner_total = sc->inner_total + 1;
    const double rel = sc->red[0] > 0.0 ? fabs(gm[kGmG + j2 + 1]) / sc->red[0] : 0.0;
    sc->relres = rel;
    int conv = 0;
    if (!(rel == rel) || !(hn == hn)) conv = 5;
    else if (rel <= sc->tol_in || hn == 0.0) conv = 1;   // hn = 0: exact within the Krylov space
    else if (sc->it >= kGmMax || sc->it >= sc->itmax_in) conv = 4;
    else {
      sc->gm_inv = 1.0 / hn;
      S2.gmT[kGmTInv] = (T)sc->gm_inv;
    }
    if (conv) {   // R y = g over the iterations of this cycle
      const int m = sc->it;
      for (int k = m - 1; k >= 0; --k) {
        double acc = gm[kGmG + k];
        for (int l = k + 1; l < m; ++l) acc -= gm[kGmH + l * kGmM1 + k] * gm[kGmY + l];
        const double d = gm[kGmH + k * kGmM1 + k];
        gm[kGmY + k] = d != 0.0 ? acc / d : 0.0;
        S2.gmT[kGmTY + k] = (T)gm[kGmY + k];
      }
    }
    sc->conv = conv;
    set_cond(S2, S2.h_inner, conv == 0);
  });
}

// x64 += sum_i y_i z_i over the cycle's iterations
template <class T>
__global__ void __launch_bounds__(256) k_gm_xupd(Dev<T> S) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= S.neq) return;
  const int m = S.sc->it;
  const size_t n = (size_t)S.neq;
  T acc = (T)0;
  for (int i = 0; i < m; ++i) acc += S.gmT[kGmTY + i] * S.gmZ[(size_t)i * n + t];
  S.xsol64[t] = S.xsol64[t] + (double)acc;
}

}  // namespace nhw
