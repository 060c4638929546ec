// krylov.cuh -- device Poisson solver: right-preconditioned BiCGSTAB with a
// vertical-line (tridiagonal per water column) preconditioner, inside an FP64
// iterative-refinement loop.  Replaces NSPCG (src/nspcg.f, serial build) and
// HYPRE Struct GMRES+SMG (src/pressure.F:260-462, parallel build); the stopping
// test is HYPRE's relative residual ||b - A x||_2 <= TOL ||b||_2, evaluated on
// the FP64 operator, and the initial guess is the previous P
// (src/pressure.F:104-113, 386-397).
//
// Vectors use the compact interior order ic = i + M*(j + N*k).  Every
// iteration kernel returns at once when the solve has already stopped
// (sc->conv != 0), so a run of iterations can be queued without host round
// trips.  Dot products are deterministic block reductions finished by the last
// block of each kernel.
#pragma once
#include "kernels.cuh"

namespace nhw {

constexpr int kRedBlocks = 152 * 8;   // bounded grid of the reduction kernels

// y = A x on the 15-point stencil; C is [NCOEF][neq] in diagonal order 1..15
template <class C, class V>
__device__ __forceinline__ V spmv_at(const C* __restrict__ Cf, const V* __restrict__ x, size_t n, int ic,
                                     int ii, int jj, int kk, int M, int N, int K) {
  const int MN = M * N;
  const bool im = ii > 0, ip = ii < M - 1, jm = jj > 0, jp = jj < N - 1, km = kk > 0, kp = kk < K - 1;
  V s = (V)Cf[ic] * x[ic];
  if (ip) s += (V)Cf[1 * n + ic] * x[ic + 1];
  if (jp) s += (V)Cf[2 * n + ic] * x[ic + M];
  if (jm && kp) s += (V)Cf[3 * n + ic] * x[ic - M + MN];
  if (im && kp) s += (V)Cf[4 * n + ic] * x[ic - 1 + MN];
  if (kp) s += (V)Cf[5 * n + ic] * x[ic + MN];
  if (ip && kp) s += (V)Cf[6 * n + ic] * x[ic + 1 + MN];
  if (jp && kp) s += (V)Cf[7 * n + ic] * x[ic + M + MN];
  if (im) s += (V)Cf[8 * n + ic] * x[ic - 1];
  if (jm) s += (V)Cf[9 * n + ic] * x[ic - M];
  if (jp && km) s += (V)Cf[10 * n + ic] * x[ic + M - MN];
  if (ip && km) s += (V)Cf[11 * n + ic] * x[ic + 1 - MN];
  if (km) s += (V)Cf[12 * n + ic] * x[ic - MN];
  if (im && km) s += (V)Cf[13 * n + ic] * x[ic - 1 - MN];
  if (jm && km) s += (V)Cf[14 * n + ic] * x[ic - M - MN];
  return s;
}

// out = M^-1 in on one column (Thomas sweeps with stored factors)
template <class T>
__device__ __forceinline__ void line_solve(const Dev<T>& S, const T* __restrict__ in, T* __restrict__ out,
                                           size_t base) {
  const size_t mn = (size_t)S.M * S.N, n = (size_t)S.neq;
  const T* a = S.coefT + 12 * n;
  T dp = (T)0;
  for (int k = 0; k < S.K; ++k) {
    const size_t ic = base + mn * k;
    const T am = k > 0 ? a[ic] : (T)0;
    dp = (in[ic] - am * dp) * S.linv[ic];
    out[ic] = dp;
  }
  T z = out[base + mn * (S.K - 1)];
  for (int k = S.K - 2; k >= 0; --k) {
    const size_t ic = base + mn * k;
    z = out[ic] - S.lcp[ic] * z;
    out[ic] = z;
  }
}

#define NHW_GRID_STRIDE(t, n) \
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < (n); t += (long long)gridDim.x * blockDim.x)

// r64 = b - A64 x64 (FP64); inner rhs rT = (T) r64; ||r64||, ||b||
template <class T>
__global__ void __launch_bounds__(256) k_res64(Dev<T> S) {
  const int M = S.M, N = S.N, K = S.K;
  const size_t n = (size_t)S.neq;
  double v[2] = {0.0, 0.0};
  NHW_GRID_STRIDE(t, (long long)n) {
    const int ic = (int)t, ii = ic % M, jj = (ic / M) % N, kk = ic / (M * N);
    const double b = S.rhs64[ic];
    const double r = b - spmv_at<double, double>(S.coef64, S.xsol64, n, ic, ii, jj, kk, M, N, K);
    S.res64[ic] = r;
    S.kr0[ic] = (T)r;   // inner right-hand side (kr0 doubles as its store)
    v[0] += r * r;
    v[1] += b * b;
  }
  reduce_finalize<2>(S, v, 0, [] __device__(const Dev<T>& S2, double* a) {
    DevScal* sc = S2.sc;
    sc->bnorm = sqrt(a[1]);
    sc->relres64 = sc->bnorm > 0.0 ? sqrt(a[0]) / sc->bnorm : 0.0;
  });
}

// start of an inner solve from c = 0: r = r0 = rT, p = v = 0
template <class T>
__global__ void __launch_bounds__(256) k_bicg_init(Dev<T> S) {
  const size_t n = (size_t)S.neq;
  double v[1] = {0.0};
  NHW_GRID_STRIDE(t, (long long)n) {
    const T r = S.kr0[t];
    S.kr[t] = r;
    S.kx[t] = (T)0;
    S.kp[t] = (T)0;
    S.kv[t] = (T)0;
    v[0] += (double)r * (double)r;
  }
  reduce_finalize<1>(S, v, 0, [] __device__(const Dev<T>& S2, double* a) {
    DevScal* sc = S2.sc;
    sc->rho = a[0];
    sc->red[0] = sqrt(a[0]);   // inner reference norm
    sc->alpha = 1.0;
    sc->omega = 1.0;
    sc->beta = 0.0;
    sc->it = 0;
    sc->relres = 1.0;
    sc->conv = (a[0] == 0.0) ? 1 : 0;
  });
}

// p = r + beta (p - omega v); ph = M^-1 p  (one column per thread)
template <class T>
__global__ void __launch_bounds__(256) k_bicg_p(Dev<T> S) {
  if (S.sc->conv) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= S.M * S.N) return;
  const T beta = (T)S.sc->beta, omega = (T)S.sc->omega;
  const size_t mn = (size_t)S.M * S.N;
  for (int k = 0; k < S.K; ++k) {
    const size_t ic = (size_t)t + mn * k;
    S.kp[ic] = S.kr[ic] + beta * (S.kp[ic] - omega * S.kv[ic]);
  }
  line_solve(S, S.kp, S.kph, (size_t)t);
}

// v = A ph; alpha = rho / (r0, v)
template <class T>
__global__ void __launch_bounds__(256) k_bicg_v(Dev<T> S) {
  if (S.sc->conv) return;
  const int M = S.M, N = S.N, K = S.K;
  const size_t n = (size_t)S.neq;
  double v[1] = {0.0};
  NHW_GRID_STRIDE(t, (long long)n) {
    const int ic = (int)t, ii = ic % M, jj = (ic / M) % N, kk = ic / (M * N);
    const T y = spmv_at<T, T>(S.coefT, S.kph, n, ic, ii, jj, kk, M, N, K);
    S.kv[ic] = y;
    v[0] += (double)S.kr0[ic] * (double)y;
  }
  reduce_finalize<1>(S, v, 0, [] __device__(const Dev<T>& S2, double* a) {
    DevScal* sc = S2.sc;
    if (a[0] == 0.0 || !(a[0] == a[0])) { sc->conv = 2; return; }
    sc->alpha = sc->rho / a[0];
  });
}

// s = r - alpha v; sh = M^-1 s
template <class T>
__global__ void __launch_bounds__(256) k_bicg_s(Dev<T> S) {
  if (S.sc->conv) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= S.M * S.N) return;
  const T alpha = (T)S.sc->alpha;
  const size_t mn = (size_t)S.M * S.N;
  for (int k = 0; k < S.K; ++k) {
    const size_t ic = (size_t)t + mn * k;
    S.ks[ic] = S.kr[ic] - alpha * S.kv[ic];
  }
  line_solve(S, S.ks, S.ksh, (size_t)t);
}

// t = A sh; omega = (t, s) / (t, t)
template <class T>
__global__ void __launch_bounds__(256) k_bicg_t(Dev<T> S) {
  if (S.sc->conv) return;
  const int M = S.M, N = S.N, K = S.K;
  const size_t n = (size_t)S.neq;
  double v[2] = {0.0, 0.0};
  NHW_GRID_STRIDE(t, (long long)n) {
    const int ic = (int)t, ii = ic % M, jj = (ic / M) % N, kk = ic / (M * N);
    const T y = spmv_at<T, T>(S.coefT, S.ksh, n, ic, ii, jj, kk, M, N, K);
    S.kt[ic] = y;
    v[0] += (double)y * (double)S.ks[ic];
    v[1] += (double)y * (double)y;
  }
  reduce_finalize<2>(S, v, 0, [] __device__(const Dev<T>& S2, double* a) {
    DevScal* sc = S2.sc;
    sc->omega = a[1] > 0.0 ? a[0] / a[1] : 0.0;
  });
}

// x += alpha ph + omega sh; r = s - omega t; convergence test
template <class T>
__global__ void __launch_bounds__(256) k_bicg_xr(Dev<T> S, double tol_in, int itmax_in) {
  if (S.sc->conv) return;
  const size_t n = (size_t)S.neq;
  const T alpha = (T)S.sc->alpha, omega = (T)S.sc->omega;
  double v[2] = {0.0, 0.0};
  NHW_GRID_STRIDE(t, (long long)n) {
    S.kx[t] = S.kx[t] + alpha * S.kph[t] + omega * S.ksh[t];
    const T r = S.ks[t] - omega * S.kt[t];
    S.kr[t] = r;
    v[0] += (double)S.kr0[t] * (double)r;
    v[1] += (double)r * (double)r;
  }
  reduce_finalize<2>(S, v, 0, [tol_in, itmax_in] __device__(const Dev<T>& S2, double* a) {
    DevScal* sc = S2.sc;
    sc->it = sc->it + 1;
    sc->total_it = sc->total_it + 1;
    const double rel = sc->red[0] > 0.0 ? sqrt(a[1]) / sc->red[0] : 0.0;
    sc->relres = rel;
    if (!(rel == rel)) { sc->conv = 5; return; }
    if (rel <= tol_in) { sc->conv = 1; return; }
    if (sc->it >= itmax_in) { sc->conv = 4; return; }
    if (a[0] == 0.0 || sc->omega == 0.0) { sc->conv = 2; return; }
    sc->beta = (a[0] / sc->rho) * (sc->alpha / sc->omega);
    sc->rho = a[0];
  });
}

// x64 += c
template <class T>
__global__ void __launch_bounds__(256) k_xupd(Dev<T> S) {
  NHW_GRID_STRIDE(t, (long long)S.neq) { S.xsol64[t] = S.xsol64[t] + (double)S.kx[t]; }
}

}  // namespace nhw
