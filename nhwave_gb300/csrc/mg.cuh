// mg.cuh -- multigrid V-cycle used as the preconditioner of the Poisson solve.
//
// The reference preconditions its Krylov solve with HYPRE's semicoarsening
// multigrid (StructSMG, src/pressure.F:406-415) or with incomplete
// factorisations in NSPCG.  This is this project's own multigrid for the same
// operator, built for the GPU:
//   * coarsening: aggregation of columns in the horizontal only (2 x 2 while a
//     direction has at least 4 cells), the vertical resolution kept on every
//     level -- the sigma-layer coupling is usually the strong one;
//   * coarse operators: Galerkin products P^T A P with piecewise-constant P,
//     which keep the 15-point pattern, hence the compact form of krylov.cuh
//     plus explicit in-level couplings (uneven last aggregates make those
//     non-uniform);
//   * smoother: red-black ("zebra") vertical-line Gauss-Seidel -- each colour
//     solves the tridiagonal (C13, C1, C6) system of its columns with the
//     neighbouring columns (the other colour) fixed; one sweep before and one
//     after the coarse-grid correction, several on the coarsest level.
// Every kernel returns at once when the Krylov solve has stopped (sc->conv).
#pragma once
#include "krylov.cuh"

namespace nhw {

template <class T>
struct MGL {
  int M, N, K, n;
  const T* coef;        // [7][n] compact operator of this level
  const T* cxr;         // [n] coupling to i+1 (nullptr: the constant cxx)
  const T* cyr;         // [n] coupling to j+1 (nullptr: the constant cyy)
  T cxx, cyy;
  const T* lcp;         // line factors of (C13, C1, C6)
  const T* linv;
  T* x;
  T* b;
  int rx, ry;           // aggregation to the next coarser level
  int Mc, Nc;
  // Level 0 only (else nullptr): C13, 1/den, c/den, C4, C5, C7, C8 of the
  // half-sweeps again, split by colour.  Slot s of colour c starts at
  // sp + (2 s + c) * K * N * Mh, Mh = (M + 1) / 2, and holds level k, row jj,
  // column ii of that colour at k * N * Mh + jj * Mh + ii / 2.
  const T* sp;
};

template <class T>
__device__ __forceinline__ T cx_p(const MGL<T>& L, int ic) { return L.cxr ? L.cxr[ic] : L.cxx; }
template <class T>
__device__ __forceinline__ T cx_m(const MGL<T>& L, int ic) { return L.cxr ? L.cxr[ic - 1] : L.cxx; }
template <class T>
__device__ __forceinline__ T cy_p(const MGL<T>& L, int ic) { return L.cyr ? L.cyr[ic] : L.cyy; }
template <class T>
__device__ __forceinline__ T cy_m(const MGL<T>& L, int ic) { return L.cyr ? L.cyr[ic - L.M] : L.cyy; }

// off-column part of (A x) at cell (ii, jj, kk): everything but C1, C6, C13;
// c4, c5, c7, c8 are the cell's cross terms
template <class T>
__device__ __forceinline__ T off_column_c(const MGL<T>& L, const T* __restrict__ x, int ic, int ii, int jj, int kk,
                                          T c4, T c5, T c7, T c8) {
  const int M = L.M, MN = L.M * L.N;
  const bool im = ii > 0, ip = ii < L.M - 1, jm = jj > 0, jp = jj < L.N - 1, km = kk > 0, kp = kk < L.K - 1;
  T s = (T)0;
  if (ip) s += cx_p(L, ic) * x[ic + 1];
  if (im) s += cx_m(L, ic) * x[ic - 1];
  if (jp) s += cy_p(L, ic) * x[ic + M];
  if (jm) s += cy_m(L, ic) * x[ic - M];
  if (kp) {
    const int u = ic + MN;
    if (ip) s += c7 * x[u + 1];
    if (im) s += c5 * x[u - 1];
    if (jp) s += c8 * x[u + M];
    if (jm) s += c4 * x[u - M];
  }
  if (km) {
    const int d = ic - MN;
    if (ip) s -= c7 * x[d + 1];
    if (im) s -= c5 * x[d - 1];
    if (jp) s -= c8 * x[d + M];
    if (jm) s -= c4 * x[d - M];
  }
  return s;
}
template <class T>
__device__ __forceinline__ T off_column(const MGL<T>& L, const T* __restrict__ x, int ic, int ii, int jj, int kk) {
  const int n = L.n;
  return off_column_c(L, x, ic, ii, jj, kk, L.coef[3 * n + ic], L.coef[4 * n + ic], L.coef[5 * n + ic],
                      L.coef[6 * n + ic]);
}

template <class T>
__device__ __forceinline__ T level_apply(const MGL<T>& L, const T* __restrict__ x, int ic, int ii, int jj, int kk) {
  const int MN = L.M * L.N;
  T s = L.coef[ic] * x[ic] + off_column(L, x, ic, ii, jj, kk);
  if (kk < L.K - 1) s += L.coef[L.n + ic] * x[ic + MN];
  if (kk > 0) s += L.coef[2 * L.n + ic] * x[ic - MN];
  return s;
}

// Neighbour value for the first post-smoothing half-sweep: x + w * P x_c,
// the coarse-grid correction applied on the fly (the swept colour recomputes
// its own columns, the other colour is corrected by the next half-sweep).
//
// P interpolates bilinearly in the horizontal between the centres of the
// aggregates (weights 3/4, 1/4 for 2 x 2 aggregates; the aggregate's own value
// at the walls), level by level in the vertical.  Restriction stays the
// aggregate sum P0^T and the coarse operator the rescaled product of P0
// (k_mg_galerkin): the piecewise-constant P0 leaves a saw-tooth in every
// corrected smooth error, which the bilinear form does not.
template <class T>
struct Prolong {
  const T* xc;    // coarse solution (nullptr: plain x)
  T w;
  int rx, ry, Mc, MNc, M, MN, Nc;
  T hx, hy;       // 1 / (2 rx), 1 / (2 ry)
  __device__ __forceinline__ T coarse(int ic) const {
    const int kk = ic / MN, r = ic - kk * MN, jj = r / M, ii = r - jj * M;
    const int I = ii / rx, J = jj / ry;
    // fine-cell centre relative to its aggregate's centre, in coarse cells
    const T ox = (T)(2 * (ii - I * rx) + 1 - rx) * hx, oy = (T)(2 * (jj - J * ry) + 1 - ry) * hy;
    int I2 = ox < (T)0 ? I - 1 : I + 1, J2 = oy < (T)0 ? J - 1 : J + 1;
    T wx = ox < (T)0 ? -ox : ox, wy = oy < (T)0 ? -oy : oy;
    if (I2 < 0 || I2 >= Mc) { I2 = I; wx = (T)0; }
    if (J2 < 0 || J2 >= Nc) { J2 = J; wy = (T)0; }
    const T* c = xc + MNc * kk;
    return ((T)1 - wy) * (((T)1 - wx) * c[I + Mc * J] + wx * c[I2 + Mc * J]) +
           wy * (((T)1 - wx) * c[I + Mc * J2] + wx * c[I2 + Mc * J2]);
  }
  __device__ __forceinline__ T operator()(const T* __restrict__ x, int ic) const {
    if (!xc) return x[ic];
    return x[ic] + w * coarse(ic);
  }
  // the horizontal part of coarse(): four offsets into a level plane of xc
  // and their weights, shared by the three levels of a neighbouring column
  struct Stencil {
    int c00, c10, c01, c11;
    T w00, w10, w01, w11;
  };
  __device__ __forceinline__ Stencil stencil(int ii, int jj) const {
    const int I = rx == 2 ? ii >> 1 : ii / rx, J = ry == 2 ? jj >> 1 : jj / ry;
    const T ox = (T)(2 * (ii - I * rx) + 1 - rx) * hx, oy = (T)(2 * (jj - J * ry) + 1 - ry) * hy;
    int I2 = ox < (T)0 ? I - 1 : I + 1, J2 = oy < (T)0 ? J - 1 : J + 1;
    T wx = ox < (T)0 ? -ox : ox, wy = oy < (T)0 ? -oy : oy;
    if (I2 < 0 || I2 >= Mc) { I2 = I; wx = (T)0; }
    if (J2 < 0 || J2 >= Nc) { J2 = J; wy = (T)0; }
    return Stencil{I + Mc * J, I2 + Mc * J, I + Mc * J2, I2 + Mc * J2,
                   ((T)1 - wx) * ((T)1 - wy), wx * ((T)1 - wy), ((T)1 - wx) * wy, wx * wy};
  }
  // (P x_c) at level kk of the column whose stencil is st
  __device__ __forceinline__ T at_coarse(const Stencil& st, int kk) const {
    const T* c = xc + MNc * kk;
    return st.w00 * c[st.c00] + st.w10 * c[st.c10] + st.w01 * c[st.c01] + st.w11 * c[st.c11];
  }
  // x + w P x_c at fine cell ic of level kk, whose column's stencil is st
  __device__ __forceinline__ T at(const T* __restrict__ x, int ic, const Stencil& st, int kk) const {
    return x[ic] + w * at_coarse(st, kk);
  }
};
template <class T>
__host__ __device__ inline Prolong<T> prolong_from(const MGL<T>& F, const MGL<T>& C, T w) {
  return Prolong<T>{C.x, w, F.rx, F.ry, C.M, C.M * C.N, F.M, F.M * F.N, C.N, (T)0.5 / (T)F.rx, (T)0.5 / (T)F.ry};
}

template <class T>
__device__ __forceinline__ T off_column_pc(const MGL<T>& L, const T* __restrict__ x, const Prolong<T>& P, int ic,
                                           int ii, int jj, int kk, T c4, T c5, T c7, T c8) {
  if (!P.xc) return off_column_c(L, x, ic, ii, jj, kk, c4, c5, c7, c8);
  const int M = L.M, MN = L.M * L.N;
  const bool im = ii > 0, ip = ii < L.M - 1, jm = jj > 0, jp = jj < L.N - 1, km = kk > 0, kp = kk < L.K - 1;
  T s = (T)0;
  // each neighbouring column: its in-level coupling, then the cross terms at k+1 and k-1
  auto column = [&](int off, T c, T cross, int ci, int cj) {
    const typename Prolong<T>::Stencil st = P.stencil(ci, cj);
    s += c * P.at(x, ic + off, st, kk);
    if (kp) s += cross * P.at(x, ic + off + MN, st, kk + 1);
    if (km) s -= cross * P.at(x, ic + off - MN, st, kk - 1);
  };
  if (ip) column(1, cx_p(L, ic), c7, ii + 1, jj);
  if (im) column(-1, cx_m(L, ic), c5, ii - 1, jj);
  if (jp) column(M, cy_p(L, ic), c8, ii, jj + 1);
  if (jm) column(-M, cy_m(L, ic), c4, ii, jj - 1);
  return s;
}
template <class T>
__device__ __forceinline__ T off_column_p(const MGL<T>& L, const T* __restrict__ x, const Prolong<T>& P, int ic,
                                          int ii, int jj, int kk) {
  const int n = L.n;
  return off_column_pc(L, x, P, ic, ii, jj, kk, L.coef[3 * n + ic], L.coef[4 * n + ic], L.coef[5 * n + ic],
                       L.coef[6 * n + ic]);
}

// Red-black line Gauss-Seidel: a half-sweep solves the columns with
// (ii + jj) % 2 == color.
//
// Right-hand sides of a half-sweep:
//   MgB            b as stored;
//   MgInP / MgInS  the BiCGSTAB vectors p = r + beta (p - omega v) and
//                  s = r - alpha v, formed on the fine level by the sweep that
//                  owns each column (colour 0 in the first half-sweep, colour 1
//                  in the second) and stored -- no launch of their own.
//
// A kernel calls bind(sc) once per thread and the bound functor per cell:
// the scalars that come from the device in FP64 (beta, omega, alpha) are
// rounded to the storage type once, not once per cell (each conversion of a
// double runs on the FP64 pipe).
template <class T>
struct MgB {
  const T* b;
  __device__ __forceinline__ MgB bind(const DevScal*) const { return *this; }
  __device__ __forceinline__ T operator()(const DevScal*, int ic, int, int, int) const { return b[ic]; }
};
template <class T>
struct MgInP {
  T* p;
  const T* r;
  const T* v;
  T beta = (T)0, omega = (T)0;   // set by bind
  __device__ __forceinline__ MgInP bind(const DevScal* sc) const {
    MgInP q = *this;
    q.beta = (T)sc->beta;
    q.omega = (T)sc->omega;
    return q;
  }
  __device__ __forceinline__ T operator()(const DevScal*, int ic, int, int, int) const {
    const T val = r[ic] + beta * (p[ic] - omega * v[ic]);
    p[ic] = val;
    return val;
  }
};
template <class T>
struct MgInS {
  T* s;
  const T* r;
  const T* v;
  T alpha = (T)0;   // set by bind
  __device__ __forceinline__ MgInS bind(const DevScal* sc) const {
    MgInS q = *this;
    q.alpha = (T)sc->alpha;
    return q;
  }
  __device__ __forceinline__ T operator()(const DevScal*, int ic, int, int, int) const {
    const T val = r[ic] - alpha * v[ic];
    s[ic] = val;
    return val;
  }
};

// GMRES: v_j = w / ||w||, formed by the sweep that owns each column and stored
// both as column j of the basis (j = sc->it, read on the device, so a
// captured iteration serves every j) and in `b`, which the post-smoothing
// half-sweeps read as the level's right-hand side
template <class T>
struct MgInV {
  const T* w;
  T* b;
  T* V;
  const T* inv;   // (T)(1 / ||w||)
  size_t n;
  __device__ __forceinline__ MgInV bind(const DevScal*) const { return *this; }
  __device__ __forceinline__ T operator()(const DevScal* sc, int ic, int, int, int) const {
    const T val = w[ic] * *inv;
    V[(size_t)sc->it * n + ic] = val;
    b[ic] = val;
    return val;
  }
};

// Same half-sweep, block-parallel: a block holds 32 columns of the colour and
// up to 32 levels (blockDim = 32 x min(K,32)); every thread forms the line
// right-hand sides of its (column, level) cells -- loads coalesced along the
// columns -- into shared memory, then one warp runs the Thomas sweeps there.
template <class T, bool kProlong, class In>
__global__ void __launch_bounds__(1024) k_mg_smooth_blk(MGL<T> L, const DevScal* sc, int color, int zero_x,
                                                        Prolong<T> P, In in) {
  if (sc->conv) return;
  const In inb = in.bind(sc);
  extern __shared__ unsigned char smem_raw[];
  T* sh = reinterpret_cast<T*>(smem_raw);
  const int K = L.K, M = L.M, MN = L.M * L.N, n = L.n;
  T* s_rhs = sh;                 // [K][32]
  T* s_a = sh + K * 32;          // C13
  T* s_inv = sh + 2 * K * 32;    // 1/den
  T* s_cp = sh + 3 * K * 32;     // c/den
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int t = blockIdx.x * 32 + tx;
  const int ncol_row0 = (M + 1 - color) / 2, ncol_row1 = (M + color) / 2, pair = ncol_row0 + ncol_row1;
  const int jp2 = t / pair, rem = t % pair;
  int jj, ii;
  if (rem < ncol_row0) { jj = 2 * jp2; ii = 2 * rem + color; }
  else { jj = 2 * jp2 + 1; ii = 2 * (rem - ncol_row0) + (1 - color); }
  const bool valid = jj < L.N && ii < M;
  const int col = ii + M * jj;
  for (int k = ty; k < K; k += blockDim.y) {
    T rhs = (T)0, a = (T)0, inv = (T)0, cp = (T)0;
    if (valid) {
      const int ic = col + MN * k;
      T off = (T)0;
      if (!zero_x) off = kProlong ? off_column_p(L, L.x, P, ic, ii, jj, k) : off_column(L, L.x, ic, ii, jj, k);
      rhs = inb(sc, ic, ii, jj, k) - off;
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
  if (ty != 0 || !valid) return;
  // the Thomas sweeps, unrolled so that the shared-memory loads of several
  // levels issue ahead of the dependent chain
  T prev = (T)0;
#pragma unroll 4
  for (int k = 0; k < K; ++k) {
    prev = (s_rhs[k * 32 + tx] - s_a[k * 32 + tx] * prev) * s_inv[k * 32 + tx];
    s_rhs[k * 32 + tx] = prev;
  }
  T z = prev;
  L.x[col + MN * (K - 1)] = z;
#pragma unroll 4
  for (int k = K - 2; k >= 0; --k) {
    z = s_rhs[k * 32 + tx] - s_cp[k * 32 + tx] * z;
    L.x[col + MN * k] = z;
  }
}

// Level-0 half-sweep on the colour-split operator (MGL::sp).  A block holds
// 32 consecutive columns of the colour in that layout, so its loads of C13,
// the line factors and the cross terms are contiguous; in the natural layout
// every other column of a row belongs to the other colour and half of each
// sector read would be the other colour's.
//
// FP32 form.  Each thread of a column forms the right-hand sides of
// kSplitLevels consecutive levels (then the next chunk, blockDim.y chunks on): x of the
// four neighbouring columns at the chunk's levels and one above and below is
// loaded once into registers and serves the in-level and cross couplings of
// every level of the chunk, and all of a chunk's loads issue before the first
// is used.  One warp then runs the Thomas sweeps in shared memory.  (C2 level
// 0, FP32, graph of 400 half-sweeps: 7.6 us per launch with levels strided
// over 7 threads per column, 5.6 us with 4 consecutive levels on each of 5.)
// The right-hand sides are summed in the order of off_column_c /
// off_column_pc, so the result is the strided kernel's, bit for bit.
constexpr int kSplitLevels = 4;      // levels per thread (a chunk)
constexpr int kSplitRegs = 56;       // no spills; 7 blocks of 32 x 5 threads fit an SM
constexpr int kSplitMaxThreads = 1024;   // 56 registers x 1024 threads fit the 64K register file
template <class T, bool kProlong, class In>
__global__ void __maxnreg__(kSplitRegs)
k_mg_smooth_split(MGL<T> L, const DevScal* sc, int color, int zero_x, Prolong<T> P, In in) {
  static_assert(sizeof(T) == 4, "the FP64 form takes k_mg_smooth_split_strided");
  if (sc->conv) return;
  const In inb = in.bind(sc);
  constexpr int LPT = kSplitLevels;
  extern __shared__ unsigned char smem_raw[];
  T* sh = reinterpret_cast<T*>(smem_raw);
  const int K = L.K, M = L.M, MN = L.M * L.N;
  T* s_rhs = sh;
  T* s_a = sh + K * 32;
  T* s_inv = sh + 2 * K * 32;
  T* s_cp = sh + 3 * K * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int Mh = (M + 1) >> 1, nmh = Mh * L.N;
  const int q = blockIdx.x * 32 + tx;
  const int jj = q / Mh, r = q - jj * Mh, ii = 2 * r + ((color + jj) & 1);
  const bool valid = jj < L.N && ii < M;
  const int col = ii + M * jj;
  const size_t cs = (size_t)K * nmh;
  const T* sp = L.sp + (size_t)color * cs + q;
  const bool im = ii > 0, ip = ii < M - 1, jm = jj > 0, jp = jj < L.N - 1;
  const T* __restrict__ x = L.x;
  // level 0 couples the columns in a level by the constants cxx, cyy (cxr,
  // cyr are null there; only coarse levels carry per-cell couplings)
  const T cxx = L.cxx, cyy = L.cyy;
  typename Prolong<T>::Stencil sxp{}, sxm{}, syp{}, sym{};
  if (kProlong && valid && !zero_x) {
    if (ip) sxp = P.stencil(ii + 1, jj);
    if (im) sxm = P.stencil(ii - 1, jj);
    if (jp) syp = P.stencil(ii, jj + 1);
    if (jm) sym = P.stencil(ii, jj - 1);
  }
  for (int k0 = ty * LPT; valid && k0 < K; k0 += blockDim.y * LPT) {
    // neighbour x at levels k0 - 1 .. k0 + LPT (slot t holds level k0 - 1 + t)
    T xp[LPT + 2], xm[LPT + 2], yp[LPT + 2], ym[LPT + 2];
#pragma unroll
    for (int t = 0; t < LPT + 2; ++t) {
      const int k = k0 - 1 + t;
      const bool in_k = !zero_x && k >= 0 && k < K;
      const int ic = col + MN * k;
      if (kProlong) {
        xp[t] = in_k && ip ? P.at(x, ic + 1, sxp, k) : (T)0;
        xm[t] = in_k && im ? P.at(x, ic - 1, sxm, k) : (T)0;
        yp[t] = in_k && jp ? P.at(x, ic + M, syp, k) : (T)0;
        ym[t] = in_k && jm ? P.at(x, ic - M, sym, k) : (T)0;
      } else {
        xp[t] = in_k && ip ? x[ic + 1] : (T)0;
        xm[t] = in_k && im ? x[ic - 1] : (T)0;
        yp[t] = in_k && jp ? x[ic + M] : (T)0;
        ym[t] = in_k && jm ? x[ic - M] : (T)0;
      }
    }
#pragma unroll
    for (int t = 0; t < LPT; ++t) {
      const int k = k0 + t;
      if (k < K) {
        const int ic = col + MN * k;
        const T* e = sp + (size_t)nmh * k;
        const T a = e[0], inv = e[2 * cs], cp = e[4 * cs];
        T off = (T)0;
        if (!zero_x) {
          const T c4 = e[6 * cs], c5 = e[8 * cs], c7 = e[10 * cs], c8 = e[12 * cs];
          const bool km = k > 0, kp = k < K - 1;
          T s = (T)0;
          if (kProlong) {   // column by column, as off_column_pc
            if (ip) { s += cxx * xp[t + 1]; if (kp) s += c7 * xp[t + 2]; if (km) s -= c7 * xp[t]; }
            if (im) { s += cxx * xm[t + 1]; if (kp) s += c5 * xm[t + 2]; if (km) s -= c5 * xm[t]; }
            if (jp) { s += cyy * yp[t + 1]; if (kp) s += c8 * yp[t + 2]; if (km) s -= c8 * yp[t]; }
            if (jm) { s += cyy * ym[t + 1]; if (kp) s += c4 * ym[t + 2]; if (km) s -= c4 * ym[t]; }
          } else {          // in-level, then the level above, then below, as off_column_c
            if (ip) s += cxx * xp[t + 1];
            if (im) s += cxx * xm[t + 1];
            if (jp) s += cyy * yp[t + 1];
            if (jm) s += cyy * ym[t + 1];
            if (kp) {
              if (ip) s += c7 * xp[t + 2];
              if (im) s += c5 * xm[t + 2];
              if (jp) s += c8 * yp[t + 2];
              if (jm) s += c4 * ym[t + 2];
            }
            if (km) {
              if (ip) s -= c7 * xp[t];
              if (im) s -= c5 * xm[t];
              if (jp) s -= c8 * yp[t];
              if (jm) s -= c4 * ym[t];
            }
          }
          off = s;
        }
        s_rhs[k * 32 + tx] = inb(sc, ic, ii, jj, k) - off;
        s_a[k * 32 + tx] = a;
        s_inv[k * 32 + tx] = inv;
        s_cp[k * 32 + tx] = cp;
      }
    }
  }
  __syncthreads();
  if (ty != 0 || !valid) return;
  // the Thomas sweeps, unrolled so that the shared-memory loads of several
  // levels issue ahead of the dependent chain
  T prev = (T)0;
#pragma unroll 4
  for (int k = 0; k < K; ++k) {
    prev = (s_rhs[k * 32 + tx] - s_a[k * 32 + tx] * prev) * s_inv[k * 32 + tx];
    s_rhs[k * 32 + tx] = prev;
  }
  T z = prev;
  L.x[col + MN * (K - 1)] = z;
#pragma unroll 4
  for (int k = K - 2; k >= 0; --k) {
    z = s_rhs[k * 32 + tx] - s_cp[k * 32 + tx] * z;
    L.x[col + MN * k] = z;
  }
}

// The same half-sweep for the FP64 form: each thread of a column forms the
// right-hand sides of the levels ty, ty + blockDim.y, ... (no register
// window: its doubles would take twice the registers, and with them fewer
// blocks fit an SM; C2 level 0, graph of 400 half-sweeps: 25.1 us per launch
// against 27.7-33.8 us for windows of 2-7 levels).  Otherwise as
// k_mg_smooth_blk.
template <class T, bool kProlong, class In>
__global__ void __launch_bounds__(1024, 2) k_mg_smooth_split_strided(MGL<T> L, const DevScal* sc, int color, int zero_x,
                                                          Prolong<T> P, In in) {
  if (sc->conv) return;
  const In inb = in.bind(sc);
  extern __shared__ unsigned char smem_raw[];
  T* sh = reinterpret_cast<T*>(smem_raw);
  const int K = L.K, M = L.M, MN = L.M * L.N;
  T* s_rhs = sh;
  T* s_a = sh + K * 32;
  T* s_inv = sh + 2 * K * 32;
  T* s_cp = sh + 3 * K * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int Mh = (M + 1) >> 1, nmh = Mh * L.N;
  const int q = blockIdx.x * 32 + tx;
  const int jj = q / Mh, r = q - jj * Mh, ii = 2 * r + ((color + jj) & 1);
  const bool valid = jj < L.N && ii < M;
  const int col = ii + M * jj;
  const size_t cs = (size_t)K * nmh;
  const T* sp = L.sp + (size_t)color * cs + q;
  for (int k = ty; k < K; k += blockDim.y) {
    T rhs = (T)0, a = (T)0, inv = (T)0, cp = (T)0;
    if (valid) {
      const int ic = col + MN * k;
      const T* e = sp + (size_t)nmh * k;
      a = e[0];
      inv = e[2 * cs];
      cp = e[4 * cs];
      T off = (T)0;
      if (!zero_x) {
        const T c4 = e[6 * cs], c5 = e[8 * cs], c7 = e[10 * cs], c8 = e[12 * cs];
        off = kProlong ? off_column_pc(L, L.x, P, ic, ii, jj, k, c4, c5, c7, c8)
                       : off_column_c(L, L.x, ic, ii, jj, k, c4, c5, c7, c8);
      }
      rhs = inb(sc, ic, ii, jj, k) - off;
    }
    s_rhs[k * 32 + tx] = rhs;
    s_a[k * 32 + tx] = a;
    s_inv[k * 32 + tx] = inv;
    s_cp[k * 32 + tx] = cp;
  }
  __syncthreads();
  if (ty != 0 || !valid) return;
  // the Thomas sweeps, unrolled so that the shared-memory loads of several
  // levels issue ahead of the dependent chain
  T prev = (T)0;
#pragma unroll 4
  for (int k = 0; k < K; ++k) {
    prev = (s_rhs[k * 32 + tx] - s_a[k * 32 + tx] * prev) * s_inv[k * 32 + tx];
    s_rhs[k * 32 + tx] = prev;
  }
  T z = prev;
  L.x[col + MN * (K - 1)] = z;
#pragma unroll 4
  for (int k = K - 2; k >= 0; --k) {
    z = s_rhs[k * 32 + tx] - s_cp[k * 32 + tx] * z;
    L.x[col + MN * k] = z;
  }
}

// Coarse-grid correction of the colour-0 cells of a level, in place:
// x += w P x_c, one thread per cell.  The first post-smoothing half-sweep
// (colour 1) re-solves its own columns from their colour-0 neighbours and the
// second one re-solves colour 0 from those, so only colour 0 needs the
// corrected values -- each of which the half-sweep would otherwise
// interpolate once for every one of the 12 off-column couplings that read it.
template <class T>
__global__ void __launch_bounds__(256) k_mg_prolong0(MGL<T> F, Prolong<T> P, const DevScal* sc) {
  if (sc->conv) return;
  const int Mh = (F.M + 1) >> 1, nq = Mh * F.N;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)nq * F.K) return;
  const int k = (int)(t / nq), q = (int)(t - (long long)k * nq);
  const int jj = q / Mh, ii = 2 * (q - jj * Mh) + (jj & 1);
  if (ii >= F.M) return;
  const int ic = ii + F.M * (jj + F.N * k);
  F.x[ic] += P.w * P.at_coarse(P.stencil(ii, jj), k);
}

// One thread block runs the V-cycle over the small coarse levels lo..nl-1
// (1024 threads = 32 columns x 32 levels per batch; __syncthreads between
// phases), replacing dozens of tiny launches.
constexpr int kCtaLevels = 8;
template <class T>
struct MGSet { MGL<T> L[kCtaLevels]; };

template <class T>
__device__ void cta_half_sweep(const MGL<T>& L, int color, int zero_x, const Prolong<T>& P, T* sh) {
  const int K = L.K, M = L.M, MN = L.M * L.N, n = L.n;
  T* s_rhs = sh;
  T* s_a = sh + K * 32;
  T* s_inv = sh + 2 * K * 32;
  T* s_cp = sh + 3 * K * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5, by = blockDim.x >> 5;
  const int ncol_row0 = (M + 1 - color) / 2, ncol_row1 = (M + color) / 2, pair = ncol_row0 + ncol_row1;
  const int ncols = pair * ((L.N + 1) / 2);
  for (int base = 0; base < ncols; base += 32) {
    const int t = base + tx;
    const int jp2 = t / pair, rem = t % pair;
    int jj, ii;
    if (rem < ncol_row0) { jj = 2 * jp2; ii = 2 * rem + color; }
    else { jj = 2 * jp2 + 1; ii = 2 * (rem - ncol_row0) + (1 - color); }
    const bool valid = t < ncols && jj < L.N && ii < M;
    const int col = ii + M * jj;
    for (int k = ty; k < K; k += by) {
      T rhs = (T)0, a = (T)0, inv = (T)0, cp = (T)0;
      if (valid) {
        const int ic = col + MN * k;
        rhs = L.b[ic] - (zero_x ? (T)0 : off_column_p(L, L.x, P, ic, ii, jj, k));
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
#pragma unroll 4
      for (int k = 0; k < K; ++k) {
        prev = (s_rhs[k * 32 + tx] - s_a[k * 32 + tx] * prev) * s_inv[k * 32 + tx];
        s_rhs[k * 32 + tx] = prev;
      }
      T z = prev;
      L.x[col + MN * (K - 1)] = z;
#pragma unroll 4
      for (int k = K - 2; k >= 0; --k) {
        z = s_rhs[k * 32 + tx] - s_cp[k * 32 + tx] * z;
        L.x[col + MN * k] = z;
      }
    }
    __syncthreads();
  }
}

template <class T>
__device__ void cta_restrict(const MGL<T>& F, const MGL<T>& C) {
  for (int ic = threadIdx.x; ic < C.n; ic += blockDim.x) {
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
        acc += F.b[f] - level_apply(F, F.x, f, i, j, k);
      }
    }
    C.b[ic] = acc;
    C.x[ic] = (T)0;
  }
  __syncthreads();
}

// V-cycle over levels set.L[0..nl-1] (set.L[0] holds its right-hand side in b;
// its x is the output); `coarse_sweeps` red-black sweeps on the last level.
template <class T>
__global__ void __launch_bounds__(1024) k_mg_cta_cycle(MGSet<T> set, int nl, const DevScal* sc, T w,
                                                       int coarse_sweeps) {
  if (sc->conv) return;
  extern __shared__ unsigned char smem_raw[];
  T* sh = reinterpret_cast<T*>(smem_raw);
  const Prolong<T> none{nullptr, (T)0, 1, 1, 1, 1, 1, 1};
  for (int l = 0; l < nl - 1; ++l) {
    cta_half_sweep(set.L[l], 0, 1, none, sh);
    cta_half_sweep(set.L[l], 1, 0, none, sh);
    cta_restrict(set.L[l], set.L[l + 1]);
  }
  const MGL<T>& cl = set.L[nl - 1];
  for (int s = 0; s < coarse_sweeps; ++s) {
    cta_half_sweep(cl, 0, s == 0 ? 1 : 0, none, sh);
    cta_half_sweep(cl, 1, 0, none, sh);
  }
  for (int l = nl - 2; l >= 0; --l) {
    const MGL<T>& F = set.L[l];
    const MGL<T>& C = set.L[l + 1];
    const Prolong<T> pr = prolong_from(F, C, w);
    cta_half_sweep(F, 1, 0, pr, sh);
    cta_half_sweep(F, 0, 0, none, sh);
  }
}

// b_c = P^T (b_f - A_f x_f), x_c = 0, right after the pre-smoothing sweep.
// That sweep starts from x = 0: colour 0 solves T0 x0 = b0 (no neighbours
// yet), then colour 1 solves its lines exactly against the new colour-0
// values.  So the residual is zero on colour 1, and on colour 0 it is minus
// the off-column part of A x, all of whose neighbours are colour 1.  The sum
// runs over the aggregate's colour-0 cells and reads neither b nor C1, C6, C13
// (the colour-split copy of the cross terms on level 0).
template <class T>
__global__ void __launch_bounds__(256) k_mg_restrict_c0(MGL<T> F, MGL<T> C, const DevScal* sc) {
  if (sc->conv) return;
  const int ic = blockIdx.x * blockDim.x + threadIdx.x;
  if (ic >= C.n) return;
  int I, J, k;
  decode(ic, C.M, C.N, I, J, k);
  const int n = F.n, Mh = (F.M + 1) >> 1;
  const size_t nmh = (size_t)Mh * F.N, cs = nmh * F.K;
  // minus the off-column part of A x at colour-0 cell (i, j) of level k
  auto cell = [&](int i, int j) -> T {
    const int f = i + F.M * (j + F.N * k);
    T c4, c5, c7, c8;
    if (F.sp) {
      const T* e = F.sp + nmh * k + (size_t)Mh * j + (i >> 1);
      c4 = e[6 * cs]; c5 = e[8 * cs]; c7 = e[10 * cs]; c8 = e[12 * cs];
    } else {
      c4 = F.coef[3 * n + f]; c5 = F.coef[4 * n + f]; c7 = F.coef[5 * n + f]; c8 = F.coef[6 * n + f];
    }
    return off_column_c(F, F.x, f, i, j, k, c4, c5, c7, c8);
  };
  T acc = (T)0;
  if (F.rx == 2 && F.ry == 2) {
    // 2 x 2: the colour-0 cells are (2I, 2J) and (2I+1, 2J+1), in the order
    // of the general loop below, written out so that both cells' loads issue
    // together
    const int i0 = 2 * I, j0 = 2 * J;
    const bool c0 = i0 < F.M && j0 < F.N, c1 = i0 + 1 < F.M && j0 + 1 < F.N;
    const T r0 = c0 ? cell(i0, j0) : (T)0, r1 = c1 ? cell(i0 + 1, j0 + 1) : (T)0;
    if (c0) acc -= r0;
    if (c1) acc -= r1;
  } else {
    for (int b = 0; b < F.ry; ++b) {
      const int j = J * F.ry + b;
      if (j >= F.N) break;
      for (int a = 0; a < F.rx; ++a) {
        const int i = I * F.rx + a;
        if (i >= F.M) break;
        if ((i + j) & 1) continue;
        acc -= cell(i, j);
      }
    }
  }
  C.b[ic] = acc;
  C.x[ic] = (T)0;
}

// Galerkin coarse operator P^T A P (piecewise-constant P), compact form + couplings
template <class T>
__global__ void __launch_bounds__(256) k_mg_galerkin(MGL<T> F, T* ccoef, T* ccxr, T* ccyr, int Mc, int Nc) {
  const int nc = Mc * Nc * F.K;
  const int ic = blockIdx.x * blockDim.x + threadIdx.x;
  if (ic >= nc) return;
  int I, J, k;
  decode(ic, Mc, Nc, I, J, k);
  const int K = F.K, n = F.n, MN = F.M * F.N;
  (void)MN;
  T d = 0, up = 0, dn = 0, xp = 0, yp = 0, xm = 0, ym = 0;
  T x7u = 0, x5u = 0, y8u = 0, y4u = 0, x7d = 0, x5d = 0, y8d = 0, y4d = 0;
  for (int b = 0; b < F.ry; ++b) {
    const int j = J * F.ry + b;
    if (j >= F.N) break;
    for (int a = 0; a < F.rx; ++a) {
      const int i = I * F.rx + a;
      if (i >= F.M) break;
      const int f = i + F.M * (j + F.N * k);
      d += F.coef[f];
      if (k < K - 1) up += F.coef[n + f];
      if (k > 0) dn += F.coef[2 * n + f];
      const T c4 = F.coef[3 * n + f], c5 = F.coef[4 * n + f], c7 = F.coef[5 * n + f], c8 = F.coef[6 * n + f];
      // in-level neighbours
      if (i + 1 < F.M) { const T c = cx_p(F, f); if ((i + 1) / F.rx == I) d += c; else xp += c; }
      if (i - 1 >= 0) { const T c = cx_m(F, f); if ((i - 1) / F.rx == I) d += c; else xm += c; }
      if (j + 1 < F.N) { const T c = cy_p(F, f); if ((j + 1) / F.ry == J) d += c; else yp += c; }
      if (j - 1 >= 0) { const T c = cy_m(F, f); if ((j - 1) / F.ry == J) d += c; else ym += c; }
      // cross terms k+1 (+c) and k-1 (-c)
      if (k < K - 1) {
        if (i + 1 < F.M) { if ((i + 1) / F.rx == I) up += c7; else x7u += c7; }
        if (i - 1 >= 0) { if ((i - 1) / F.rx == I) up += c5; else x5u += c5; }
        if (j + 1 < F.N) { if ((j + 1) / F.ry == J) up += c8; else y8u += c8; }
        if (j - 1 >= 0) { if ((j - 1) / F.ry == J) up += c4; else y4u += c4; }
      }
      if (k > 0) {
        if (i + 1 < F.M) { if ((i + 1) / F.rx == I) dn -= c7; else x7d -= c7; }
        if (i - 1 >= 0) { if ((i - 1) / F.rx == I) dn -= c5; else x5d -= c5; }
        if (j + 1 < F.N) { if ((j + 1) / F.ry == J) dn -= c8; else y8d -= c8; }
        if (j - 1 >= 0) { if ((j - 1) / F.ry == J) dn -= c4; else y4d -= c4; }
      }
    }
  }
  // Rescaled horizontal couplings.  Across an aggregate boundary the product
  // sums ry (x faces) or rx (y faces) fine couplings, each ~ h_y dz / h_x, so
  // the coarse x coupling comes out rx times what the same operator
  // discretised on the coarse cells has (2 h_y dz / (2 h_x) for 2 x 2); the
  // vertical couplings and the x-z / y-z cross terms come out at the coarse
  // discretisation's scale.  Too-strong horizontal couplings halve the
  // correction of horizontally smooth errors on every level, which a uniform
  // correction weight cannot undo without over-correcting the vertical.  So
  // the in-level couplings are scaled by 1/rx and 1/ry, and the removed part
  // goes to the diagonal: the row sums stay those of the product.
  const T sx = (T)1 / (T)F.rx, sy = (T)1 / (T)F.ry;
  d += ((T)1 - sx) * (xp + xm) + ((T)1 - sy) * (yp + ym);
  xp *= sx;
  yp *= sy;
  const bool top = (k == K - 1);
  ccoef[ic] = d;
  ccoef[nc + ic] = up;
  ccoef[2 * nc + ic] = dn;
  ccoef[3 * nc + ic] = top ? -y4d : y4u;
  ccoef[4 * nc + ic] = top ? -x5d : x5u;
  ccoef[5 * nc + ic] = top ? -x7d : x7u;
  ccoef[6 * nc + ic] = top ? -y8d : y8u;
  ccxr[ic] = xp;
  ccyr[ic] = yp;
}

// line factors of one level (C13, C1, C6), one column per thread
template <class T>
__global__ void __launch_bounds__(256) k_mg_factor(MGL<T> L, T* lcp, T* linv) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= L.M * L.N) return;
  const int MN = L.M * L.N, n = L.n;
  T cpm = (T)0;   // in the storage type, as the factors are stored
  for (int k = 0; k < L.K; ++k) {
    const int ic = col + MN * k;
    const T a = k > 0 ? L.coef[2 * n + ic] : (T)0;
    const T b = L.coef[ic];
    const T c = k < L.K - 1 ? L.coef[n + ic] : (T)0;
    const T inv = (T)1 / (b - a * cpm);
    cpm = c * inv;
    lcp[ic] = cpm;
    linv[ic] = inv;
  }
}

// p = r + beta (p - omega v)   /   s = r - alpha v   (cell kernels when MG preconditions)
template <class T>
__global__ void __launch_bounds__(256) k_bicg_p_cell(Dev<T> S) {
  if (S.sc->conv) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= S.neq) return;
  const T beta = (T)S.sc->beta, omega = (T)S.sc->omega;
  S.kp[t] = S.kr[t] + beta * (S.kp[t] - omega * S.kv[t]);
}
template <class T>
__global__ void __launch_bounds__(256) k_bicg_s_cell(Dev<T> S) {
  if (S.sc->conv) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= S.neq) return;
  S.ks[t] = S.kr[t] - (T)S.sc->alpha * S.kv[t];
}

}  // namespace nhw
