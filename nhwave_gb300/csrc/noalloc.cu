// noalloc.cu -- nhw_estimate_dt_noalloc: the Courant time step of
// estimate_dt computed on device arrays that the caller owns, with the
// reduction's scratch in a fixed device array of this library instead of
// memory that the library allocates.
//
// Who needs it: a host model that keeps its fields in device memory that it
// does not get from cudaMalloc -- a Fortran code whose arrays belong to the
// OpenACC or CUDA Fortran runtime, a framework whose caching allocator owns
// the GPU -- and that cannot let a library call cudaMalloc/cudaFree behind
// its back: those calls synchronise the device, stalling the caller's other
// streams, and they draw on a memory budget that such callers fix up front.
// The handle-based entry points allocate a scenario arena at nhw_create; this
// one allocates nothing and keeps no per-call state on the host.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/nhwave_gb300.h"
#include "state.h"

namespace nhw {

void set_last_error(const std::string& s);

namespace {

constexpr int kNaThreads = 256;
constexpr int kNaCellsPerThread = 8;
constexpr long long kNaCellsPerBlock = (long long)kNaThreads * kNaCellsPerThread;   // 2048
constexpr int kNaMaxBlocks = 8192;                                                   // partial minima held
constexpr long long kNaMaxCells = kNaMaxBlocks * kNaCellsPerBlock;                   // 16,777,216
constexpr int kNaCounter = kNaMaxBlocks;                                             // counter slot

// The scratch: one partial minimum per block, then a 256-byte line whose
// first word counts the blocks that have finished.  65,792 bytes, held on
// every device that loads the library until the process exits.  Host code
// must not use this name as an address; it takes the address from
// cudaGetSymbolAddress (scratch_on_current_device).
static __device__ __align__(256) double g_dt_scratch[kNaMaxBlocks + 32];

// Running minimum m updated by a candidate x the way the reference does
// (src/nhwave.F:3730-3746, `if(dxonu<tmp2) tmp2=dxonu`): a NaN candidate fails
// the comparison and leaves m as it was.
__device__ __forceinline__ double na_min(double m, double x) { return x < m ? x : m; }
__device__ __forceinline__ double na_max(double a, double b) { return a > b ? a : b; }

__device__ __forceinline__ double block_min(double m) {
  __shared__ double sh[kNaThreads / 32];
  for (int o = 16; o > 0; o >>= 1) m = na_min(m, __shfl_down_sync(0xffffffffu, m, o));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) sh[warp] = m;
  __syncthreads();
  if (threadIdx.x == 0)
    for (int w = 1; w < kNaThreads / 32; ++w) m = na_min(m, sh[w]);
  return m;   // valid in thread 0
}

// Same arithmetic as the handle's estimate_dt (src/nhwave.F:3694-3874 with
// viscous and slide limits off): tmp2 = min over interior cells of
// dx/max(|U|+sqrt(g D), Small), dy/max(|V|+sqrt(g D), Small) and
// dsig(k) D/max(|W|, Small); dt = min(1.05 dt_old, CFL tmp2, Large, DT_MAX).
// Arrays are the reference's ghosted Fortran ones: U(Mloc,Nloc,Kloc),
// D(Mloc,Nloc), dsig(Kloc) with Mloc = Mglob+4 (two ghost cells a side).
__global__ void __launch_bounds__(kNaThreads)
k_dt_min_noalloc(const double* __restrict__ U, const double* __restrict__ V, const double* __restrict__ W,
                 const double* __restrict__ D, const double* __restrict__ dsig, int M, int N, int K, double dx,
                 double dy, double cfl, double dt_old, double dt_max, double* __restrict__ dt_out,
                 double* __restrict__ scratch) {
  const long long Ml = M + 2 * NG, Nl = N + 2 * NG;
  const long long n = (long long)M * N * K;
  double m = kLarge;
#pragma unroll
  for (int q = 0; q < kNaCellsPerThread; ++q) {
    const long long t = ((long long)blockIdx.x * kNaCellsPerThread + q) * kNaThreads + threadIdx.x;
    if (t < n) {
      const long long i = NG + t % M, r = t / M;
      const long long j = NG + r % N, k = NG + r / N;
      const long long c2 = i + Ml * j, c3 = c2 + Ml * Nl * k;
      const double Dq = D[c2];
      double tmp1 = na_max(fabs(U[c3]) + sqrt(kGrav * Dq), kSmall);
      m = na_min(m, dx / tmp1);
      tmp1 = na_max(fabs(V[c3]) + sqrt(kGrav * Dq), kSmall);
      m = na_min(m, dy / tmp1);
      tmp1 = na_max(fabs(W[c3]), kSmall);
      m = na_min(m, dsig[k] * Dq / tmp1);
    }
  }
  m = block_min(m);
  __shared__ bool last;
  if (threadIdx.x == 0) {
    scratch[blockIdx.x] = m;
    __threadfence();
    const unsigned prev = atomicAdd(reinterpret_cast<unsigned*>(scratch + kNaCounter), 1u);
    last = prev == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  m = kLarge;
  for (unsigned b = threadIdx.x; b < gridDim.x; b += kNaThreads)
    m = na_min(m, reinterpret_cast<volatile double*>(scratch)[b]);
  m = block_min(m);
  if (threadIdx.x == 0) {
    const double dt_growth = (double)1.05f * dt_old;
    dt_out[0] = na_min(na_min(na_min(dt_growth, cfl * m), kLarge), dt_max);
  }
}

constexpr int kNaDevices = 64;
std::mutex g_na_mu;
double* g_na_ptr[kNaDevices] = {};

// Device address of g_dt_scratch on the current device, looked up once per
// device (the first call on a device does this set-up).
int scratch_on_current_device(double** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_last_error(std::string("nhw_estimate_dt_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
    return NHW_ERR_CUDA;
  }
  std::lock_guard<std::mutex> g(g_na_mu);
  if (dev >= 0 && dev < kNaDevices && g_na_ptr[dev]) {
    *out = g_na_ptr[dev];
    return NHW_OK;
  }
  void* p = nullptr;
  e = cudaGetSymbolAddress(&p, g_dt_scratch);
  if (e != cudaSuccess || !p) {
    set_last_error(std::string("nhw_estimate_dt_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    return NHW_ERR_CUDA;
  }
  if (dev >= 0 && dev < kNaDevices) g_na_ptr[dev] = static_cast<double*>(p);
  *out = static_cast<double*>(p);
  return NHW_OK;
}

// Device memory of the current device, or managed memory.  Device memory of
// another GPU is refused: without peer access the kernel's loads would fault.
bool on_device(const void* p, int dev) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type == cudaMemoryTypeManaged) return true;
  return a.type == cudaMemoryTypeDevice && a.device == dev;
}

}  // namespace
}  // namespace nhw

extern "C" int nhw_estimate_dt_noalloc(const double* U, const double* V, const double* W, const double* D,
                                       const double* dsig, int32_t Mglob, int32_t Nglob, int32_t Kglob,
                                       double dx, double dy, double cfl, double dt_old, double dt_max,
                                       double* dt_out, void* stream) {
  using namespace nhw;
  if (!U || !V || !W || !D || !dsig || !dt_out) {
    set_last_error("nhw_estimate_dt_noalloc: null array");
    return NHW_ERR_ARG;
  }
  if (Mglob < 1 || Nglob < 1 || Kglob < 1 || !(dx > 0.0) || !(dy > 0.0)) {
    set_last_error("nhw_estimate_dt_noalloc: grid sizes and dx, dy must be positive");
    return NHW_ERR_ARG;
  }
  const long long n = (long long)Mglob * Nglob * Kglob;
  if (n > kNaMaxCells) {
    set_last_error("nhw_estimate_dt_noalloc: Mglob*Nglob*Kglob = " + std::to_string(n) +
                   " interior cells exceeds the limit of " + std::to_string(kNaMaxCells) +
                   " that its static device scratch holds");
    return NHW_ERR_ARG;
  }
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    set_last_error("nhw_estimate_dt_noalloc: no current CUDA device");
    return NHW_ERR_CUDA;
  }
  for (const void* p : {(const void*)U, (const void*)V, (const void*)W, (const void*)D, (const void*)dsig,
                        (const void*)dt_out})
    if (!on_device(p, dev)) {
      set_last_error("nhw_estimate_dt_noalloc: every array must be device memory of the current device "
                     "(device " + std::to_string(dev) + ") or managed memory");
      return NHW_ERR_ARG;
    }
  double* scratch = nullptr;
  int rc = scratch_on_current_device(&scratch);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // the blocks-done counter must start at zero; partial minima are all rewritten
  cudaError_t e = cudaMemsetAsync(scratch + kNaCounter, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) {
    set_last_error(std::string("nhw_estimate_dt_noalloc: cudaMemsetAsync: ") + cudaGetErrorString(e));
    return NHW_ERR_CUDA;
  }
  const unsigned nb = (unsigned)((n + kNaCellsPerBlock - 1) / kNaCellsPerBlock);
  k_dt_min_noalloc<<<nb, kNaThreads, 0, s>>>(U, V, W, D, dsig, Mglob, Nglob, Kglob, dx, dy, cfl, dt_old, dt_max,
                                             dt_out, scratch);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_last_error(std::string("nhw_estimate_dt_noalloc: launch: ") + cudaGetErrorString(e));
    return NHW_ERR_CUDA;
  }
  return NHW_OK;
}
