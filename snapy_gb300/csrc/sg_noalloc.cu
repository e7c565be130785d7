// sg_max_dt_noalloc: the time step of a set of blocks with no allocation at
// all -- no handle, no cudaMalloc, no library allocator.
//
// Who needs it: callers that own every byte of device memory they touch and
// may not ask the runtime for more -- a host model that hands this library
// views into its own pre-allocated arena, or a serving loop that admitted a
// request against a fixed HBM budget and must not grow past it mid-request.
// The handle path (sg_create / sg_max_dt) allocates a small reduction buffer
// per handle; this entry point keeps its reduction scratch in a file-scope
// __device__ array instead, which every GPU that loads the library holds
// until the process exits (SG_NOALLOC_MAX_BLOCKS x 16 bytes).
//
// The scratch is shared by every call: the first kernel of each call clears
// the slots it uses, so a call never sees the previous call's values, but two
// calls whose kernels overlap on the GPU (different streams, no ordering)
// race on it.  Callers serialise them (one stream, or events).
//
// The device address of the array is looked up once per device, on the
// first call made with that device current (cudaGetSymbolAddress); make that
// first call before any stream capture.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <mutex>

#include "../../include/snapy_gb300.h"
#include "sg_device.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kMaxDevices = 64;

// [0, MAX): the ordered keys of each block's minimum dt; [MAX, 2 MAX): its
// NaN flag
static __device__ __align__(256) unsigned long long
    g_dt_scratch[2 * SG_NOALLOC_MAX_BLOCKS];

struct NoallocParams {
  int32_t nblock;
  int32_t dtype;
  double cfl;
  sg_dt_block blk[SG_NOALLOC_MAX_BLOCKS];
};

__device__ __forceinline__ unsigned long long order_key(double x) {
  unsigned long long k = __double_as_longlong(x);
  return (k >> 63) ? ~k : (k | 0x8000000000000000ull);
}

__device__ __forceinline__ double order_unkey(unsigned long long k) {
  return __longlong_as_double((k >> 63) ? (k & 0x7fffffffffffffffull) : ~k);
}

__global__ void noalloc_clear(unsigned long long* scratch, int nblock) {
  int b = threadIdx.x;
  if (b < nblock) {
    scratch[b] = order_key(INFINITY);
    scratch[SG_NOALLOC_MAX_BLOCKS + b] = 0ull;
  }
}

// the per-cell bound of HydroImpl::max_time_step (src/hydro/hydro.cpp:316-398)
// over the interior of block blockIdx.y, as the handle path's reduction
template <typename T>
__global__ void __launch_bounds__(kThreads)
    noalloc_reduce(NoallocParams p, unsigned long long* scratch) {
  const int b = blockIdx.y;
  const sg_dt_block& B = p.blk[b];
  const int nc1 = B.nc1, nc2 = B.nc2, nc3 = B.nc3, ng = B.ng;
  const int nx1 = nc1 > 1 ? nc1 - 2 * ng : 1, nx2 = nc2 > 1 ? nc2 - 2 * ng : 1,
            nx3 = nc3 > 1 ? nc3 - 2 * ng : 1;
  const int o1 = nc1 > 1 ? ng : 0, o2 = nc2 > 1 ? ng : 0, o3 = nc3 > 1 ? ng : 0;
  const size_t plane = (size_t)nc1 * nc2 * nc3;
  const size_t ncell = (size_t)nx1 * nx2 * nx3;
  const T* u = static_cast<const T*>(B.u);
  const T gammad = T(B.gammad);
  double dtm = INFINITY;
  int nan = 0;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < ncell;
       e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % nx1) + o1;
    const int j = (int)((e / nx1) % nx2) + o2;
    const int k = (int)(e / ((size_t)nx1 * nx2)) + o3;
    const size_t c = ((size_t)k * nc2 + j) * nc1 + i;
    T uc[sg::NHYDRO], w[sg::NHYDRO];
#pragma unroll
    for (int v = 0; v < sg::NHYDRO; ++v) uc[v] = u[v * plane + c];
    // FP32 blocks under gravity hold anomalies about the FP64 base: the
    // totals are formed as the handle path's reduction forms them
    if (B.base) uc[sg::IDN] = T(B.base[i]) + uc[sg::IDN];
    sg::cons2prim<T>(uc, w, gammad);
    if (B.base) w[sg::IPR] = T(B.base[nc1 + i]) + w[sg::IPR];
    const T cs = sqrt(gammad * w[sg::IPR] / w[sg::IDN]);
    if (nc1 > 1 && (B.implicit & 1) && !(nc2 == 1 && nc3 == 1))
      dtm = fmin(dtm, (double)(T(B.dx1) / (fabs(w[sg::IVX]) * T(p.cfl / 1.0))));
    else if (nc1 > 1)
      dtm = fmin(dtm, (double)(T(B.dx1) / (fabs(w[sg::IVX]) + cs)));
    if (nc2 > 1) dtm = fmin(dtm, (double)(T(B.dx2) / (fabs(w[sg::IVY]) + cs)));
    if (nc3 > 1) dtm = fmin(dtm, (double)(T(B.dx3) / (fabs(w[sg::IVZ]) + cs)));
#pragma unroll
    for (int v = 0; v < sg::NHYDRO; ++v) nan |= isnan(w[v]) ? 1 : 0;
    nan |= isnan(cs) ? 1 : 0;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    dtm = fmin(dtm, __shfl_xor_sync(0xffffffffu, dtm, o));
    nan |= __shfl_xor_sync(0xffffffffu, nan, o);
  }
  __shared__ double s_dt[kThreads / 32];
  __shared__ int s_n[kThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    s_dt[wid] = dtm;
    s_n[wid] = nan;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 1; q < (int)(blockDim.x >> 5); ++q) {
      dtm = fmin(dtm, s_dt[q]);
      nan |= s_n[q];
    }
    atomicMin(&scratch[b], order_key(fmin(dtm, B.dt_src)));
    if (nan) atomicOr(&scratch[SG_NOALLOC_MAX_BLOCKS + b], 1ull);
  }
}

__global__ void noalloc_finish(NoallocParams p, const int32_t* redo,
                               const unsigned long long* scratch,
                               double* dt_out) {
  int b = threadIdx.x;
  if (b >= p.nblock) return;
  double f = redo ? pow(2., -(double)redo[b]) : 1.;
  dt_out[b] = scratch[SG_NOALLOC_MAX_BLOCKS + b]
                  ? __longlong_as_double(0x7ff8000000000000ll)
                  : f * p.cfl * order_unkey(scratch[b]);
}

// the scratch's device address, looked up once per device
std::mutex g_mu;
unsigned long long* g_addr[kMaxDevices] = {nullptr};

}  // namespace

// defined in sg_api.cu: records the message of a failed call
extern "C" int sg_fail_message(int code, const char* msg);

extern "C" int sg_max_dt_noalloc(const sg_dt_block* blocks, int32_t nblock,
                                 int32_t dtype, double cfl,
                                 const int32_t* redo_dev, double* dt_out_dev,
                                 sg_stream_t stream) {
  if (!blocks || !dt_out_dev || nblock <= 0)
    return sg_fail_message(SG_ERR_ARG, "sg_max_dt_noalloc: null argument or "
                                       "nblock <= 0");
  if (nblock > SG_NOALLOC_MAX_BLOCKS)
    return sg_fail_message(SG_ERR_ARG, "sg_max_dt_noalloc: more blocks than "
                                       "SG_NOALLOC_MAX_BLOCKS in one call");
  if (dtype != SG_F64 && dtype != SG_F32)
    return sg_fail_message(SG_ERR_ARG, "sg_max_dt_noalloc: dtype");
  NoallocParams p;
  p.nblock = nblock;
  p.dtype = dtype;
  p.cfl = cfl;
  size_t max_cells = 1;
  for (int b = 0; b < nblock; ++b) {
    const sg_dt_block& B = blocks[b];
    if (!B.u || B.nc1 < 1 || B.nc2 < 1 || B.nc3 < 1 || B.ng < 0)
      return sg_fail_message(SG_ERR_ARG, "sg_max_dt_noalloc: a block has a null "
                                         "state or a bad size");
    if (B.base && dtype != SG_F32)
      return sg_fail_message(SG_ERR_ARG, "sg_max_dt_noalloc: a hydrostatic "
                                         "base is only used by FP32 blocks");
    p.blk[b] = B;
    // no source-term bound: 0, negative, NaN or +inf all mean none
    if (!(B.dt_src > 0.) || isinf(B.dt_src)) p.blk[b].dt_src = INFINITY;
    size_t cells = (size_t)B.nc1 * B.nc2 * B.nc3;
    if (cells > max_cells) max_cells = cells;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return sg_fail_message(SG_ERR_CUDA, "sg_max_dt_noalloc: cudaGetDevice");
  unsigned long long* scratch;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
      void* ptr = nullptr;
      e = cudaGetSymbolAddress(&ptr, g_dt_scratch);
      if (e != cudaSuccess)
        return sg_fail_message(SG_ERR_CUDA, "sg_max_dt_noalloc: "
                                            "cudaGetSymbolAddress failed");
      g_addr[dev] = static_cast<unsigned long long*>(ptr);
    }
    scratch = g_addr[dev];
  }
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  noalloc_clear<<<1, SG_NOALLOC_MAX_BLOCKS, 0, s>>>(scratch, nblock);
  int gx = (int)((max_cells + kThreads - 1) / kThreads);
  if (gx > 64) gx = 64;
  if (dtype == SG_F64)
    noalloc_reduce<double><<<dim3(gx, nblock), kThreads, 0, s>>>(p, scratch);
  else
    noalloc_reduce<float><<<dim3(gx, nblock), kThreads, 0, s>>>(p, scratch);
  noalloc_finish<<<1, SG_NOALLOC_MAX_BLOCKS, 0, s>>>(p, redo_dev, scratch,
                                                     dt_out_dev);
  e = cudaGetLastError();
  if (e != cudaSuccess)
    return sg_fail_message(SG_ERR_CUDA, "sg_max_dt_noalloc: launch failed");
  return 0;
}
