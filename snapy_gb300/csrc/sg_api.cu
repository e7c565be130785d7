// C ABI of the batched hydro stage (include/snapy_gb300.h): handle and
// buffer bookkeeping on the host, launches on the caller's stream, and the
// two tiny finishing kernels of the per-step reductions.
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <array>
#include <string>
#include <vector>

#include "../../include/snapy_gb300.h"
#include "sg_types.h"

using sg::BlockDev;
using sg::StageParams;

// per-precision launchers (sg_stage.cu compiled for double and for float)
#define SG_DECLARE(sfx)                                                        \
  extern "C" size_t sg_stage_smem##sfx(int nc1, int tj, int has2, int wb,      \
                                       int cov, int visc);                     \
  extern "C" int sg_launch_stage##sfx(const BlockDev*, StageParams, size_t,    \
                                      cudaStream_t);                           \
  extern "C" int sg_launch_ghost##sfx(const BlockDev*, int, int, size_t,       \
                                      cudaStream_t);                           \
  extern "C" int sg_launch_prim##sfx(const BlockDev*, int, int, void* const*,  \
                                     size_t, cudaStream_t);                    \
  extern "C" int sg_launch_init##sfx(const BlockDev*, int, int,                \
                                     double* const*, size_t,                   \
                                     cudaStream_t);                            \
  extern "C" int sg_launch_vic##sfx(const BlockDev*, StageParams, size_t,     \
                                    size_t, int, int*, cudaStream_t,           \
                                    cudaEvent_t*);                             \
  extern "C" int sg_launch_x3##sfx(const BlockDev*, StageParams, size_t,      \
                                   cudaStream_t);                              \
  extern "C" int sg_launch_reduce##sfx(const BlockDev*, int, int,              \
                                       unsigned long long*, int*, size_t,      \
                                       cudaStream_t);                          \
  extern "C" int sg_launch_budget_totals##sfx(const BlockDev*, int, int,       \
                                              double*, cudaStream_t);          \
  extern "C" int sg_launch_budget_boundary##sfx(const BlockDev*, int, double*, \
                                                int, cudaStream_t);           \
  extern "C" int sg_launch_scalar##sfx(const BlockDev*, StageParams, size_t,  \
                                       size_t, cudaStream_t);                  \
  extern "C" int sg_launch_scalar_ghost##sfx(const BlockDev*, int, int,       \
                                             size_t, cudaStream_t);             \
  extern "C" int sg_launch_psw_rcp##sfx(const double*, double*, size_t,       \
                                        cudaStream_t);
SG_DECLARE(_f64)
SG_DECLARE(_f32)

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(SG_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

constexpr unsigned long long kKeyInf = 0xfff0000000000000ull;  // key(+inf)

__device__ __forceinline__ double unkey(unsigned long long k) {
  return __longlong_as_double((k >> 63) ? (k & 0x7fffffffffffffffull) : ~k);
}

// dt[b] = (2^-redo[b] cfl) dt_min[b]  (meshblock_advance.cpp:61-72); a NaN
// anywhere makes the step's dt NaN, as torch's min does
__global__ void finish_dt_kernel(int nblock, unsigned long long* red, int* nan,
                                 const int32_t* redo, double cfl,
                                 double* dt_out) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nblock) return;
  double dtm = unkey(red[4 * b]);
  double f = redo ? pow(2., -(double)redo[b]) : 1.;
  dt_out[b] = nan[b] ? __longlong_as_double(0x7ff8000000000000ll) : f * cfl * dtm;
  red[4 * b] = red[4 * b + 1] = red[4 * b + 2] = kKeyInf;
  nan[b] = 0;
}

// meshblock_redo.cpp:106-114: a floor hit when min rho (p) is not above
// 1.001 x its floor (a NaN compares false, so it is a hit too); bit 3: NaN
__global__ void finish_check_kernel(int nblock, unsigned long long* red,
                                    int* nan, int* status, double dfloor,
                                    double pfloor, int32_t* flags,
                                    int32_t* redo = nullptr,
                                    int32_t* state = nullptr,
                                    int max_redo = 0) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nblock) return;
  double rmin = unkey(red[4 * b + 1]), pmin = unkey(red[4 * b + 2]);
  int f = 0;
  if (!(rmin > 1.001 * dfloor)) f |= 1;
  if (!(pmin > 1.001 * pfloor)) f |= 1;
  if (nan[b]) f |= 1 | 8;
  // bit 5: a column of the vertical implicit solve failed this step; bit 6:
  // a tile's shared-memory staging did not arrive in time (the stage kernel
  // gave up on it)
  if (status[b] & ~sg::kStatusStaging) f |= 32;
  if (status[b] & sg::kStatusStaging) f |= 64;
  status[b] = 0;
  flags[b] = f;
  // the retry decision (MeshBlockImpl::apply_redo): a flagged block counts
  // a redo and is restored (state 1), or is terminated past max_redo (state
  // -1, kept from then on: its last accepted state is restored at every
  // later check); an accepted step clears the count
  if (redo) {
    if (state[b] == -1) {
    } else if (f) {
      const int r = redo[b] + 1;
      redo[b] = r;
      state[b] = r > max_redo ? -1 : 1;
    } else {
      redo[b] = 0;
      state[b] = 0;
    }
  }
  red[4 * b] = red[4 * b + 1] = red[4 * b + 2] = kKeyInf;
  nan[b] = 0;
}

// the step-start state back into the current buffer of every block whose
// retry state is not 0 (4-byte words: both storage types)
__global__ void restore_kernel(const BlockDev* __restrict__ tab, int cur,
                               int base, const int32_t* state, int esz) {
  const int b = blockIdx.y;
  if (state[b] == 0) return;
  const BlockDev& B = tab[b];
  const size_t words = (size_t)5 * B.nc1 * B.nc2 * B.nc3 * esz / 4;
  const uint32_t* src = static_cast<const uint32_t*>(B.buf[base]);
  uint32_t* dst = static_cast<uint32_t*>(B.buf[cur]);
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < words;
       q += (size_t)gridDim.x * blockDim.x)
    dst[q] = src[q];
  if (B.nscalar > 0) {  // the scalars' step-start state too
    const size_t sw = (size_t)B.nscalar * B.nc1 * B.nc2 * B.nc3 * esz / 4;
    const uint32_t* ss = static_cast<const uint32_t*>(B.sbuf[base]);
    uint32_t* sd = static_cast<uint32_t*>(B.sbuf[cur]);
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < sw;
         q += (size_t)gridDim.x * blockDim.x)
      sd[q] = ss[q];
  }
}

// the x1 geometry constants of the gravity-work correction for interior
// cell k of a block (BlockDev::x1tab); the stage kernel formerly evaluated
// these per cell and launch, with the same operations
__global__ void x1tab_kernel(const double* x1f, const double* x1v, int ng,
                             int nx1, double grav1, double* tab,
                             float* tab32) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nx1) return;
  const int i = ng + k;
  const double* x = x1v + ng;
  double w0 = 0., w1 = 0., w2 = 0., gvar = 0.;
  if (nx1 >= 3) {
    if (k == 0) {
      double a = x[1] - x[0], b2 = x[2] - x[1];
      w0 = -(2. * a + b2) / (a * (a + b2));
      w1 = (a + b2) / (a * b2);
      w2 = -(a / ((a + b2) * b2));
    } else if (k == nx1 - 1) {
      double c = x[nx1 - 2] - x[nx1 - 3], d = x[nx1 - 1] - x[nx1 - 2];
      w0 = d / (c * (c + d));
      w1 = -((c + d) / (c * d));
      w2 = (c + 2. * d) / ((c + d) * d);
    } else {
      double hm = x[k] - x[k - 1], hp = x[k + 1] - x[k];
      w0 = -hp / (hm * (hm + hp));
      w1 = (hp - hm) / (hm * hp);
      w2 = hm / (hp * (hm + hp));
    }
    double h = x1f[i + 1] - x1f[i];
    gvar = grav1 * (h * h / 12.);
  }
  double* t = tab + 6 * k;
  t[0] = w0;
  t[1] = w1;
  t[2] = w2;
  t[3] = gvar;
  t[4] = grav1 * (x1f[i + 1] - x1v[i]);
  t[5] = grav1 * (x1f[i] - x1v[i]);
  if (tab32) {  // the same values rounded to FP32, and the covariance dx
    float* f = tab32 + 8 * k;
    for (int q = 0; q < 6; ++q) f[q] = (float)t[q];
    f[6] = (float)(x1v[i + 1] - x1v[i - 1]);
    f[7] = 0.f;
  }
}

// acc[k] += counts[k] over the nblock * kCountSlots monitor counts
__global__ void add_counts_kernel(int n, const unsigned long long* counts,
                                  int64_t* acc) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) acc[k] += (int64_t)counts[k];
}

__global__ void init_red_kernel(int n, unsigned long long* red, int* nan) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n) return;
  red[4 * b] = red[4 * b + 1] = red[4 * b + 2] = red[4 * b + 3] = kKeyInf;
  nan[b] = 0;
}

}  // namespace

struct sg_handle {
  sg_scheme scheme;
  std::vector<BlockDev> host;
  BlockDev* dev = nullptr;
  unsigned long long* red = nullptr;  // 4 keys per block
  int* nan = nullptr;
  void** ptrs = nullptr;  // device array of nblock pointers (sg_prim)
  void** ptrs_host = nullptr;  // pinned staging
  int32_t nblock = 0, ntile = 0;
  int32_t cur = 0, base = 0;  // current buffer, stage-0 buffer
  bool bound_all = false, dirty = true;
  size_t smem = 0, max_plane = 0, max_cells = 0;
  int32_t max_nc1 = 0;
  int32_t launches = 0;
  int* status = nullptr;  // per-block solve status bits (VIC failures)
  unsigned long long* fallbacks = nullptr;  // per block: refined-solve
                                            // columns solved directly
  unsigned long long* counts = nullptr;  // per block, kCountSlots: the
                                         // current step's monitor counts
  std::vector<double*> x1tabs;  // per-block geometry tables (gravity)
  bool has3 = false;            // a 3-D block: the x3 sweep runs
  bool visc3 = false;           // a 3-D block with viscosity: the prep runs
  size_t sum_icols = 0;         // implicit columns of all blocks
  int wide = 0;  // enough columns for a thread per column in the finish
  int wide_auto = 0;  // that rule's own answer (finish form 0)
  bool implicit = false;
  int vic_kinds = 0;  // bit 0: a block with the full 5x5 matrix, bit 1: 3x3
  bool ref32 = false;  // an FP32 block under gravity: base_ref_kernel runs
  int asm_kinds = 0;   // implicit blocks assembled in FP64 (bit 0), FP32 (1)
  int refine = 0;  // corrections of the refined implicit solve (0: direct)
  // the partitioned form of the scheme-9 solve of FP64-assembled blocks:
  // the requested mode (sg_set_sweep: 0 serial, 1 partitioned, 2 the
  // autotuner's choice), whether it runs now, and its region (per block,
  // at psw_off[b]; the blocks it serves: FP64-assembled, scheme 9, at least
  // kPswMinLayers layers)
  int psw_mode = 0;
  int psw_on = 0;
  double* psw_mem = nullptr;
  std::vector<size_t> psw_off;
  int any_f32 = 0;  // a block assembles its implicit blocks in FP32
  size_t max_icells = 0, max_icols = 0;
  std::vector<sg_block_desc> descs;   // as created (tile re-layout)
  int32_t finish = 0;  // implicit finish form: 0 auto, 1 warp, 2 thread
  std::vector<size_t> scratch_bytes;  // per block: vic_bytes + the x3 part
  std::vector<size_t> vic_bytes;
  std::vector<size_t> dv3_bytes;  // per block: the x3 part of the scratch
  bool scalars = false;           // some block transports passive scalars
  int device = 0;
  // per-kernel timing (sg_set_timing): events recorded between the launches
  // of each eager sg_stage, reused from a pool; each pending interval is
  // (kernel, start event, end event)
  bool timing = false;
  std::vector<cudaEvent_t> events;
  size_t events_used = 0;
  struct Interval {
    int kernel, e0, e1;
  };
  std::vector<Interval> pending;
};

namespace {

bool f64(const sg_handle* h) { return h->scheme.dtype == SG_F64; }

size_t stage_smem(const sg_handle* h, const sg_block_desc& d, int tj) {
  int has2 = d.nc2 > 1, wb = d.grav1 != 0., cov = d.flux_cov && d.nc1 >= 3;
  int visc = d.nu_iso > 0.;
  return f64(h) ? sg_stage_smem_f64(d.nc1, tj, has2, wb, cov, visc)
                : sg_stage_smem_f32(d.nc1, tj, has2, wb, cov, visc);
}

// tile width: enough CTAs to cover the SMs, shared memory within one CTA's
// opt-in limit (2 CTAs per SM where it fits)
int choose_tj(const sg_handle* h, const sg_block_desc& d, int nblock) {
  if (d.nc2 <= 1) return 1;
  int nx2 = d.nc2 - 2 * d.ng;
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
  int best = 1;
  for (int tj : {8, 4, 2, 1}) {
    if (stage_smem(h, d, tj) > 110 * 1024) continue;
    long tiles = (long)((nx2 + tj - 1) / tj) * std::max(1, d.nc3 - 2 * d.ng) *
                 nblock;
    if (tiles >= 2L * sms) return tj;
    best = tj;
  }
  return best;
}

int upload(sg_handle* h, cudaStream_t s) {
  if (!h->dirty) return 0;
  for (int b = 0; b < h->nblock; ++b) {
    for (int q = 0; q < 3; ++q)
      if (!h->host[b].buf[q])
        return fail(SG_ERR_STATE, "block %d buffer %d is not bound", b, q);
    if ((h->host[b].implicit && !h->host[b].vic) ||
        (h->host[b].nc3 > 1 && !h->host[b].dv3))
      return fail(SG_ERR_STATE, "block %d: the scratch (implicit solve, x3 "
                  "faces) is not bound (sg_bind_scratch)", b);
    if (h->host[b].implicit && h->host[b].step[0] && !h->host[b].t1)
      return fail(SG_ERR_STATE, "block %d: the x1 step field of an implicit "
                  "block needs its scratch (sg_bind_step_fields)", b);
    if (h->host[b].nscalar > 0 &&
        (!h->host[b].sbuf[0] || !h->host[b].mflux[0]))
      return fail(SG_ERR_STATE, "block %d: its scalar buffers or scratch are "
                  "not bound (sg_bind_scalars, sg_bind_scratch)", b);
  }
  cudaError_t e = cudaMemcpyAsync(h->dev, h->host.data(),
                                  sizeof(BlockDev) * h->nblock,
                                  cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "upload block table");
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "upload block table");
  h->dirty = false;
  return 0;
}

// the tiles of every block for the tile widths tj (null or 0: the library's
// choice), each clamped to the block's x2 extent and halved until its tile
// fits the opt-in shared memory
int relayout(sg_handle* h, const int32_t* tj) {
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin,
                         h->device);
  int tile = 0;
  size_t smem = 0;
  for (int b = 0; b < h->nblock; ++b) {
    const sg_block_desc& d = h->descs[b];
    BlockDev& B = h->host[b];
    const int nx2 = d.nc2 > 1 ? d.nc2 - 2 * d.ng : 1;
    const int nx3 = d.nc3 > 1 ? d.nc3 - 2 * d.ng : 1;
    int t = tj && tj[b] > 0 ? tj[b] : (d.tj > 0 ? d.tj : choose_tj(h, d, h->nblock));
    if (d.nc2 <= 1) t = 1;
    if (t > nx2) t = nx2;
    while (t > 1 && (long)stage_smem(h, d, t) > optin) t = (t + 1) / 2;
    const size_t sm = stage_smem(h, d, t);
    if ((long)sm > optin)
      return fail(SG_ERR_UNSUPPORTED, "block %d: a tile needs %zu B of "
                  "shared memory (limit %d)", b, sm, optin);
    B.tj = t;
    B.ntile = nx3 * ((nx2 + t - 1) / t);
    B.tile0 = tile;
    tile += B.ntile;
    smem = std::max(smem, sm);
  }
  h->ntile = tile;
  h->smem = smem;
  h->dirty = true;
  return 0;
}

}  // namespace

extern "C" {

const char* sg_last_error(void) { return g_err.c_str(); }

int sg_set_solve(sg_handle* h, int32_t corrections) {
  if (!h || corrections < -1 || corrections > 3)
    return fail(SG_ERR_ARG, "sg_set_solve: %d corrections (-1 to 3)",
                corrections);
  h->refine = h->any_f32 ? corrections : 0;
  return 0;
}

namespace {
// does block b take the partitioned form: FP64-assembled scheme 9 with
// enough layers for four chunks
bool psw_block(const sg_handle* h, int b) {
  const BlockDev& B = h->host[b];
  return B.implicit == 9 && !B.implicit_f32 &&
         B.nc1 - 2 * B.ng >= sg::kPswMinLayers;
}

// point the served blocks at their regions (on) or at none (off)
void psw_apply(sg_handle* h, int on) {
  for (int b = 0; b < h->nblock; ++b)
    h->host[b].psw = on && psw_block(h, b) ? h->psw_mem + h->psw_off[b] : nullptr;
  h->psw_on = on;
  h->dirty = true;
}
}  // namespace

int sg_set_sweep(sg_handle* h, int32_t mode) {
  if (!h || mode < 0 || mode > 2)
    return fail(SG_ERR_ARG, "sg_set_sweep: mode %d (0 serial, 1 partitioned, "
                "2 autotuned)", mode);
  if (mode != 0 && !h->psw_mem) {
    // the region: per served block 50 doubles per interior cell and an int
    // per interior column, 16-byte aligned
    size_t total = 0;
    h->psw_off.assign(h->nblock, 0);
    for (int b = 0; b < h->nblock; ++b) {
      if (!psw_block(h, b)) continue;
      const BlockDev& B = h->host[b];
      const size_t n = B.nc1 - 2 * B.ng;
      const size_t cols = (size_t)(B.nc2 > 1 ? B.nc2 - 2 * B.ng : 1) *
                          (B.nc3 > 1 ? B.nc3 - 2 * B.ng : 1);
      h->psw_off[b] = total;
      size_t bytes = (sg::kPswDoublesPerCell * n * cols) * sizeof(double) +
                     cols * sizeof(int);
      total += (bytes + 15) / 16 * 2;  // in doubles
    }
    if (total) {
      cudaError_t e = cudaMalloc(&h->psw_mem, total * sizeof(double));
      if (e != cudaSuccess) return cuda_fail(e, "sg_set_sweep: region");
    }
  }
  h->psw_mode = mode;
  // a block table without served blocks keeps the serial solve
  psw_apply(h, mode == 1 && h->psw_mem ? 1 : 0);
  return 0;
}

int sg_psw_rcp(const double* x, double* r, int64_t n, sg_stream_t stream) {
  if (n < 0 || (n > 0 && (!x || !r)))
    return fail(SG_ERR_ARG, "sg_psw_rcp: null or negative size");
  if (n == 0) return 0;
  int e = sg_launch_psw_rcp_f64(x, r, (size_t)n,
                                reinterpret_cast<cudaStream_t>(stream));
  return e ? cuda_fail((cudaError_t)e, "sg_psw_rcp") : 0;
}

int sg_add_step_counts(sg_handle* h, int64_t* acc_dev, sg_stream_t stream) {
  if (!h || !acc_dev) return fail(SG_ERR_ARG, "sg_add_step_counts: null");
  const int n = sg::kCountSlots * h->nblock;
  add_counts_kernel<<<(n + 127) / 128, 128, 0,
                      reinterpret_cast<cudaStream_t>(stream)>>>(n, h->counts,
                                                                acc_dev);
  cudaError_t e = cudaGetLastError();
  return e != cudaSuccess ? cuda_fail(e, "sg_add_step_counts") : 0;
}

int sg_sweep(const sg_handle* h, int32_t* on) {
  if (!h || !on) return fail(SG_ERR_ARG, "sg_sweep: null");
  *on = h->psw_on;
  return 0;
}

int sg_solve_fallbacks(sg_handle* h, int64_t* counts) {
  if (!h || !counts) return fail(SG_ERR_ARG, "sg_solve_fallbacks: null");
  cudaError_t e = cudaMemcpy(counts, h->fallbacks,
                             sizeof(unsigned long long) * h->nblock,
                             cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "sg_solve_fallbacks");
  return 0;
}

int sg_set_schedule(sg_handle* h, const int32_t* tj, int32_t finish) {
  if (!h || finish < 0 || finish > 2)
    return fail(SG_ERR_ARG, "sg_set_schedule: finish form %d", finish);
  int rc = relayout(h, tj);
  if (rc) return rc;
  h->finish = finish;
  h->wide = finish == 0 ? h->wide_auto : (finish == 2 ? 1 : 0);
  return 0;
}

int sg_autotune(sg_handle* h, int32_t reps, int32_t* tj_out,
                int32_t* finish_out, double* ms_out, sg_stream_t stream) {
  if (!h) return fail(SG_ERR_ARG, "sg_autotune: null handle");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cs) != cudaSuccess ||
      cs != cudaStreamCaptureStatusNone)
    return fail(SG_ERR_STATE, "sg_autotune: not inside a stream capture");
  if (reps < 1) reps = 1;
  int rc = upload(h, s);
  if (rc) return rc;
  const int nb = h->nblock;
  // the trials leave the step fields, the status bits and the state alone:
  // fields out of the table, status saved, and the trials write only the
  // rotation's free buffer (and the solve's scratch)
  std::vector<std::array<double*, 4>> saved(nb);
  for (int b = 0; b < nb; ++b) {
    BlockDev& B = h->host[b];
    saved[b] = {B.step[0], B.step[1], B.step[2], B.t1};
    B.step[0] = B.step[1] = B.step[2] = B.t1 = nullptr;
  }
  std::vector<int32_t> prev_tj(nb);
  for (int b = 0; b < nb; ++b) prev_tj[b] = h->host[b].tj;
  int* st_save = nullptr;
  double* dt = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaMalloc(&st_save, sizeof(int) * nb);
  if (e == cudaSuccess) e = cudaMalloc(&dt, sizeof(double) * nb);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(st_save, h->status, sizeof(int) * nb,
                        cudaMemcpyDeviceToDevice, s);
  std::vector<int32_t> best_tj = prev_tj;
  double best_ms = 1e300, best_vic = 0.;
  int best_finish = h->finish;
  if (e == cudaSuccess) {
    h->dirty = true;
    rc = upload(h, s);
    // a realistic dt: the blocks' own CFL step
    if (!rc) rc = sg_max_dt(h, nullptr, dt, stream);
    StageParams p;
    memset(&p, 0, sizeof(p));
    p.nblock = nb;
    p.in = p.u0 = h->cur;
    p.out = h->cur != h->base ? 3 - h->cur - h->base : (h->cur + 1) % 3;
    p.riemann = h->scheme.riemann;
    p.shock = h->scheme.shock;
    p.scale = h->scheme.scale;
    p.w0 = h->scheme.wght[0][0];
    p.w1 = h->scheme.wght[0][1];
    p.w2 = h->scheme.wght[0][2];
    p.dt = dt;
    p.first = 1;
    p.status = h->status;
    p.refine = h->refine;
    p.psw = h->psw_on;
    p.fallbacks = h->fallbacks;
    p.max_nc1 = h->max_nc1;
    p.visc3 = h->visc3;
    p.vic_kinds = h->vic_kinds;
    p.ref32 = h->ref32;
    p.asm_kinds = h->asm_kinds;
    auto stage = [&]() -> int {
      p.ntile = h->ntile;
      int r = 0;
      if (h->has3)
        r = f64(h) ? sg_launch_x3_f64(h->dev, p, h->max_cells, s)
                   : sg_launch_x3_f32(h->dev, p, h->max_cells, s);
      if (!r)
        r = f64(h) ? sg_launch_stage_f64(h->dev, p, h->smem, s)
                   : sg_launch_stage_f32(h->dev, p, h->smem, s);
      return r ? cuda_fail((cudaError_t)r, "sg_autotune: trial stage") : 0;
    };
    auto vic = [&]() -> int {
      int r = f64(h) ? sg_launch_vic_f64(h->dev, p, h->max_icells, h->max_icols,
                                         h->wide, h->status, s, nullptr)
                     : sg_launch_vic_f32(h->dev, p, h->max_icells, h->max_icols,
                                         h->wide, h->status, s, nullptr);
      return r ? cuda_fail((cudaError_t)r, "sg_autotune: trial solve") : 0;
    };
    auto timed = [&](auto&& launch, double* ms) -> int {
      int r = launch();  // warm
      if (r) return r;
      cudaEventRecord(e0, s);
      for (int k = 0; k < reps && !r; ++k) r = launch();
      cudaEventRecord(e1, s);
      if (r) return r;
      cudaError_t x = cudaEventSynchronize(e1);
      if (x != cudaSuccess) return cuda_fail(x, "sg_autotune: trial timing");
      float f = 0.f;
      cudaEventElapsedTime(&f, e0, e1);
      *ms = f / reps;
      return 0;
    };
    // (1) the tile width, the same request for every block
    std::vector<std::vector<int32_t>> tried;
    for (int c : {1, 2, 3, 4, 6, 8, 12, 16, 24, 32}) {
      if (rc) break;
      std::vector<int32_t> req(nb, c);
      rc = relayout(h, req.data());
      if (rc) break;
      std::vector<int32_t> got(nb);
      for (int b = 0; b < nb; ++b) got[b] = h->host[b].tj;
      bool seen = false;
      for (auto& t : tried) seen = seen || t == got;
      if (seen) continue;
      tried.push_back(got);
      rc = upload(h, s);
      double ms = 0.;
      if (!rc) rc = timed(stage, &ms);
      if (rc) break;
      if (ms < best_ms) {
        best_ms = ms;
        best_tj = got;
      }
    }
    if (!rc) rc = relayout(h, best_tj.data());
    if (!rc) rc = upload(h, s);
    // (2) the implicit solve's finish: a warp per column or a thread per
    // column (the stage's explicit tendency is in the scratch first), and
    // with sg_set_sweep mode 2 its solve serial or partitioned
    if (!rc && h->implicit) {
      rc = stage();
      double best = 1e300;
      int best_sweep = h->psw_on;
      const bool both = h->psw_mode == 2 && h->psw_mem;
      for (int sweep = both ? 0 : h->psw_on; sweep <= (both ? 1 : h->psw_on);
           ++sweep) {
        if (both) {
          psw_apply(h, sweep);
          if (!rc) rc = upload(h, s);
          p.psw = sweep;
        }
        for (int form : {1, 2}) {
          if (rc) break;
          h->wide = form == 2;
          double ms = 0.;
          rc = timed(vic, &ms);
          if (!rc && ms < best) {
            best = ms;
            best_finish = form;
            best_vic = ms;
            best_sweep = sweep;
          }
        }
      }
      h->finish = best_finish;
      h->wide = best_finish == 2;
      if (both) {
        psw_apply(h, best_sweep);
        if (!rc) rc = upload(h, s);
      }
    }
    if (!rc) {
      e = cudaMemcpyAsync(h->status, st_save, sizeof(int) * nb,
                          cudaMemcpyDeviceToDevice, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) rc = cuda_fail(e, "sg_autotune: restore");
    }
  } else {
    rc = cuda_fail(e, "sg_autotune: setup");
  }
  for (int b = 0; b < nb; ++b) {
    BlockDev& B = h->host[b];
    B.step[0] = saved[b][0];
    B.step[1] = saved[b][1];
    B.step[2] = saved[b][2];
    B.t1 = saved[b][3];
  }
  if (rc) relayout(h, prev_tj.data());
  h->dirty = true;
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(st_save);
  cudaFree(dt);
  if (rc) return rc;
  rc = upload(h, s);
  if (rc) return rc;
  for (int b = 0; b < nb && tj_out; ++b) tj_out[b] = h->host[b].tj;
  if (finish_out) *finish_out = h->finish;
  if (ms_out) {
    ms_out[0] = best_ms;
    ms_out[1] = best_vic;
  }
  return 0;
}

// records `msg` as the calling thread's last error for entry points defined
// in other translation units; returns `code`
int sg_fail_message(int code, const char* msg) { return fail(code, "%s", msg); }
const char* sg_version(void) { return "snapy_gb300 0.1 (sm_103a)"; }

int sg_create(const sg_scheme* scheme, const sg_block_desc* blocks,
              int32_t nblock, sg_handle** out) {
  if (!scheme || !blocks || !out || nblock <= 0)
    return fail(SG_ERR_ARG, "sg_create: null argument or nblock <= 0");
  if (scheme->dtype != SG_F64 && scheme->dtype != SG_F32)
    return fail(SG_ERR_ARG, "sg_create: dtype must be SG_F64 or SG_F32");
  if (scheme->riemann != SG_HLLC && scheme->riemann != SG_LMARS)
    return fail(SG_ERR_UNSUPPORTED, "sg_create: riemann solver %d",
                scheme->riemann);
  if (scheme->nstage != 3)
    return fail(SG_ERR_UNSUPPORTED, "sg_create: only 3-stage rk3 is built");
  auto* h = new sg_handle();
  h->scheme = *scheme;
  cudaGetDevice(&h->device);
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin,
                         h->device);
  h->nblock = nblock;
  h->host.resize(nblock);
  h->descs.assign(blocks, blocks + nblock);
  int tile = 0;
  for (int b = 0; b < nblock; ++b) {
    const sg_block_desc& d = blocks[b];
    if (d.ng != 3) {
      sg_destroy(h);
      return fail(SG_ERR_UNSUPPORTED, "block %d: nghost %d (3 is built)", b,
                  d.ng);
    }
    if (d.nc1 < 2 * d.ng + 1 || d.nc2 < 1 || d.nc3 < 1 ||
        (d.nc2 > 1 && d.nc2 < 2 * d.ng + 1)) {
      sg_destroy(h);
      return fail(SG_ERR_ARG, "block %d: sizes (%d, %d, %d)", b, d.nc3, d.nc2,
                  d.nc1);
    }
    for (int f = 0; f < 6; ++f)
      if (d.bc[f] < SG_BC_NONE || d.bc[f] > SG_BC_EXTRAPOLATION) {
        sg_destroy(h);
        return fail(SG_ERR_ARG, "block %d: boundary kind %d", b, d.bc[f]);
      }
    BlockDev& B = h->host[b];
    memset(&B, 0, sizeof(B));
    B.nc1 = d.nc1, B.nc2 = d.nc2, B.nc3 = d.nc3, B.ng = d.ng;
    for (int f = 0; f < 6; ++f) B.bc[f] = d.bc[f];
    B.dx1 = d.dx1, B.dx2 = d.dx2, B.dx3 = d.dx3;
    B.gammad = d.gammad;
    B.cfl = scheme->cfl;
    B.grav1 = d.grav1;
    B.nu_iso = d.nu_iso;
    B.flux_cov = d.flux_cov;
    B.wb_wall_clamp = d.wb_wall_clamp;
    B.x1f = d.x1f;
    B.x1v = d.x1v;
    B.implicit = d.implicit_scheme;
    B.vic = nullptr;
    if (d.implicit_scheme != 0) {
      if (d.implicit_scheme != 9 && d.implicit_scheme != 1) {
        sg_destroy(h);
        return fail(SG_ERR_UNSUPPORTED, "block %d: implicit-scheme %d (the "
                    "full 5x5 scheme 9 and the partial 3x3 scheme 1 are "
                    "built)", b, d.implicit_scheme);
      }
      h->vic_kinds |= d.implicit_scheme == 9 ? 1 : 2;
      if (d.grav1 == 0. || d.bc[0] != SG_BC_REFLECTING ||
          d.bc[1] != SG_BC_REFLECTING || d.nc1 - 2 * d.ng < 3) {
        sg_destroy(h);
        return fail(SG_ERR_UNSUPPORTED, "block %d: the vertical implicit solve "
                    "needs const-gravity, reflecting x1 walls and nx1 >= 3", b);
      }
      h->implicit = true;
    }
    B.dt_src = INFINITY;
    if (d.nu_iso > 0.) {  // DiffusionImpl::max_time_step, kinematic nu
      int ndim = 0;
      double dxm = 1.7976931348623157e308;
      const double dxs[3] = {d.dx1, d.dx2, d.dx3};
      const int ns[3] = {d.nc1, d.nc2, d.nc3};
      for (int q = 0; q < 3; ++q)
        if (ns[q] > 1) {
          ++ndim;
          if (dxs[q] < dxm) dxm = dxs[q];
        }
      B.dt_src = dxm * dxm / (2. * ndim * d.nu_iso);
    }
    if ((d.grav1 != 0. || (d.flux_cov && d.nc2 > 1)) && (!d.x1f || !d.x1v)) {
      sg_destroy(h);
      return fail(SG_ERR_ARG, "block %d: gravity and the covariance row need "
                  "the x1 geometry (x1f, x1v)", b);
    }
    if (d.grav1 != 0. && scheme->dtype == SG_F32) {
      // FP32 under gravity stores anomalies about an FP64 hydrostatic base;
      // the anomaly Riemann solver is LMARS's (its face pressure is affine
      // in the two sides' pressures)
      if (!d.base) {
        sg_destroy(h);
        return fail(SG_ERR_ARG, "block %d: FP32 with gravity needs the FP64 "
                    "hydrostatic base (sg_block_desc.base)", b);
      }
      if (scheme->riemann != SG_LMARS) {
        sg_destroy(h);
        return fail(SG_ERR_UNSUPPORTED, "block %d: FP32 with gravity is built "
                    "for the lmars solver", b);
      }
    } else if (d.base) {
      sg_destroy(h);
      return fail(SG_ERR_ARG, "block %d: a hydrostatic base is only used by "
                  "FP32 blocks with gravity", b);
    }
    B.base = d.base;
    if (d.implicit_precision != SG_F64 && d.implicit_precision != SG_F32) {
      sg_destroy(h);
      return fail(SG_ERR_ARG, "block %d: implicit_precision %d", b,
                  d.implicit_precision);
    }
    if (d.implicit_precision == SG_F32 && scheme->dtype != SG_F32) {
      sg_destroy(h);
      return fail(SG_ERR_UNSUPPORTED, "block %d: implicit-precision float32 "
                  "needs the FP32 state (dynamics/precision float32)", b);
    }
    B.implicit_f32 = d.implicit_scheme != 0 && d.implicit_precision == SG_F32;
    if (d.implicit_scheme != 0) h->asm_kinds |= B.implicit_f32 ? 2 : 1;
    if (d.nscalar < 0 || d.nscalar > 16) {
      sg_destroy(h);
      return fail(SG_ERR_ARG, "block %d: nscalar %d (0 to 16)", b, d.nscalar);
    }
    B.nscalar = d.nscalar;
    if (d.nscalar > 0) h->scalars = true;
    if (B.implicit_f32) {
      h->any_f32 = 1;
      h->refine = 2;
    }
    B.x1tab = nullptr;
    B.refb = nullptr;
    B.x1tab32 = nullptr;
    if (d.grav1 != 0.) {
      const int nx1 = d.nc1 - 2 * d.ng;
      // FP32: the geometry table in FP32 and the base reference table
      // follow the geometry table
      const bool r32 = scheme->dtype == SG_F32;
      const size_t nref = r32 ? 4 * (size_t)nx1 + 1 + 5 * ((size_t)d.nc1 + 1) : 0;
      double* t = nullptr;
      cudaError_t e = cudaMalloc(&t, sizeof(double) * (6 * (size_t)nx1 + nref));
      if (e == cudaSuccess) {
        h->x1tabs.push_back(t);
        float* t32 = r32 ? reinterpret_cast<float*>(t + 6 * (size_t)nx1) : nullptr;
        x1tab_kernel<<<(nx1 + 127) / 128, 128>>>(d.x1f, d.x1v, d.ng, nx1,
                                                 d.grav1, t, t32);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
      }
      if (e != cudaSuccess) {
        int rc = cuda_fail(e, "sg_create: x1 geometry table");
        sg_destroy(h);
        return rc;
      }
      B.x1tab = t;
      if (r32) {
        B.x1tab32 = reinterpret_cast<const float*>(t + 6 * (size_t)nx1);
        B.refb = t + 10 * (size_t)nx1;
        h->ref32 = true;
      }
    }
    if (d.grav1 != 0. && (d.bc[0] == SG_BC_PERIODIC || d.bc[1] == SG_BC_PERIODIC)) {
      sg_destroy(h);
      return fail(SG_ERR_UNSUPPORTED, "block %d: gravity with a periodic x1", b);
    }
    B.tj = d.tj > 0 ? d.tj : choose_tj(h, d, nblock);
    int nx2 = d.nc2 > 1 ? d.nc2 - 2 * d.ng : 1;
    int nx3 = d.nc3 > 1 ? d.nc3 - 2 * d.ng : 1;
    // tiles: tj-wide x2 strips of every interior x3 plane
    B.ntile = nx3 * ((nx2 + B.tj - 1) / B.tj);
    if (d.nc3 > 1) h->has3 = true;
    B.tile0 = tile;
    tile += B.ntile;
    size_t sm = stage_smem(h, d, B.tj);
    if ((long)sm > optin) {
      sg_destroy(h);
      return fail(SG_ERR_UNSUPPORTED,
                  "block %d: a tile needs %zu B of shared memory (limit %d)",
                  b, sm, optin);
    }
    h->smem = std::max(h->smem, sm);
    size_t plane = (size_t)d.nc1 * d.nc2 * d.nc3;
    h->max_plane = std::max(h->max_plane, plane);
    h->max_cells = std::max(h->max_cells, plane);
    h->max_nc1 = std::max(h->max_nc1, d.nc1);
    size_t icols = (size_t)(d.nc2 > 1 ? d.nc2 - 2 * d.ng : 1) *
                   (size_t)(d.nc3 > 1 ? d.nc3 - 2 * d.ng : 1);
    size_t icells = (size_t)(d.nc1 - 2 * d.ng) * icols;
    // the block's scratch: the implicit solve's FP64 arrays, then (3-D) the
    // x3 flux differences a3 dF3 of every interior cell in the storage type
    size_t vic_bytes = d.implicit_scheme ? icells * sg::kVicDoublesPerCell *
                                               sizeof(double)
                                         : 0;
    if (d.implicit_scheme && d.implicit_precision == SG_F32)
      vic_bytes += (icells * sg::kVicFloatsPerCell +
                    icols * sg::kVicFloatsPerColumn) * sizeof(float);
    vic_bytes = (vic_bytes + 15) / 16 * 16;  // the x3 part starts aligned
    const size_t esz = f64(h) ? 8 : 4;
    size_t dv3_bytes = d.nc3 > 1 ? 5 * icells * esz : 0;
    dv3_bytes = (dv3_bytes + 15) / 16 * 16;
    if (d.nc3 > 1 && d.nu_iso > 0.) {
      // the viscous prep planes and the x3 viscous momentum differences
      const size_t cells3 = (size_t)d.nc1 * d.nc2 * d.nc3;
      dv3_bytes += (5 * cells3 * esz + 15) / 16 * 16 + (3 * icells * esz + 15) / 16 * 16;
      h->visc3 = true;
    }
    // passive scalars: the FP64 mass flux and the scalars' face fluxes along
    // x1 and x2 over the padded block
    const size_t cells = (size_t)d.nc1 * d.nc2 * d.nc3;
    size_t sc_bytes = d.nscalar > 0 ? (4 + 5 * (size_t)d.nscalar) * cells * 8 : 0;
    h->vic_bytes.push_back(vic_bytes);
    h->dv3_bytes.push_back(dv3_bytes);
    h->scratch_bytes.push_back(vic_bytes + dv3_bytes + sc_bytes);
    if (d.implicit_scheme) {
      h->max_icells = std::max(h->max_icells, icells);
      h->max_icols = std::max(h->max_icols, icols);
      h->sum_icols += icols;
    }
  }
  h->ntile = tile;
  {
    // a full warp of columns for every SM sub-partition
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
    h->wide_auto = h->sum_icols >= (size_t)32 * 4 * sms;
    h->wide = h->wide_auto;
  }
  cudaError_t e = cudaMalloc(&h->dev, sizeof(BlockDev) * nblock);
  if (e == cudaSuccess)
    e = cudaMalloc(&h->red, sizeof(unsigned long long) * 4 * nblock);
  if (e == cudaSuccess) e = cudaMalloc(&h->nan, sizeof(int) * nblock);
  if (e == cudaSuccess) e = cudaMalloc(&h->ptrs, sizeof(void*) * nblock);
  if (e == cudaSuccess) e = cudaMalloc(&h->status, sizeof(int) * nblock);
  if (e == cudaSuccess) e = cudaMemset(h->status, 0, sizeof(int) * nblock);
  if (e == cudaSuccess)
    e = cudaMalloc(&h->fallbacks, sizeof(unsigned long long) * nblock);
  if (e == cudaSuccess)
    e = cudaMemset(h->fallbacks, 0, sizeof(unsigned long long) * nblock);
  if (e == cudaSuccess)
    e = cudaMalloc(&h->counts, sizeof(unsigned long long) * sg::kCountSlots * nblock);
  if (e == cudaSuccess)
    e = cudaMemset(h->counts, 0, sizeof(unsigned long long) * sg::kCountSlots * nblock);
  if (e == cudaSuccess) e = cudaMallocHost(&h->ptrs_host, sizeof(void*) * nblock);
  if (e != cudaSuccess) {
    sg_destroy(h);
    return cuda_fail(e, "sg_create");
  }
  init_red_kernel<<<(nblock + 127) / 128, 128>>>(nblock, h->red, h->nan);
  e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    sg_destroy(h);
    return cuda_fail(e, "sg_create");
  }
  *out = h;
  return 0;
}

int sg_destroy(sg_handle* h) {
  if (!h) return 0;
  if (h->dev) cudaFree(h->dev);
  if (h->red) cudaFree(h->red);
  if (h->nan) cudaFree(h->nan);
  if (h->ptrs) cudaFree(h->ptrs);
  if (h->status) cudaFree(h->status);
  if (h->fallbacks) cudaFree(h->fallbacks);
  if (h->counts) cudaFree(h->counts);
  if (h->ptrs_host) cudaFreeHost(h->ptrs_host);
  for (cudaEvent_t e : h->events) cudaEventDestroy(e);
  for (double* t : h->x1tabs) cudaFree(t);
  if (h->psw_mem) cudaFree(h->psw_mem);
  delete h;
  return 0;
}

int sg_bind(sg_handle* h, int32_t block, void* b0, void* b1, void* b2) {
  if (!h || block < 0 || block >= h->nblock)
    return fail(SG_ERR_ARG, "sg_bind: block %d out of range", block);
  if (!b0 || !b1 || !b2 || b0 == b1 || b1 == b2 || b0 == b2)
    return fail(SG_ERR_ARG, "sg_bind: three distinct non-null buffers needed");
  size_t align = f64(h) ? 8 : 4;
  for (void* p : {b0, b1, b2})
    if (reinterpret_cast<uintptr_t>(p) % align)
      return fail(SG_ERR_ARG, "sg_bind: misaligned buffer");
  BlockDev& B = h->host[block];
  B.buf[0] = b0, B.buf[1] = b1, B.buf[2] = b2;
  h->dirty = true;
  return 0;
}

int sg_scratch_bytes(const sg_handle* h, int32_t block, size_t* bytes) {
  if (!h || !bytes || block < 0 || block >= h->nblock)
    return fail(SG_ERR_ARG, "sg_scratch_bytes: block %d", block);
  *bytes = h->scratch_bytes[block];
  return 0;
}

int sg_bind_scratch(sg_handle* h, int32_t block, void* scratch, size_t bytes) {
  if (!h || block < 0 || block >= h->nblock)
    return fail(SG_ERR_ARG, "sg_bind_scratch: block %d", block);
  if (bytes < h->scratch_bytes[block] || (h->scratch_bytes[block] && !scratch))
    return fail(SG_ERR_ARG, "sg_bind_scratch: block %d needs %zu bytes, got %zu",
                block, h->scratch_bytes[block], bytes);
  if (reinterpret_cast<uintptr_t>(scratch) % 16)
    return fail(SG_ERR_ARG, "sg_bind_scratch: misaligned scratch");
  BlockDev& B = h->host[block];
  B.vic = B.implicit ? static_cast<double*>(scratch) : nullptr;
  B.dv3 = B.nc3 > 1 ? static_cast<unsigned char*>(scratch) + h->vic_bytes[block]
                    : nullptr;
  B.visc3 = B.dv3v = nullptr;
  if (B.nc3 > 1 && B.nu_iso > 0.) {
    const size_t esz = f64(h) ? 8 : 4;
    const size_t icells = (size_t)(B.nc1 - 2 * B.ng) *
                          (B.nc2 > 1 ? B.nc2 - 2 * B.ng : 1) * (B.nc3 - 2 * B.ng);
    const size_t cells3 = (size_t)B.nc1 * B.nc2 * B.nc3;
    unsigned char* v = static_cast<unsigned char*>(B.dv3) +
                       (5 * icells * esz + 15) / 16 * 16;
    B.visc3 = v;
    B.dv3v = v + (5 * cells3 * esz + 15) / 16 * 16;
  }
  if (B.nscalar > 0) {
    double* sc = reinterpret_cast<double*>(static_cast<unsigned char*>(scratch) +
                                           h->vic_bytes[block] +
                                           h->dv3_bytes[block]);
    const size_t plane = (size_t)B.nc1 * B.nc2 * B.nc3;
    const size_t ns = B.nscalar;
    for (int d = 0; d < 3; ++d) {
      B.mflux[d] = sc + d * plane;
      B.sflux[d] = sc + (3 + d * ns) * plane;
    }
    B.sds = sc + (3 + 3 * ns) * plane;
    B.vicq = sc + (3 + 4 * ns) * plane;
    B.stheta = sc + (4 + 4 * ns) * plane;
  }
  h->dirty = true;
  return 0;
}

int sg_bind_scalars(sg_handle* h, int32_t block, void* s0, void* s1, void* s2) {
  if (!h || block < 0 || block >= h->nblock)
    return fail(SG_ERR_ARG, "sg_bind_scalars: block %d", block);
  BlockDev& B = h->host[block];
  if (B.nscalar == 0)
    return fail(SG_ERR_ARG, "sg_bind_scalars: block %d has no scalars", block);
  if (!s0 || !s1 || !s2)
    return fail(SG_ERR_ARG, "sg_bind_scalars: null buffer");
  B.sbuf[0] = s0;
  B.sbuf[1] = s1;
  B.sbuf[2] = s2;
  h->dirty = true;
  return 0;
}

int sg_step_scratch_bytes(const sg_handle* h, int32_t block, size_t* bytes) {
  if (!h || !bytes || block < 0 || block >= h->nblock)
    return fail(SG_ERR_ARG, "sg_step_scratch_bytes: block %d", block);
  const BlockDev& B = h->host[block];
  size_t nx1 = B.nc1 - 2 * B.ng;
  size_t ncols = (B.nc2 > 1 ? B.nc2 - 2 * B.ng : 1) *
                 (size_t)(B.nc3 > 1 ? B.nc3 - 2 * B.ng : 1);
  *bytes = B.implicit ? 5 * (nx1 + 1) * ncols * sizeof(double) : 0;
  return 0;
}

int sg_bind_step_fields(sg_handle* h, int32_t block, double* s1, double* s2,
                        double* s3, void* scratch, size_t bytes) {
  if (!h || block < 0 || block >= h->nblock)
    return fail(SG_ERR_ARG, "sg_bind_step_fields: block %d", block);
  BlockDev& B = h->host[block];
  if ((s2 && B.nc2 <= 1) || (s3 && B.nc3 <= 1))
    return fail(SG_ERR_ARG, "sg_bind_step_fields: block %d has no x%d faces",
                block, s2 && B.nc2 <= 1 ? 2 : 3);
  for (double* f : {s1, s2, s3})
    if (reinterpret_cast<uintptr_t>(f) % 8)
      return fail(SG_ERR_ARG, "sg_bind_step_fields: misaligned field");
  size_t need = 0;
  sg_step_scratch_bytes(h, block, &need);
  if (s1 && need) {
    if (!scratch || bytes < need)
      return fail(SG_ERR_ARG, "sg_bind_step_fields: block %d needs %zu bytes "
                  "of scratch, got %zu", block, need, bytes);
    if (reinterpret_cast<uintptr_t>(scratch) % 16)
      return fail(SG_ERR_ARG, "sg_bind_step_fields: misaligned scratch");
  }
  B.step[0] = s1;
  B.step[1] = s2;
  B.step[2] = s3;
  B.t1 = s1 && need ? static_cast<double*>(scratch) : nullptr;
  h->dirty = true;
  // the table goes to the device now when it can: a replayed graph reads it
  // without another sg_stage call to upload it
  for (int b = 0; b < h->nblock; ++b)
    for (int q = 0; q < 3; ++q)
      if (!h->host[b].buf[q]) return 0;
  return upload(h, nullptr);
}

int sg_budget_totals(sg_handle* h, double* out_dev, sg_stream_t stream) {
  if (!h || !out_dev) return fail(SG_ERR_ARG, "sg_budget_totals: null");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  int rc = upload(h, s);
  if (rc) return rc;
  rc = f64(h) ? sg_launch_budget_totals_f64(h->dev, h->nblock, h->cur, out_dev, s)
              : sg_launch_budget_totals_f32(h->dev, h->nblock, h->cur, out_dev, s);
  if (rc) return cuda_fail((cudaError_t)rc, "sg_budget_totals");
  return 0;
}

int sg_budget_boundary(sg_handle* h, double* out_dev, int32_t accumulate,
                       sg_stream_t stream) {
  if (!h || !out_dev) return fail(SG_ERR_ARG, "sg_budget_boundary: null");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  int rc = upload(h, s);
  if (rc) return rc;
  rc = f64(h) ? sg_launch_budget_boundary_f64(h->dev, h->nblock, out_dev,
                                              accumulate, s)
              : sg_launch_budget_boundary_f32(h->dev, h->nblock, out_dev,
                                              accumulate, s);
  if (rc) return cuda_fail((cudaError_t)rc, "sg_budget_boundary");
  return 0;
}

int sg_set_current(sg_handle* h, int32_t current) {
  if (!h || current < 0 || current > 2)
    return fail(SG_ERR_ARG, "sg_set_current: %d", current);
  h->cur = h->base = current;
  return 0;
}

int sg_current(const sg_handle* h, int32_t* current) {
  if (!h || !current) return fail(SG_ERR_ARG, "sg_current: null");
  *current = h->cur;
  return 0;
}

int sg_tile(const sg_handle* h, int32_t block, int32_t* tj) {
  if (!h || !tj || block < 0 || block >= h->nblock)
    return fail(SG_ERR_ARG, "sg_tile: block %d", block);
  *tj = h->host[block].tj;
  return 0;
}

int sg_launches_per_stage(const sg_handle* h, int32_t* n) {
  if (!h || !n) return fail(SG_ERR_ARG, "sg_launches_per_stage: null");
  *n = h->launches;
  return 0;
}

namespace {
// an event of the timing pool (created on first use, reused after each
// sg_kernel_times)
int take_event(sg_handle* h, int* idx) {
  if (h->events_used == h->events.size()) {
    cudaEvent_t e;
    cudaError_t err = cudaEventCreate(&e);
    if (err != cudaSuccess) return cuda_fail(err, "sg_stage: timing event");
    h->events.push_back(e);
  }
  *idx = (int)h->events_used++;
  return 0;
}
}  // namespace

int sg_set_timing(sg_handle* h, int32_t on) {
  if (!h) return fail(SG_ERR_ARG, "sg_set_timing: null");
  h->timing = on != 0;
  return 0;
}

int sg_kernel_times(sg_handle* h, double* ms, int64_t* launches) {
  if (!h || !ms || !launches) return fail(SG_ERR_ARG, "sg_kernel_times: null");
  for (int k = 0; k < SG_NKERNEL; ++k) ms[k] = 0., launches[k] = 0;
  for (const auto& iv : h->pending) {
    cudaError_t e = cudaEventSynchronize(h->events[iv.e1]);
    float t = 0.f;
    if (e == cudaSuccess)
      e = cudaEventElapsedTime(&t, h->events[iv.e0], h->events[iv.e1]);
    if (e != cudaSuccess) {
      h->pending.clear();
      h->events_used = 0;
      return cuda_fail(e, "sg_kernel_times");
    }
    ms[iv.kernel] += t;
    launches[iv.kernel] += 1;
  }
  h->pending.clear();
  h->events_used = 0;
  return 0;
}

namespace {
// the buffers of a stage: in = current, u0 = the stage-0 state, out = the
// remaining one (never the input, which other tiles read as a stencil)
void plan(const sg_handle* h, int stage, int* in, int* u0, int* out) {
  *in = h->cur;
  *u0 = stage == 0 ? h->cur : h->base;
  int o = 0;
  while (o == *in || o == *u0) ++o;
  *out = o;
}
}  // namespace

int sg_advance(sg_handle* h, int32_t stage) {
  if (!h || stage < 0 || stage >= h->scheme.nstage)
    return fail(SG_ERR_ARG, "sg_advance: stage %d", stage);
  int in, u0, out;
  plan(h, stage, &in, &u0, &out);
  if (stage == 0) h->base = h->cur;
  h->cur = out;
  return 0;
}

int sg_rotation(const sg_handle* h, int32_t* cur, int32_t* base) {
  if (!h || !cur || !base) return fail(SG_ERR_ARG, "sg_rotation: null");
  *cur = h->cur;
  *base = h->base;
  return 0;
}

int sg_set_rotation(sg_handle* h, int32_t cur, int32_t base) {
  if (!h || cur < 0 || cur > 2 || base < 0 || base > 2)
    return fail(SG_ERR_ARG, "sg_set_rotation: %d %d", cur, base);
  h->cur = cur;
  h->base = base;
  return 0;
}

int sg_stage(sg_handle* h, int32_t stage, const double* dt_dev,
             sg_stream_t stream) {
  if (!h || !dt_dev) return fail(SG_ERR_ARG, "sg_stage: null argument");
  if (stage < 0 || stage >= h->scheme.nstage)
    return fail(SG_ERR_ARG, "sg_stage: stage %d of %d", stage,
                h->scheme.nstage);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  int rc = upload(h, s);
  if (rc) return rc;
  int in, u0, out;
  plan(h, stage, &in, &u0, &out);
  StageParams p;
  memset(&p, 0, sizeof(p));
  p.nblock = h->nblock;
  p.ntile = h->ntile;
  p.in = in, p.u0 = u0, p.out = out;
  p.riemann = h->scheme.riemann;
  p.shock = h->scheme.shock;
  p.scale = h->scheme.scale;
  p.w0 = h->scheme.wght[stage][0];
  p.w1 = h->scheme.wght[stage][1];
  p.w2 = h->scheme.wght[stage][2];
  p.dt = dt_dev;
  p.first = stage == 0;
  p.status = h->status;
  p.refine = h->refine;
  p.counts = h->counts;
  p.psw = h->psw_on;
  p.fallbacks = h->fallbacks;
  p.max_nc1 = h->max_nc1;
  p.visc3 = h->visc3;
  p.vic_kinds = h->vic_kinds;
  p.ref32 = h->ref32;
  p.asm_kinds = h->asm_kinds;
  // events between the launches when timing is on and the stream is not
  // being captured: ev[0] (x3 ev[6]) stage ev[1] (assemble ev[2] solve
  // ev[3] finish ev[4]) (scalars ev[7]) ghost ev[5]
  cudaEvent_t ev[8] = {};
  int eidx[8] = {};
  bool timed = false;
  if (h->timing) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess)
      return cuda_fail(cudaGetLastError(), "sg_stage: capture query");
    timed = cs == cudaStreamCaptureStatusNone;
  }
  if (timed) {
    for (int k = 0; k < 8; ++k) {
      rc = take_event(h, &eidx[k]);
      if (rc) return rc;
      ev[k] = h->events[eidx[k]];
    }
    cudaEventRecord(ev[0], s);
  }
  if (stage == 0) {
    // the monitor's counts start over with the step (a rejected attempt's
    // counts are gone when its retry begins)
    cudaError_t ze = cudaMemsetAsync(
        h->counts, 0, sizeof(unsigned long long) * sg::kCountSlots * h->nblock, s);
    if (ze != cudaSuccess) return cuda_fail(ze, "sg_stage: monitor counts");
  }
  int launches = h->ref32 ? 3 : 2;  // (with the base reference's refresh)
  if (h->has3) {
    // the x3 faces of the 3-D blocks: their flux differences, which the
    // stage kernel adds to its divergence after x1 and x2
    rc = f64(h) ? sg_launch_x3_f64(h->dev, p, h->max_cells, s)
                : sg_launch_x3_f32(h->dev, p, h->max_cells, s);
    if (rc) return cuda_fail((cudaError_t)rc, "sg_stage: x3 sweep");
    if (timed) cudaEventRecord(ev[6], s);
    launches += h->visc3 ? 2 : 1;  // with viscosity its prep first
  }
  rc = f64(h) ? sg_launch_stage_f64(h->dev, p, h->smem, s)
              : sg_launch_stage_f32(h->dev, p, h->smem, s);
  if (rc) return cuda_fail((cudaError_t)rc, "sg_stage: stage kernel");
  if (timed) cudaEventRecord(ev[1], s);
  if (h->implicit) {
    rc = f64(h) ? sg_launch_vic_f64(h->dev, p, h->max_icells, h->max_icols,
                                    h->wide, h->status, s,
                                    timed ? ev + 2 : nullptr)
                : sg_launch_vic_f32(h->dev, p, h->max_icells, h->max_icols,
                                    h->wide, h->status, s,
                                    timed ? ev + 2 : nullptr);
    if (rc) return cuda_fail((cudaError_t)rc, "sg_stage: implicit solve");
    if (timed) cudaEventRecord(ev[4], s);
    // assembly, solve, finish; the refined solve adds its FP32 sweep and a
    // residual and a correction per correction
    // (a wide batch's finish is three launches)
    launches += 3 + (h->wide ? 2 : 0) + (h->vic_kinds == 3 ? 1 : 0) +
                (h->asm_kinds == 3 ? 1 : 0) +
                (h->refine > 0 ? 2 + 2 * h->refine : (h->refine < 0 ? 3 : 0)) +
                (h->psw_on ? 1 : 0);
  }
  if (h->scalars) {
    // the passive scalars on the stage's mass flux: face fluxes, update
    // (implicit blocks: the transport tendency, then the solve's transfer
    // and the update per column)
    rc = f64(h) ? sg_launch_scalar_f64(h->dev, p, h->max_plane,
                                       h->implicit ? h->max_icols : 0, s)
                : sg_launch_scalar_f32(h->dev, p, h->max_plane,
                                       h->implicit ? h->max_icols : 0, s);
    if (rc) return cuda_fail((cudaError_t)rc, "sg_stage: scalars");
    if (timed) cudaEventRecord(ev[7], s);
    // fluxes, the limiter's theta, its ghosts and the scaling, the update
    // (implicit blocks: and the solve's transfer)
    launches += h->implicit ? 6 : 5;
  }
  rc = f64(h) ? sg_launch_ghost_f64(h->dev, h->nblock, out, h->max_plane, s)
              : sg_launch_ghost_f32(h->dev, h->nblock, out, h->max_plane, s);
  if (rc) return cuda_fail((cudaError_t)rc, "sg_stage: ghost kernel");
  if (h->scalars) {
    rc = f64(h) ? sg_launch_scalar_ghost_f64(h->dev, h->nblock, out,
                                             h->max_plane, s)
                : sg_launch_scalar_ghost_f32(h->dev, h->nblock, out,
                                             h->max_plane, s);
    if (rc) return cuda_fail((cudaError_t)rc, "sg_stage: scalar ghosts");
    launches += 1;
  }
  if (timed) {
    cudaEventRecord(ev[5], s);
    if (h->has3) {
      h->pending.push_back({SG_KERNEL_X3, eidx[0], eidx[6]});
      h->pending.push_back({SG_KERNEL_STAGE, eidx[6], eidx[1]});
    } else {
      h->pending.push_back({SG_KERNEL_STAGE, eidx[0], eidx[1]});
    }
    int last = eidx[1];  // the event before the scalars or the ghosts
    if (h->implicit) {
      h->pending.push_back({SG_KERNEL_VIC_ASSEMBLE, eidx[1], eidx[2]});
      h->pending.push_back({SG_KERNEL_VIC_SOLVE, eidx[2], eidx[3]});
      h->pending.push_back({SG_KERNEL_VIC_FINISH, eidx[3], eidx[4]});
      last = eidx[4];
    }
    if (h->scalars) {
      h->pending.push_back({SG_KERNEL_SCALAR, last, eidx[7]});
      last = eidx[7];
    }
    h->pending.push_back({SG_KERNEL_GHOST, last, eidx[5]});
  }
  if (stage == 0) h->base = h->cur;
  h->cur = out;
  h->launches = launches;
  return 0;
}

int sg_fill_ghosts(sg_handle* h, sg_stream_t stream) {
  if (!h) return fail(SG_ERR_ARG, "sg_fill_ghosts: null");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  int rc = upload(h, s);
  if (rc) return rc;
  rc = f64(h) ? sg_launch_ghost_f64(h->dev, h->nblock, h->cur, h->max_plane, s)
              : sg_launch_ghost_f32(h->dev, h->nblock, h->cur, h->max_plane, s);
  if (rc) return cuda_fail((cudaError_t)rc, "sg_fill_ghosts");
  if (h->scalars) {
    rc = f64(h) ? sg_launch_scalar_ghost_f64(h->dev, h->nblock, h->cur,
                                             h->max_plane, s)
                : sg_launch_scalar_ghost_f32(h->dev, h->nblock, h->cur,
                                             h->max_plane, s);
    if (rc) return cuda_fail((cudaError_t)rc, "sg_fill_ghosts: scalars");
  }
  return 0;
}

int sg_max_dt(sg_handle* h, const int32_t* redo_dev, double* dt_out,
              sg_stream_t stream) {
  if (!h || !dt_out) return fail(SG_ERR_ARG, "sg_max_dt: null");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  int rc = upload(h, s);
  if (rc) return rc;
  rc = f64(h) ? sg_launch_reduce_f64(h->dev, h->nblock, h->cur, h->red,
                                     h->nan, h->max_cells, s)
              : sg_launch_reduce_f32(h->dev, h->nblock, h->cur, h->red,
                                     h->nan, h->max_cells, s);
  if (rc) return cuda_fail((cudaError_t)rc, "sg_max_dt: reduce");
  finish_dt_kernel<<<(h->nblock + 127) / 128, 128, 0, s>>>(
      h->nblock, h->red, h->nan, redo_dev, h->scheme.cfl, dt_out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "sg_max_dt: finish");
  return 0;
}

int sg_check(sg_handle* h, int32_t* flags, sg_stream_t stream) {
  if (!h || !flags) return fail(SG_ERR_ARG, "sg_check: null");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  int rc = upload(h, s);
  if (rc) return rc;
  rc = f64(h) ? sg_launch_reduce_f64(h->dev, h->nblock, h->cur, h->red,
                                     h->nan, h->max_cells, s)
              : sg_launch_reduce_f32(h->dev, h->nblock, h->cur, h->red,
                                     h->nan, h->max_cells, s);
  if (rc) return cuda_fail((cudaError_t)rc, "sg_check: reduce");
  finish_check_kernel<<<(h->nblock + 127) / 128, 128, 0, s>>>(
      h->nblock, h->red, h->nan, h->status, h->scheme.density_floor,
      h->scheme.pressure_floor, flags);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "sg_check: finish");
  return 0;
}

int sg_check_retry(sg_handle* h, int32_t* flags, int32_t* redo,
                   int32_t max_redo, int32_t* state, sg_stream_t stream) {
  if (!h || !flags || !redo || !state)
    return fail(SG_ERR_ARG, "sg_check_retry: null");
  if (max_redo < 0) return fail(SG_ERR_ARG, "sg_check_retry: max_redo %d", max_redo);
  if (h->cur == h->base)
    return fail(SG_ERR_STATE, "sg_check_retry: no step since the last one "
                "began (the current buffer is the step-start buffer)");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  int rc = upload(h, s);
  if (rc) return rc;
  rc = f64(h) ? sg_launch_reduce_f64(h->dev, h->nblock, h->cur, h->red,
                                     h->nan, h->max_cells, s)
              : sg_launch_reduce_f32(h->dev, h->nblock, h->cur, h->red,
                                     h->nan, h->max_cells, s);
  if (rc) return cuda_fail((cudaError_t)rc, "sg_check_retry: reduce");
  finish_check_kernel<<<(h->nblock + 127) / 128, 128, 0, s>>>(
      h->nblock, h->red, h->nan, h->status, h->scheme.density_floor,
      h->scheme.pressure_floor, flags, redo, state, max_redo);
  int gx = (int)std::min<size_t>((h->max_plane * 5 + 255) / 256, 1024);
  restore_kernel<<<dim3(gx, h->nblock), 256, 0, s>>>(
      h->dev, h->cur, h->base, state, f64(h) ? 8 : 4);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "sg_check_retry");
  return 0;
}

int sg_init_from_prim(sg_handle* h, double* const* w_in,
                      sg_stream_t stream) {
  if (!h || !w_in) return fail(SG_ERR_ARG, "sg_init_from_prim: null");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  int rc = upload(h, s);
  if (rc) return rc;
  cudaError_t e = cudaStreamSynchronize(s);  // the staging buffer is reused
  if (e != cudaSuccess) return cuda_fail(e, "sg_init_from_prim");
  for (int b = 0; b < h->nblock; ++b) {
    if (!w_in[b]) return fail(SG_ERR_ARG, "sg_init_from_prim: block %d", b);
    h->ptrs_host[b] = w_in[b];
  }
  e = cudaMemcpyAsync(h->ptrs, h->ptrs_host, sizeof(void*) * h->nblock,
                      cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "sg_init_from_prim: pointers");
  double* const* win = reinterpret_cast<double* const*>(h->ptrs);
  rc = f64(h) ? sg_launch_init_f64(h->dev, h->nblock, h->cur, win,
                                   h->max_plane, s)
              : sg_launch_init_f32(h->dev, h->nblock, h->cur, win,
                                   h->max_plane, s);
  if (rc) return cuda_fail((cudaError_t)rc, "sg_init_from_prim");
  h->base = h->cur;
  return 0;
}

int sg_restore(sg_handle* h) {
  if (!h) return fail(SG_ERR_ARG, "sg_restore: null");
  h->cur = h->base;
  return 0;
}

int sg_prim(sg_handle* h, void* const* w_out, sg_stream_t stream) {
  if (!h || !w_out) return fail(SG_ERR_ARG, "sg_prim: null");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  int rc = upload(h, s);
  if (rc) return rc;
  cudaError_t e = cudaStreamSynchronize(s);  // the staging buffer is reused
  if (e != cudaSuccess) return cuda_fail(e, "sg_prim");
  for (int b = 0; b < h->nblock; ++b) h->ptrs_host[b] = w_out[b];
  e = cudaMemcpyAsync(h->ptrs, h->ptrs_host, sizeof(void*) * h->nblock,
                      cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "sg_prim: pointers");
  rc = f64(h) ? sg_launch_prim_f64(h->dev, h->nblock, h->cur, h->ptrs,
                                   h->max_plane, s)
              : sg_launch_prim_f32(h->dev, h->nblock, h->cur, h->ptrs,
                                   h->max_plane, s);
  if (rc) return cuda_fail((cudaError_t)rc, "sg_prim");
  return 0;
}

}  // extern "C"
