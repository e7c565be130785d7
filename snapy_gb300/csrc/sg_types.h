// Host/device shared descriptors of the batched hydro stage.
//
// A batch is a set of equal-scheme blocks (a MeshBlock, an ensemble member or
// a served request) that advance the same RK stage in ONE launch.  Each block
// owns three rotating state buffers in HBM; a stage reads buf[in] (stencil),
// buf[u0] (the stage-0 state, pointwise) and writes buf[out].  The rotation is
// uniform across the batch, so the block table stays constant on the device
// and a captured CUDA graph replays without host writes.
#pragma once

#include <stdint.h>

namespace sg {

enum BcKind : int32_t {
  kBcNone = 0,  // no boundary function (custom no-op): ghosts keep their bits
  kBcReflecting = 1,
  kBcPeriodic = 2,
  kBcExtrapolation = 3,
};

enum RiemannKind : int32_t { kHllc = 0, kLmars = 1 };

// one block of the batch, as the device sees it
struct BlockDev {
  void* buf[3];         // (nvar, nc3, nc2, nc1) state buffers, storage dtype
  int32_t nc1, nc2, nc3, ng;
  int32_t tj;           // x2 columns per tile
  int32_t ntile;        // tiles of this block
  int32_t tile0;        // first tile index of this block in the batch
  int32_t bc[6];        // BcKind per face: x1 in/out, x2 in/out, x3 in/out
  double dx1, dx2, dx3;
  double gammad;
  double cfl;
  // the Straka-class physics: x1 gravity (0 = off), kinematic viscosity,
  // the x2-face covariance row and the well-balanced wall clamp
  double grav1;
  double nu_iso;
  int32_t flux_cov;
  int32_t wb_wall_clamp;
  // FP64 x1 geometry of the padded block: faces [nc1 + 1], centres [nc1]
  const double* x1f;
  const double* x1v;
  // the sources' time-step bound (the viscous dx^2 / (2 ndim nu)), or +inf
  double dt_src;
  // the vertical implicit correction: scheme (0 off, 9 the full 5x5 blocks,
  // 1 the partial 3x3 blocks of rows and columns {rho, m1, E})
  // and its FP64 scratch (kVicDoublesPerCell per interior cell), laid out
  // as in vic_scratch()
  int32_t implicit;
  int32_t implicit_f32;  // implicit-precision float32: FP32 block assembly
  double* vic;
  // the layer-parallel (partitioned) form of the scheme-9 solve of an
  // FP64-assembled block (sg_set_sweep): its region, per interior cell the
  // E and F blocks (25 doubles each), then one int per interior column
  // (1: the serial solve redoes the column); null: the serial solve alone
  double* psw;
  // FP32 under gravity: the state buffers hold anomalies u - u_b about an
  // FP64 hydrostatic base that depends on x1 only, laid out as
  //   rho_b[nc1] | p_b[nc1] | e_b[nc1] = p_b / (gamma - 1) | pf_b[nc1 + 1]
  //   (the base pressure at x1 face f, between cells f - 1 and f) |
  //   r_b[nc1] = rho_b g1 - (pf_b[i + 1] - pf_b[i]) / dx1
  // (null: the buffers hold totals)
  const double* base;
  // FP32 under gravity: the base's own well-balanced reference, refreshed
  // every stage from `base` (base_ref_kernel): refb[0] the base's top face
  // pressure (FP64), then as floats, with N = nc1: pbf [N + 1] and p_b [N]
  // rounded to FP32, Eb [N + 1] (the base's scanned face pressure - pf_b),
  // per cell Cmid, Clo, Chi, Cst [N] (the base parts of the mid, lower,
  // upper and stencil cell pressures, relative to p_b), rho_b and r_b [N]
  // rounded to FP32, and the top face's base pressure and exponential
  // factor; and x1tab32, the x1 geometry table in FP32 (8 floats per
  // interior cell: x1tab's 6, then x1v[i + 1] - x1v[i - 1]); null otherwise
  double* refb;
  const float* x1tab32;
  // with gravity: per interior x1 cell k, 6 FP64 constants of the geometry
  // (the corrected-PE slope weights w0, w1, w2, grav1 h^2 / 12, and
  // grav1 (x1f[i+1] - x1v[i]), grav1 (x1f[i] - x1v[i]) for i = ng + k)
  const double* x1tab;
  // 3-D: a3 (F3[k+1] - F3[k]) of every interior cell and variable, in the
  // storage type, laid out (v, k, j, i) over the interior; written by the x3
  // sweep, added to the divergence by the stage kernel
  void* dv3;
  // 3-D with viscosity: per cell of the block (ghosts included, set on the
  // interior extended by one cell) the velocity divergence and the centred
  // derivatives dv1/dx3, dv2/dx3, dv3/dx1, dv3/dx2, five planes in the
  // storage type (visc3_kernel); and a3 (V3[k+1] - V3[k]) of the x3 faces'
  // viscous momentum rows (IVX, IVY, IVZ), laid out like dv3
  void* visc3;
  void* dv3v;
  // the FluxRegister's FP64 step fields S_d (5, nc3, nc2, nc1), face f
  // along d below cell f (null: not requested), and, for an implicit block
  // with S_1, the stage's x1 totals T_1 staged for the solve's posts,
  // laid out (v, column, face) over the interior columns and nx1 + 1 faces
  double* step[3];
  double* t1;
  // passive scalars: their three buffers (nscalar, nc3, nc2, nc1) in the
  // storage type, rotated with buf; the stage's FP64 mass flux along x1, x2
  // and x3 (face f below cell f, written by the stage kernel and the x3
  // sweep) and the scalars' FP64 face fluxes (nscalar rows of the same
  // layout), in the scratch
  int32_t nscalar;
  void* sbuf[3];
  double* mflux[3];
  double* sflux[3];
  // an implicit block's scalars: their transport tendency ds (nscalar rows,
  // FP64) and the solve's clamped dry transfer q of each x1 face (the
  // finish kernel's, face f below cell f), for the transfer's share
  double* sds;
  double* vicq;
  // with the covariance row: the positivity limiter's theta of each scalar
  // (nscalar rows, FP64), ghosts filled like the scalars'
  double* stheta;
};

// offsets into BlockDev::base
__host__ __device__ inline const double* base_rho(const double* b, int nc1) { return b; }
__host__ __device__ inline const double* base_p(const double* b, int nc1) { return b + nc1; }
__host__ __device__ inline const double* base_e(const double* b, int nc1) { return b + 2 * nc1; }
__host__ __device__ inline const double* base_pf(const double* b, int nc1) { return b + 3 * nc1; }
__host__ __device__ inline const double* base_r(const double* b, int nc1) { return b + 4 * nc1 + 1; }

// doubles of VIC scratch per interior cell: du, du0 (5 each), the blocks
// a, b, c (25 each), the solution and the two Woodbury vectors (5 each)
constexpr int kVicDoublesPerCell = 100;
// implicit-precision float32 blocks add, after the FP64 part, a part for
// the refined solve: per interior cell the blocks A, B, C in FP32 (28 each:
// 25 and a pad), the factors of the FP32 sweep's pivot blocks (32), its C'
// blocks (28) and the residuals of the three right-hand sides (16: 15 and
// a pad); per
// interior column the largest update of each right-hand side in the last
// pass (3), the largest |x| of each after the first (3) and the direct-solve
// mask (1 int: 0 accepted, 1 left to the FP64 solve, 2 left by the
// partitioned FP64 solve to the serial one, 3 solved by the partitioned one)
constexpr int kVicFloatsPerCell = 160;
// the partitioned form of the scheme-9 solve: columns of fewer layers take
// the serial solve; its region holds two 5x5 blocks per interior cell
constexpr int kPswMinLayers = 16;
constexpr int kPswDoublesPerCell = 50;
constexpr int kVicFloatsPerColumn = 7;

// the monitor's counts of a step, per block (the RegisterMonitor counters
// src/hydro/hydro.cpp:175-192 that this path can raise): HLLC faces whose
// contact pressure was clamped to zero, and columns the implicit solve
// left to its FP64 retry; zeroed at each step's first stage
constexpr int kCountPstar = 0;
constexpr int kCountFp64Columns = 1;
constexpr int kCountSlots = 2;

// a tile's bulk-copy wait ran out (status bit; the step is rejected)
constexpr int32_t kStatusStaging = 1 << 30;

// what a stage launch needs besides the table
struct StageParams {
  int32_t nblock;
  int32_t ntile;        // total tiles (grid size)
  int32_t in, u0, out;  // buffer indices
  int32_t riemann;      // RiemannKind
  int32_t shock;        // 1: every row weno5
  int32_t scale;        // InterpOptions::scale
  double w0, w1, w2;    // RK weights of this stage
  const double* dt;     // device scalar: the host dt or a captured graph's
  int32_t first;        // stage 0: the step fields start from zero
  int32_t refine;       // corrections of the refined implicit solve of
                        // implicit-precision float32 blocks (0: direct)
  unsigned long long* fallbacks;  // per block: columns the refined solve left
                                  // to the direct FP64 solve (a running count)
  unsigned long long* counts;     // per block, kCountSlots: this step's
                                  // monitor counts (null: none kept)
  int32_t* status;      // per-block status bits (kStatusStaging: a tile's
                        // staging wait ran out)
  int32_t smem_rows;    // x1 lines held in shared memory per tile
  int32_t max_nc1;
  int32_t visc3;        // some 3-D block has viscosity: visc3_kernel runs
  int32_t asm_kinds;    // implicit blocks: bit 0 some assemble in FP64,
                        // bit 1 some in FP32 (one kernel each)
  int32_t ref32;        // some FP32 block keeps its reference in FP32
                        // (base_ref_kernel runs before the stage kernel)
  int32_t psw;          // some block has the partitioned solve on
                        // (vic_psolve_kernel runs before the serial one)
  int32_t vic_kinds;    // implicit blocks: bit 0 some with the full 5x5
                        // matrix (scheme 9), bit 1 some with the partial
                        // 3x3 one (scheme 1)
};

}  // namespace sg
