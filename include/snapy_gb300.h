/*
 * snapy_gb300 -- C ABI of the GB300-native MeshBlock hydro stage.
 *
 * A drop-in for the native dispatch boundary of snapy's hydro stage: one call
 * advances every block of a batch by one RK stage on a caller-provided CUDA
 * stream, reading the time step from device memory (so a captured CUDA graph
 * replays with any dt).  Plain pointers and sizes only; no torch types.
 *
 * Reference interfaces replaced (paths inside the snapy project):
 *   sg_create / sg_bind   MeshBlockImpl construction + StateStore adoption
 *                         (src/mesh/meshblock.hpp:142-392,
 *                          src/mesh/state_store.hpp:24-125)
 *   sg_stage              StageExecutor::run_stage -> stage_advance /
 *                         stage_combine / stage_boundaries
 *                         (src/mesh/stage_executor.cpp:809,
 *                          src/mesh/meshblock_advance.cpp:145,314,398), which
 *                         dispatch call_recon (src/recon/recon_dispatch.hpp:13),
 *                         call_riemann (src/riemann/riemann.hpp:161-171) and
 *                         the torch divergence / RK combine
 *   sg_max_dt             MeshBlockImpl::max_time_step
 *                         (src/mesh/meshblock_advance.cpp:61-72,
 *                          src/hydro/hydro.cpp:316-398)
 *   sg_check              MeshBlockImpl::local_redo_flag_tensor
 *                         (src/mesh/meshblock_redo.cpp:95-150)
 *   sg_restore            MeshBlockImpl::apply_redo's StateStore::restore
 *                         (src/mesh/meshblock_redo.cpp:58-60)
 *   sg_prim               EquationOfStateImpl::forward, U->W
 *                         (src/eos/equation_of_state.cpp:283-289)
 *   sg_fill_ghosts        MeshBlockImpl::apply_boundaries
 *                         (src/mesh/meshblock_exchange.cpp:214-286)
 *
 * Every function returns 0 on success and a positive code on error; the
 * message of the last error of the calling thread is sg_last_error().
 */
#ifndef SNAPY_GB300_H
#define SNAPY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sg_handle sg_handle;
typedef struct CUstream_st* sg_stream_t; /* a cudaStream_t */

enum { SG_F64 = 0, SG_F32 = 1 };
enum { SG_HLLC = 0, SG_LMARS = 1 };
enum {
  SG_BC_NONE = 0,
  SG_BC_REFLECTING = 1,
  SG_BC_PERIODIC = 2,
  SG_BC_EXTRAPOLATION = 3
};
enum {
  SG_OK = 0,
  SG_ERR_ARG = 1,
  SG_ERR_CUDA = 2,
  SG_ERR_UNSUPPORTED = 3,
  SG_ERR_STATE = 4
};

/* the scheme shared by every block of a batch (one deck) */
typedef struct sg_scheme {
  int32_t dtype;   /* SG_F64 / SG_F32: storage and compute of the stage */
  int32_t riemann; /* SG_HLLC / SG_LMARS */
  int32_t shock;   /* reconstruct shock: every row weno5 */
  int32_t scale;   /* reconstruct scale (WENO prologue) */
  int32_t nstage;  /* 3 for rk3 */
  double wght[3][3]; /* per stage (w0, w1, w2): u <- w0 u0 + w1 u + w2 du */
  double cfl;
  double density_floor, pressure_floor;
} sg_scheme;

/* one block: padded sizes (nx + 2 ng on an active axis, else 1) */
typedef struct sg_block_desc {
  int32_t nc1, nc2, nc3, ng;
  int32_t bc[6]; /* x1-inner, x1-outer, x2-inner, x2-outer, x3-in, x3-out */
  double dx1, dx2, dx3;
  double gammad;
  int32_t tj; /* x2 columns per tile, 0 = the library's choice */
  /* forcing/const-gravity/grav1 (0: none); with it the x1 reconstruction is
   * the well-balanced one (src/recon/well_balanced_x1.cpp) */
  double grav1;
  double nu_iso;         /* forcing/diffusion/nu_iso (0: none) */
  int32_t flux_cov;      /* dynamics/flux-covariance */
  int32_t wb_wall_clamp; /* dynamics/wb-wall-clamp */
  /* FP64 x1 geometry on the device: faces [nc1 + 1] and centres [nc1]
   * (the reference's linspace faces), read by the covariance row and the
   * gravity work; may be null without gravity and covariance */
  const double* x1f;
  const double* x1v;
  /* integration/implicit-scheme: 0 (none), 9 (the full 5x5 vertical
   * implicit solve) or 1 (the partial 3x3 blocks of rows and columns
   * {rho, m1, E}, the tangential momenta folded into the density column and
   * carried by the face mass transfers; assembled in either precision,
   * solved in FP64; the refined FP32 solve is scheme 9's).  Both need
   * const-gravity and reflecting x1 walls
   * (src/implicit/implicit_hydro.hpp:25-41) */
  int32_t implicit_scheme;
  /* SG_F32 with gravity: the FP64 hydrostatic base the FP32 state is stored
   * about (the buffers hold u - u_b), 5 nc1 + 1 device doubles:
   *   rho_b[nc1] | p_b[nc1] | e_b[nc1] = p_b/(gamma-1) |
   *   pf_b[nc1+1] (face f between cells f-1 and f) |
   *   r_b[nc1] = rho_b grav1 - (pf_b[i+1] - pf_b[i]) / dx1
   * The contents may be written after sg_create, before sg_init_from_prim.
   * Must be null otherwise. */
  const double* base;
  /* integration/implicit-precision: SG_F64 (default) or SG_F32, which
   * assembles the implicit blocks in FP32 (SG_F32 storage only); the
   * block-tridiagonal solve is refined to the FP64 solution (sg_set_solve,
   * below) or is the direct FP64 solve */
  int32_t implicit_precision;
  /* scalar/nvar: passive scalars transported by the stage's mass flux
   * (ScalarImpl, src/scalar/scalar.cpp:90-211); 0 for none.  Built for 1-D
   * and 2-D blocks without the implicit solve */
  int32_t nscalar;
} sg_block_desc;

int sg_create(const sg_scheme* scheme, const sg_block_desc* blocks,
              int32_t nblock, sg_handle** out);
int sg_destroy(sg_handle* h);
/* three device buffers per block, each (5, nc3, nc2, nc1) of the dtype; the
 * current state must be in buffer `current` (0..2) */
int sg_bind(sg_handle* h, int32_t block, void* buf0, void* buf1, void* buf2);
/* a block's three scalar buffers, each (nscalar, nc3, nc2, nc1) of the
 * dtype: the tracer densities s (scalar_s), rotated with the state buffers
 * (MeshBlockImpl's scalar StateStore rows, src/mesh/state_store.hpp) */
int sg_bind_scalars(sg_handle* h, int32_t block, void* s0, void* s1, void* s2);
/* the FP64 scratch of a block's vertical implicit solve (0 bytes without
 * one): the caller allocates it, 16-byte aligned, and binds it before the
 * first sg_stage (ImplicitHydroImpl::prepare, src/implicit/implicit_hydro.hpp) */
int sg_scratch_bytes(const sg_handle* h, int32_t block, size_t* bytes);
int sg_bind_scratch(sg_handle* h, int32_t block, void* scratch, size_t bytes);
int sg_set_current(sg_handle* h, int32_t current);
int sg_current(const sg_handle* h, int32_t* current);
/* the buffer rotation: `cur` holds the current state, `base` the stage-0
 * state of the step.  sg_advance does sg_stage's bookkeeping without a launch
 * (the replay of a captured stage); sg_set_rotation restores a saved one */
int sg_rotation(const sg_handle* h, int32_t* cur, int32_t* base);
int sg_set_rotation(sg_handle* h, int32_t cur, int32_t base);
int sg_advance(sg_handle* h, int32_t stage);
/* one RK stage of every block; dt_dev points at nblock device doubles */
int sg_stage(sg_handle* h, int32_t stage, const double* dt_dev,
             sg_stream_t stream);
/* ghost cells of the current buffer from the boundary functions */
int sg_fill_ghosts(sg_handle* h, sg_stream_t stream);
/* dt_dev_out[b] = cfl 2^-redo[b] min over block b (no host sync) */
int sg_max_dt(sg_handle* h, const int32_t* redo_dev, double* dt_dev_out,
              sg_stream_t stream);
/* per-block retry flags into flags_dev (int32[nblock]): bit 0 floor, bit 3
 * NaN, bit 5 a failed column of the implicit solve (meshblock_redo.cpp),
 * bit 6 a tile whose shared-memory staging did not arrive within the stage
 * kernel's bounded wait (the tile was not computed) */
int sg_check(sg_handle* h, int32_t* flags_dev, sg_stream_t stream);
/* The retry decision on the device, after a step (MeshBlockImpl::apply_redo
 * with local_redo_flag_tensor's flags, src/mesh/meshblock_redo.cpp:32-150):
 * sg_check's flags into flags_dev, then per block a flagged block counts a
 * redo (redo_dev[b] += 1) and gets its step-start state back in the current
 * buffer, state_dev[b] = 1, or -1 once redo_dev[b] exceeds max_redo; a
 * terminated block stays terminated and keeps its last accepted state
 * (restored at every later call).  A block without flags gets redo_dev[b]
 * = 0, state_dev[b] = 0.  sg_max_dt with the same redo_dev gives the
 * retried blocks dt x 2^-redo.  No host read: a captured step graph can
 * end with it.  Call it after a step's last stage, before the next step. */
int sg_check_retry(sg_handle* h, int32_t* flags_dev, int32_t* redo_dev,
                   int32_t max_redo, int32_t* state_dev, sg_stream_t stream);
/* initialize (MeshBlockImpl::initialize, src/mesh/meshblock.cpp:306-420):
 * the boundary functions fill the ghosts of the FP64 primitives w_in[b]
 * (device pointers in a host array, written in place), and the current
 * buffers <- W->U of them */
int sg_init_from_prim(sg_handle* h, double* const* w_in, sg_stream_t stream);
/* the current buffer becomes the stage-0 state again (a rejected step) */
int sg_restore(sg_handle* h);
/* primitives of the current state: w_out[b] are device pointers (host array) */
int sg_prim(sg_handle* h, void* const* w_out, sg_stream_t stream);
/* x2 columns per tile the library picked for block b */
int sg_tile(const sg_handle* h, int32_t block, int32_t* tj);
/* kernels launched by the last sg_stage call */
int sg_launches_per_stage(const sg_handle* h, int32_t* n);
/* Per-kernel device time of sg_stage (no counterpart in the reference, whose
 * profiling is host-side timers).  With timing on, each sg_stage that is not
 * being captured into a graph records events around its launches on its
 * stream; sg_kernel_times waits for them and returns, per kernel, the summed
 * milliseconds and the launch count since the previous call (arrays of
 * SG_NKERNEL).  Call it now and then while timing: the events of every
 * timed stage are held until it is called. */
enum {
  SG_KERNEL_STAGE = 0,        /* reconstruction, fluxes, sources, update */
  SG_KERNEL_VIC_ASSEMBLE = 1, /* implicit solve: block rows of each cell */
  SG_KERNEL_VIC_SOLVE = 2,    /* implicit solve: block-Thomas sweep */
  SG_KERNEL_VIC_FINISH = 3,   /* implicit solve: redistribution, update */
  SG_KERNEL_GHOST = 4,        /* ghost fill of the new state */
  SG_KERNEL_X3 = 5,           /* x3 faces of 3-D blocks */
  SG_KERNEL_SCALAR = 6,       /* passive scalars: face fluxes and update */
  SG_NKERNEL = 7
};
int sg_set_timing(sg_handle* h, int32_t on);
int sg_kernel_times(sg_handle* h, double* ms, int64_t* launches);

/* The schedule autotuner (no counterpart in the reference, whose stage is a
 * fixed chain of library calls).  sg_autotune times the stage's kernels on
 * this handle's own blocks and current state: every tile width of
 * 1, 2, 3, 4, 6, 8, 12, 16, 24, 32 x2 columns (the same request for every block, each
 * clamped to its x2 extent and halved until its tile fits the shared
 * memory), then, with an implicit solve, its finish as a warp per column
 * and as a thread per column, and keeps the fastest.  The results do not
 * depend on either choice (same operations, same order).  The trial
 * launches read the current state and write only the rotation's free
 * buffer and the solve's scratch; the step fields and the status bits are
 * left as they were.  Not inside a stream capture; graphs captured before
 * must be captured again.  Outputs (each may be null): tj_out[nblock] the
 * tile widths, *finish_out the finish form (1 warp, 2 thread; 0 when there
 * is no solve), ms_out[2] the best stage and solve milliseconds per launch.
 * sg_set_schedule applies a stored choice (tj null or 0: the library's
 * rule; finish 0: the library's rule). */
/* The implicit solve of integration/implicit-precision float32 blocks.  By
 * default it is refined: the block-tridiagonal system of each column is
 * solved by the block-Thomas sweep in FP32, then corrected `corrections`
 * times (default 2, at most 3) with FP64 residuals (mixed-precision
 * iterative refinement, the scheme of LAPACK's dsgesv), the solution
 * accumulating in FP64.  A column whose FP32 factorisation fails, or whose
 * last correction leaves an estimated error above 2^-44 of its solution,
 * takes the direct FP64 solve.  corrections 0 runs the direct FP64 solve for
 * every column (the FP64 blocks' solve, bitwise).  corrections -1 is the
 * reference's own FP32 compute of the implicit solve (PrecisionPolicy's
 * kImplicit row in FP32, src/mesh/precision_policy.hpp:31-71): the FP32
 * sweep and its Woodbury step, no corrections, the direct FP64 solve for
 * the columns whose FP32 sweep fails (the reference's FP64 retry,
 * integration/implicit-fallback-fp64).  FP64 blocks always run the direct
 * solve.  The refined and direct forms agree to FP64 roundoff of the
 * solution; the FP32 form to FP32 roundoff times the condition of the
 * column.  Not inside a stream capture; graphs captured before must be
 * captured again. */
int sg_set_solve(sg_handle* h, int32_t corrections);
/* per block, the running count of columns the refined solve left to the
 * direct FP64 solve (ImplicitHydroImpl's "implicit.fp64_columns" monitor,
 * src/hydro/hydro.cpp:460-466); waits for the device */
int sg_solve_fallbacks(sg_handle* h, int64_t* counts);
/* The order of elimination of the scheme-9 solve of FP64-assembled blocks
 * (replaces the serial ForwardSweep column loop of
 * src/implicit/forward_sweep_impl.h:30-131 and the back substitution of
 * src/implicit/vic_kernels.h:100-160 for such blocks; the reference has only
 * the serial order).  mode 0: the serial block-Thomas sweep, bit for bit the
 * reference's operation order (the default).  mode 1: the partitioned form,
 * for batches with too few columns to fill the GPU: each column in four
 * chunks swept at once by one warp, then a 3-row system of the separator
 * layers; the same solution to rounding (within 1e-12 relative), not bit
 * for bit.  mode 2: sg_autotune times both and keeps the faster (the
 * serial sweep until it runs).  Columns shorter than 16 layers, scheme-1
 * and FP32-assembled blocks always take their own solve; a column whose
 * partitioned solve fails any check is solved again serially, which
 * decides its failure as the reference does, and counts in
 * sg_solve_fallbacks.  Modes 1 and 2 allocate the form's region (400 B per
 * interior cell of the served blocks) on first use.  Not inside a stream
 * capture; graphs captured before must be captured again. */
int sg_set_sweep(sg_handle* h, int32_t mode);
/* The RegisterMonitor counts of the last step (src/hydro/flux_register.hpp
 * :61-178, the counters of src/hydro/hydro.cpp:175-192 that this path can
 * raise): acc_dev[2 b + 0] += the x1/x2/x3 interior faces of block b whose
 * HLLC contact pressure was clamped to zero (riemann.pstar_clamp),
 * acc_dev[2 b + 1] += its columns the implicit solve left to the FP64 retry
 * (implicit.fp64_columns).  acc_dev: 2 nblock device int64.  The counts
 * start over at each step's first stage, so a rejected attempt's are gone
 * when its retry begins, and an accepted step's stay until the next step
 * (the monitor's census of accepted steps).  On the stream, no host sync. */
int sg_add_step_counts(sg_handle* h, int64_t* acc_dev, sg_stream_t stream);
/* whether the partitioned form runs now (1) or the serial one (0) */
int sg_sweep(const sg_handle* h, int32_t* on);
/* A check of the partitioned form's reciprocal (no counterpart in the
 * reference): r[i] = its 1 / x[i] for n device doubles x, on the stream,
 * for comparison with the IEEE division. */
int sg_psw_rcp(const double* x, double* r, int64_t n, sg_stream_t stream);
int sg_autotune(sg_handle* h, int32_t reps, int32_t* tj_out,
                int32_t* finish_out, double* ms_out, sg_stream_t stream);
int sg_set_schedule(sg_handle* h, const int32_t* tj, int32_t finish);

/* The FluxRegister's step fields (src/hydro/flux_register.hpp:337-349,
 * request_step_field / step_field / end_stage):
 *   S_d <- w1_s S_d + w2_s dt T_d   after every stage s, S_d = 0 at stage 0,
 * in FP64 whatever the storage type, where T_d is the stage's face-flux
 * total of direction d (1 = x1, 2 = x2, 3 = x3): the Riemann flux, the
 * diffusion energy row, the prescribed wall faces (rows IDN and IPR zero on
 * a reflecting wall) and, with the implicit solve, its x1 face transfers
 * ("vic.mass_dry" on row IDN, "vic.momentum_t" on rows IVY and IVZ,
 * src/implicit/implicit_hydro.cpp:625-673).  Each field is
 * (5, nc3, nc2, nc1) FP64 on the device; the face of index f along d is
 * the face below cell f, and the faces of the interior cells (f = ng ..
 * nc_d - ng along d, interior across) are written, the rest never.  Under
 * SG_F32 with a base the normal-momentum row is the total flux (the base
 * face pressure added back in FP64).  s1, s2, s3 may each be null (not
 * requested); a direction the block does not have must be null.  An
 * implicit block with s1 also needs sg_step_scratch_bytes of FP64 scratch
 * (16-byte aligned), where its stage stages T_1 for the solve's posts.
 * The fields are read from the device table, so binding takes effect from
 * the next stage, captured graphs included. */
int sg_step_scratch_bytes(const sg_handle* h, int32_t block, size_t* bytes);
int sg_bind_step_fields(sg_handle* h, int32_t block, double* s1, double* s2,
                        double* s3, void* scratch, size_t bytes);
/* The budget sums (BudgetConsumer::totals and ::boundary,
 * src/diagnostics/budget.cpp:68-155), FP64 on the device, 5 rows per block
 * (mass, momentum 1-3, energy), out[5 b + row]:
 *   totals:   sum over the interior cells of the current state's total u
 *             (the base added back under SG_F32) times the cell volume;
 *   boundary: the outward transfer of the step fields through the block's
 *             boundary faces (reflecting and extrapolation faces; periodic
 *             faces and faces with no boundary function are not boundary),
 *             sum of sign A_f S_d with sign -1 on a lower, +1 on an upper
 *             face; accumulate != 0 adds it to out (the consumer's pending
 *             sum), else stores it. */
int sg_budget_totals(sg_handle* h, double* out_dev, sg_stream_t stream);
int sg_budget_boundary(sg_handle* h, double* out_dev, int32_t accumulate,
                       sg_stream_t stream);
const char* sg_last_error(void);
const char* sg_version(void);

/* ---------------------------------------------------------------------
 * The cubed sphere: shallow water on six gnomonic-equiangle panels of n x n
 * cells (nghost 3, one radial cell), all in one handle.  The state is one
 * buffer (6, 4, n + 6, n + 6) of the dtype per RK buffer: the geopotential
 * Phi, the radial and the two covariant tangential momenta.  Replaces, for
 * this layout, the hydro stage with the gnomonic coordinate
 * (src/coord/gnomonic_equiangle.cpp:357-521, shallow_roe with dir yz,
 * src/riemann/riemann_kernels.h:447-495), the seam flux single-valuing
 * (src/layout/seam_register.cpp:35) and the cross-panel ghost exchange
 * with edge interpolation (src/layout/cubed_sphere_layout.cpp:563-803,
 * src/coord/gnomonic_equiangle.cpp:307-325,536-609) -- the exchange here is
 * one gather over the six panels of this GPU.
 * --------------------------------------------------------------------- */
typedef struct sg_cs_handle sg_cs_handle;
typedef struct sg_cs_desc {
  int32_t n, ng, dtype, nstage;
  double wght[3][3];
  double cfl;
  /* FP64 geometry on the device, one block of nc = n + 6: cos_c, sin_c, vol,
   * x_ov_rD, y_ov_rC, width2, width3 ([nc][nc] each, x3 index slowest), then
   * cos_f2, sin_f2, area2 ([nc][nc + 1] each), cos_f3, sin_f3, area3
   * ([nc + 1][nc] each) */
  const double* geo;
  /* the seam halo: nghost rows of 24 doubles (dst, src0, src1 flat cell
   * indices (panel nc + k) nc + j, the fraction x toward src1, per source
   * its cosine and unit alpha/beta tangents, the ghost's tangents) */
  const double* ghost_tab;
  int32_t nghost;
  /* the seam faces the non-owning panel takes: nseam rows of 18 doubles
   * (dst direction 2|3, dst flat face, src direction, src flat face, sign,
   * the source face cosine, source tangents, destination tangents) */
  const double* seam_tab;
  int32_t nseam;
  /* SG_F32: a reference geopotential Phi0 (> 0): the state's Phi row holds
   * the anomaly Phi - Phi0, and the pressure Phi^2 / 2 is carried as the
   * anomaly Phi0 Phi' + Phi'^2 / 2 (0: totals); SG_F64 ignores it and runs
   * the reference's form on totals */
  double phi_ref;
  /* SG_CS_SHALLOW_ROE (the reference's shallow_roe_impl, dir yz) or
   * SG_CS_HLLC (shallow-water HLLC, Toro 2001: no reference counterpart) */
  int32_t riemann;
  /* the face-state exchange at the seams (HydroImpl::forward's cross-panel
   * sync of hydro_wl / hydro_wr, src/hydro/hydro_forward.cpp:719-757): one
   * row of 16 doubles per seam face, 24 n rows ordered (panel, side L R B
   * T, along): the neighbour panel, its side (0..3 for L R B T) and the
   * face's along index on that side (whose interior-side state the
   * neighbour's own reconstruction gives), a 0, then the 3 x 3 map of
   * contravariant velocities (radial, alpha, beta) from the neighbour's
   * face frame to this panel's at the shared face point (row major), then
   * 3 unused */
  const double* seam_state_tab;
  int32_t nseam_state;
} sg_cs_desc;
enum { SG_CS_SHALLOW_ROE = 0, SG_CS_HLLC = 1 };

int sg_cs_create(const sg_cs_desc* desc, sg_cs_handle** out);
int sg_cs_destroy(sg_cs_handle* h);
/* the face-flux scratch the caller allocates and binds with the buffers */
int sg_cs_scratch_bytes(const sg_cs_handle* h, size_t* bytes);
int sg_cs_bind(sg_cs_handle* h, void* buf0, void* buf1, void* buf2,
               void* scratch, size_t bytes);
int sg_cs_set_current(sg_cs_handle* h, int32_t current);
int sg_cs_rotation(const sg_cs_handle* h, int32_t* cur, int32_t* base);
int sg_cs_set_rotation(sg_cs_handle* h, int32_t cur, int32_t base);
int sg_cs_advance(sg_cs_handle* h, int32_t stage);
/* one RK stage of all six panels, ending with the seam halo fill of the
 * new state; dt_dev points at one device double */
int sg_cs_stage(sg_cs_handle* h, int32_t stage, const double* dt_dev,
                sg_stream_t stream);
/* the seam halo of the current buffer (after loading a state) */
int sg_cs_fill_seams(sg_cs_handle* h, sg_stream_t stream);
/* dt_dev = cfl min over the interior of width / (|v| + sqrt(Phi)) */
int sg_cs_max_dt(sg_cs_handle* h, double* dt_dev, sg_stream_t stream);
/* The FluxRegister's step fields of the six panels (FluxRegister::end_stage
 * after reconcile_panel_seams, src/hydro/flux_register.hpp:241-402,
 * src/layout/seam_register.cpp:35): every stage sets S_d <- w1 S_d +
 * w2 dt T_d on each interior face, FP64, from the stage's final face
 * fluxes (seam faces single-valued); S_d = 0 at stage 0.  s2 and s3 are
 * device doubles laid out (6, 4, nc, nc + 1) and (6, 4, nc + 1, nc),
 * nc = n + 6 (face j of row k at [k][j]); both null unbinds.  An FP32
 * state's normal-momentum rows get the constant phi_ref^2 / 2 of the
 * pressure added back in FP64, so the fields mean what FP64's do. */
int sg_cs_bind_step_fields(sg_cs_handle* h, double* s2, double* s3);
/* The budget's row totals of the current state (BudgetConsumer's totals,
 * src/diagnostics/budget.cpp:68-200): out[4] = sum over the interior cells
 * of u V per variable (Phi, the radial and the two tangential momenta),
 * FP64, an FP32 state's Phi with phi_ref added back; one fixed reduction
 * order, so the sums repeat exactly.  out is device memory. */
int sg_cs_budget_totals(sg_cs_handle* h, double* out, sg_stream_t stream);

/* Allocation-free time step.  No counterpart in the reference: it is for
 * callers that may not allocate device memory at all (a host that hands in
 * views of its own pre-allocated arena, a serving loop held to a fixed HBM
 * budget).  It computes what sg_max_dt computes for up to
 * SG_NOALLOC_MAX_BLOCKS blocks described by value, with its reduction scratch
 * in a file-scope device array (SG_NOALLOC_MAX_BLOCKS x 16 bytes per GPU);
 * more blocks are refused with an error.  The scratch is cleared by each
 * call's first kernel; calls that overlap on the GPU race on it, so the
 * caller serialises them.  The first call on each device looks the array's
 * address up and must come before any stream capture on that device. */
#define SG_NOALLOC_MAX_BLOCKS 64
typedef struct sg_dt_block {
  const void* u;      /* current conserved state, (5, nc3, nc2, nc1) */
  int32_t nc1, nc2, nc3, ng;
  double dx1, dx2, dx3, gammad;
  double dt_src;      /* source-term bound, e.g. the diffusion limit
                         dx_min^2 / (2 ndim nu); 0, negative, NaN or +inf:
                         no bound */
  int32_t implicit;   /* the deck's implicit-scheme number (0: none); bit 0
                         (the vertical solve, as in scheme 9) drops the x1
                         acoustic bound for blocks with more than one column,
                         as sg_max_dt does */
  const double* base; /* FP32 blocks under gravity: the FP64 hydrostatic base
                         (rho_b | p_b | ..., nc1 each) that the state's
                         anomalies are about, as in sg_block_desc.base;
                         NULL otherwise (refused for FP64 blocks) */
} sg_dt_block;
int sg_max_dt_noalloc(const sg_dt_block* blocks, int32_t nblock, int32_t dtype,
                      double cfl, const int32_t* redo_dev, double* dt_out_dev,
                      sg_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif
