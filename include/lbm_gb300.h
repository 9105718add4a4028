/*
 * lbm_gb300 -- C-ABI of the GB300 D2Q9 TRT lattice update.
 *
 * Every entry point takes plain device pointers, sizes and a CUDA stream
 * (cudaStream_t passed as void*; NULL = legacy default stream), returns an
 * int status (LBM_OK = 0) and never synchronises the device unless stated.
 * Arrays use the reference layout of jviquerat/lbm: distributions
 * g[q][i][j] (9 x nx x ny, j fastest), rho[i][j], u[d][i][j], BC vectors
 * u_left/u_right[d][j], u_top/u_bot[d][i], rho_right[j]
 * (lbm/src/core/lattice.py:155-174).  Link lists are int32 triples (i, j, q)
 * in the order produced by lattice.add_obstacle (lattice.py:328-344); negative
 * i/j wrap like NumPy indices.  On error, lbm_last_error_string() describes
 * the failure of the calling thread's last call.
 *
 * The library owns no caller memory.  Scratch used by the fused engine lives
 * in buffers the caller passes in lbm_problem (see lbm_problem_scratch_bytes).
 */
#ifndef LBM_GB300_H
#define LBM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes --------------------------------------------------------- */
#define LBM_OK 0
#define LBM_ERR_ARG 1          /* bad size, pointer, enum or alignment        */
#define LBM_ERR_CUDA 2         /* a CUDA runtime call failed                   */
#define LBM_ERR_NONFINITE 3    /* NaN/Inf detected in the distributions        */
#define LBM_ERR_UNSUPPORTED 5  /* valid request outside what this build does   */

/* ---- enums ---------------------------------------------------------------- */
/* Storage/compute forms of the fused engine. */
#define LBM_PREC_F64 0   /* FP64 storage, FP64 arithmetic                           */
#define LBM_PREC_F32 1   /* FP32 storage of f - w*rho0, FP32 arithmetic              */
#define LBM_PREC_F16S 2  /* FP16 storage of f - w*rho0, FP32 arithmetic              */
#define LBM_PREC_BF16S 3 /* BF16 storage of f - w*rho0, FP32 arithmetic              */
/* 64-bit fixed-point storage of f (Q3.60: f * 2^60 as int64, |f| < 8;
 * resolution 2^-60, sums exact) with the bulk collision in integer arithmetic
 * and FP64 at wall and link cells.  Needs rho0 in [3/4, 3/2] and om_p, om_m in
 * [1/1024, 1.999]; a cell whose rho leaves (9/16, 15/4) or whose |j| or |u|
 * leaves the range is reported like a non-finite value and stored as
 * INT64_MIN, which unpacks to NaN.  No counterpart in the reference (its FP64
 * path computes in FP64). */
#define LBM_PREC_Q60 4
/* FP16 / BF16 storage of f - w*rho0 as LBM_PREC_F16S / LBM_PREC_BF16S, with
 * stochastic rounding of every update (deterministic: the random bits hash
 * the cell and the iteration).  No counterpart in the reference. */
#define LBM_PREC_F16SR 5
#define LBM_PREC_BF16SR 6

/* Wall operations (Zou-He), lbm/src/core/nb.py:121-247. */
#define LBM_WALL_LEFT_VELOCITY 0
#define LBM_WALL_RIGHT_VELOCITY 1
#define LBM_WALL_RIGHT_PRESSURE 2
#define LBM_WALL_TOP_VELOCITY 3
#define LBM_WALL_BOTTOM_VELOCITY 4

/* Corners, lbm/src/core/nb.py:250-344. */
#define LBM_CORNER_BOTTOM_LEFT 0
#define LBM_CORNER_TOP_LEFT 1
#define LBM_CORNER_TOP_RIGHT 2
#define LBM_CORNER_BOTTOM_RIGHT 3

/* Fused-step modes. */
#define LBM_MODE_COLLIDE_FROM_G 0  /* macro+equilibrium+collide of g (first step)   */
#define LBM_MODE_STEP 1            /* stream+BC of f_in, then macro+eq+collide      */
#define LBM_MODE_FINISH 2          /* stream+BC of f_in into g_out, no collision    */

/* 2 (lbm_batch_config.bulk_tma added). */
int lbm_abi_version(void);
const char* lbm_last_error_string(void);
/* Number of SMs and name of the current device (for logs/tuning). */
int lbm_device_info(int* sm_count, char* name, int name_len);

/* ---- kernel-level entry points (FP64, one per reference function) ---------- */
/* lattice.macro, lbm/src/core/lattice.py:178-189. */
int lbm_macro_f64(const double* g, double* rho, double* u, int nx, int ny, void* stream);
/* nb_equilibrium, lbm/src/core/nb.py:7-17. */
int lbm_equilibrium_f64(const double* u, const double* rho, double* g_eq, int nx, int ny,
                        void* stream);
/* nb_col_str, lbm/src/core/nb.py:21-45 (collide into g_up, stream into g in place). */
int lbm_collision_stream_f64(double* g, const double* g_eq, double* g_up, double om_p,
                             double om_m, int nx, int ny, void* stream);
/* nb_bounce_back_obstacle, lbm/src/core/nb.py:77-117.  links: n x 3 int32
 * (i, j, q); p: n IBB distances (ignored when ibb == 0).  Links are applied in
 * order (the last link that writes a population wins, as in the serial
 * reference loop). */
int lbm_bounce_back_f64(int ibb, const int32_t* links, int64_t n, const double* p,
                        const double* g_up, double* g, int nx, int ny, void* stream);
/* nb_drag_lift, lbm/src/core/nb.py:49-73.  Writes the raw momentum-exchange
 * sums out[0] = fx, out[1] = fy (device pointer); the caller normalises
 * C = -2 F / (R_ref L_ref U_ref^2).  Deterministic (fixed-order FP64 tree).
 * scratch: device buffer of at least lbm_drag_lift_scratch_bytes(n) bytes. */
size_t lbm_drag_lift_scratch_bytes(int64_t n);
int lbm_drag_lift_f64(const int32_t* links, int64_t n, const double* g_up, const double* g,
                      int nx, int ny, double* out, void* scratch, void* stream);
/* Same result as lbm_drag_lift_f64, for callers that cannot provide device
 * memory (their device memory belongs to another allocator, or they must not
 * allocate after start-up).  No counterpart in the reference.  The block
 * partials live in a fixed 64 KiB array inside the library's device image,
 * held by every GPU that loads the library until exit; at most
 * LBM_DRAG_NOALLOC_MAX_LINKS links per call (more: LBM_ERR_ARG).  The first
 * call in each CUDA context (the device's primary context, or a context the
 * host made current) looks up the array's device address in that context;
 * make that first call before any stream capture.  All calls share the
 * array: calls that overlap on the GPU (different streams, or different host
 * threads) race and must be serialised by the caller.  Allocates nothing. */
#define LBM_DRAG_NOALLOC_MAX_LINKS 1048576
int lbm_drag_lift_f64_noalloc(const int32_t* links, int64_t n, const double* g_up,
                              const double* g, int nx, int ny, double* out, void* stream);
/* buff.mv_avg (lbm/src/utils/buff.py:35-77) after each of n adds, on the
 * device.  hist: [4][cap] doubles, the histories buff, avg1, avg2, avg3 of
 * the reference (each starting with two zeros; add m is stored at index
 * m + 1).  The caller has stored adds k0 + 1 .. k0 + n in hist[0] and has
 * made k0 adds before (k0 + n + 2 <= cap).  For each add t: obs[t] (the
 * returned average), growth[t] and cv[t] (the obs_cv flag after it); the
 * averages are appended to avg1..avg3.  state: [2] ints, the convergence
 * counter and flag, carried between calls (zero at the start).  Sums are in
 * NumPy's pairwise order, so every value equals the reference's bit for bit. */
int lbm_mv_avg_chunk(double* hist, int64_t cap, int64_t k0, int32_t n, double dt, double cv_ct,
                     int32_t cv_nb, int32_t* state, double* obs, double* growth, int32_t* cv,
                     void* stream);
/* Zou-He walls, lbm/src/core/nb.py:121-247.  wall: LBM_WALL_*; vec is the
 * wall's (2 x len) velocity vector; rho_right only for RIGHT_PRESSURE. */
int lbm_zou_he_f64(int wall, double* u, double* rho, double* g, const double* vec,
                   const double* rho_right, int nx, int ny, void* stream);
/* Zou-He corners, lbm/src/core/nb.py:250-344.  corner: LBM_CORNER_*. */
int lbm_zou_he_corner_f64(int corner, double* u, double* rho, double* g, int nx, int ny,
                          void* stream);

/* ---- fused engine ---------------------------------------------------------- */
/*
 * One call advances the lattice by n_steps reference iterations
 * (lbm/src/core/run.py:24-54: macro, equilibrium, collide-stream, set_bc,
 * observables) with the state held as post-collision populations (pull
 * scheme).  Step k of the call reads f[(parity + k) & 1] and writes
 * f[(parity + k + 1) & 1].
 *
 * Special cells = every wall cell plus every fluid cell that owns an obstacle
 * link; they are re-done by a second kernel that applies, in reference order,
 * the links (IBB/BB), the wall operations and the corners.  The host supplies
 * the special-cell table (linear cell indices i*ny + j, each once; the
 * Python host sorts them, which keeps a warp's cells close together), CSR
 * offsets into the link arrays and the special index of each corner's
 * x-neighbour.
 */
typedef struct lbm_problem {
  int32_t nx, ny;
  int32_t precision;        /* LBM_PREC_*                                        */
  int32_t ibb;              /* 1: interpolated bounce-back, 0: halfway BB       */
  double om_p, om_m;        /* TRT relaxation rates (lattice.py:127-131)        */
  double rho0;              /* storage shift for the shifted forms              */

  /* BC program: wall operations in application order, then corners. */
  int32_t n_wall_ops;
  int32_t wall_ops[5];
  int32_t n_corner_ops;
  int32_t corner_ops[4];
  int32_t corner_nb_special[4];  /* special index of each corner's x-neighbour   */
  int32_t corner_special[4];     /* special index of each corner cell            */

  /* Distributions (storage type per precision), 9 * nx * ny elements each. */
  void* f[2];

  /* BC vectors at iteration it: value = base + scale[it - scale_it0] * vec.
   * Packed layout (doubles): u_left[2*ny] | u_right[2*ny] | u_top[2*nx] |
   * u_bot[2*nx] | rho_right[ny].  vec may be NULL (constant BCs). */
  const double* bc_base;
  const double* bc_vec;
  const double* bc_scale;   /* one scalar per iteration                         */
  int64_t bc_scale_it0;
  int64_t bc_scale_len;

  /* Special cells and links. */
  int32_t n_special;
  const int32_t* special_cell;        /* [n_special] linear index i*ny + j       */
  const int32_t* special_link_start;  /* [n_special + 1]                         */
  int32_t n_links;
  const int32_t* link_cell;    /* [n_links] linear index of the (wrapped) cell   */
  const int32_t* link_q;       /* [n_links] link direction (toward the solid)    */
  const int32_t* link_nb1;     /* [n_links] linear index of x + c_qb (wrapped)   */
  const int32_t* link_nb2;     /* [n_links] linear index of x + 2 c_qb (wrapped) */
  const double* link_p;        /* [n_links] IBB distance                         */
  const int32_t* special_link_ids; /* [sum of CSR] link ids per special cell     */
  int32_t n_obstacles;
  const int32_t* obstacle_link_start; /* [n_obstacles + 1] link id ranges        */

  /* Scratch (caller-allocated, lbm_problem_scratch_bytes). */
  void* scratch;
  size_t scratch_bytes;

  /* Optional outputs. */
  double* drag_hist;        /* [drag_cap][n_obstacles][2] raw (fx, fy)          */
  int64_t drag_cap;         /* ring size in iterations                          */
  double* rho_out;          /* [nx*ny]   macro rho (see flags)                  */
  double* u_out;            /* [2*nx*ny] macro u                                */
  double* g_out;            /* [9*nx*ny] post-BC g (FINISH / COLLIDE_FROM_G in) */
  uint32_t* status_flags;   /* [1] device word; bit 0 = non-finite detected,
                             * bit 3 = a bulk-kernel pipeline wait timed out */

  /* Row pitch of f[0]/f[1] in elements (0 = ny).  The distributions are
   * stored as [q][i][j] with rows of row_pitch >= ny elements; padding a
   * row to a multiple of 16 bytes lets the bulk kernel use 16-byte vectors
   * for any ny.  link_cell/link_nb1/link_nb2 are indices i * row_pitch + j in
   * that layout; special_cell, g_out, rho_out and u_out use i * ny + j. */
  int32_t row_pitch;

  /* Optional IBB coefficients, [3][n_links] doubles (NULL: computed from
   * link_p in the kernel).  For link k with p = link_p[k], pp = 2p:
   *   p <  1/2: c1 = p(pp+1), c2 = (1+pp)(1-pp), c3 = p(1-pp),
   *             g[qb] = c1 g_up[q,x] + c2 g_up[q,x+c_qb] - c3 g_up[q,x+2c_qb]
   *   p >= 1/2: c1 = 1/(p(pp+1)), c2 = (pp-1)/p, c3 = (1-pp)/(1+pp),
   *             g[qb] = c1 g_up[q,x] + c2 g_up[qb,x] + c3 g_up[qb,x+c_qb]
   * (the factors of nb.py:98-104 in the reference's evaluation order). */
  const double* link_coef;
} lbm_problem;

/* Flags for lbm_advance. */
#define LBM_FLAG_MACRO_LAST 1u   /* write rho_out/u_out on the last step's macro */
#define LBM_FLAG_CHECK_FINITE 2u /* set status bit 0 on NaN/Inf (cheap)          */
#define LBM_FLAG_WALL_MACRO 4u   /* FINISH: write rho/u written by wall ops      */
/* 16-bit forms: step with the register-pipelined bulk kernel (16-byte global
 * loads, warp-shuffle halos) instead of the default TMA-staged one
 * (cp.async.bulk into shared-memory stages); both give the same bits. */
#define LBM_FLAG_BULK_REGISTERS 8u
/* Test of the failure path only: the TMA-staged kernel's producer withholds
 * each block's first tile, so that the consumers' bounded wait (0.5 s) runs
 * out; the kernel then sets status bit 3 and returns, and the context stays
 * usable.  No result of such a step is meaningful. */
#define LBM_FLAG_TEST_STALL 16u

size_t lbm_problem_scratch_bytes(const lbm_problem* p);
/* Advance n_steps iterations: each is one pass of the reference's run() loop
 * body (run.py:24-54: lattice.macro, equilibrium, collision_stream, then the
 * app's set_bc -- bounce_back_obstacle, zou_he_* walls and corners -- and
 * the drag_lift observable; nb.py:7-344), fused into three kernels.  it0 is
 * the reference iteration number of the
 * first collision performed by this call (its BCs use iteration it0 - 1 and
 * its drag output lands in drag_hist[(it0 - 1) % drag_cap]).  parity selects
 * which of f[0]/f[1] holds the input.  mode: LBM_MODE_*.  For
 * LBM_MODE_COLLIDE_FROM_G the input is g_out (the post-BC g) and n_steps must
 * be 1; LBM_MODE_FINISH must have n_steps == 1 and writes g_out. */
int lbm_advance(const lbm_problem* p, int mode, int64_t it0, int n_steps, int parity,
                uint32_t flags, void* stream);
/* Same as lbm_advance(mode = LBM_MODE_STEP) but launched as a cached CUDA
 * graph of n_steps iterations (captured on first use per (problem, n_steps,
 * parity); a graph is re-captured when the problem descriptor changes). */
int lbm_advance_graph(const lbm_problem* p, int64_t it0, int n_steps, int parity,
                      uint32_t flags, void* stream);
/* Per-kernel timing (measurement helper, no counterpart in the reference):
 * runs n_steps LBM_MODE_STEP iterations (no graph) with CUDA events around
 * each kernel and synchronises.  ms_out[0..2] = average
 * milliseconds of the bulk, special-cell and drag kernels per step,
 * ms_out[3] = kernels launched per step. */
int lbm_profile_steps(const lbm_problem* p, int64_t it0, int n_steps, int parity, uint32_t flags,
                      double* ms_out, void* stream);
/* FP64 pipe throughput of the current device: independent DFMA chains timed
 * with CUDA events (the second roofline of the FP64 form).  Synchronises.
 * scratch: device buffer of lbm_measure_dfma_scratch_bytes() bytes.  No
 * counterpart in the reference (measurement helper). */
size_t lbm_measure_dfma_scratch_bytes(void);
int lbm_measure_dfma_rate(double* ginstr_per_s, void* scratch, size_t scratch_bytes,
                          void* stream);
/* Drop every cached graph (call before freeing buffers a graph refers to). */
int lbm_graph_cache_clear(void);

/* ---- batched lattices ------------------------------------------------------ */
/*
 * Many independent lattices of one storage form advanced together: per
 * iteration one persistent bulk kernel over a work queue of tiles of every
 * lattice, one persistent special-cell kernel, one drag kernel.  Each
 * lattice keeps its own buffers, tables and scratch (its lbm_problem); the
 * batch owns the tile tables and a shared iteration counter (workspace from
 * lbm_batch_create, released by lbm_batch_destroy).  A lattice gives the same
 * bits in a batch as alone.  No counterpart in the reference, which runs one
 * case per process.
 */
typedef struct lbm_batch lbm_batch;
typedef struct lbm_batch_config {
  int32_t bulk_threads;          /* threads per bulk block = groups per tile (x32) */
  int32_t bulk_blocks_per_sm;    /* persistent bulk grid = SMs x this              */
  int32_t special_blocks_per_sm; /* persistent special-cell grid = SMs x this      */
  int32_t scalar_tile_cells;     /* cells per tile of lattices without 16-byte rows */
  int32_t persistent;            /* 1: persistent blocks pull tiles from an atomic
                                    queue; 0: one block per tile                  */
  int32_t vec_bytes;             /* 8 or 16: bytes per vector access of the bulk
                                    kernel (cells per thread = this / element)    */
  int32_t tile_rounds;           /* 1..64: a vector bulk tile is this many block-
                                    widths of groups (a thread loops over them)   */
  int32_t bulk_tma;              /* 1 (16-bit forms only): the bulk phase runs the
                                    TMA-staged persistent kernel, on tiles of its
                                    own size; 2: the same with half the warps per
                                    block (two blocks per SM, room for another
                                    batch's kernels beside them); bulk_threads,
                                    bulk_blocks_per_sm, vec_bytes and tile_rounds
                                    then do not apply                          */
} lbm_batch_config;
int lbm_batch_create(lbm_batch** out, const lbm_problem* cases, int32_t n_cases,
                     const lbm_batch_config* cfg);
int lbm_batch_destroy(lbm_batch* b);
/* out6: lattices, bulk tiles, special tiles, drag items, SMs, kernels per step. */
int lbm_batch_info(const lbm_batch* b, int64_t* out6);
/* Advance every lattice by n_steps iterations (it0: first collided
 * iteration; parity: which of each lattice's f[0]/f[1] holds the input). */
int lbm_batch_advance(lbm_batch* b, int64_t it0, int n_steps, int parity, void* stream);
/* Same, as a CUDA graph of n_steps iterations cached per (n_steps, parity). */
int lbm_batch_advance_graph(lbm_batch* b, int64_t it0, int n_steps, int parity, void* stream);

/* ---- adjoint (FP64) ---------------------------------------------------------- */
/*
 * Discrete adjoint of one fused step, for the gradient of a drag/lift
 * objective J = sum over iterations it in [obj_it_first, obj_it_last] of
 * sum_o (obj_w[o] fx_o(it) + obj_w[n_obstacles + o] fy_o(it)), fx/fy the raw
 * momentum-exchange sums of nb_drag_lift (nb.py:49-73), with respect to the
 * TRT rate om_p (om_m = 1 / (lambda / (1/om_p - 1/2) + 1/2), lambda = 1/4,
 * lattice.py:127-131) and to every entry of the packed BC vectors.  Needs an
 * FP64 problem whose four walls all carry a Zou-He operation and whose four
 * corners are applied.  No counterpart in the reference (it has no gradient).
 */
typedef struct lbm_adjoint {
  int64_t obj_it_first, obj_it_last;
  const double* obj_w;          /* [2 * n_obstacles] weights of fx, then fy      */
  const uint8_t* is_special;    /* [nx*ny] 1 for the special cells               */
  double* adj_pulled;           /* [9*nx*ny] scratch                             */
  double* link_adj;             /* [3*n_links] scratch                           */
  double* corner_seed;          /* [12] scratch                                  */
  double* grad_bc_base;         /* [4ny+4nx+ny] += dJ/d BC value                  */
  double* grad_bc_vec;          /* [4ny+4nx+ny] += scale(it) dJ/d BC value        */
  double* grad_omega;           /* [grad_omega_len] += per-block parts of dJ/d om_p */
  int32_t grad_omega_len;
} lbm_adjoint;
size_t lbm_adjoint_omega_slots(const lbm_problem* p);
/* Step `it` (the forward step that reads x_prev = g_up(it-1), applies the
 * BCs and drag of iteration it-1 and collides iteration it): lam_out =
 * dJ/dx_prev given lam_in = dJ/d g_up(it).  FP64 arrays, reference layout. */
int lbm_adjoint_step(const lbm_problem* p, const lbm_adjoint* adj, int64_t it,
                     const double* x_prev, const double* lam_in, double* lam_out, void* stream);
/* Recompute one checkpoint segment: with states[0] (FP64, reference layout)
 * = x(it_first), write x(it_first + m) into states + m * stride for
 * m = 1 .. n_steps - 1 (forward steps without drag history).  stride >=
 * 9 * nx * ny elements.  Uses the problem's scratch: one recompute at a time
 * per problem; it may run on another stream than lbm_adjoint_sweep, which
 * does not touch the scratch.  No counterpart in the reference. */
int lbm_adjoint_recompute(const lbm_problem* p, int64_t it_first, int n_steps, double* states,
                          int64_t stride, void* stream);
/* Reverse sweep over a recomputed segment: lbm_adjoint_step for it =
 * it_first + n_steps down to it_first + 1 with x_prev = states + (it - 1 -
 * it_first) * stride and lambda ping-ponging between lam0/lam1: lam[parity]
 * holds dJ/dx(it_first + n_steps) on entry and lam[parity ^ (n_steps & 1)]
 * holds dJ/dx(it_first) on return.  No counterpart in the reference. */
int lbm_adjoint_sweep(const lbm_problem* p, const lbm_adjoint* adj, int64_t it_first,
                      int n_steps, const double* states, int64_t stride, double* lam0,
                      double* lam1, int parity, void* stream);
/* First collision (from the initial g0): adds its om_p term, lam_out = dJ/dg0. */
int lbm_adjoint_initial(const lbm_problem* p, const lbm_adjoint* adj, const double* g0,
                        const double* lam_in, double* lam_out, void* stream);

/* Convert distributions between the FP64 reference layout (lattice.g,
 * float64 [9][nx][ny], lattice.py:155-157) and a storage form (shifted forms
 * store kScale (f - w_q * rho0), kScale = 2^10 for FP16, 1 otherwise).  g has rows of ny, f rows of
 * row_pitch (0 = ny); padding elements of f are left untouched. */
int lbm_pack_f64(int precision, const double* g, void* f, int nx, int ny, int row_pitch, double rho0,
                 void* stream);
int lbm_unpack_f64(int precision, const void* f, double* g, int nx, int ny, int row_pitch,
                   double rho0, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* LBM_GB300_H */
