// Fused D2Q9 TRT lattice update (pull scheme), all storage forms.
//
// One reference iteration (lbm/src/core/run.py:24-54) is split at the
// collision: the state kept in HBM is the post-collision population g_up of
// the previous iteration.  Iteration `it` then reads g_up(it-1), streams it
// (pull), applies set_bc(it-1) and the drag/lift of it-1, and takes macro,
// equilibrium and collision of g(it) to write g_up(it).  Three kernels do
// this (in enqueues of several steps the drag kernel of step k runs on a
// second stream beside the bulk kernel of step k + 1):
//
//   k_bulk    every cell not on a wall: pull 9 values, collide, write 9
//             (k_bulk_q60 for the plain form, the TMA-staged k_bulk_tma or
//             the register-pipelined k_bulk_vec for the 16-bit forms).
//   k_special every wall cell and every cell owning an obstacle link (a short
//             sorted list): pull, links (IBB/BB), Zou-He walls in the app's
//             order, corners, per-link drag terms, collide.  It overwrites
//             what k_bulk wrote at link cells.
//   k_drag    per obstacle (one block each), a fixed-order FP64 sum of the
//             per-link terms.
//
// Edge populations without an in-domain source keep the previous post-BC
// value (nb.py:38-45 streams interior slices only); k_special keeps those
// values, and the previous macro rho/u of every special cell that corners
// read (nb.py:254-257), in ping-pong scratch buffers.
#include "lbm_fused.cuh"
#include "lbm_tma.cuh"

#include <math.h>
#include <string.h>

namespace lbm {

template <class St, int MODE>
__global__ void __launch_bounds__(256) k_bulk(FusedArgs a) {
  const long long cell = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell < a.Ns) bulk_cell<St, MODE>(a, cell);
  if (a.advance_at == 0) advance_counter(a.it_dev, a.step_done);
}

// Resident 128-thread blocks per SM the vectorised bulk kernel is compiled for.
#ifndef LBM_VEC_MIN_BLOCKS
#define LBM_VEC_MIN_BLOCKS 1
#endif
template <class St, int V>
__global__ void __launch_bounds__(128, LBM_VEC_MIN_BLOCKS) k_bulk_vec(FusedArgs a) {
  const long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  bulk_group_vec<St, V>(a, gi);
  if (a.advance_at == 0) advance_counter(a.it_dev, a.step_done);
}

// TMA-staged bulk kernel of the 16-bit forms (lbm_tma.cuh): one lattice,
// tiles of consecutive cells over the interior columns.
template <class St, class Sh>
__global__ void __launch_bounds__(Sh::kThreads, 1) k_bulk_tma(FusedArgs a, int n_tiles) {
  const LatticeTiles<Sh> src{a, a.sy, (long long)(a.nx - 1) * a.sy};
  bulk_tma_body<St, Sh>(src, n_tiles, a.status);
  if (a.advance_at == 0) advance_counter(a.it_dev, a.step_done);
}

// Q3.60 bulk kernel: block b covers column i = b / jb, rows
// j = (b mod jb) * 256 + threadIdx.x (block-uniform index arithmetic).
// Five resident 256-thread blocks per SM (48 registers, a few spilled
// values): measured 6 % faster than four (64 registers) and than six on the
// GB300, where the kernel is co-limited by HBM and the IMAD.WIDE pipe.
#ifndef LBM_Q60_MIN_BLOCKS
#define LBM_Q60_MIN_BLOCKS 5
#endif
__global__ void __launch_bounds__(256, LBM_Q60_MIN_BLOCKS) k_bulk_q60(FusedArgs a, int jb) {
  const int i = blockIdx.x / jb;
  const int j = (blockIdx.x - i * jb) * 256 + threadIdx.x;
  bulk_q60_ij(a, i, j);
  if (a.advance_at == 0) advance_counter(a.it_dev, a.step_done);
}

template <class St, int MODE>
__global__ void __launch_bounds__(128, LBM_SPECIAL_MIN_BLOCKS) k_special(FusedArgs a) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < a.n_special) special_cell<St, MODE>(a, s);
  if (a.advance_at == 1) advance_counter(a.it_dev, a.step_done);
}

// One block of 256 threads per obstacle.
__global__ void __launch_bounds__(256) k_drag(FusedArgs a) {
  if ((int)blockIdx.x < a.n_obs) drag_obstacle(a, blockIdx.x);
  if (a.advance_at == 2) advance_counter(a.it_dev, a.step_done);
}

__global__ void k_set_it(long long* it_dev, unsigned* done, long long value) {
  *it_dev = value;
  *done = 0;
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
template <class St, class Sh>
static int tma_blocks_per_sm() {
  static int per_sm[64] = {};
  return tma_prepare((const void*)k_bulk_tma<St, Sh>, Sh::kThreads, Sh::kSmem, per_sm);
}

// lane (optional): the drag kernel of a step goes to lane->sd beside the next
// step's bulk kernel; *drag_pending tells whether a drag kernel of this
// enqueue is on lane->sd.
template <class St, int MODE>
static void launch_mode(const FusedArgs& a0, cudaStream_t st, cudaEvent_t* ev, DragLane* lane,
                        bool* drag_pending) {
  FusedArgs a = a0;
  const bool with_special = a.n_special > 0;
  const bool with_drag = MODE != LBM_MODE_COLLIDE_FROM_G && a.drag_hist && a.n_obs > 0 && a.n_links > 0;
  const bool side = lane && with_drag && with_special && MODE == LBM_MODE_STEP && !ev;
  const int tb = 256;
  const long long nb = (a.Ns + tb - 1) / tb;
  // 16-bit storage forms: the TMA-staged kernel, or with
  // LBM_FLAG_BULK_REGISTERS the register-pipelined one with 16-byte vectors
  // (8 cells per thread; 4-cell vectors: 108-118 vs 103-112 us).  FP32 takes
  // the one-cell-per-thread kernel, measured faster on 8192x2048 (176 vs
  // 190 us per bulk launch with 4-cell vectors).
  constexpr int kVec = 16 / (int)sizeof(typename St::S);
  constexpr bool kUseVec = MODE == LBM_MODE_STEP && St::kShift && sizeof(typename St::S) == 2;
  a.advance_at = with_drag && !side ? 2 : (with_special ? 1 : 0);
  a.drag_it_offset = side ? 2 : 1;
  if (ev) cudaEventRecord(ev[0], st);
  if (St::kFixed && MODE == LBM_MODE_STEP) {
    const int jb = (a.ny + 255) / 256;
    k_bulk_q60<<<(unsigned)((long long)a.nx * jb), 256, 0, st>>>(a, jb);
  } else {
    bool launched = false;
    if constexpr (kUseVec) {
      if (a.sy % kVec == 0 && a.bulk_tma && a.nx > 2) {
        using Sh = typename TmaShapeOf<St>::type;
        const long long cells = (long long)(a.nx - 2) * a.sy;
        const int n_tiles = (int)((cells + Sh::kCells - 1) / Sh::kCells);
        const int slots = tma_blocks_per_sm<St, Sh>() * device_sm_count();
        k_bulk_tma<St, Sh><<<n_tiles < slots ? n_tiles : slots, Sh::kThreads, Sh::kSmem, st>>>(
            a, n_tiles);
        launched = true;
      } else if (a.sy % kVec == 0) {
        const long long groups = (long long)a.nx * (a.sy / kVec);
        k_bulk_vec<St, kVec><<<(unsigned)((groups + 127) / 128), 128, 0, st>>>(a);
        launched = true;
      }
    }
    if (!launched) k_bulk<St, MODE><<<(unsigned)nb, tb, 0, st>>>(a);
  }
  if (ev) cudaEventRecord(ev[1], st);
  if (with_special) {
    const int ts = 128;
    // the previous step's drag kernel reads the per-link terms written here
    if (side && *drag_pending) cudaStreamWaitEvent(st, lane->ev_drag, 0);
    k_special<St, MODE><<<(a.n_special + ts - 1) / ts, ts, 0, st>>>(a);
  }
  if (ev) cudaEventRecord(ev[2], st);
  if (with_drag && side) {
    cudaEventRecord(lane->ev_special, st);
    cudaStreamWaitEvent(lane->sd, lane->ev_special, 0);
    k_drag<<<a.n_obs, 256, 0, lane->sd>>>(a);
    cudaEventRecord(lane->ev_drag, lane->sd);
    *drag_pending = true;
  } else if (with_drag) {
    k_drag<<<a.n_obs, 256, 0, st>>>(a);
  }
  if (ev) cudaEventRecord(ev[3], st);
}

template <class St>
static void launch_store(const FusedArgs& a, int mode, cudaStream_t st, cudaEvent_t* ev,
                         DragLane* lane, bool* drag_pending) {
  switch (mode) {
    case LBM_MODE_COLLIDE_FROM_G:
      launch_mode<St, LBM_MODE_COLLIDE_FROM_G>(a, st, ev, lane, drag_pending);
      break;
    case LBM_MODE_STEP: launch_mode<St, LBM_MODE_STEP>(a, st, ev, lane, drag_pending); break;
    default: launch_mode<St, LBM_MODE_FINISH>(a, st, ev, lane, drag_pending); break;
  }
}

int fused_kernels_per_step(const lbm_problem* p, int mode) {
  int n = 1 + (p->n_special > 0 ? 1 : 0);
  if (mode != LBM_MODE_COLLIDE_FROM_G && p->drag_hist && p->n_obstacles > 0 && p->n_links > 0) n++;
  return n;
}

// Scratch layout: iteration counter and step-done count (256 B) |
// stale[2][9][n_special] | mac[2][3][n_special] | link_force[2][n_links]
// (doubles).
size_t fused_scratch_bytes(const lbm_problem* p) {
  size_t ns = (size_t)(p->n_special > 0 ? p->n_special : 0);
  size_t nl = (size_t)(p->n_links > 0 ? p->n_links : 0);
  return 256 + sizeof(double) * (2 * 9 * ns + 2 * 3 * ns + 2 * nl) + 256;
}

// Integer coefficients of the Q3.60 collision, rounded from the FP64 rates
// in extended precision (om_p, om_m in [1/1024, 1.999], checked by
// problem_check, keep every split half inside 32 bits).
CoefQ60 make_coef_q60(double om_p, double om_m) {
  const long double op = om_p, om = om_m;
  auto fix = [](long double v, int e) { return split((long long)llroundl(ldexpl(v, e))); };
  CoefQ60 k;
  k.alpha = fix((1.0L - op) / 2.0L, 64);
  k.beta = fix((1.0L - om) / 2.0L, 64);
  k.a0 = fix(1.0L - op, 63);
  k.wp = fix(op / 9.0L, 64);
  k.wm = fix(om / 3.0L, 63);
  k.c1 = fix(op / 2.0L, 63);
  k.third = fix(1.0L / 3.0L, 64);
  return k;
}

FusedArgs make_args(const lbm_problem* p, int mode, unsigned flags) {
  FusedArgs a;
  memset(&a, 0, sizeof(a));
  a.nx = p->nx;
  a.ny = p->ny;
  a.N = (long long)p->nx * p->ny;
  a.sy = p->row_pitch > 0 ? p->row_pitch : p->ny;
  a.Ns = (long long)p->nx * a.sy;
  const bool unshifted = p->precision == LBM_PREC_F64 || p->precision == LBM_PREC_Q60;
  const double rho0 = unshifted ? 0.0 : p->rho0;
  a.kd = make_coef<double>(p->om_p, p->om_m, rho0);
  a.kf = make_coef<float>(p->om_p, p->om_m, rho0);
  if (p->precision == LBM_PREC_Q60) a.kq = make_coef_q60(p->om_p, p->om_m);
  a.n_wall_ops = p->n_wall_ops;
  for (int w = 0; w < 5; ++w) a.wall_ops[w] = p->wall_ops[w];
  a.n_corner_ops = p->n_corner_ops;
  for (int w = 0; w < 4; ++w) {
    a.corner_ops[w] = p->corner_ops[w];
    a.corner_nb_special[w] = p->corner_nb_special[w];
    a.corner_special[w] = p->corner_special[w];
  }
  a.ibb = p->ibb;
  a.bc_base = p->bc_base;
  a.bc_vec = p->bc_vec;
  a.bc_scale = p->bc_scale;
  a.bc_scale_it0 = p->bc_scale_it0;
  a.bc_scale_len = p->bc_scale_len;
  a.n_special = p->n_special;
  a.special_cell = p->special_cell;
  a.special_link_start = p->special_link_start;
  a.special_link_ids = p->special_link_ids;
  a.link_cell = p->link_cell;
  a.link_q = p->link_q;
  a.link_nb1 = p->link_nb1;
  a.link_nb2 = p->link_nb2;
  a.link_p = p->link_p;
  a.link_coef = p->link_coef;
  a.n_links = p->n_links;
  char* base = (char*)(((uintptr_t)p->scratch + 255) & ~(uintptr_t)255);
  a.it_dev = (long long*)base;
  a.step_done = (unsigned*)(base + 8);
  double* sc = (double*)(base + 256);
  const size_t ns = (size_t)p->n_special;
  a.stale[0] = sc;
  a.stale[1] = sc + 9 * ns;
  a.mac[0] = sc + 18 * ns;
  a.mac[1] = sc + 21 * ns;
  a.link_force = sc + 24 * ns;
  a.drag_hist = p->drag_hist;
  a.drag_cap = p->drag_cap > 0 ? p->drag_cap : 1;
  a.drag_it_offset = 1;
  a.n_obs = p->n_obstacles;
  a.obs_start = p->obstacle_link_start;
  a.rho_out = p->rho_out;
  a.u_out = p->u_out;
  a.g_out = p->g_out;
  a.status = p->status_flags;
  a.mode = mode;
  a.advance_at = 0;
  a.check_finite = (flags & LBM_FLAG_CHECK_FINITE) && p->status_flags ? 1 : 0;
  a.bulk_tma = (flags & LBM_FLAG_BULK_REGISTERS) ? 0 : 1;
  a.tma_stall = (flags & LBM_FLAG_TEST_STALL) ? 1 : 0;
  a.wall_macro = (flags & LBM_FLAG_WALL_MACRO) && p->rho_out && p->u_out ? 1 : 0;
  return a;
}

// Enqueue n_steps steps.  set_it: write it0 into the device counter first
// (left out when a graph that must not bake the start iteration is captured).
int fused_enqueue(const lbm_problem* p, int mode, long long it0, int n_steps, int parity,
                  unsigned flags, bool set_it, cudaStream_t st, cudaEvent_t* ev) {
  FusedArgs a = make_args(p, mode, flags);
  if (set_it) k_set_it<<<1, 1, 0, st>>>(a.it_dev, a.step_done, it0);
  // per-kernel timing (ev) keeps every kernel on st, and so does a single
  // step (its drag kernel has no next bulk kernel to run beside before the
  // join)
  DragLane* lane = ev || !LBM_DRAG_SIDE || n_steps < 2 ? nullptr : drag_lane();
  bool drag_pending = false;
  for (int k = 0; k < n_steps; ++k) {
    const int par = (parity + k) & 1;  // f[par] holds g_up of the previous iteration
    a.fin = p->f[par];
    a.fout = p->f[par ^ 1];
    a.write_macro = (flags & LBM_FLAG_MACRO_LAST) && k == n_steps - 1 && p->rho_out && p->u_out;
    cudaEvent_t* e = ev ? ev + 4 * k : nullptr;
    switch (p->precision) {
      case LBM_PREC_F64: launch_store<StoreF64>(a, mode, st, e, lane, &drag_pending); break;
      case LBM_PREC_F32: launch_store<StoreF32>(a, mode, st, e, lane, &drag_pending); break;
      case LBM_PREC_F16S: launch_store<StoreF16>(a, mode, st, e, lane, &drag_pending); break;
      case LBM_PREC_Q60: launch_store<StoreQ60>(a, mode, st, e, lane, &drag_pending); break;
      case LBM_PREC_F16SR: launch_store<StoreF16SR>(a, mode, st, e, lane, &drag_pending); break;
      case LBM_PREC_BF16SR: launch_store<StoreBF16SR>(a, mode, st, e, lane, &drag_pending); break;
      default: launch_store<StoreBF16>(a, mode, st, e, lane, &drag_pending); break;
    }
  }
  if (drag_pending) cudaStreamWaitEvent(st, lane->ev_drag, 0);  // join
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("lbm_advance: launch failed: %s", cudaGetErrorString(e));
    return LBM_ERR_CUDA;
  }
  return LBM_OK;
}

template <class St>
static int tile_cells_of(bool half) {
  using Sh = typename TmaShapeOf<St>::type;
  return half ? TmaHalf<Sh>::type::kCells : Sh::kCells;
}

int fused_enqueue_chain(const lbm_problem* p, long long it0, int n_steps, double* states,
                        long long stride, cudaStream_t st) {
  FusedArgs a = make_args(p, LBM_MODE_STEP, 0);
  a.drag_hist = nullptr;
  a.write_macro = 0;
  for (int m = 1; m < n_steps; ++m) {
    if (m == 1) k_set_it<<<1, 1, 0, st>>>(a.it_dev, a.step_done, it0 + 1);
    a.fin = states + (m - 1) * stride;
    a.fout = states + m * stride;
    launch_store<StoreF64>(a, LBM_MODE_STEP, st, nullptr, nullptr, nullptr);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("lbm_adjoint_recompute: launch failed: %s", cudaGetErrorString(e));
    return LBM_ERR_CUDA;
  }
  return LBM_OK;
}

int tma_tile_cells(int precision, bool half) {
  switch (precision) {
    case LBM_PREC_F16S: return tile_cells_of<StoreF16>(half);
    case LBM_PREC_F16SR: return tile_cells_of<StoreF16SR>(half);
    case LBM_PREC_BF16S: return tile_cells_of<StoreBF16>(half);
    case LBM_PREC_BF16SR: return tile_cells_of<StoreBF16SR>(half);
    default: return 0;
  }
}

int fused_set_it(const lbm_problem* p, long long value, cudaStream_t st) {
  char* base = (char*)(((uintptr_t)p->scratch + 255) & ~(uintptr_t)255);
  k_set_it<<<1, 1, 0, st>>>((long long*)base, (unsigned*)(base + 8), value);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("lbm_advance: launch failed: %s", cudaGetErrorString(e));
    return LBM_ERR_CUDA;
  }
  return LBM_OK;
}

}  // namespace lbm
