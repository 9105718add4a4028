// Kernel-level entry points: one CUDA kernel per reference function, FP64.
//
// These restate lbm/src/core/nb.py and lattice.macro operation by operation
// so that an app calling the lattice methods in any order gets the reference
// result.  This translation unit is compiled with -fmad=false: every product
// and sum is rounded on its own as in NumPy, so the results equal the CPU
// restatement bit for bit (division and square root are IEEE in both).
#include <cuda.h>

#include <mutex>

#include "lbm_device.cuh"
#include "lbm_internal.h"

namespace lbm {
namespace {

#define IDX(q, i, j) (((long long)(q) * nx + (i)) * ny + (j))

// lattice.macro, lattice.py:178-189 (sum over q in order, then divide).
__global__ void k_macro(const double* __restrict__ g, double* __restrict__ rho,
                        double* __restrict__ u, int nx, int ny) {
  const long long N = (long long)nx * ny;
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= N) return;
  double r = g[c];
#pragma unroll
  for (int q = 1; q < 9; ++q) r += g[q * N + c];
  double jx = 0.0, jy = 0.0;
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    jx += (double)cx(q) * g[q * N + c];
    jy += (double)cy(q) * g[q * N + c];
  }
  rho[c] = r;
  u[c] = jx / r;
  u[N + c] = jy / r;
}

// nb_equilibrium, nb.py:7-17.
__global__ void k_equilibrium(const double* __restrict__ u, const double* __restrict__ rho,
                              double* __restrict__ g_eq, int nx, int ny) {
  const long long N = (long long)nx * ny;
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= N) return;
  const double ux = u[c], uy = u[N + c];
  const double v = 1.5 * (ux * ux + uy * uy);
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    const double t = 3.0 * (ux * (double)cx(q) + uy * (double)cy(q));
    const double e = 1.0 + t + 0.5 * (t * t) - v;
    g_eq[q * N + c] = e * (rho[c] * wgt(q));
  }
}

// nb_col_str collision part, nb.py:24-35.
__global__ void k_collide(const double* __restrict__ g, const double* __restrict__ g_eq,
                          double* __restrict__ g_up, double om_p, double om_m, int nx, int ny) {
  const long long N = (long long)nx * ny;
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= N) return;
  const double a = 1.0 - 0.5 * (om_p + om_m);
  const double b = 0.5 * (om_p - om_m);
  const double cc = 0.5 * (om_p + om_m);
  g_up[c] = (1.0 - om_p) * g[c] + om_p * g_eq[c];
#pragma unroll
  for (int q = 1; q < 9; ++q) {
    const int qb = opp(q);
    g_up[q * N + c] = a * g[q * N + c] - b * g[qb * N + c] + cc * g_eq[q * N + c] +
                      b * g_eq[qb * N + c];
  }
}

// nb_col_str streaming part, nb.py:26 and 37-45: shift-copy on interior
// slices, edge entries without a source untouched.
__global__ void k_stream(double* __restrict__ g, const double* __restrict__ g_up, int nx, int ny) {
  const long long N = (long long)nx * ny;
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= N) return;
  const int i = (int)(c / ny), j = (int)(c - (long long)i * ny);
  g[c] = g_up[c];
#pragma unroll
  for (int q = 1; q < 9; ++q) {
    const int si = i - cx(q), sj = j - cy(q);
    if (si < 0 || si >= nx || sj < 0 || sj >= ny) continue;
    g[q * N + c] = g_up[IDX(q, si, sj)];
  }
}

__device__ __forceinline__ int wrap(int k, int n) { return k < 0 ? k + n : k; }

// nb_bounce_back_obstacle, nb.py:77-117 (one thread per link; the host keeps
// at most one link per (cell, q)).
__global__ void k_bounce_back(int ibb, const int32_t* __restrict__ links, long long n,
                              const double* __restrict__ p_ibb, const double* __restrict__ g_up,
                              double* __restrict__ g, int nx, int ny) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int i0 = links[3 * k], j0 = links[3 * k + 1], q = links[3 * k + 2];
  if (q < 1 || q > 8) return;
  const int qb = opp(q);
  const int i = wrap(i0, nx), j = wrap(j0, ny);
  if (i < 0 || i >= nx || j < 0 || j >= ny) return;  // the host rejects these links
  if (ibb) {
    const int im = wrap(i0 + cx(qb), nx), jm = wrap(j0 + cy(qb), ny);
    if (im < 0 || im >= nx || jm < 0 || jm >= ny) return;
    const double p = p_ibb[k];
    const double pp = 2.0 * p;
    if (p < 0.5) {
      const int imm = wrap(i0 + 2 * cx(qb), nx), jmm = wrap(j0 + 2 * cy(qb), ny);
      if (imm < 0 || imm >= nx || jmm < 0 || jmm >= ny) return;
      g[IDX(qb, i, j)] = p * (pp + 1.0) * g_up[IDX(q, i, j)] +
                         (1.0 + pp) * (1.0 - pp) * g_up[IDX(q, im, jm)] -
                         p * (1.0 - pp) * g_up[IDX(q, imm, jmm)];
    } else {
      g[IDX(qb, i, j)] = (1.0 / (p * (pp + 1.0))) * g_up[IDX(q, i, j)] +
                         ((pp - 1.0) / p) * g_up[IDX(qb, i, j)] +
                         ((1.0 - pp) / (1.0 + pp)) * g_up[IDX(qb, im, jm)];
    }
  } else {
    g[IDX(qb, i, j)] = g_up[IDX(q, i, j)];
  }
}

// nb_drag_lift, nb.py:49-73: per-block fixed-order trees, then one block
// sums the block partials in order.
__global__ void k_drag_partial(const int32_t* __restrict__ links, long long n,
                               const double* __restrict__ g_up, const double* __restrict__ g,
                               int nx, int ny, double* __restrict__ part) {
  __shared__ double sx[256], sy[256];
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double fx = 0.0, fy = 0.0;
  if (k < n) {
    const int i = wrap(links[3 * k], nx), j = wrap(links[3 * k + 1], ny), q = links[3 * k + 2];
    if (i >= 0 && i < nx && j >= 0 && j < ny && q >= 1 && q <= 8) {
      const double g0 = g_up[IDX(q, i, j)] + g[IDX(opp(q), i, j)];
      fx = g0 * (double)cx(q);
      fy = g0 * (double)cy(q);
    }
  }
  sx[threadIdx.x] = fx;
  sy[threadIdx.x] = fy;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      sx[threadIdx.x] += sx[threadIdx.x + w];
      sy[threadIdx.x] += sy[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = sx[0];
    part[2 * blockIdx.x + 1] = sy[0];
  }
}

__global__ void k_drag_final(const double* __restrict__ part, int nb, double* __restrict__ out) {
  __shared__ double sx[256], sy[256];
  double fx = 0.0, fy = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    fx += part[2 * b];
    fy += part[2 * b + 1];
  }
  sx[threadIdx.x] = fx;
  sy[threadIdx.x] = fy;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      sx[threadIdx.x] += sx[threadIdx.x + w];
      sy[threadIdx.x] += sy[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = sx[0];
    out[1] = sy[0];
  }
}

// Zou-He walls: one thread per wall cell, arithmetic from lbm_device.cuh.
__global__ void k_zou_he(int wall, double* __restrict__ u, double* __restrict__ rho,
                         double* __restrict__ g, const double* __restrict__ vec,
                         const double* __restrict__ rho_right, int nx, int ny) {
  const long long N = (long long)nx * ny;
  const bool vertical = wall == LBM_WALL_LEFT_VELOCITY || wall == LBM_WALL_RIGHT_VELOCITY ||
                        wall == LBM_WALL_RIGHT_PRESSURE;
  const int len = vertical ? ny : nx;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= len) return;
  int i, j;
  if (vertical) {
    i = wall == LBM_WALL_LEFT_VELOCITY ? 0 : nx - 1;
    j = t;
  } else {
    i = t;
    j = wall == LBM_WALL_TOP_VELOCITY ? ny - 1 : 0;
  }
  const long long c = (long long)i * ny + j;
  CellBC<double> s;
#pragma unroll
  for (int q = 0; q < 9; ++q) s.g[q] = g[q * N + c];
  s.rho = rho[c];
  s.ux = u[c];
  s.uy = u[N + c];
  switch (wall) {
    case LBM_WALL_LEFT_VELOCITY: zh_left<double>(s, vec[t], vec[len + t]); break;
    case LBM_WALL_RIGHT_VELOCITY: zh_right<double>(s, vec[t], vec[len + t]); break;
    case LBM_WALL_RIGHT_PRESSURE: zh_right_pressure<double>(s, rho_right[t], vec[len + t]); break;
    case LBM_WALL_TOP_VELOCITY: zh_top<double>(s, vec[t], vec[len + t]); break;
    default: zh_bottom<double>(s, vec[t], vec[len + t]); break;
  }
#pragma unroll
  for (int q = 0; q < 9; ++q) g[q * N + c] = s.g[q];
  rho[c] = s.rho;
  u[c] = s.ux;
  u[N + c] = s.uy;
}

__global__ void k_corner(int corner, double* __restrict__ u, double* __restrict__ rho,
                         double* __restrict__ g, int nx, int ny) {
  const long long N = (long long)nx * ny;
  const int lx = nx - 1, ly = ny - 1;
  const int i = (corner == LBM_CORNER_BOTTOM_LEFT || corner == LBM_CORNER_TOP_LEFT) ? 0 : lx;
  const int j = (corner == LBM_CORNER_BOTTOM_LEFT || corner == LBM_CORNER_BOTTOM_RIGHT) ? 0 : ly;
  const int in = i == 0 ? 1 : lx - 1;
  const long long c = (long long)i * ny + j, cn = (long long)in * ny + j;
  CellBC<double> s;
#pragma unroll
  for (int q = 0; q < 9; ++q) s.g[q] = g[q * N + c];
  zh_corner<double>(corner, s, rho[cn], u[cn], u[N + cn]);
#pragma unroll
  for (int q = 0; q < 9; ++q) g[q * N + c] = s.g[q];
  rho[c] = s.rho;
  u[c] = s.ux;
  u[N + c] = s.uy;
}

inline unsigned blocks_for(long long n, int tb) { return (unsigned)((n + tb - 1) / tb); }

int check_grid(const char* fn, int nx, int ny) {
  if (nx < 3 || ny < 3 || (long long)nx * ny > (1LL << 31) - 1) {
    set_error("%s: lattice %d x %d outside 3 <= n, nx*ny < 2^31", fn, nx, ny);
    return LBM_ERR_ARG;
  }
  return LBM_OK;
}

}  // namespace
}  // namespace lbm

using namespace lbm;

#define LBM_LAUNCH_CHECK(what)                                                      \
  do {                                                                              \
    cudaError_t e_ = cudaGetLastError();                                            \
    if (e_ != cudaSuccess) {                                                        \
      set_error("%s: %s", what, cudaGetErrorString(e_));                           \
      return LBM_ERR_CUDA;                                                          \
    }                                                                               \
  } while (0)

extern "C" int lbm_macro_f64(const double* g, double* rho, double* u, int nx, int ny, void* stream) {
  if (int rc = check_grid("lbm_macro_f64", nx, ny)) return rc;
  if (!g || !rho || !u) { set_error("lbm_macro_f64: null pointer"); return LBM_ERR_ARG; }
  const long long N = (long long)nx * ny;
  k_macro<<<blocks_for(N, 256), 256, 0, (cudaStream_t)stream>>>(g, rho, u, nx, ny);
  LBM_LAUNCH_CHECK("lbm_macro_f64");
  return LBM_OK;
}

extern "C" int lbm_equilibrium_f64(const double* u, const double* rho, double* g_eq, int nx, int ny,
                                   void* stream) {
  if (int rc = check_grid("lbm_equilibrium_f64", nx, ny)) return rc;
  if (!g_eq || !rho || !u) { set_error("lbm_equilibrium_f64: null pointer"); return LBM_ERR_ARG; }
  const long long N = (long long)nx * ny;
  k_equilibrium<<<blocks_for(N, 256), 256, 0, (cudaStream_t)stream>>>(u, rho, g_eq, nx, ny);
  LBM_LAUNCH_CHECK("lbm_equilibrium_f64");
  return LBM_OK;
}

extern "C" int lbm_collision_stream_f64(double* g, const double* g_eq, double* g_up, double om_p,
                                        double om_m, int nx, int ny, void* stream) {
  if (int rc = check_grid("lbm_collision_stream_f64", nx, ny)) return rc;
  if (!g || !g_eq || !g_up) { set_error("lbm_collision_stream_f64: null pointer"); return LBM_ERR_ARG; }
  const long long N = (long long)nx * ny;
  cudaStream_t st = (cudaStream_t)stream;
  k_collide<<<blocks_for(N, 256), 256, 0, st>>>(g, g_eq, g_up, om_p, om_m, nx, ny);
  k_stream<<<blocks_for(N, 256), 256, 0, st>>>(g, g_up, nx, ny);
  LBM_LAUNCH_CHECK("lbm_collision_stream_f64");
  return LBM_OK;
}

extern "C" int lbm_bounce_back_f64(int ibb, const int32_t* links, int64_t n, const double* p,
                                   const double* g_up, double* g, int nx, int ny, void* stream) {
  if (int rc = check_grid("lbm_bounce_back_f64", nx, ny)) return rc;
  if (n < 0 || (n > 0 && (!links || !g_up || !g || (ibb && !p)))) {
    set_error("lbm_bounce_back_f64: bad arguments (n=%lld)", (long long)n);
    return LBM_ERR_ARG;
  }
  if (n == 0) return LBM_OK;
  k_bounce_back<<<blocks_for(n, 128), 128, 0, (cudaStream_t)stream>>>(ibb, links, n, p, g_up, g, nx, ny);
  LBM_LAUNCH_CHECK("lbm_bounce_back_f64");
  return LBM_OK;
}

extern "C" size_t lbm_drag_lift_scratch_bytes(int64_t n) {
  long long nb = n > 0 ? (n + 255) / 256 : 1;
  return (size_t)(2 * nb * sizeof(double));
}

extern "C" int lbm_drag_lift_f64(const int32_t* links, int64_t n, const double* g_up, const double* g,
                                 int nx, int ny, double* out, void* scratch, void* stream) {
  if (int rc = check_grid("lbm_drag_lift_f64", nx, ny)) return rc;
  if (n < 0 || !out || !scratch || (n > 0 && (!links || !g_up || !g))) {
    set_error("lbm_drag_lift_f64: bad arguments");
    return LBM_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const long long nb = n > 0 ? (n + 255) / 256 : 1;
  if (nb > (1LL << 30)) { set_error("lbm_drag_lift_f64: too many links"); return LBM_ERR_ARG; }
  double* part = (double*)scratch;
  k_drag_partial<<<(unsigned)nb, 256, 0, st>>>(links, n, g_up, g, nx, ny, part);
  k_drag_final<<<1, 256, 0, st>>>(part, (int)nb, out);
  LBM_LAUNCH_CHECK("lbm_drag_lift_f64");
  return LBM_OK;
}

// ---- drag/lift without caller memory ------------------------------------------
// Some callers cannot hand the library a scratch buffer: a host whose device
// memory is owned by another allocator (a framework's caching allocator, a
// Fortran or game-engine runtime that budgets all device memory at start-up)
// or a real-time loop that must not allocate after set-up.  For them the
// block partials of the drag/lift reduction live in this fixed array, part of
// the library's device image: every GPU that loads the library holds its
// 64 KiB until the process exits.  The host must not pass the symbol itself
// to a kernel (on the host it names a stand-in, not device memory); its
// device address is fetched with cudaGetSymbolAddress once per CUDA context
// (each context that loads the library has its own copy of the array).
#define LBM_NOALLOC_MAX_BLOCKS (LBM_DRAG_NOALLOC_MAX_LINKS / 256)
static __device__ __align__(256) double g_drag_noalloc_part[2 * LBM_NOALLOC_MAX_BLOCKS];

namespace {
// Contexts are told apart by the driver's context id (cuCtxGetId), which is
// unique for the life of the process: a context destroyed and re-created
// (cudaDeviceReset, or a host that makes its own driver context current)
// gets a new id and a fresh look-up.  The driver entry points come through
// the runtime, so the library does not link libcuda.
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);
struct NoallocEntry {
  unsigned long long ctx_id;
  double* addr;
};
std::mutex g_noalloc_mu;
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;
NoallocEntry g_noalloc_cache[64];
int g_noalloc_n = 0;

// Id of the calling thread's current context (made current by the runtime
// if none is); false if the driver cannot tell.
bool current_context_id(unsigned long long* id) {
  if (!g_ctx_get_current || !g_ctx_get_id) {
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) !=
            cudaSuccess ||
        q1 != cudaDriverEntryPointSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) !=
            cudaSuccess ||
        q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
      return false;
    g_ctx_get_current = (CtxGetCurrentFn)f1;
    g_ctx_get_id = (CtxGetIdFn)f2;
  }
  CUcontext ctx = nullptr;
  if (g_ctx_get_current(&ctx) != CUDA_SUCCESS) return false;
  if (!ctx) {
    // No context on this thread yet: bind the current device's primary
    // context, as the runtime's first call on the thread would.
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaSetDevice(dev) != cudaSuccess) return false;
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx) return false;
  }
  return g_ctx_get_id(ctx, id) == CUDA_SUCCESS;
}
}  // namespace

extern "C" int lbm_drag_lift_f64_noalloc(const int32_t* links, int64_t n, const double* g_up,
                                         const double* g, int nx, int ny, double* out,
                                         void* stream) {
  if (int rc = check_grid("lbm_drag_lift_f64_noalloc", nx, ny)) return rc;
  if (n < 0 || !out || (n > 0 && (!links || !g_up || !g))) {
    set_error("lbm_drag_lift_f64_noalloc: bad arguments");
    return LBM_ERR_ARG;
  }
  if (n > LBM_DRAG_NOALLOC_MAX_LINKS) {
    set_error("lbm_drag_lift_f64_noalloc: %lld links exceed the fixed scratch limit of %d links; "
              "use lbm_drag_lift_f64 with a caller buffer",
              (long long)n, (int)LBM_DRAG_NOALLOC_MAX_LINKS);
    return LBM_ERR_ARG;
  }
  double* part = nullptr;
  {
    // One-time set-up per context, with that context current.
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    unsigned long long ctx_id = 0;
    if (!current_context_id(&ctx_id)) {
      set_error("lbm_drag_lift_f64_noalloc: no usable current CUDA context");
      return LBM_ERR_CUDA;
    }
    for (int k = 0; k < g_noalloc_n; ++k)
      if (g_noalloc_cache[k].ctx_id == ctx_id) part = g_noalloc_cache[k].addr;
    if (!part) {
      void* addr = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&addr, g_drag_noalloc_part);
      if (e != cudaSuccess || !addr) {
        set_error("lbm_drag_lift_f64_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
        return LBM_ERR_CUDA;
      }
      part = (double*)addr;
      // A full table keeps its entries; later contexts look the address up on every call.
      if (g_noalloc_n < 64) g_noalloc_cache[g_noalloc_n++] = NoallocEntry{ctx_id, part};
    }
  }
  // k_drag_partial writes all nb partials before k_drag_final reads them
  // (same stream), so nothing from the previous call has to be cleared.
  cudaStream_t st = (cudaStream_t)stream;
  const long long nb = n > 0 ? (n + 255) / 256 : 1;
  k_drag_partial<<<(unsigned)nb, 256, 0, st>>>(links, n, g_up, g, nx, ny, part);
  k_drag_final<<<1, 256, 0, st>>>(part, (int)nb, out);
  LBM_LAUNCH_CHECK("lbm_drag_lift_f64_noalloc");
  return LBM_OK;
}

// ---- observable buffer: buff.mv_avg for a chunk of adds ----------------------
// lbm/src/utils/buff.py:35-77.  After add number k (k = 1, 2, ...) the
// reference computes, with it_s = floor(4k/5) and windows [it_s, k) of its
// histories (each starts with two zeros, so add m is stored at index m + 1):
//   obs1 = sum(buff[it_s:k]) / (k - it_s + 1)    appended to avg1
//   obs2 = sum(avg1[it_s:k]) / (k - it_s + 1)    appended to avg2
//   obs3 = sum(avg2[it_s:k]) / (k - it_s + 1)    appended to avg3
//   obs  = sum(avg3[it_s:k]) / (k - it_s + 1)    returned
// and, for k > 10, growth = (avg3[k] - avg3[it_s]) / ((k - it_s + 1) dt) with
// the convergence counter.  A level's window for add k reads the level below
// up to index k - 1, i.e. values of adds <= k - 2, so each level of a chunk
// of adds is computed in parallel (one thread per add) once the level below
// is complete.  Sums follow NumPy's order for a contiguous float64 slice
// (pairwise summation: blocks of at most 128 values summed with eight
// accumulators, longer ranges split in two with the first length a multiple
// of 8), so every value equals the reference's bit for bit.
namespace lbm {
namespace mvavg {

__device__ double pw_block(const double* a, long long n) {
  if (n < 8) {
    double r = 0.0;
    for (long long i = 0; i < n; ++i) r += a[i];
    return r;
  }
  double r0 = a[0], r1 = a[1], r2 = a[2], r3 = a[3], r4 = a[4], r5 = a[5], r6 = a[6], r7 = a[7];
  long long i = 8;
  for (; i < n - (n % 8); i += 8) {
    r0 += a[i];
    r1 += a[i + 1];
    r2 += a[i + 2];
    r3 += a[i + 3];
    r4 += a[i + 4];
    r5 += a[i + 5];
    r6 += a[i + 6];
    r7 += a[i + 7];
  }
  double res = ((r0 + r1) + (r2 + r3)) + ((r4 + r5) + (r6 + r7));
  for (; i < n; ++i) res += a[i];
  return res;
}

__device__ __forceinline__ long long pw_split(long long n) {
  long long n2 = n / 2;
  return n2 - n2 % 8;
}

// Pairwise sum of a[0..n) without recursion: a stack of the ranges whose
// left half is being summed (at most 57 levels for any 64-bit length).
__device__ double pw_sum(const double* a, long long n) {
  if (n <= 128) return pw_block(a, n);
  const double* sa[64];
  long long sn[64];
  double sl[64];
  bool sdone[64];
  int top = 0;
  sa[0] = a;
  sn[0] = n;
  sdone[0] = false;
  for (;;) {
    // descend into left halves down to a block
    while (sn[top] > 128) {
      const long long n2 = pw_split(sn[top]);
      sa[top + 1] = sa[top];
      sn[top + 1] = n2;
      sdone[top + 1] = false;
      ++top;
    }
    double v = pw_block(sa[top], sn[top]);
    --top;
    // go up: a finished left half starts its right sibling, a finished
    // right half completes its parent
    for (;;) {
      if (top < 0) return v;
      if (!sdone[top]) {
        const long long n2 = pw_split(sn[top]);
        sl[top] = v;
        sdone[top] = true;
        sa[top + 1] = sa[top] + n2;
        sn[top + 1] = sn[top] - n2;
        sdone[top + 1] = false;
        ++top;
        break;
      }
      v = sl[top] + v;
      --top;
    }
  }
}

// Level `level` (1..4) of adds k0 + 1 .. k0 + n.  hist: [4][cap] (buff, avg1,
// avg2, avg3).  Levels 1-3 append to the next history; level 4 writes obs.
__global__ void k_mv_avg_level(double* hist, long long cap, long long k0, int n, int level,
                               double* obs) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const long long k = k0 + 1 + t;
  const long long it_s = (4 * k) / 5;
  const double v = pw_sum(hist + (long long)(level - 1) * cap + it_s, k - it_s) /
                   (double)(k - it_s + 1);
  if (level < 4) hist[(long long)level * cap + k + 1] = v;
  else obs[t] = v;
}

// Growth rates and the convergence counter, in order (one thread).
// state: [0] counter, [1] converged flag (kept across calls).
__global__ void k_mv_avg_growth(const double* hist, long long cap, long long k0, int n, double dt,
                                double cv_ct, int cv_nb, int* state, double* growth, int* cv) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  const double* avg3 = hist + 3 * cap;
  int cnt = state[0], flag = state[1];
  for (int t = 0; t < n; ++t) {
    const long long k = k0 + 1 + t;
    double g = 0.0;
    if (k > 10) {
      const long long it_s = (4 * k) / 5;
      const double db = avg3[k] - avg3[it_s];
      g = db / ((double)(k - it_s + 1) * dt);
      cnt = fabs(g) < cv_ct ? cnt + 1 : 0;
      if (cnt > cv_nb) flag = 1;
    }
    growth[t] = g;
    cv[t] = flag;
  }
  state[0] = cnt;
  state[1] = flag;
}

}  // namespace mvavg
}  // namespace lbm

extern "C" int lbm_mv_avg_chunk(double* hist, int64_t cap, int64_t k0, int32_t n, double dt,
                                double cv_ct, int32_t cv_nb, int32_t* state, double* obs,
                                double* growth, int32_t* cv, void* stream) {
  if (!hist || !state || !obs || !growth || !cv || n < 0 || k0 < 0 || k0 + n + 2 > cap) {
    set_error("lbm_mv_avg_chunk: bad arguments (k0 %lld, n %d, capacity %lld)", (long long)k0,
              (int)n, (long long)cap);
    return LBM_ERR_ARG;
  }
  if (n == 0) return LBM_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const int tb = 128;
  for (int level = 1; level <= 4; ++level)
    lbm::mvavg::k_mv_avg_level<<<(n + tb - 1) / tb, tb, 0, st>>>(hist, cap, k0, n, level, obs);
  lbm::mvavg::k_mv_avg_growth<<<1, 1, 0, st>>>(hist, cap, k0, n, dt, cv_ct, cv_nb, state, growth, cv);
  LBM_LAUNCH_CHECK("lbm_mv_avg_chunk");
  return LBM_OK;
}

extern "C" int lbm_zou_he_f64(int wall, double* u, double* rho, double* g, const double* vec,
                              const double* rho_right, int nx, int ny, void* stream) {
  if (int rc = check_grid("lbm_zou_he_f64", nx, ny)) return rc;
  if (wall < LBM_WALL_LEFT_VELOCITY || wall > LBM_WALL_BOTTOM_VELOCITY) {
    set_error("lbm_zou_he_f64: unknown wall %d", wall);
    return LBM_ERR_ARG;
  }
  if (!u || !rho || !g || !vec || (wall == LBM_WALL_RIGHT_PRESSURE && !rho_right)) {
    set_error("lbm_zou_he_f64: null pointer");
    return LBM_ERR_ARG;
  }
  const bool vertical = wall <= LBM_WALL_RIGHT_PRESSURE;
  const int len = vertical ? ny : nx;
  k_zou_he<<<blocks_for(len, 128), 128, 0, (cudaStream_t)stream>>>(wall, u, rho, g, vec, rho_right, nx, ny);
  LBM_LAUNCH_CHECK("lbm_zou_he_f64");
  return LBM_OK;
}

extern "C" int lbm_zou_he_corner_f64(int corner, double* u, double* rho, double* g, int nx, int ny,
                                     void* stream) {
  if (int rc = check_grid("lbm_zou_he_corner_f64", nx, ny)) return rc;
  if (corner < 0 || corner > 3 || !u || !rho || !g) {
    set_error("lbm_zou_he_corner_f64: bad arguments");
    return LBM_ERR_ARG;
  }
  k_corner<<<1, 1, 0, (cudaStream_t)stream>>>(corner, u, rho, g, nx, ny);
  LBM_LAUNCH_CHECK("lbm_zou_he_corner_f64");
  return LBM_OK;
}
