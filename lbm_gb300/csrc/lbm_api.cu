// C-ABI front of liblbm_gb300: argument checks, error strings, the fused
// engine entry points, the CUDA-graph cache and storage-form conversion.
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <mutex>
#include <vector>

#include "lbm_device.cuh"
#include "lbm_internal.h"

namespace lbm {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int problem_check(const lbm_problem* p, const char* fn) {
  if (!p) { set_error("%s: null problem", fn); return LBM_ERR_ARG; }
  if (p->nx < 4 || p->ny < 4 || (long long)p->nx * p->ny > (1LL << 31) - 1) {
    set_error("%s: lattice %d x %d outside 4 <= n, nx*ny < 2^31", fn, p->nx, p->ny);
    return LBM_ERR_ARG;
  }
  if (p->precision < LBM_PREC_F64 || p->precision > LBM_PREC_BF16SR) {
    set_error("%s: unknown precision %d", fn, p->precision);
    return LBM_ERR_ARG;
  }
  if (p->precision == LBM_PREC_Q60 &&
      !(p->rho0 >= 0.75 && p->rho0 <= 1.5 && p->om_p >= 1.0 / 1024 && p->om_p <= 1.999 &&
        p->om_m >= 1.0 / 1024 && p->om_m <= 1.999)) {
    set_error("%s: the Q3.60 form needs rho0 in [0.75, 1.5] and om_p, om_m in [1/1024, 1.999] "
              "(rho0 %g, om_p %g, om_m %g)", fn, p->rho0, p->om_p, p->om_m);
    return LBM_ERR_UNSUPPORTED;
  }
  if (p->row_pitch != 0 &&
      (p->row_pitch < p->ny || (long long)p->nx * p->row_pitch > (1LL << 31) - 1)) {
    set_error("%s: row pitch %d below ny %d or too large", fn, p->row_pitch, p->ny);
    return LBM_ERR_ARG;
  }
  if (!p->f[0] || !p->f[1] || !p->bc_base || !p->scratch) {
    set_error("%s: null distribution, BC or scratch pointer", fn);
    return LBM_ERR_ARG;
  }
  if (p->scratch_bytes < fused_scratch_bytes(p)) {
    set_error("%s: scratch of %zu bytes, %zu needed", fn, p->scratch_bytes, fused_scratch_bytes(p));
    return LBM_ERR_ARG;
  }
  if (p->n_wall_ops < 0 || p->n_wall_ops > 5 || p->n_corner_ops < 0 || p->n_corner_ops > 4) {
    set_error("%s: bad BC program size", fn);
    return LBM_ERR_ARG;
  }
  for (int w = 0; w < p->n_wall_ops; ++w)
    if (p->wall_ops[w] < LBM_WALL_LEFT_VELOCITY || p->wall_ops[w] > LBM_WALL_BOTTOM_VELOCITY) {
      set_error("%s: unknown wall op %d", fn, p->wall_ops[w]);
      return LBM_ERR_ARG;
    }
  for (int w = 0; w < p->n_corner_ops; ++w) {
    const int c = p->corner_ops[w];
    if (c < 0 || c > 3 || p->corner_special[c] < 0 || p->corner_special[c] >= p->n_special ||
        p->corner_nb_special[c] < 0 || p->corner_nb_special[c] >= p->n_special) {
      set_error("%s: bad corner op %d", fn, c);
      return LBM_ERR_ARG;
    }
  }
  if (p->n_special < 2 * (p->nx + p->ny) - 4 || !p->special_cell || !p->special_link_start) {
    set_error("%s: the special-cell table must hold every wall cell", fn);
    return LBM_ERR_ARG;
  }
  if (p->n_links < 0 || (p->n_links > 0 && (!p->link_cell || !p->link_q || !p->special_link_ids ||
                                            !p->link_nb1 || !p->link_nb2 ||
                                            (p->ibb && !p->link_p)))) {
    set_error("%s: bad link table", fn);
    return LBM_ERR_ARG;
  }
  if (p->drag_hist && (p->drag_cap <= 0 || p->n_obstacles < 0 ||
                       (p->n_obstacles > 0 && !p->obstacle_link_start))) {
    set_error("%s: bad drag history", fn);
    return LBM_ERR_ARG;
  }
  if (p->bc_vec && (!p->bc_scale || p->bc_scale_len <= 0)) {
    set_error("%s: bc_vec given without a scale table", fn);
    return LBM_ERR_ARG;
  }
  return LBM_OK;
}

namespace {

// ---- CUDA-graph cache -------------------------------------------------------
struct GraphEntry {
  lbm_problem prob;
  int n_steps, parity;
  unsigned flags;
  int device;
  cudaGraphExec_t exec;
  unsigned long long last_use;
};

std::mutex g_mu;
std::vector<GraphEntry> g_cache;
unsigned long long g_clock = 0;
cudaStream_t g_capture_stream[64] = {};
const size_t kMaxGraphs = 16;

}  // namespace
}  // namespace lbm

using namespace lbm;

extern "C" int lbm_abi_version(void) { return 2; }

extern "C" const char* lbm_last_error_string(void) { return g_err; }

extern "C" int lbm_device_info(int* sm_count, char* name, int name_len) {
  int dev = 0;
  LBM_CUDA_CHECK(cudaGetDevice(&dev), "lbm_device_info");
  cudaDeviceProp prop;
  LBM_CUDA_CHECK(cudaGetDeviceProperties(&prop, dev), "lbm_device_info");
  if (sm_count) *sm_count = prop.multiProcessorCount;
  if (name && name_len > 0) {
    strncpy(name, prop.name, (size_t)name_len - 1);
    name[name_len - 1] = 0;
  }
  return LBM_OK;
}

extern "C" size_t lbm_problem_scratch_bytes(const lbm_problem* p) {
  return p ? fused_scratch_bytes(p) : 0;
}

extern "C" int lbm_advance(const lbm_problem* p, int mode, int64_t it0, int n_steps, int parity,
                           uint32_t flags, void* stream) {
  if (int rc = problem_check(p, "lbm_advance")) return rc;
  if (mode < LBM_MODE_COLLIDE_FROM_G || mode > LBM_MODE_FINISH || n_steps < 1 ||
      (mode != LBM_MODE_STEP && n_steps != 1) || (parity != 0 && parity != 1)) {
    set_error("lbm_advance: bad mode %d / n_steps %d / parity %d", mode, n_steps, parity);
    return LBM_ERR_ARG;
  }
  if (mode != LBM_MODE_STEP && !p->g_out) {
    set_error("lbm_advance: mode %d needs g_out", mode);
    return LBM_ERR_ARG;
  }
  return fused_enqueue(p, mode, it0, n_steps, parity, flags, true, (cudaStream_t)stream);
}

extern "C" int lbm_profile_steps(const lbm_problem* p, int64_t it0, int n_steps, int parity,
                                 uint32_t flags, double* ms_out, void* stream) {
  if (int rc = problem_check(p, "lbm_profile_steps")) return rc;
  if (n_steps < 1 || n_steps > 100000 || (parity != 0 && parity != 1) || !ms_out) {
    set_error("lbm_profile_steps: bad n_steps %d / parity %d / output", n_steps, parity);
    return LBM_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  std::vector<cudaEvent_t> ev(4 * (size_t)n_steps, nullptr);
  for (auto& e : ev) {
    cudaError_t err = cudaEventCreate(&e);
    if (err != cudaSuccess) {
      for (auto& x : ev)
        if (x) cudaEventDestroy(x);
      set_error("lbm_profile_steps: event create: %s", cudaGetErrorString(err));
      return LBM_ERR_CUDA;
    }
  }
  int rc = fused_enqueue(p, LBM_MODE_STEP, it0, n_steps, parity, flags, true, st, ev.data());
  double sums[3] = {0.0, 0.0, 0.0};
  if (rc == LBM_OK) {
    cudaError_t err = cudaEventSynchronize(ev.back());
    for (int k = 0; k < n_steps && err == cudaSuccess; ++k) {
      for (int s = 0; s < 3 && err == cudaSuccess; ++s) {
        float ms = 0.f;
        err = cudaEventElapsedTime(&ms, ev[4 * k + s], ev[4 * k + s + 1]);
        sums[s] += ms;
      }
    }
    if (err != cudaSuccess) {
      set_error("lbm_profile_steps: %s", cudaGetErrorString(err));
      rc = LBM_ERR_CUDA;
    }
  }
  for (auto& e : ev) cudaEventDestroy(e);
  for (int s = 0; s < 3; ++s) ms_out[s] = sums[s] / n_steps;
  ms_out[3] = (double)fused_kernels_per_step(p, LBM_MODE_STEP);
  return rc;
}

extern "C" int lbm_graph_cache_clear(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto& e : g_cache) cudaGraphExecDestroy(e.exec);
  g_cache.clear();
  return LBM_OK;
}

extern "C" int lbm_advance_graph(const lbm_problem* p, int64_t it0, int n_steps, int parity,
                                 uint32_t flags, void* stream) {
  if (int rc = problem_check(p, "lbm_advance_graph")) return rc;
  if (n_steps < 1 || (parity != 0 && parity != 1)) {
    set_error("lbm_advance_graph: bad n_steps %d / parity %d", n_steps, parity);
    return LBM_ERR_ARG;
  }
  int dev = 0;
  LBM_CUDA_CHECK(cudaGetDevice(&dev), "lbm_advance_graph");
  if (dev < 0 || dev >= 64) { set_error("lbm_advance_graph: device %d", dev); return LBM_ERR_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lk(g_mu);
  GraphEntry* hit = nullptr;
  for (auto& e : g_cache) {
    if (e.device == dev && e.n_steps == n_steps && e.parity == parity && e.flags == flags &&
        memcmp(&e.prob, p, sizeof(lbm_problem)) == 0) {
      hit = &e;
      break;
    }
  }
  if (!hit) {
    if (!g_capture_stream[dev])
      LBM_CUDA_CHECK(cudaStreamCreateWithFlags(&g_capture_stream[dev], cudaStreamNonBlocking),
                     "lbm_advance_graph: capture stream");
    cudaStream_t cs = g_capture_stream[dev];
    LBM_CUDA_CHECK(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal),
                   "lbm_advance_graph: begin capture");
    int rc = fused_enqueue(p, LBM_MODE_STEP, 0, n_steps, parity, flags, false, cs);
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(cs, &graph);
    if (rc != LBM_OK) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (e != cudaSuccess) {
      set_error("lbm_advance_graph: end capture: %s", cudaGetErrorString(e));
      return LBM_ERR_CUDA;
    }
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      set_error("lbm_advance_graph: instantiate: %s", cudaGetErrorString(e));
      return LBM_ERR_CUDA;
    }
    if (g_cache.size() >= kMaxGraphs) {
      size_t old = 0;
      for (size_t k = 1; k < g_cache.size(); ++k)
        if (g_cache[k].last_use < g_cache[old].last_use) old = k;
      cudaGraphExecDestroy(g_cache[old].exec);
      g_cache.erase(g_cache.begin() + (long)old);
    }
    GraphEntry ent;
    memcpy(&ent.prob, p, sizeof(lbm_problem));
    ent.n_steps = n_steps;
    ent.parity = parity;
    ent.flags = flags;
    ent.device = dev;
    ent.exec = exec;
    g_cache.push_back(ent);
    hit = &g_cache.back();
  }
  hit->last_use = ++g_clock;
  if (int rc = fused_set_it(p, it0, st)) return rc;
  LBM_CUDA_CHECK(cudaGraphLaunch(hit->exec, st), "lbm_advance_graph: launch");
  return LBM_OK;
}

// ---- FP64 pipe throughput ---------------------------------------------------------
namespace lbm {
namespace {
// Eight independent FMA chains per thread, 32 DFMA per loop trip.
__global__ void k_dfma_rate(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
      x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
}  // namespace
}  // namespace lbm

extern "C" int lbm_measure_dfma_rate(double* ginstr_per_s, void* scratch, size_t scratch_bytes,
                                     void* stream) {
  int dev = 0, sms = 0;
  LBM_CUDA_CHECK(cudaGetDevice(&dev), "lbm_measure_dfma_rate");
  LBM_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev),
                 "lbm_measure_dfma_rate");
  const int threads = 256, blocks = sms * 8, iters = 2000;
  if (!ginstr_per_s || !scratch || scratch_bytes < (size_t)blocks * threads * sizeof(double)) {
    set_error("lbm_measure_dfma_rate: needs %zu bytes of scratch",
              (size_t)blocks * threads * sizeof(double));
    return LBM_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  cudaEvent_t e0, e1;
  LBM_CUDA_CHECK(cudaEventCreate(&e0), "lbm_measure_dfma_rate");
  LBM_CUDA_CHECK(cudaEventCreate(&e1), "lbm_measure_dfma_rate");
  float ms = 0.f;
  cudaError_t err = cudaSuccess;
  for (int rep = 0; rep < 3 && err == cudaSuccess; ++rep) {  // last of three (warm clocks)
    cudaEventRecord(e0, st);
    k_dfma_rate<<<blocks, threads, 0, st>>>((double*)scratch, iters, 0.999999, 1e-7);
    cudaEventRecord(e1, st);
    err = cudaEventSynchronize(e1);
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (err != cudaSuccess) {
    set_error("lbm_measure_dfma_rate: %s", cudaGetErrorString(err));
    return LBM_ERR_CUDA;
  }
  *ginstr_per_s = (double)blocks * threads * iters * 32.0 / (ms * 1e-3) / 1e9;
  return LBM_OK;
}

size_t lbm_measure_dfma_scratch_bytes(void) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return 0;
  return (size_t)sms * 8 * 256 * sizeof(double);
}

// ---- storage-form conversion ---------------------------------------------------
namespace lbm {
namespace {
// g: FP64 reference layout [q][i][j] (rows of ny); f: storage layout (rows of
// sy >= ny).  One thread per cell of the reference layout.
template <class St>
__global__ void k_pack(const double* __restrict__ g, typename St::S* __restrict__ f, int nx, int ny,
                       int sy, double rho0) {
  const long long n = (long long)nx * ny, ns = (long long)nx * sy;
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const long long i = c / ny, s = i * sy + (c - i * ny);
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    const double v = (g[q * n + c] - (St::kShift ? wgt(q) * rho0 : 0.0)) * (double)St::kScale;
    St::store(f + q * ns + s, (typename St::T)v);
  }
}
template <class St>
__global__ void k_unpack(const typename St::S* __restrict__ f, double* __restrict__ g, int nx,
                         int ny, int sy, double rho0) {
  const long long n = (long long)nx * ny, ns = (long long)nx * sy;
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const long long i = c / ny, s = i * sy + (c - i * ny);
#pragma unroll
  for (int q = 0; q < 9; ++q)
    g[q * n + c] = (double)St::load(f + q * ns + s) * (double)St::kInvScale +
                   (St::kShift ? wgt(q) * rho0 : 0.0);
}

int check_conv(const char* fn, const void* g, const void* f, int nx, int ny, int sy) {
  if (!g || !f || nx < 1 || ny < 1 || (sy != 0 && sy < ny) ||
      (long long)nx * (sy > 0 ? sy : ny) > (1LL << 31) - 1) {
    set_error("%s: bad arguments", fn);
    return LBM_ERR_ARG;
  }
  return LBM_OK;
}
}  // namespace
}  // namespace lbm

extern "C" int lbm_pack_f64(int precision, const double* g, void* f, int nx, int ny, int row_pitch,
                            double rho0, void* stream) {
  if (int rc = check_conv("lbm_pack_f64", g, f, nx, ny, row_pitch)) return rc;
  const int sy = row_pitch > 0 ? row_pitch : ny;
  cudaStream_t st = (cudaStream_t)stream;
  const unsigned nb = (unsigned)(((long long)nx * ny + 255) / 256);
  switch (precision) {
    case LBM_PREC_F64: k_pack<StoreF64><<<nb, 256, 0, st>>>(g, (double*)f, nx, ny, sy, rho0); break;
    case LBM_PREC_F32: k_pack<StoreF32><<<nb, 256, 0, st>>>(g, (float*)f, nx, ny, sy, rho0); break;
    case LBM_PREC_F16S:
    case LBM_PREC_F16SR: k_pack<StoreF16><<<nb, 256, 0, st>>>(g, (__half*)f, nx, ny, sy, rho0); break;
    case LBM_PREC_BF16S:
    case LBM_PREC_BF16SR:
      k_pack<StoreBF16><<<nb, 256, 0, st>>>(g, (__nv_bfloat16*)f, nx, ny, sy, rho0);
      break;
    case LBM_PREC_Q60: k_pack<StoreQ60><<<nb, 256, 0, st>>>(g, (long long*)f, nx, ny, sy, rho0); break;
    default: set_error("lbm_pack_f64: unknown precision %d", precision); return LBM_ERR_ARG;
  }
  LBM_CUDA_CHECK(cudaGetLastError(), "lbm_pack_f64");
  return LBM_OK;
}

extern "C" int lbm_unpack_f64(int precision, const void* f, double* g, int nx, int ny,
                              int row_pitch, double rho0, void* stream) {
  if (int rc = check_conv("lbm_unpack_f64", g, f, nx, ny, row_pitch)) return rc;
  const int sy = row_pitch > 0 ? row_pitch : ny;
  cudaStream_t st = (cudaStream_t)stream;
  const unsigned nb = (unsigned)(((long long)nx * ny + 255) / 256);
  switch (precision) {
    case LBM_PREC_F64:
      k_unpack<StoreF64><<<nb, 256, 0, st>>>((const double*)f, g, nx, ny, sy, rho0);
      break;
    case LBM_PREC_F32:
      k_unpack<StoreF32><<<nb, 256, 0, st>>>((const float*)f, g, nx, ny, sy, rho0);
      break;
    case LBM_PREC_F16S:
    case LBM_PREC_F16SR:
      k_unpack<StoreF16><<<nb, 256, 0, st>>>((const __half*)f, g, nx, ny, sy, rho0);
      break;
    case LBM_PREC_BF16S:
    case LBM_PREC_BF16SR:
      k_unpack<StoreBF16><<<nb, 256, 0, st>>>((const __nv_bfloat16*)f, g, nx, ny, sy, rho0);
      break;
    case LBM_PREC_Q60:
      k_unpack<StoreQ60><<<nb, 256, 0, st>>>((const long long*)f, g, nx, ny, sy, rho0);
      break;
    default: set_error("lbm_unpack_f64: unknown precision %d", precision); return LBM_ERR_ARG;
  }
  LBM_CUDA_CHECK(cudaGetLastError(), "lbm_unpack_f64");
  return LBM_OK;
}
