// Batched lattices: many independent lattices (uneven sizes, Reynolds
// numbers, geometry and boundary programs, one storage form) advanced
// together, one iteration per three launches, each a persistent kernel
// whose blocks pull tiles from an atomic work queue:
//
//   k_batch_bulk     tiles of bulk cells of every lattice (16-byte vector
//                    groups where ny % V == 0, single cells otherwise), or
//                    k_batch_bulk_tma: the TMA-staged persistent kernel of
//                    the 16-bit forms (lbm_tma.cuh) over every lattice's tiles
//   k_batch_special  tiles of special cells of every lattice
//   k_batch_drag     one block per (lattice, obstacle)
//
// The per-cell work is the single-lattice code of lbm_fused.cuh, reading the
// lattice's FusedArgs from a device array (one array per ping-pong parity),
// so a lattice advanced in a batch gives the same bits as when advanced alone.
// All lattices share one device iteration counter.
#include <string.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "lbm_fused.cuh"
#include "lbm_tma.cuh"

struct lbm_batch {
  int n_cases;
  int precision;
  lbm_batch_config cfg;
  int sm_count;
  lbm::FusedArgs* d_args;   // [2][n_cases]
  int4* d_bulk_tiles;       // (case, first, count, vectorised); TMA: (case, first cell, cells, 2)
  int n_bulk_tiles;
  int4* d_special_tiles;    // (case, first, count, links in the tile)
  int n_special_tiles;
  int2* d_drag_items;       // (case, obstacle)
  int n_drag_items;
  unsigned* d_queue;        // [0] bulk queue, [1] special queue, [2] step-done count
  long long* d_it;          // shared iteration counter
  int any_scalar;
  // graph cache (one per (n_steps, parity))
  std::vector<int> g_steps, g_parity;
  std::vector<cudaGraphExec_t> g_exec;
};

namespace lbm {
namespace {


// One vector group per thread per round; a tile is tile_rounds block-widths
// of groups (whole warps in every round: only a lattice's last tile is
// shorter, and the groups past the lattice's end are inactive).
template <class St, int V>
__device__ __forceinline__ void bulk_tile_vec(const FusedArgs& a, const int4& tl) {
  for (int g = 0; g < tl.z; g += blockDim.x) bulk_group_vec<St, V>(a, (long long)tl.y + g + threadIdx.x);
}

// VB: bytes per vector access (a group of VB / sizeof(element) cells per
// thread; lbm_batch_config.vec_bytes).  kVecOnly: every tile is a vector
// tile (no scalar path compiled in).
template <class St, int VB, bool kVecOnly>
__global__ void __launch_bounds__(256) k_batch_bulk(const FusedArgs* __restrict__ args,
                                                    const int4* __restrict__ tiles, int n_tiles,
                                                    unsigned* queue, long long* it_dev, int last) {
  constexpr int V = VB / (int)sizeof(typename St::S);
  if (blockIdx.x == 0 && threadIdx.x == 0)
    queue[1] = 0;  // the special phase of this iteration starts from tile 0
  // the next tile is taken while this one is processed
  __shared__ int t_sh;
  if (threadIdx.x == 0) t_sh = (int)atomicAdd(&queue[0], 1u);
  __syncthreads();
  for (int t = t_sh; t < n_tiles;) {
    int next = 0;
    if (threadIdx.x == 0) next = (int)atomicAdd(&queue[0], 1u);
    const int4 tl = tiles[t];
    const FusedArgs& a = args[tl.x];
    if (tl.w) {
      bulk_tile_vec<St, V>(a, tl);
    } else if (!kVecOnly) {
      for (int k = threadIdx.x; k < tl.z; k += blockDim.x)
        bulk_cell<St, LBM_MODE_STEP>(a, (long long)tl.y + k);
    }
    __syncthreads();
    if (threadIdx.x == 0) t_sh = next;
    __syncthreads();
    t = t_sh;
  }
  if (last) advance_counter(it_dev, queue + 2);
}

// Same work as k_batch_bulk with one block per tile (the hardware block
// scheduler distributes the tiles; no queue).
template <class St, int VB, bool kVecOnly>
__global__ void __launch_bounds__(256) k_batch_bulk_grid(const FusedArgs* __restrict__ args,
                                                         const int4* __restrict__ tiles,
                                                         unsigned* queue, long long* it_dev,
                                                         int last) {
  constexpr int V = VB / (int)sizeof(typename St::S);
  if (blockIdx.x == 0 && threadIdx.x == 0) queue[1] = 0;
  const int4 tl = tiles[blockIdx.x];
  const FusedArgs& a = args[tl.x];
  if (tl.w) {
    bulk_tile_vec<St, V>(a, tl);
  } else if (!kVecOnly) {
    for (int k = threadIdx.x; k < tl.z; k += blockDim.x)
      bulk_cell<St, LBM_MODE_STEP>(a, (long long)tl.y + k);
  }
  if (last) advance_counter(it_dev, queue + 2);
}

template <class St>
__global__ void __launch_bounds__(128, LBM_SPECIAL_MIN_BLOCKS) k_batch_special_grid(const FusedArgs* __restrict__ args,
                                                            const int4* __restrict__ tiles,
                                                            unsigned* queue, long long* it_dev,
                                                            int last) {
  if (blockIdx.x == 0 && threadIdx.x == 0) queue[0] = 0;
  const int4 tl = tiles[blockIdx.x];
  if ((int)threadIdx.x < tl.z) special_cell<St, LBM_MODE_STEP>(args[tl.x], tl.y + threadIdx.x);
  if (last) advance_counter(it_dev, queue + 2);
}

template <class St>
__global__ void __launch_bounds__(128, LBM_SPECIAL_MIN_BLOCKS) k_batch_special(const FusedArgs* __restrict__ args,
                                                       const int4* __restrict__ tiles, int n_tiles,
                                                       unsigned* queue, long long* it_dev,
                                                       int last) {
  // The next iteration's bulk queue (lbm_batch_create refuses the persistent
  // schedule for a batch without special tiles, where nothing would reset it).
  if (blockIdx.x == 0 && threadIdx.x == 0) queue[0] = 0;
  __shared__ int t_sh;
  if (threadIdx.x == 0) t_sh = (int)atomicAdd(&queue[1], 1u);
  __syncthreads();
  for (int t = t_sh; t < n_tiles;) {
    int next = 0;
    if (threadIdx.x == 0) next = (int)atomicAdd(&queue[1], 1u);
    const int4 tl = tiles[t];
    for (int k = threadIdx.x; k < tl.z; k += blockDim.x)
      special_cell<St, LBM_MODE_STEP>(args[tl.x], tl.y + k);
    __syncthreads();
    if (threadIdx.x == 0) t_sh = next;
    __syncthreads();
    t = t_sh;
  }
  if (last) advance_counter(it_dev, queue + 2);
}

// TMA-staged bulk phase: persistent blocks over every lattice's tiles (tiles
// of the largest lattices first, taken round-robin by block).
template <class St, class Sh>
__global__ void __launch_bounds__(Sh::kThreads, Sh::kMinBlocks) k_batch_bulk_tma(
    const FusedArgs* __restrict__ args, const int4* __restrict__ tiles, int n_tiles,
    unsigned* queue, long long* it_dev, int last) {
  if (blockIdx.x == 0 && threadIdx.x == 0)
    queue[1] = 0;  // the special phase of this iteration starts from tile 0
  const BatchTiles src{args, tiles};
  bulk_tma_body<St, Sh>(src, n_tiles, args[0].status);
  if (last) advance_counter(it_dev, queue + 2);
}

// One block of 256 threads per (lattice, obstacle) item.  It runs on a second
// stream after the special-cell kernel has advanced the shared counter
// (FusedArgs.drag_it_offset 2), beside the next iteration's bulk phase.
__global__ void __launch_bounds__(256) k_batch_drag(const FusedArgs* __restrict__ args,
                                                    const int2* __restrict__ items, int n_items) {
  if ((int)blockIdx.x < n_items) {
    const int2 it = items[blockIdx.x];
    drag_obstacle(args[it.x], it.y);
  }
}

// The TMA-staged bulk phase: as many persistent blocks as fit on the GPU.
template <class St, class Sh>
void launch_batch_tma(const lbm_batch* b, const FusedArgs* args, int last, cudaStream_t st) {
  static int per_sm[64] = {};
  const int slots =
      tma_prepare((const void*)k_batch_bulk_tma<St, Sh>, Sh::kThreads, Sh::kSmem, per_sm) *
      b->sm_count;
  k_batch_bulk_tma<St, Sh><<<b->n_bulk_tiles < slots ? b->n_bulk_tiles : slots, Sh::kThreads,
                             Sh::kSmem, st>>>(args, b->d_bulk_tiles, b->n_bulk_tiles, b->d_queue,
                                              b->d_it, last);
}

template <class St, int VB, bool kVecOnly>
void enqueue_store_vb(const lbm_batch* b, int n_steps, int parity, cudaStream_t st) {
  const int gb = b->sm_count * b->cfg.bulk_blocks_per_sm;
  const int gs = b->sm_count * b->cfg.special_blocks_per_sm;
  // The special-cell kernel (the bulk kernel without special cells)
  // advances the shared iteration counter; the drag kernel of iteration k
  // runs on a second stream beside the bulk phase of k + 1 and is waited for
  // by the special phase of k + 1, which rewrites the per-link terms.
  const bool drag = b->n_drag_items > 0, special = b->n_special_tiles > 0;
  const int bulk_last = !special, special_last = special;
  DragLane* lane = drag && LBM_DRAG_SIDE && n_steps > 1 ? drag_lane() : nullptr;
  bool drag_pending = false;
  auto wait_drag = [&]() {
    if (drag_pending) cudaStreamWaitEvent(st, lane->ev_drag, 0);
  };
  auto launch_drag = [&](const FusedArgs* args) {
    if (!drag) return;
    if (lane) {
      cudaEventRecord(lane->ev_special, st);
      cudaStreamWaitEvent(lane->sd, lane->ev_special, 0);
      k_batch_drag<<<b->n_drag_items, 256, 0, lane->sd>>>(args, b->d_drag_items, b->n_drag_items);
      cudaEventRecord(lane->ev_drag, lane->sd);
      drag_pending = true;
    } else {
      k_batch_drag<<<b->n_drag_items, 256, 0, st>>>(args, b->d_drag_items, b->n_drag_items);
    }
  };
  for (int k = 0; k < n_steps; ++k) {
    const FusedArgs* args = b->d_args + (size_t)((parity + k) & 1) * b->n_cases;
    if constexpr (sizeof(typename St::S) == 2 && St::kShift) {
      if (b->cfg.bulk_tma) {
        using Full = typename TmaShapeOf<St>::type;
        using Half = typename TmaHalf<Full>::type;
        if (b->cfg.bulk_tma == 2)
          launch_batch_tma<St, Half>(b, args, bulk_last, st);
        else
          launch_batch_tma<St, Full>(b, args, bulk_last, st);
        if (special) {
          wait_drag();
          if (b->cfg.persistent)
            k_batch_special<St><<<gs, 128, 0, st>>>(args, b->d_special_tiles, b->n_special_tiles,
                                                    b->d_queue, b->d_it, special_last);
          else
            k_batch_special_grid<St><<<b->n_special_tiles, 128, 0, st>>>(
                args, b->d_special_tiles, b->d_queue, b->d_it, special_last);
        }
        launch_drag(args);
        continue;
      }
    }
    if (b->cfg.persistent) {
      k_batch_bulk<St, VB, kVecOnly><<<gb, b->cfg.bulk_threads, 0, st>>>(
          args, b->d_bulk_tiles, b->n_bulk_tiles, b->d_queue, b->d_it, bulk_last);
      if (special) {
        wait_drag();
        k_batch_special<St><<<gs, 128, 0, st>>>(args, b->d_special_tiles, b->n_special_tiles,
                                                b->d_queue, b->d_it, special_last);
      }
    } else {
      k_batch_bulk_grid<St, VB, kVecOnly><<<b->n_bulk_tiles, b->cfg.bulk_threads, 0, st>>>(
          args, b->d_bulk_tiles, b->d_queue, b->d_it, bulk_last);
      if (special) {
        wait_drag();
        k_batch_special_grid<St><<<b->n_special_tiles, 128, 0, st>>>(
            args, b->d_special_tiles, b->d_queue, b->d_it, special_last);
      }
    }
    launch_drag(args);
  }
  if (drag_pending) cudaStreamWaitEvent(st, lane->ev_drag, 0);  // join
}

template <class St>
void enqueue_store(const lbm_batch* b, int n_steps, int parity, cudaStream_t st) {
  if (b->cfg.vec_bytes == 8) {
    if (b->any_scalar) enqueue_store_vb<St, 8, false>(b, n_steps, parity, st);
    else enqueue_store_vb<St, 8, true>(b, n_steps, parity, st);
  } else {
    if (b->any_scalar) enqueue_store_vb<St, 16, false>(b, n_steps, parity, st);
    else enqueue_store_vb<St, 16, true>(b, n_steps, parity, st);
  }
}

int batch_enqueue(const lbm_batch* b, int n_steps, int parity, cudaStream_t st) {
  switch (b->precision) {
    case LBM_PREC_F64: enqueue_store<StoreF64>(b, n_steps, parity, st); break;
    case LBM_PREC_F32: enqueue_store<StoreF32>(b, n_steps, parity, st); break;
    case LBM_PREC_F16S: enqueue_store<StoreF16>(b, n_steps, parity, st); break;
    case LBM_PREC_Q60: enqueue_store<StoreQ60>(b, n_steps, parity, st); break;
    case LBM_PREC_F16SR: enqueue_store<StoreF16SR>(b, n_steps, parity, st); break;
    case LBM_PREC_BF16SR: enqueue_store<StoreBF16SR>(b, n_steps, parity, st); break;
    default: enqueue_store<StoreBF16>(b, n_steps, parity, st); break;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("lbm_batch: launch failed: %s", cudaGetErrorString(e));
    return LBM_ERR_CUDA;
  }
  return LBM_OK;
}

// queue[0]: bulk tile queue, [1]: special tile queue, [2]: step-done count.
__global__ void k_batch_set_it(long long* it, long long v, unsigned* queue) {
  *it = v;
  queue[0] = 0;
  queue[1] = 0;
  queue[2] = 0;
}

void batch_free(lbm_batch* b) {
  if (!b) return;
  for (auto e : b->g_exec) cudaGraphExecDestroy(e);
  cudaFree(b->d_args);
  cudaFree(b->d_bulk_tiles);
  cudaFree(b->d_special_tiles);
  cudaFree(b->d_drag_items);
  cudaFree(b->d_queue);
  cudaFree(b->d_it);
  delete b;
}

}  // namespace
}  // namespace lbm

using namespace lbm;

extern "C" int lbm_batch_create(lbm_batch** out, const lbm_problem* cases, int32_t n_cases,
                                const lbm_batch_config* cfg) {
  if (!out || !cases || n_cases < 1 || !cfg) {
    set_error("lbm_batch_create: bad arguments");
    return LBM_ERR_ARG;
  }
  *out = nullptr;
  if (cfg->bulk_threads < 32 || cfg->bulk_threads > 256 || cfg->bulk_threads % 32 ||
      cfg->bulk_blocks_per_sm < 1 || cfg->bulk_blocks_per_sm > 32 ||
      cfg->special_blocks_per_sm < 1 || cfg->special_blocks_per_sm > 32 ||
      cfg->scalar_tile_cells < 32 || cfg->scalar_tile_cells > (1 << 20) ||
      (cfg->persistent != 0 && cfg->persistent != 1) ||
      (cfg->vec_bytes != 8 && cfg->vec_bytes != 16) || cfg->tile_rounds < 1 ||
      cfg->tile_rounds > 64 || cfg->bulk_tma < 0 || cfg->bulk_tma > 2) {
    set_error("lbm_batch_create: bad config (threads %d, blocks/SM %d/%d, tile %d)",
              cfg->bulk_threads, cfg->bulk_blocks_per_sm, cfg->special_blocks_per_sm,
              cfg->scalar_tile_cells);
    return LBM_ERR_ARG;
  }
  const int prec = cases[0].precision;
  for (int c = 0; c < n_cases; ++c) {
    if (int rc = problem_check(&cases[c], "lbm_batch_create")) return rc;
    if (cases[c].precision != prec) {
      set_error("lbm_batch_create: lattice %d has another storage form", c);
      return LBM_ERR_ARG;
    }
  }
  const int V = (prec == LBM_PREC_F64 || prec == LBM_PREC_Q60)
                    ? 1
                    : cfg->vec_bytes / (prec == LBM_PREC_F32 ? 4 : 2);
  const int tma_cells = cfg->bulk_tma ? tma_tile_cells(prec, cfg->bulk_tma == 2) : 0;
  if (cfg->bulk_tma && !tma_cells) {
    set_error("lbm_batch_create: bulk_tma needs a 16-bit storage form");
    return LBM_ERR_ARG;
  }
  std::vector<FusedArgs> args(2 * (size_t)n_cases);
  std::vector<int4> bulk, special;
  std::vector<int2> drag;
  // Largest lattices first: their tiles are taken early, so the queue ends
  // with small lattices and the last blocks finish together.
  std::vector<int> order(n_cases);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    return (long long)cases[x].nx * cases[x].ny > (long long)cases[y].nx * cases[y].ny;
  });
  for (int c : order) {
    const lbm_problem& p = cases[c];
    for (int par = 0; par < 2; ++par) {
      FusedArgs a = make_args(&p, LBM_MODE_STEP, LBM_FLAG_CHECK_FINITE);
      a.fin = p.f[par];
      a.fout = p.f[par ^ 1];
      a.advance_at = -1;  // the batch kernels advance the shared counter
      a.drag_it_offset = 2;  // k_batch_drag runs after the special phase advanced it
      a.write_macro = 0;
      args[(size_t)par * n_cases + c] = a;
    }
    const int sy = p.row_pitch > 0 ? p.row_pitch : p.ny;
    const long long N = (long long)p.nx * sy;  // storage cells, padding included
    if (tma_cells) {
      if (sy % 8) {
        set_error("lbm_batch_create: bulk_tma needs rows padded to 16 bytes (lattice %d)", c);
        return LBM_ERR_ARG;
      }
      // the interior columns 1 .. nx-2, tma_cells per tile
      for (long long x = sy; x < N - sy; x += tma_cells)
        bulk.push_back(make_int4(c, (int)x, (int)std::min<long long>(tma_cells, N - sy - x), 2));
    } else if (V > 1 && sy % V == 0) {
      const long long groups = (long long)p.nx * (sy / V);
      // tile_rounds block-widths of groups per tile
      const int tg = cfg->bulk_threads * cfg->tile_rounds;
      for (long long g = 0; g < groups; g += tg)
        bulk.push_back(make_int4(c, (int)g, (int)std::min<long long>(tg, groups - g), 1));
    } else {
      for (long long x = 0; x < N; x += cfg->scalar_tile_cells)
        bulk.push_back(make_int4(c, (int)x, (int)std::min<long long>(cfg->scalar_tile_cells, N - x), 0));
    }
    // special tiles carry their number of links (w), the longest chains
    std::vector<int> link_start((size_t)p.n_special + 1, 0);
    if (p.n_links > 0 &&
        cudaMemcpy(link_start.data(), p.special_link_start, link_start.size() * sizeof(int),
                   cudaMemcpyDeviceToHost) != cudaSuccess)
      std::fill(link_start.begin(), link_start.end(), 0);
    for (int s = 0; s < p.n_special; s += 128) {
      const int n = std::min(128, p.n_special - s);
      special.push_back(make_int4(c, s, n, link_start[s + n] - link_start[s]));
    }
    if (p.drag_hist && p.n_links > 0)
      for (int o = 0; o < p.n_obstacles; ++o) drag.push_back(make_int2(c, o));
  }
  // Special tiles with the most links first (stable): their chains are the
  // longest, so they start in the first wave and the short wall tiles fill
  // in behind them.
#ifndef LBM_SPECIAL_TILE_ORDER
#define LBM_SPECIAL_TILE_ORDER 1
#endif
  if (LBM_SPECIAL_TILE_ORDER)
    std::stable_sort(special.begin(), special.end(),
                     [](const int4& x, const int4& y) { return x.w > y.w; });
  // The persistent bulk kernel's tile queue (queue[0]) is reset for the next
  // iteration by the special-cell kernel, so that schedule needs special
  // tiles.  Every lattice has them today (problem_check asks for at least the
  // wall cells), and this check keeps that dependency explicit.
  if (cfg->persistent && special.empty()) {
    set_error("lbm_batch_create: the persistent schedule needs special cells in some lattice");
    return LBM_ERR_ARG;
  }
  lbm_batch* b = new lbm_batch();
  b->n_cases = n_cases;
  b->precision = prec;
  b->cfg = *cfg;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, dev);
  b->any_scalar = 0;
  for (const int4& t : bulk) b->any_scalar |= t.w == 0;
  b->n_bulk_tiles = (int)bulk.size();
  b->n_special_tiles = (int)special.size();
  b->n_drag_items = (int)drag.size();
  cudaError_t e = cudaSuccess;
  auto alloc_copy = [&](void** dst, const void* src, size_t bytes) {
    if (e != cudaSuccess) return;
    e = cudaMalloc(dst, bytes > 0 ? bytes : 16);
    if (e == cudaSuccess && bytes > 0) e = cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
  };
  alloc_copy((void**)&b->d_args, args.data(), args.size() * sizeof(FusedArgs));
  alloc_copy((void**)&b->d_bulk_tiles, bulk.data(), bulk.size() * sizeof(int4));
  alloc_copy((void**)&b->d_special_tiles, special.data(), special.size() * sizeof(int4));
  alloc_copy((void**)&b->d_drag_items, drag.data(), drag.size() * sizeof(int2));
  if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_queue, 4 * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemset(b->d_queue, 0, 4 * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_it, sizeof(long long));
  if (e == cudaSuccess) e = cudaMemset(b->d_it, 0, sizeof(long long));
  if (e != cudaSuccess) {
    set_error("lbm_batch_create: %s", cudaGetErrorString(e));
    batch_free(b);
    return LBM_ERR_CUDA;
  }
  // Every lattice reads the shared counter.
  for (auto& a : args) {
    a.it_dev = b->d_it;
    a.step_done = b->d_queue + 2;
  }
  e = cudaMemcpy(b->d_args, args.data(), args.size() * sizeof(FusedArgs), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    set_error("lbm_batch_create: %s", cudaGetErrorString(e));
    batch_free(b);
    return LBM_ERR_CUDA;
  }
  *out = b;
  return LBM_OK;
}

extern "C" int lbm_batch_destroy(lbm_batch* b) {
  batch_free(b);
  return LBM_OK;
}

extern "C" int lbm_batch_info(const lbm_batch* b, int64_t* out6) {
  if (!b || !out6) { set_error("lbm_batch_info: bad arguments"); return LBM_ERR_ARG; }
  out6[0] = b->n_cases;
  out6[1] = b->n_bulk_tiles;
  out6[2] = b->n_special_tiles;
  out6[3] = b->n_drag_items;
  out6[4] = b->sm_count;
  out6[5] = 1 + (b->n_special_tiles > 0 ? 1 : 0) + (b->n_drag_items > 0 ? 1 : 0);
  return LBM_OK;
}

extern "C" int lbm_batch_advance(lbm_batch* b, int64_t it0, int n_steps, int parity,
                                 void* stream) {
  if (!b || n_steps < 1 || (parity != 0 && parity != 1)) {
    set_error("lbm_batch_advance: bad arguments");
    return LBM_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  k_batch_set_it<<<1, 1, 0, st>>>(b->d_it, it0, b->d_queue);
  return batch_enqueue(b, n_steps, parity, st);
}

extern "C" int lbm_batch_advance_graph(lbm_batch* b, int64_t it0, int n_steps, int parity,
                                       void* stream) {
  if (!b || n_steps < 1 || (parity != 0 && parity != 1)) {
    set_error("lbm_batch_advance_graph: bad arguments");
    return LBM_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  cudaGraphExec_t exec = nullptr;
  for (size_t k = 0; k < b->g_exec.size(); ++k)
    if (b->g_steps[k] == n_steps && b->g_parity[k] == parity) exec = b->g_exec[k];
  if (!exec) {
    cudaStream_t cs;
    LBM_CUDA_CHECK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "lbm_batch_advance_graph");
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
      cudaStreamDestroy(cs);
      set_error("lbm_batch_advance_graph: begin capture: %s", cudaGetErrorString(e));
      return LBM_ERR_CUDA;
    }
    int rc = batch_enqueue(b, n_steps, parity, cs);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(cs, &g);
    cudaStreamDestroy(cs);
    if (rc != LBM_OK) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      set_error("lbm_batch_advance_graph: %s", cudaGetErrorString(e));
      return LBM_ERR_CUDA;
    }
    b->g_steps.push_back(n_steps);
    b->g_parity.push_back(parity);
    b->g_exec.push_back(exec);
  }
  k_batch_set_it<<<1, 1, 0, st>>>(b->d_it, it0, b->d_queue);
  LBM_CUDA_CHECK(cudaGetLastError(), "lbm_batch_advance_graph");
  LBM_CUDA_CHECK(cudaGraphLaunch(exec, st), "lbm_batch_advance_graph: launch");
  return LBM_OK;
}
