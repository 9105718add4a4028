// TMA-staged bulk update of the 16-bit storage forms, shared by the
// single-lattice kernel (lbm_fused.cu) and the batched one (lbm_batch.cu).
//
// A persistent kernel: block b takes tiles b, b + gridDim.x, ... of at most
// Sh::kCells consecutive storage cells of one lattice's interior columns
// (1 .. nx-2).  For a tile of len cells starting at cell c0, the pull sources
// of plane q are the cells c0 - c_x sy - c_y + [0, len): one producer thread
// copies the range c0 - c_x sy + [-8, len + 8) of each plane (one 16-byte
// vector of halo on either side, clipped to the plane) from HBM into a
// shared-memory stage with cp.async.bulk, which completes on the stage's
// `full` mbarrier.  The stages rotate, so several tiles' loads are in flight
// while the consumer warps work: each consumer thread reads its group's nine
// vectors and six halo cells from the stage, arrives on the stage's `empty`
// mbarrier (batched tiles: after the update, see BatchTiles), and runs
// bulk_group_vec_update (the update of the register-pipelined kernel, so
// both give the same bits).  Every wait is bounded (kWaitNs): a wait that
// runs out sets status bit 3 and the thread leaves its loop.  Before the
// block exits, the producer waits (bounded) for the last copies it issued,
// so that none lands in a freed block (LBM_FLAG_TEST_STALL exercises that
// path).
//
// Alignment: lattice rows are padded to a multiple of 8 elements (16 bytes),
// so c0, len, sy and the plane size are multiples of 8 elements; every copy
// starts and ends on a 16-byte boundary of the plane (the planes start on
// 256-byte boundaries) and of its stage row (rows of kRow elements, kRow a
// multiple of 8, at offset 0 or 8).
#pragma once

#include "lbm_fused.cuh"

namespace lbm {

constexpr int kTmaBarBytes = 128;  // the stages' mbarriers
constexpr unsigned long long kWaitNs = 500ull * 1000 * 1000;

// Shape of the kernel: W consumer warps of V cells per thread (tiles of
// W * 32 * V cells), NST stages, plus one producer warp; compiled for MB
// resident blocks per SM.  Each plane's copy is widened by kHalo elements
// (16 bytes) on either side.
template <int W, int V, int NST, int MB = 1>
struct TmaShape {
  static constexpr int kWarps = W, kV = V, kStages = NST, kMinBlocks = MB;
  static constexpr int kConsumers = W * 32;
  static constexpr int kThreads = kConsumers + 32;
  static constexpr int kCells = kConsumers * V;
  static constexpr int kHalo = 8;
  static constexpr int kRow = kCells + 2 * kHalo;  // elements per plane and stage
  // barriers | one FusedArgs per stage (batched tiles) | stages
  static constexpr size_t kArgsBytes = (size_t)NST * sizeof(FusedArgs);
  static constexpr size_t kSmem = kTmaBarBytes + kArgsBytes + (size_t)NST * 9 * kRow * 2;
  static_assert(16 * NST <= kTmaBarBytes, "two mbarriers per stage");
  static_assert(kSmem <= 227 * 1024, "stages exceed the shared memory of a block");
  static_assert(V == 4 || V == 8, "8- or 16-byte vectors");
};
// Per form, the fastest shape measured on 8192x2048 (bulk kernel, us per
// launch; the register-pipelined kernel in brackets): FP16 8 warps x 8 cells,
// 4 stages of 37 KB: 95.9 (104.4); BF16 12 x 4, 6 stages of 28 KB: 97.7
// (104.3); FP16 and BF16 with stochastic rounding 16 x 4, 4 stages of
// 37 KB: 97.0 (109.2) and 96.9 (111.0).  One block per SM in each case.
#if defined(LBM_TMA_WARPS)  // one shape for every form (tuning builds)
template <class St>
struct TmaShapeOf {
  using type = TmaShape<LBM_TMA_WARPS, LBM_TMA_V, LBM_TMA_STAGES>;
};
#else
template <class St>
struct TmaShapeOf {
  using type = TmaShape<16, 4, 4>;
};
template <>
struct TmaShapeOf<StoreF16> {
  using type = TmaShape<8, 8, 4>;
};
template <>
struct TmaShapeOf<StoreBF16> {
  using type = TmaShape<12, 4, 6>;
};
#endif
// Half the consumer warps of the form's shape (tiles half as long, half the
// shared memory): two blocks per SM, which leaves room for the blocks of
// another batch's kernels beside them (batches advanced concurrently).
template <class Sh>
struct TmaHalf {
  using type = TmaShape<Sh::kWarps / 2, Sh::kV, Sh::kStages, 2>;
};

__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Wait for the phase of the given parity to complete; false after kWaitNs.
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  do {
    if (mbar_try_wait(bar, parity)) return true;
  } while (global_ns() - t0 < kWaitNs);
  return false;
}
// HBM -> shared memory bulk copy (16-byte aligned addresses, size a multiple
// of 16), completing `bytes` of transaction count on bar.
__device__ __forceinline__ void bulk_load(unsigned dst, const void* src, unsigned bytes,
                                          unsigned bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}

// Source range of plane q for the tile at c0 (len cells), clipped to the
// plane: [lo, hi) in plane elements, and where lo lands in the stage row.
struct TmaRange {
  long long lo, hi;
  int dst;
};
__device__ __forceinline__ TmaRange tma_range(int q, long long c0, long long len, int sy,
                                              long long Ns, int halo) {
  const long long s0 = c0 - (long long)cx(q) * sy - halo;
  TmaRange r;
  r.lo = s0 < 0 ? 0 : s0;
  const long long h = s0 + len + 2 * halo;
  r.hi = h > Ns ? Ns : h;
  r.dst = (int)(r.lo - s0);
  return r;
}

static_assert(sizeof(FusedArgs) % 16 == 0, "FusedArgs records are copied with cp.async.bulk");

// Tiles of one lattice: kCells consecutive cells from column 1's first cell.
// The lattice's FusedArgs is the kernel parameter.
template <class Sh>
struct LatticeTiles {
  static constexpr bool kStageArgs = false;
  const FusedArgs& a;
  long long c_begin, c_end;
  __device__ __forceinline__ const FusedArgs& args(int) const { return a; }
  __device__ __forceinline__ long long first(int t) const {
    return c_begin + (long long)t * Sh::kCells;
  }
  __device__ __forceinline__ int count(int t) const {
    const long long left = c_end - first(t);
    return left < Sh::kCells ? (int)left : Sh::kCells;
  }
};

// Tiles of a batch: (lattice, first cell, cells, -) records.  The producer
// copies each tile's FusedArgs into its stage with the populations, so that
// the consumers read it from shared memory (read from global memory, every
// field would be loaded again after each store: the compiler cannot tell
// the records from the distributions they point to).
struct BatchTiles {
  static constexpr bool kStageArgs = true;
  const FusedArgs* a;
  const int4* tiles;
  __device__ __forceinline__ const FusedArgs& args(int t) const { return a[tiles[t].x]; }
  __device__ __forceinline__ long long first(int t) const { return tiles[t].y; }
  __device__ __forceinline__ int count(int t) const { return tiles[t].z; }
};

// Barrier set-up of a TMA-staged block: a `full` mbarrier per stage (one
// arrival, the producer's, plus the copies' bytes) and an `empty` one (one
// arrival per consumer thread).  Every thread calls it.
template <class Sh>
__device__ __forceinline__ void tma_init(unsigned full0, unsigned empty0) {
  if (threadIdx.x == 0) {
    for (int s = 0; s < Sh::kStages; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, Sh::kConsumers);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
}

// The producer thread: for tile k of this block, wait until the consumers
// have released stage k % NST, then copy the tile's nine source ranges (and,
// with Src::kStageArgs, its FusedArgs) into it.
template <class S, class Sh, class Src>
__device__ __forceinline__ void tma_produce(const Src& src, int n_tiles, unsigned* status,
                                            unsigned full0, unsigned empty0, S* stage,
                                            FusedArgs* stage_args) {
  constexpr int NST = Sh::kStages, kRow = Sh::kRow;
  constexpr bool kStageArgs = Src::kStageArgs;
  int k = 0;
  bool ok = true;
  for (int t = blockIdx.x; t < n_tiles; t += gridDim.x, ++k) {
    const int s = k % NST;
    if (k >= NST && !mbar_wait(empty0 + 8 * s, ((k / NST) - 1) & 1)) {
      ok = false;
      break;
    }
    const FusedArgs& a = src.args(t);
    if (a.tma_stall && k == 0) continue;  // failure-path test: tile 0 never arrives
    const S* fin = (const S*)a.fin;
    const long long Ns = a.Ns, c0 = src.first(t);
    const int sy = a.sy, len = src.count(t);
    unsigned bytes = kStageArgs ? (unsigned)sizeof(FusedArgs) : 0u;
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      const TmaRange r = tma_range(q, c0, len, sy, Ns, Sh::kHalo);
      bytes += (unsigned)(r.hi - r.lo) * (unsigned)sizeof(S);
    }
    mbar_expect_tx(full0 + 8 * s, bytes);
    if (kStageArgs)
      bulk_load(smem_addr(stage_args + s), &a, (unsigned)sizeof(FusedArgs), full0 + 8 * s);
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      const TmaRange r = tma_range(q, c0, len, sy, Ns, Sh::kHalo);
      bulk_load(smem_addr(stage + (size_t)(s * 9 + q) * kRow + r.dst), fin + q * Ns + r.lo,
                (unsigned)(r.hi - r.lo) * (unsigned)sizeof(S), full0 + 8 * s);
    }
  }
  if (!ok && status) atomicOr(status, 8u);
  // The block must not exit with copies in flight: wait (bounded) for the
  // last tiles issued into each stage.  After a normal run the consumers
  // have waited for them already and these waits return at once; after a
  // consumer gave up they keep the copies from landing in a freed block.
  for (int kk = k - NST < 0 ? 0 : k - NST; kk < k; ++kk)
    mbar_wait(full0 + 8 * (kk % NST), (kk / NST) & 1);
}

// The kernel body; every thread of the block calls it.  status: where a
// timed-out wait is reported.
template <class St, class Sh, class Src>
__device__ __forceinline__ void bulk_tma_body(const Src& src, int n_tiles, unsigned* status) {
  using S = typename St::S;
  using T = typename St::T;
  constexpr int V = Sh::kV, NST = Sh::kStages, kConsumers = Sh::kConsumers, kRow = Sh::kRow;
  constexpr int kHalo = Sh::kHalo;
  using P = Pack<S, V>;
  static_assert(sizeof(S) == 2, "16-bit storage forms only");
  constexpr bool kStageArgs = Src::kStageArgs;
  extern __shared__ __align__(128) unsigned char smem[];
  const unsigned full0 = smem_addr(smem), empty0 = full0 + 8 * NST;
  FusedArgs* stage_args = reinterpret_cast<FusedArgs*>(smem + kTmaBarBytes);
  S* stage = reinterpret_cast<S*>(smem + kTmaBarBytes + Sh::kArgsBytes);
  const int tid = threadIdx.x;
  tma_init<Sh>(full0, empty0);
  if (tid == kConsumers) {
    tma_produce<S, Sh>(src, n_tiles, status, full0, empty0, stage, stage_args);
  } else if (tid < kConsumers) {
    int k = 0;
    for (int t = blockIdx.x; t < n_tiles; t += gridDim.x, ++k) {
      const int s = k % NST;
      if (!mbar_wait(full0 + 8 * s, (k / NST) & 1)) {
        if (status) atomicOr(status, 8u);
        break;
      }
      const FusedArgs& a = kStageArgs ? stage_args[s] : src.args(t);
      const int sy = a.sy;
      const int off = tid * V;
      const long long c = src.first(t) + off;
      const bool act = off < src.count(t);
      const int i = (int)(c / sy);
      const int j0 = (int)(c - (long long)i * sy);
      P in[9];
      T halo[9];
#pragma unroll
      for (int q = 0; q < 9; ++q) {
        const S* row = stage + (size_t)(s * 9 + q) * kRow + kHalo + off;
        if (act) in[q] = *reinterpret_cast<const P*>(row);
        if (cy(q) == 1)  // cell j0 pulls from j0 - 1 (zero at a column start)
          halo[q] = act && j0 > 0 ? St::load(row - 1) : T(0);
        else if (cy(q) == -1)  // cell j0 + V - 1 pulls from j0 + V (zero past the column)
          halo[q] = act && j0 + V < sy ? St::load(row + V) : T(0);
        else
          halo[q] = T(0);
      }
      // With the FusedArgs in the stage, the stage is released after the
      // update (its record is read until then), else as soon as the
      // populations are in registers.
      if (!kStageArgs) mbar_arrive(empty0 + 8 * s);
      if (act) bulk_group_vec_update<St, V>(a, i, j0, in, halo);
      if (kStageArgs) mbar_arrive(empty0 + 8 * s);
    }
  }
}

// Host: SMs of the current device (cached per device).
inline int device_sm_count() {
  static int count[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return 1;
  if (!count[dev]) {
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    count[dev] = n > 0 ? n : 1;
  }
  return count[dev];
}

// Host: opts a TMA-staged kernel into its dynamic shared memory and returns
// how many of its blocks fit on one SM (once per device; cache[64] per
// kernel).
inline int tma_prepare(const void* kernel, int threads, size_t smem, int* cache) {
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return 1;
  if (!cache[dev]) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, smem);
    cache[dev] = n > 0 ? n : 1;
  }
  return cache[dev];
}

// Cells per tile of the form's TMA-staged kernel (half: of its half-width
// shape; 0: the form has none).
int tma_tile_cells(int precision, bool half = false);

}  // namespace lbm
