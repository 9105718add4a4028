// Device-side work units of the fused lattice update, shared by the
// single-lattice kernels (lbm_fused.cu) and the batched persistent kernels
// (lbm_batch.cu).  See lbm_fused.cu for the scheme.
#pragma once
#include <type_traits>

#include "lbm_device.cuh"
#include "lbm_internal.h"

namespace lbm {

struct alignas(16) FusedArgs {
  int nx, ny;
  long long N;          // nx * ny: plane size of the FP64 reference-layout arrays
  int sy;               // row pitch of the distribution storage (>= ny)
  long long Ns;         // nx * sy: plane size of the distribution storage
  Coef<double> kd;
  Coef<float> kf;
  CoefQ60 kq;
  const void* fin;
  void* fout;
  // BC program
  int n_wall_ops;
  int wall_ops[5];
  int n_corner_ops;
  int corner_ops[4];
  int corner_nb_special[4];
  int corner_special[4];
  int ibb;
  // BC vectors: value(it) = base + scale[it - scale_it0] * vec
  const double* bc_base;
  const double* bc_vec;
  const double* bc_scale;
  long long bc_scale_it0, bc_scale_len;
  // Device iteration counter: the iteration whose collision the running step
  // does.  The step's last kernel advances it when its last block finishes
  // (advance_counter), so every kernel of a step reads the same value and a
  // captured graph replays correctly from any starting iteration.
  long long* it_dev;
  unsigned* step_done;  // blocks of the last kernel that have finished
  int advance_at;       // kernel that advances: 0 bulk, 1 special, 2 drag, -1 none
  // special cells / links
  int n_special;
  const int* special_cell;
  const int* special_link_start;
  const int* special_link_ids;
  const int* link_cell;
  const int* link_q;
  const int* link_nb1;
  const int* link_nb2;
  const double* link_p;
  const double* link_coef;  // [3][n_links] IBB coefficients, or NULL
  // scratch: halves alternate with the parity of the iteration number
  double* stale[2];         // [9][n_special] post-BC g of an iteration
  double* mac[2];           // [3][n_special] macro rho, ux, uy of an iteration
  double* link_force;       // [2][n_links]
  int n_links;
  // drag/lift history
  double* drag_hist;
  long long drag_cap;
  // 1: the drag kernel runs before the step advances the iteration counter;
  // 2: after (on a second stream, beside the next step's bulk kernel)
  int drag_it_offset;
  int n_obs;
  const int* obs_start;
  // outputs
  double* rho_out;
  double* u_out;
  double* g_out;
  unsigned* status;
  int bulk_tma;  // 16-bit forms: TMA-staged bulk kernel (else register-pipelined)
  int tma_stall;  // LBM_FLAG_TEST_STALL: the producer withholds each block's first tile
  int mode;
  int write_macro;
  int wall_macro;
  int check_finite;
};

// Called by every block of a step's last kernel after its work: the last
// block to arrive advances the iteration counter.  Every block has read the
// counter before it arrives; no block waits for another.
__device__ __forceinline__ void advance_counter(long long* it_dev, unsigned* done) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned n = gridDim.x * gridDim.y * gridDim.z;
    if (atomicAdd(done, 1u) == n - 1) {
      *done = 0;
      *it_dev += 1;
      __threadfence();
    }
  }
}

template <typename T>
__device__ __forceinline__ const Coef<T>& coef(const FusedArgs& a);
template <>
__device__ __forceinline__ const Coef<double>& coef<double>(const FusedArgs& a) { return a.kd; }
template <>
__device__ __forceinline__ const Coef<float>& coef<float>(const FusedArgs& a) { return a.kf; }

// Scale of the BC vectors at iteration bc_it (status bit 1 if not covered).
__device__ __forceinline__ double bc_scale_at(const FusedArgs& a, long long bc_it) {
  if (!a.bc_vec) return 0.0;
  long long idx = bc_it - a.bc_scale_it0;
  if (idx < 0 || idx >= a.bc_scale_len) {
    if (a.status) atomicOr(a.status, 2u);
    return 0.0;
  }
  return a.bc_scale[idx];
}

__device__ __forceinline__ double bc_value(const FusedArgs& a, double s, int off) {
  double b = a.bc_base[off];
  return a.bc_vec ? fma(s, a.bc_vec[off], b) : b;
}

// ---------------------------------------------------------------------------
// Bulk kernel: every non-wall cell.
// ---------------------------------------------------------------------------
// Bulk cell of the Q3.60 form (LBM_MODE_STEP): pull the 9 integers,
// integer collision (collide_q60), store the 9 integers.  A cell outside the
// range of the form stores kQ60Bad (NaN when converted back) and sets status
// bit 0 when finite checks are on.
__device__ __forceinline__ void q60_collide_store(const FusedArgs& a, int i, int j,
                                                  long long cell, long long (&x)[9]);

__device__ __forceinline__ void bulk_q60_ij(const FusedArgs& a, int i, int j) {
  if (i <= 0 || i >= a.nx - 1 || j <= 0 || j >= a.ny - 1) return;
  const long long Ns = a.Ns, sy = a.sy;
  const long long cell = (long long)i * sy + j;
  const long long* fin = (const long long*)a.fin;
  long long x[9];
  x[0] = __ldg(fin + cell);
  x[1] = __ldg(fin + 1 * Ns + cell - sy);
  x[2] = __ldg(fin + 2 * Ns + cell + sy);
  x[3] = __ldg(fin + 3 * Ns + cell - 1);
  x[4] = __ldg(fin + 4 * Ns + cell + 1);
  x[5] = __ldg(fin + 5 * Ns + cell - sy - 1);
  x[6] = __ldg(fin + 6 * Ns + cell + sy + 1);
  x[7] = __ldg(fin + 7 * Ns + cell + sy - 1);
  x[8] = __ldg(fin + 8 * Ns + cell - sy + 1);
  q60_collide_store(a, i, j, cell, x);
}

// Integer collision of interior cell (i, j) from its nine pulled populations
// and the stores (shared by the register-pipelined and TMA-staged kernels).
__device__ __forceinline__ void q60_collide_store(const FusedArgs& a, int i, int j,
                                                  long long cell, long long (&x)[9]) {
  const long long Ns = a.Ns;
  long long rho, jx, jy;
  const bool ok = collide_q60(x, a.kq, rho, jx, jy);
  if (a.write_macro) {
    const long long rc = (long long)i * a.ny + j;
    const double r = ok ? q60_to_double(rho) : q60_to_double(kQ60Bad);
    a.rho_out[rc] = r;
    a.u_out[rc] = q60_to_double(jx) / r;
    a.u_out[a.N + rc] = q60_to_double(jy) / r;
  }
  if (!ok) {
    if (a.check_finite) atomicOr(a.status, 1u);
#pragma unroll
    for (int q = 0; q < 9; ++q) x[q] = kQ60Bad;
  }
  long long* fout = (long long*)a.fout;
#pragma unroll
  for (int q = 0; q < 9; ++q) fout[q * Ns + cell] = x[q];
}

__device__ __forceinline__ void bulk_cell_q60(const FusedArgs& a, long long cell) {
  const int i = (int)(cell / a.sy);
  bulk_q60_ij(a, i, (int)(cell - (long long)i * a.sy));
}

template <class St, int MODE>
__device__ __forceinline__ void bulk_cell(const FusedArgs& a, long long cell) {
  using S = typename St::S;
  using T = typename St::T;
  if constexpr (St::kFixed && MODE == LBM_MODE_STEP) {
    bulk_cell_q60(a, cell);
    return;
  }
  // cell: index in the storage layout (i * sy + j); padding cells j >= ny
  // are skipped.  Reference-layout arrays (g_out, rho_out, u_out) use
  // rc = i * ny + j.
  const long long N = a.N, Ns = a.Ns;
  const int i = (int)(cell / a.sy);
  const int j = (int)(cell - (long long)i * a.sy);
  if (j >= a.ny) return;
  const long long rc = (long long)i * a.ny + j;
  const S* fin = (const S*)a.fin;
  const Coef<T>& k = coef<T>(a);
  T d[9];
  if (MODE == LBM_MODE_COLLIDE_FROM_G) {
    // Input is the full post-BC g (FP64) of every cell, edges included.
#pragma unroll
    for (int q = 0; q < 9; ++q)
      d[q] = St::kShift ? (T)(a.g_out[q * N + rc] - wgt(q) * a.kd.rho0) * St::kScale
                        : (T)a.g_out[q * N + rc];
  } else {
    if (i == 0 || i == a.nx - 1 || j == 0 || j == a.ny - 1) return;
    const long long sy = a.sy;
    d[0] = St::load(fin + cell);
    d[1] = St::load(fin + 1 * Ns + cell - sy);
    d[2] = St::load(fin + 2 * Ns + cell + sy);
    d[3] = St::load(fin + 3 * Ns + cell - 1);
    d[4] = St::load(fin + 4 * Ns + cell + 1);
    d[5] = St::load(fin + 5 * Ns + cell - sy - 1);
    d[6] = St::load(fin + 6 * Ns + cell + sy + 1);
    d[7] = St::load(fin + 7 * Ns + cell + sy - 1);
    d[8] = St::load(fin + 8 * Ns + cell - sy + 1);
    if (MODE == LBM_MODE_FINISH) {
#pragma unroll
      for (int q = 0; q < 9; ++q)
        a.g_out[q * N + rc] = (double)(St::kShift ? d[q] * St::kInvScale + k.w[q] : d[q]);
      return;
    }
  }
  Moments<T, St::kShift> m = moments<T, St::kShift>(d, k.rho0, St::kInvScale);
  if (a.write_macro) {
    a.rho_out[rc] = (double)m.rho;
    a.u_out[rc] = (double)m.ux;
    a.u_out[N + rc] = (double)m.uy;
  }
  if (a.check_finite && !isfinite(m.rho + m.ux + m.uy)) atomicOr(a.status, 1u);
  collide<T, St::kShift>(d, m, k);
  S* fout = (S*)a.fout;
  unsigned r = St::kStochastic ? sr_seed(cell, *a.it_dev) : 0u;
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    if (St::kStochastic) r = xorshift32(r);
    St::store_r(fout + q * Ns + cell, d[q], r);
  }
}

// ---------------------------------------------------------------------------
// Bulk kernel, vectorised: each thread updates V consecutive cells of one
// column (j0 .. j0+V-1, j0 a multiple of V) with one 16-byte load and one
// 16-byte store per population plane.  Planes shifted along y (c_y = +-1)
// need one cell beyond the thread's group: it comes from the neighbouring
// lane's registers by a warp shuffle, or from memory for the first/last lane
// of the warp.  Needs sy % V == 0 (the storage rows are padded so that
// groups never straddle two columns); wall cells inside a group are computed
// with placeholder values and then overwritten by k_special, as in k_bulk,
// and padding cells (j >= ny) hold values no real cell ever reads.
// ---------------------------------------------------------------------------
// 1: the vectorised bulk kernels of the FP32-arithmetic forms update a pair
// of cells with packed FP32 instructions (moments2 / collide2); 0: one cell
// at a time.
#ifndef LBM_VEC_PAIRED
#define LBM_VEC_PAIRED 1
#endif

template <typename S, int V>
struct alignas(sizeof(S) * V) Pack {
  S v[V];
};

template <class St, int V>
__device__ __forceinline__ void bulk_group_vec_update(const FusedArgs& a, int i, int j0,
                                                      const Pack<typename St::S, V> (&in)[9],
                                                      const typename St::T (&halo)[9]);

// gi: group index within the lattice; every lane of the warp must call this
// (the halo shuffles use the full mask), lanes past the last group included.
template <class St, int V>
__device__ __forceinline__ void bulk_group_vec(const FusedArgs& a, long long gi) {
  using S = typename St::S;
  using T = typename St::T;
  using P = Pack<S, V>;
  const long long Ns = a.Ns;
  const int sy = a.sy;
  const int G = sy / V;
  const bool valid = gi >= 0 && gi < (long long)a.nx * G;
  const int i = valid ? (int)(gi / G) : 0;
  const int j0 = valid ? (int)(gi - (long long)i * G) * V : 0;
  const bool active = valid && i > 0 && i < a.nx - 1;
  const unsigned lane = threadIdx.x & 31u;
  const S* fin = (const S*)a.fin;

  P in[9];
  T halo[9];  // the cell just outside the group for planes with c_y != 0
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    const long long base = q * Ns + (long long)(i - cx(q)) * sy + j0;
    if (active) {
      in[q] = *reinterpret_cast<const P*>(fin + base);
    } else {
#pragma unroll
      for (int e = 0; e < V; ++e) in[q].v[e] = S();
    }
    if (cy(q) == 1) {
      // cell j0 pulls from j0 - 1: last element of the previous lane's group
      T h = __shfl_up_sync(0xffffffffu, (T)St::load(&in[q].v[V - 1]), 1);
      if (lane == 0) h = (active && j0 > 0) ? St::load(fin + base - 1) : T(0);
      halo[q] = h;
    } else if (cy(q) == -1) {
      // cell j0 + V - 1 pulls from j0 + V: first element of the next lane's group
      T h = __shfl_down_sync(0xffffffffu, (T)St::load(&in[q].v[0]), 1);
      if (lane == 31) h = (active && j0 + V < sy) ? St::load(fin + base + V) : T(0);
      halo[q] = h;
    } else {
      halo[q] = T(0);
    }
  }
  if (!active) return;
  bulk_group_vec_update<St, V>(a, i, j0, in, halo);
}

// The update of one vector group (cells j0 .. j0+V-1 of column i) from its
// nine source vectors and halo cells (planes with c_y = +1: in[q].v[e] is the
// source of cell j0+e+1 and halo[q] that of j0; c_y = -1: in[q].v[e] feeds
// j0+e-1 and halo[q] feeds j0+V-1; c_y = 0: in[q].v[e] feeds j0+e).  Shared
// by the register-pipelined and the TMA-staged bulk kernels.
template <class St, int V>
__device__ __forceinline__ void bulk_group_vec_update(const FusedArgs& a, int i, int j0,
                                                      const Pack<typename St::S, V> (&in)[9],
                                                      const typename St::T (&halo)[9]) {
  using S = typename St::S;
  using T = typename St::T;
  using P = Pack<S, V>;
  const long long N = a.N, Ns = a.Ns;
  const int ny = a.ny, sy = a.sy;
  const Coef<T>& k = coef<T>(a);

  P out[9];
  // Cells are updated two at a time so that each plane's pair of results is
  // converted and rounded by one packed instruction (St::store_pair).  The
  // random stream of a pair starts from its first cell's storage index, so
  // the bits do not depend on V.
  const unsigned it_hash = St::kStochastic ? sr_iter(*a.it_dev) : 0u;
  if constexpr (LBM_VEC_PAIRED && std::is_same<T, float>::value) {
    // Both cells of a pair in packed FP32 (moments2 / collide2).
#pragma unroll
    for (int e = 0; e < V; e += 2) {
      unsigned r = St::kStochastic ? sr_cell((long long)i * sy + j0 + e, it_hash) : 0u;
      float2 d2[9];
#pragma unroll
      for (int q = 0; q < 9; ++q) {
        T v[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int c = e + h;
          if (cy(q) == 1) {
            v[h] = c == 0 ? halo[q] : St::load(&in[q].v[c - 1]);
          } else if (cy(q) == -1) {
            v[h] = c == V - 1 ? halo[q] : St::load(&in[q].v[c + 1]);
          } else {
            v[h] = St::load(&in[q].v[c]);
          }
        }
        d2[q] = make_float2(v[0], v[1]);
      }
      const Moments2 m = moments2<St::kShift>(d2, k.rho0, St::kInvScale);
      const int ja = j0 + e, jb = ja + 1;
      if (a.write_macro) {
        if (ja < ny) {
          const long long rc = (long long)i * ny + ja;
          a.rho_out[rc] = (double)m.rho.x;
          a.u_out[rc] = (double)m.ux.x;
          a.u_out[N + rc] = (double)m.uy.x;
        }
        if (jb < ny) {
          const long long rc = (long long)i * ny + jb;
          a.rho_out[rc] = (double)m.rho.y;
          a.u_out[rc] = (double)m.ux.y;
          a.u_out[N + rc] = (double)m.uy.y;
        }
      }
      // Wall cells are checked by k_special, which recomputes them.
      if (a.check_finite) {
        const float2 chk = add2(add2(m.rho, m.ux), m.uy);
        if ((ja > 0 && ja < ny - 1 && !isfinite(chk.x)) ||
            (jb > 0 && jb < ny - 1 && !isfinite(chk.y)))
          atomicOr(a.status, 1u);
      }
      collide2(d2, m, k);
#pragma unroll
      for (int q = 0; q < 9; ++q) {
        // padding (j >= ny): keep the stored deviations at zero
        if (ja >= ny) d2[q].x = 0.0f;
        if (jb >= ny) d2[q].y = 0.0f;
        if (St::kStochastic) r = lcg32(r);
        St::store_pair(&out[q].v[e], d2[q].x, d2[q].y, r);
      }
    }
  } else {
#pragma unroll
  for (int e = 0; e < V; e += 2) {
    unsigned r = St::kStochastic ? sr_cell((long long)i * sy + j0 + e, it_hash) : 0u;
    T dd[2][9];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int c = e + h;
      T* d = dd[h];
#pragma unroll
      for (int q = 0; q < 9; ++q) {
        if (cy(q) == 1) {
          d[q] = c == 0 ? halo[q] : St::load(&in[q].v[c - 1]);
        } else if (cy(q) == -1) {
          d[q] = c == V - 1 ? halo[q] : St::load(&in[q].v[c + 1]);
        } else {
          d[q] = St::load(&in[q].v[c]);
        }
      }
      Moments<T, St::kShift> m = moments<T, St::kShift>(d, k.rho0, St::kInvScale);
      const int j = j0 + c;
      if (j < ny && a.write_macro) {
        const long long rc = (long long)i * ny + j;
        a.rho_out[rc] = (double)m.rho;
        a.u_out[rc] = (double)m.ux;
        a.u_out[N + rc] = (double)m.uy;
      }
      // Wall cells are checked by k_special, which recomputes them.
      if (a.check_finite && j > 0 && j < ny - 1 && !isfinite(m.rho + m.ux + m.uy))
        atomicOr(a.status, 1u);
      collide<T, St::kShift>(d, m, k);
      if (j >= ny) {
        // padding: keep the stored deviations at zero (never read by a cell)
#pragma unroll
        for (int q = 0; q < 9; ++q) d[q] = T(0);
      }
    }
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      if (St::kStochastic) r = lcg32(r);
      St::store_pair(&out[q].v[e], dd[0][q], dd[1][q], r);
    }
  }
  }
  S* fout = (S*)a.fout;
#pragma unroll
  for (int q = 0; q < 9; ++q)
    *reinterpret_cast<P*>(fout + q * Ns + (long long)i * sy + j0) = out[q];
}

// ---------------------------------------------------------------------------
// Special cells.
// ---------------------------------------------------------------------------
// Full (unshifted) population q from the storage form, in the form's
// arithmetic type (no add at all for the plain FP64 form).
template <class St>
__device__ __forceinline__ typename St::T full_value(const typename St::S* p, int q,
                                                     typename St::T rho0) {
  using T = typename St::T;
  const T v = St::load(p);
  return St::kShift ? v * St::kInvScale + T(wgt(q)) * rho0 : v;
}

// Resident 128-thread blocks per SM that the special-cell kernels are
// compiled for (register cap 65536 / (128 x this)).
#ifndef LBM_SPECIAL_MIN_BLOCKS
#define LBM_SPECIAL_MIN_BLOCKS 5
#endif

__device__ __forceinline__ bool is_corner_neighbour(const FusedArgs& a, int s) {
  bool r = false;
  for (int w = 0; w < a.n_corner_ops; ++w) r |= a.corner_nb_special[a.corner_ops[w]] == s;
  return r;
}

// Post-BC state of special cell s without corners (pull, links, wall ops),
// in the storage form's arithmetic type T (FP64 for the plain form, FP32 for
// the reduced forms).
template <class St>
__device__ void bc_chain(const FusedArgs& a, long long it, int s, CellBC<typename St::T>& c) {
  using S = typename St::S;
  using T = typename St::T;
  const long long Ns = a.Ns;  // link cells and neighbours are storage indices
  const int ny = a.ny, nx = a.nx;
  const int cell = a.special_cell[s];
  const int i = cell / ny, j = cell - i * ny;
  const S* fin = (const S*)a.fin;
  const T rho0 = St::kShift ? T(a.kd.rho0) : T(0);
  const double* stale_in = a.stale[(it - 1) & 1];
  const double* mac_in = a.mac[(it - 1) & 1];
  const double bs = bc_scale_at(a, it - 1);
  // Pull (or keep the stale post-BC value where the source is outside).
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    const int si = i - cx(q), sj = j - cy(q);
    if (si >= 0 && si < nx && sj >= 0 && sj < ny) {
      c.g[q] = full_value<St>(fin + q * Ns + (long long)si * a.sy + sj, q, rho0);
    } else {
      c.g[q] = (T)stale_in[(long long)q * a.n_special + s];
    }
  }
  // rho/u before the wall operations are only ever read by a corner, from
  // its x-neighbour (nb.py:254-257); other cells never use them.
  if (is_corner_neighbour(a, s)) {
    c.rho = (T)mac_in[s];
    c.ux = (T)mac_in[a.n_special + s];
    c.uy = (T)mac_in[2 * a.n_special + s];
  } else {
    c.rho = c.ux = c.uy = T(0);
  }
  // Obstacle links, in reference order (nb.py:77-117).
  const int l0 = a.special_link_start[s], l1 = a.special_link_start[s + 1];
  for (int l = l0; l < l1; ++l) {
    const int k = a.special_link_ids[l];
    const int q = a.link_q[k], qb = opp(q);
    const long long x = a.link_cell[k];
    const T up_q_x = full_value<St>(fin + q * Ns + x, q, rho0);
    T v = up_q_x;
    if (a.ibb) {
      const T p = (T)a.link_p[k];
      const long long x1 = a.link_nb1[k];
      T c1, c2, c3;
      if (a.link_coef) {
        c1 = (T)a.link_coef[k];
        c2 = (T)a.link_coef[a.n_links + k];
        c3 = (T)a.link_coef[2 * a.n_links + k];
      } else {
        ibb_coefs<T>(p, c1, c2, c3);
      }
      // p < 1/2: c1 f_q(x) + c2 f_q(x1) - c3 f_q(x2);
      // else:    c1 f_q(x) + c2 f_qb(x) + c3 f_qb(x1).  One load pattern.
      const bool near = p < T(0.5);
      const int qy = near ? q : qb;
      const long long y1 = qy * Ns + (near ? x1 : x);
      const long long y2 = qy * Ns + (near ? a.link_nb2[k] : x1);
      const T u1 = full_value<St>(fin + y1, qy, rho0);
      const T u2 = full_value<St>(fin + y2, qy, rho0);
      v = c1 * up_q_x + c2 * u1 + (near ? -c3 : c3) * u2;
    }
    set_pop<T>(c.g, qb, v);
  }
  // Zou-He walls in the app's order (nb.py:121-247).
  const int off_ur = 2 * ny, off_ut = 4 * ny, off_ub = 4 * ny + 2 * nx, off_rr = 4 * ny + 4 * nx;
  for (int w = 0; w < a.n_wall_ops; ++w) {
    switch (a.wall_ops[w]) {
      case LBM_WALL_LEFT_VELOCITY:
        if (i == 0) zh_left<T>(c, (T)bc_value(a, bs, j), (T)bc_value(a, bs, ny + j));
        break;
      case LBM_WALL_RIGHT_VELOCITY:
        if (i == nx - 1)
          zh_right<T>(c, (T)bc_value(a, bs, off_ur + j), (T)bc_value(a, bs, off_ur + ny + j));
        break;
      case LBM_WALL_RIGHT_PRESSURE:
        if (i == nx - 1)
          zh_right_pressure<T>(c, (T)bc_value(a, bs, off_rr + j),
                               (T)bc_value(a, bs, off_ur + ny + j));
        break;
      case LBM_WALL_TOP_VELOCITY:
        if (j == ny - 1)
          zh_top<T>(c, (T)bc_value(a, bs, off_ut + i), (T)bc_value(a, bs, off_ut + nx + i));
        break;
      case LBM_WALL_BOTTOM_VELOCITY:
        if (j == 0)
          zh_bottom<T>(c, (T)bc_value(a, bs, off_ub + i), (T)bc_value(a, bs, off_ub + nx + i));
        break;
      default:
        break;
    }
  }
}

__device__ __forceinline__ bool on_wall_op(const FusedArgs& a, int i, int j) {
  for (int w = 0; w < a.n_wall_ops; ++w) {
    const int op = a.wall_ops[w];
    if (op == LBM_WALL_LEFT_VELOCITY && i == 0) return true;
    if ((op == LBM_WALL_RIGHT_VELOCITY || op == LBM_WALL_RIGHT_PRESSURE) && i == a.nx - 1) return true;
    if (op == LBM_WALL_TOP_VELOCITY && j == a.ny - 1) return true;
    if (op == LBM_WALL_BOTTOM_VELOCITY && j == 0) return true;
  }
  return false;
}

template <class St>
__device__ __forceinline__ void special_collide(const FusedArgs& a, int s, int cell,
                                                long long scell, CellBC<typename St::T>& c);

template <class St, int MODE>
__device__ __forceinline__ void special_cell(const FusedArgs& a, int s) {
  using S = typename St::S;
  using T = typename St::T;
  const long long N = a.N;
  const int ny = a.ny;
  const int cell = a.special_cell[s];  // reference layout i * ny + j
  const int i = cell / ny, j = cell - i * ny;
  const long long scell = (long long)i * a.sy + j;  // storage layout
  const Coef<T>& k = coef<T>(a);
  const T rho0 = St::kShift ? T(a.kd.rho0) : T(0);
  const long long it = *a.it_dev;
  CellBC<T> c;
  if (MODE == LBM_MODE_COLLIDE_FROM_G) {
#pragma unroll
    for (int q = 0; q < 9; ++q) c.g[q] = (T)a.g_out[q * N + cell];
  } else {
    bc_chain<St>(a, it, s, c);
    // Corners (nb.py:250-344): rho/u of the x-neighbour after its wall ops.
    for (int w = 0; w < a.n_corner_ops; ++w) {
      const int cn = a.corner_ops[w];
      if (a.corner_special[cn] != s) continue;
      CellBC<T> nb;
      bc_chain<St>(a, it, a.corner_nb_special[cn], nb);
      zh_corner<T>(cn, c, nb.rho, nb.ux, nb.uy);
    }
    // Per-link momentum exchange terms (nb.py:49-73) with the post-BC g,
    // accumulated in FP64 for every form.
    const int l0 = a.special_link_start[s], l1 = a.special_link_start[s + 1];
    const S* fin = (const S*)a.fin;
    for (int l = l0; l < l1; ++l) {
      const int kk = a.special_link_ids[l];
      const int q = a.link_q[kk];
      const double g0 =
          (double)full_value<St>(fin + q * a.Ns + scell, q, rho0) + (double)get_pop<T>(c.g, opp(q));
      a.link_force[kk] = g0 * (double)cx(q);
      a.link_force[a.n_links + kk] = g0 * (double)cy(q);
    }
    if (MODE == LBM_MODE_FINISH) {
#pragma unroll
      for (int q = 0; q < 9; ++q) a.g_out[q * N + cell] = (double)c.g[q];
      bool corner_cell = false;
      for (int w = 0; w < a.n_corner_ops; ++w) corner_cell |= (a.corner_special[a.corner_ops[w]] == s);
      if (a.wall_macro && (corner_cell || on_wall_op(a, i, j))) {
        a.rho_out[cell] = (double)c.rho;
        a.u_out[cell] = (double)c.ux;
        a.u_out[N + cell] = (double)c.uy;
      }
      return;
    }
  }
  // Keep the post-BC value of the populations the next iteration cannot pull
  // (sources outside the lattice: only on walls).
  double* stale_out = a.stale[it & 1];
  double* mac_out = a.mac[it & 1];
#pragma unroll
  for (int q = 1; q < 9; ++q) {
    const int si = i - cx(q), sj = j - cy(q);
    if (si < 0 || si >= a.nx || sj < 0 || sj >= ny)
      stale_out[(long long)q * a.n_special + s] = (double)c.g[q];
  }
  if constexpr (St::kFixed) {
    // Q3.60: the post-BC populations (FP64) are converted and collided in
    // integer arithmetic like the bulk; macro values (few cells) in FP64.
    long long x[9];
    bool ok = true;
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      x[q] = q60_from_double((double)c.g[q]);
      ok &= x[q] != kQ60Bad;
    }
    const bool corner_nb = is_corner_neighbour(a, s);
    if (corner_nb || a.write_macro) {
      Moments<double, false> m = moments<double, false>(c.g, 0.0);
      if (corner_nb) {
        mac_out[s] = m.rho;
        mac_out[a.n_special + s] = m.ux;
        mac_out[2 * a.n_special + s] = m.uy;
      }
      if (a.write_macro) {
        a.rho_out[cell] = m.rho;
        a.u_out[cell] = m.ux;
        a.u_out[N + cell] = m.uy;
      }
    }
    long long rq, jxq, jyq;
    ok = ok && collide_q60(x, a.kq, rq, jxq, jyq);
    if (!ok) {
      if (a.check_finite) atomicOr(a.status, 1u);
#pragma unroll
      for (int q = 0; q < 9; ++q) x[q] = kQ60Bad;
    }
    long long* fout = (long long*)a.fout;
#pragma unroll
    for (int q = 0; q < 9; ++q) fout[q * a.Ns + scell] = x[q];
  } else {
    special_collide<St>(a, s, cell, scell, c);
  }
}

// Macro + collision of a special cell in the storage form's arithmetic.
template <class St>
__device__ __forceinline__ void special_collide(const FusedArgs& a, int s, int cell,
                                                long long scell, CellBC<typename St::T>& c) {
  using S = typename St::S;
  using T = typename St::T;
  const long long N = a.N;
  const Coef<T>& k = coef<T>(a);
  const T rho0 = St::kShift ? T(a.kd.rho0) : T(0);
  const long long it = *a.it_dev;
  double* mac_out = a.mac[it & 1];
  T d[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) d[q] = St::kShift ? (c.g[q] - T(wgt(q)) * rho0) * St::kScale : c.g[q];
  Moments<T, St::kShift> m = moments<T, St::kShift>(d, k.rho0, St::kInvScale);
  if (is_corner_neighbour(a, s)) {
    mac_out[s] = (double)m.rho;
    mac_out[a.n_special + s] = (double)m.ux;
    mac_out[2 * a.n_special + s] = (double)m.uy;
  }
  if (a.write_macro) {
    a.rho_out[cell] = (double)m.rho;
    a.u_out[cell] = (double)m.ux;
    a.u_out[N + cell] = (double)m.uy;
  }
  if (a.check_finite && !isfinite(m.rho + m.ux + m.uy)) atomicOr(a.status, 1u);
  collide<T, St::kShift>(d, m, k);
  S* fout = (S*)a.fout;
  unsigned r = St::kStochastic ? sr_seed(scell, *a.it_dev) : 0u;
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    if (St::kStochastic) r = xorshift32(r);
    St::store_r(fout + q * a.Ns + scell, d[q], r);
  }
}

// Per-obstacle drag/lift: one block of 256 threads per obstacle, a
// fixed-order FP64 sum (thread t adds links t, t + 256, ... in order, each
// warp reduces by a fixed shuffle tree, warp 0 adds the eight warp sums in
// order), so the result does not depend on scheduling.
__device__ __forceinline__ void drag_obstacle(const FusedArgs& a, int o) {
  const double* link_force = a.link_force;
  const int n_links = a.n_links;
  long long slot = (*a.it_dev - a.drag_it_offset) % a.drag_cap;
  if (slot < 0) slot += a.drag_cap;
  const int l0 = a.obs_start[o], l1 = a.obs_start[o + 1];
  double fx = 0.0, fy = 0.0;
  for (int l = l0 + (int)threadIdx.x; l < l1; l += blockDim.x) {
    fx += link_force[l];
    fy += link_force[n_links + l];
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    fx += __shfl_down_sync(0xffffffffu, fx, off);
    fy += __shfl_down_sync(0xffffffffu, fy, off);
  }
  __shared__ double wx[8], wy[8];
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  if (lane == 0) {
    wx[warp] = fx;
    wy[warp] = fy;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double sx = wx[0], sy = wy[0];
    for (unsigned w = 1; w < (blockDim.x >> 5); ++w) {
      sx += wx[w];
      sy += wy[w];
    }
    double* out = a.drag_hist + slot * 2 * a.n_obs;
    out[2 * o] = sx;
    out[2 * o + 1] = sy;
  }
}

}  // namespace lbm

namespace lbm {
// Kernel arguments of one lattice from its C-ABI description (lbm_fused.cu).
FusedArgs make_args(const lbm_problem* p, int mode, unsigned flags);
// Host: a second stream and two events per thread and device.  The drag/lift
// sums of step k run on it beside the bulk kernel of step k + 1 (they read
// only the per-link terms of step k, which the special-cell kernel of step
// k + 1 overwrites after waiting for them); the caller's stream joins it at
// the end of each enqueue.
#ifndef LBM_DRAG_SIDE
#define LBM_DRAG_SIDE 1  // 0: every kernel of a step on the caller's stream
#endif
struct DragLane {
  cudaStream_t sd;
  cudaEvent_t ev_special, ev_drag;
};
inline DragLane* drag_lane() {
  thread_local DragLane lanes[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  DragLane& l = lanes[dev];
  if (!l.sd) {
    cudaStream_t sd = nullptr;
    if (cudaStreamCreateWithFlags(&sd, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
    if (cudaEventCreateWithFlags(&l.ev_special, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&l.ev_drag, cudaEventDisableTiming) != cudaSuccess) {
      cudaStreamDestroy(sd);
      return nullptr;
    }
    l.sd = sd;
  }
  return &l;
}

}  // namespace lbm
