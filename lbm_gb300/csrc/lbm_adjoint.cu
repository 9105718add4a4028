// Hand-written discrete adjoint of the FP64 fused lattice update.
//
// Forward step n (lbm_fused.cu): x(n) = F(x(n-1)) with x = post-collision
// populations g_up; inside F: pull, set_bc(n-1) (IBB/BB links, Zou-He walls,
// corners), drag/lift of iteration n-1 from x(n-1) and the post-BC g, then
// macro/equilibrium/TRT collision.  One adjoint step maps lambda(n) =
// dJ/dx(n) to lambda(n-1) = dJ/dx(n-1), adds the drag objective terms of
// iteration n-1 and accumulates the gradients with respect to the TRT rate
// om_p (om_m follows from om_p, lattice.py:127-131) and to every entry of the
// packed BC vectors of iteration n-1:
//
//   k_adj_cells    one launch over every cell:
//                  - bulk cells (one per thread): recompute the pulled
//                    values, apply the transposed collision Jacobian
//                    (hand-derived: linear pair part plus a rank-3 update
//                    through rho, jx, jy), store the adjoint of each pulled
//                    value; d/d om_p terms;
//                  - special cells other than corners (one per warp):
//                    collision transposed, drag seeds, then the chain
//                    reversed op by op.  The BC ops are small, so each op's
//                    transposed Jacobian is taken with forward-mode dual
//                    numbers, one Jacobian column per lane, on the same
//                    templated code the forward uses; the IBB rows are
//                    written out by hand;
//                  - the four corners (one per warp): their chain reversed
//                    (corner op, walls, links).  The corner op reads rho/u of
//                    the x-neighbour; the neighbour's warp recomputes that
//                    seed itself, so no cell waits for another.
//   k_adj_gather   lambda(n-1)[q, y] = adjoint of the value pulled by cell
//                  y + c_q (the transpose of the pull).
//   k_adj_links    add the IBB and drag terms that read x(n-1) directly.
//
// Supported boundary programs: every wall carries a Zou-He operation and all
// four corners are applied, so no edge value is ever carried over from the
// previous iteration (the stale values and the pre-BC rho/u of the forward
// have zero adjoint).
#include <string.h>

#include "lbm_fused.cuh"

namespace lbm {
namespace {

// ---------------------------------------------------------------------------
// Dual numbers (value, derivative) for the BC ops' Jacobian columns.
// ---------------------------------------------------------------------------
struct Dual {
  double v, d;
  __device__ Dual() : v(0.0), d(0.0) {}
  __device__ Dual(double x) : v(x), d(0.0) {}  // NOLINT: constants lift implicitly
  __device__ Dual(double x, double dx) : v(x), d(dx) {}
};
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
  const double q = a.v / b.v;
  return Dual(q, (a.d - q * b.d) / b.v);
}

// Packed BC layout offsets (u_left | u_right | u_top | u_bot | rho_right).
struct BcOff {
  int ul, ur, ut, ub, rr;
};
__device__ __forceinline__ BcOff bc_off(int nx, int ny) {
  return BcOff{0, 2 * ny, 4 * ny, 4 * ny + 2 * nx, 4 * ny + 4 * nx};
}

// Packed indices of the two BC values a wall op of cell (i, j) reads.
__device__ __forceinline__ void wall_param_index(int op, int i, int j, int nx, int ny, int& k0,
                                                 int& k1) {
  const BcOff o = bc_off(nx, ny);
  switch (op) {
    case LBM_WALL_LEFT_VELOCITY: k0 = o.ul + j; k1 = o.ul + ny + j; break;
    case LBM_WALL_RIGHT_VELOCITY: k0 = o.ur + j; k1 = o.ur + ny + j; break;
    case LBM_WALL_RIGHT_PRESSURE: k0 = o.rr + j; k1 = o.ur + ny + j; break;
    case LBM_WALL_TOP_VELOCITY: k0 = o.ut + i; k1 = o.ut + nx + i; break;
    default: k0 = o.ub + i; k1 = o.ub + nx + i; break;
  }
}

__device__ __forceinline__ bool wall_touches(int op, int i, int j, int nx, int ny) {
  switch (op) {
    case LBM_WALL_LEFT_VELOCITY: return i == 0;
    case LBM_WALL_RIGHT_VELOCITY:
    case LBM_WALL_RIGHT_PRESSURE: return i == nx - 1;
    case LBM_WALL_TOP_VELOCITY: return j == ny - 1;
    default: return j == 0;
  }
}

template <typename T>
__device__ __forceinline__ void apply_wall(int op, CellBC<T>& c, T p0, T p1) {
  switch (op) {
    case LBM_WALL_LEFT_VELOCITY: zh_left<T>(c, p0, p1); break;
    case LBM_WALL_RIGHT_VELOCITY: zh_right<T>(c, p0, p1); break;
    case LBM_WALL_RIGHT_PRESSURE: zh_right_pressure<T>(c, p0, p1); break;
    case LBM_WALL_TOP_VELOCITY: zh_top<T>(c, p0, p1); break;
    default: zh_bottom<T>(c, p0, p1); break;
  }
}

// Transposed Jacobian-vector product of a BC op by forward-mode columns,
// warp-cooperative: every lane of the warp calls it with the same arguments;
// lane k < 12 + np propagates the derivative with respect to input k (one
// Jacobian column), and the column-adjoint dot products are exchanged by
// shuffles.  in: state before the op; adj: adjoint of the state after it
// (replaced by the adjoint of the state before it); params/adj_params: np op
// parameters.  kind < 5: wall op `kind`; kind 5 + c: corner c with params
// (rho, ux, uy) of the x-neighbour.
__device__ void op_transpose(int kind, const CellBC<double>& in, const double* params, int np,
                             CellBC<double>& adj, double* adj_params) {
  const int k = threadIdx.x & 31;
  double s = 0.0;
  if (k < 12 + np) {
    CellBC<Dual> c;
#pragma unroll
    for (int q = 0; q < 9; ++q) c.g[q] = Dual(in.g[q], k == q ? 1.0 : 0.0);
    c.rho = Dual(in.rho, k == 9 ? 1.0 : 0.0);
    c.ux = Dual(in.ux, k == 10 ? 1.0 : 0.0);
    c.uy = Dual(in.uy, k == 11 ? 1.0 : 0.0);
    Dual p[3];
    for (int m = 0; m < np; ++m) p[m] = Dual(params[m], k == 12 + m ? 1.0 : 0.0);
    if (kind < 5) {
      apply_wall<Dual>(kind, c, p[0], p[1]);
    } else {
      zh_corner<Dual>(kind - 5, c, p[0], p[1], p[2]);
    }
    s = c.rho.d * adj.rho + c.ux.d * adj.ux + c.uy.d * adj.uy;
#pragma unroll
    for (int q = 0; q < 9; ++q) s += c.g[q].d * adj.g[q];
  }
#pragma unroll
  for (int q = 0; q < 9; ++q) adj.g[q] = __shfl_sync(0xffffffffu, s, q);
  adj.rho = __shfl_sync(0xffffffffu, s, 9);
  adj.ux = __shfl_sync(0xffffffffu, s, 10);
  adj.uy = __shfl_sync(0xffffffffu, s, 11);
  for (int m = 0; m < 3; ++m) {
    const double v = __shfl_sync(0xffffffffu, s, 12 + m);
    if (m < np) adj_params[m] = v;
  }
}

// ---------------------------------------------------------------------------
// Transposed TRT collision (FP64, unshifted), with the d/d om_p term.
// Forward (lbm_device.cuh:collide): moments rho = sum d, j = sum c d,
// u = j / rho; R = rho - 1.5 (jx ux + jy uy); per pair (q, qb):
//   P = R + 4.5 Q, M = wm cj, up_q = a d_q + mb d_qb + wp P + M,
//   up_qb = a d_qb + mb d_q + wp P - M; up_0 = a0 d_0 + p0 R.
// ---------------------------------------------------------------------------
struct TrtRates {
  double a, mb, a0, p0, wp1, wm1, wp2, wm2;     // as Coef<double>
  double da, dmb, da0, dp0, dwp1, dwm1, dwp2, dwm2;  // d/d om_p
};

__host__ TrtRates make_rates(double om_p, double om_m, double lambda_trt) {
  TrtRates r;
  // om_m(om_p): tau_m = lambda / (1/om_p - 1/2) + 1/2, om_m = 1/tau_m
  const double tau_p = 1.0 / om_p;
  const double tau_m = 1.0 / om_m;
  const double dtaum_dtaup = -lambda_trt / ((tau_p - 0.5) * (tau_p - 0.5));
  const double dom_m = (-1.0 / (tau_m * tau_m)) * dtaum_dtaup * (-1.0 / (om_p * om_p));
  const double w1 = 1.0 / 9.0, w2 = 1.0 / 36.0, w0 = 4.0 / 9.0;
  r.a = 1.0 - 0.5 * (om_p + om_m);
  r.mb = -0.5 * (om_p - om_m);
  r.a0 = 1.0 - om_p;
  r.p0 = om_p * w0;
  r.wp1 = om_p * w1;
  r.wm1 = 3.0 * om_m * w1;
  r.wp2 = om_p * w2;
  r.wm2 = 3.0 * om_m * w2;
  r.da = -0.5 * (1.0 + dom_m);
  r.dmb = -0.5 * (1.0 - dom_m);
  r.da0 = -1.0;
  r.dp0 = w0;
  r.dwp1 = w1;
  r.dwm1 = 3.0 * w1 * dom_m;
  r.dwp2 = w2;
  r.dwm2 = 3.0 * w2 * dom_m;
  return r;
}

// d: post-BC populations; lam: adjoint of the post-collision populations.
// Returns the adjoint of d in adj and d(lam . up)/d om_p.
__device__ __forceinline__ double collide_transpose(const double d[9], const double lam[9],
                                                    const TrtRates& k, double adj[9]) {
  const double rho = (((d[0] + (d[1] + d[2])) + (d[3] + d[4])) + (d[5] + d[6])) + (d[7] + d[8]);
  const double jx = ((d[1] - d[2]) + (d[5] - d[6])) + (d[8] - d[7]);
  const double jy = ((d[3] - d[4]) + (d[5] - d[6])) - (d[8] - d[7]);
  const double r = 1.0 / rho;
  const double ux = jx * r, uy = jy * r;
  const double Qx = jx * ux, Qy = jy * uy;
  const double j5 = jx + jy, u5 = ux + uy, Q5 = j5 * u5;
  const double j7 = jy - jx, u7 = uy - ux, Q7 = j7 * u7;
  const double R = rho - 1.5 * (Qx + Qy);
  // pairs: (1,2) Qx jx; (3,4) Qy jy; (5,6) Q5 j5; (7,8) Q7 j7
  const double s12 = lam[1] + lam[2], t12 = lam[1] - lam[2];
  const double s34 = lam[3] + lam[4], t34 = lam[3] - lam[4];
  const double s56 = lam[5] + lam[6], t56 = lam[5] - lam[6];
  const double s78 = lam[7] + lam[8], t78 = lam[7] - lam[8];
  // d/d om_p of lam . up
  double dom = lam[0] * (k.da0 * d[0] + k.dp0 * R);
#define LBM_PAIR_DOM(q, qb, Q, cj, dwp, dwm)                                      \
  dom += lam[q] * (k.da * d[q] + k.dmb * d[qb] + (dwp) * (R + 4.5 * (Q)) + (dwm) * (cj)) + \
         lam[qb] * (k.da * d[qb] + k.dmb * d[q] + (dwp) * (R + 4.5 * (Q)) - (dwm) * (cj));
  LBM_PAIR_DOM(1, 2, Qx, jx, k.dwp1, k.dwm1)
  LBM_PAIR_DOM(3, 4, Qy, jy, k.dwp1, k.dwm1)
  LBM_PAIR_DOM(5, 6, Q5, j5, k.dwp2, k.dwm2)
  LBM_PAIR_DOM(7, 8, Q7, j7, k.dwp2, k.dwm2)
#undef LBM_PAIR_DOM
  // adjoints of the intermediate quantities
  const double aR = k.p0 * lam[0] + k.wp1 * (s12 + s34) + k.wp2 * (s56 + s78);
  const double aQx = 4.5 * k.wp1 * s12 - 1.5 * aR;
  const double aQy = 4.5 * k.wp1 * s34 - 1.5 * aR;
  const double aQ5 = 4.5 * k.wp2 * s56;
  const double aQ7 = 4.5 * k.wp2 * s78;
  double ajx = k.wm1 * t12 + aQx * ux;
  double ajy = k.wm1 * t34 + aQy * uy;
  double aux = aQx * jx;
  double auy = aQy * jy;
  const double aj5 = k.wm2 * t56 + aQ5 * u5, au5 = aQ5 * j5;
  const double aj7 = k.wm2 * t78 + aQ7 * u7, au7 = aQ7 * j7;
  ajx += aj5 - aj7;
  ajy += aj5 + aj7;
  aux += au5 - au7;
  auy += au5 + au7;
  ajx += aux * r;
  ajy += auy * r;
  const double ar = aux * jx + auy * jy;
  const double arho = aR - ar * r * r;
  // linear (pair) part plus the moment terms
  adj[0] = k.a0 * lam[0] + arho;
  adj[1] = k.a * lam[1] + k.mb * lam[2] + arho + ajx;
  adj[2] = k.a * lam[2] + k.mb * lam[1] + arho - ajx;
  adj[3] = k.a * lam[3] + k.mb * lam[4] + arho + ajy;
  adj[4] = k.a * lam[4] + k.mb * lam[3] + arho - ajy;
  adj[5] = k.a * lam[5] + k.mb * lam[6] + arho + ajx + ajy;
  adj[6] = k.a * lam[6] + k.mb * lam[5] + arho - ajx - ajy;
  adj[7] = k.a * lam[7] + k.mb * lam[8] + arho - ajx + ajy;
  adj[8] = k.a * lam[8] + k.mb * lam[7] + arho + ajx - ajy;
  return dom;
}

struct AdjArgs {
  FusedArgs f;        // forward description (f.fin = x(n-1), FP64)
  TrtRates k;
  const double* lam_in;   // [9][N] lambda(n)
  double* lam_out;        // [9][N] lambda(n-1)
  double* adj_pulled;     // [9][N]
  double* link_adj;       // [3][n_links]
  double* corner_seed;    // [4][3]
  double* grad_bc_base;
  double* grad_bc_vec;
  double* grad_omega;     // per-block partial sums
  const unsigned char* is_special;  // [N]
  const double* obj_w;    // [2][n_obs] weights of fx, fy
  int in_window;          // the drag of iteration it-1 enters the objective
  long long it;           // forward step n
};

__device__ __forceinline__ double block_sum(double v, double* sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  return sh[0];
}

// ---------------------------------------------------------------------------
// Bulk cell: transposed collision of the pulled values (one thread per cell).
__device__ __forceinline__ double adj_bulk_cell(const AdjArgs& A, long long cell) {
  const FusedArgs& a = A.f;
  const long long N = a.N;
  if (cell >= N) return 0.0;
  const int i = (int)(cell / a.ny), j = (int)(cell - (long long)i * a.ny);
  if (i <= 0 || i >= a.nx - 1 || j <= 0 || j >= a.ny - 1 || A.is_special[cell]) return 0.0;
  const double* x = (const double*)a.fin;
  const long long ny = a.ny;
  double d[9], lam[9], adj[9];
  d[0] = x[cell];
  d[1] = x[1 * N + cell - ny];
  d[2] = x[2 * N + cell + ny];
  d[3] = x[3 * N + cell - 1];
  d[4] = x[4 * N + cell + 1];
  d[5] = x[5 * N + cell - ny - 1];
  d[6] = x[6 * N + cell + ny + 1];
  d[7] = x[7 * N + cell + ny - 1];
  d[8] = x[8 * N + cell - ny + 1];
#pragma unroll
  for (int q = 0; q < 9; ++q) lam[q] = A.lam_in[q * N + cell];
  const double dom = collide_transpose(d, lam, A.k, adj);
#pragma unroll
  for (int q = 0; q < 9; ++q) A.adj_pulled[q * N + cell] = adj[q];
  return dom;
}

// Op list of special cell s: links [0, nl), wall ops touching the cell, then
// the corner (if any).  chain_prefix(K) = state after the first K ops.
struct OpList {
  int nl;       // links
  int l0;       // first entry in special_link_ids
  int walls[5];
  int nw;
  int corner;   // -1 if none
};

__device__ OpList op_list(const FusedArgs& a, int s, int i, int j) {
  OpList o;
  o.l0 = a.special_link_start[s];
  o.nl = a.special_link_start[s + 1] - o.l0;
  o.nw = 0;
  for (int w = 0; w < a.n_wall_ops; ++w)
    if (wall_touches(a.wall_ops[w], i, j, a.nx, a.ny)) o.walls[o.nw++] = a.wall_ops[w];
  o.corner = -1;
  for (int w = 0; w < a.n_corner_ops; ++w)
    if (a.corner_special[a.corner_ops[w]] == s) o.corner = a.corner_ops[w];
  return o;
}

__device__ __forceinline__ double xval(const FusedArgs& a, int q, long long x) {
  return ((const double*)a.fin)[q * a.N + x];
}

// The two BC values of wall op `op` at (i, j) for iteration it - 1.
__device__ __forceinline__ void wall_params(const AdjArgs& A, int op, int i, int j, double p[2]) {
  int k0, k1;
  wall_param_index(op, i, j, A.f.nx, A.f.ny, k0, k1);
  const double bs = bc_scale_at(A.f, A.it - 1);
  p[0] = bc_value(A.f, bs, k0);
  p[1] = bc_value(A.f, bs, k1);
}

// IBB/BB value of link k (nb.py:77-117) and its three read coefficients.
__device__ __forceinline__ void link_rows(const FusedArgs& a, int k, double coef[3]) {
  if (!a.ibb) {
    coef[0] = 1.0; coef[1] = 0.0; coef[2] = 0.0;
    return;
  }
  const double p = a.link_p[k];
  const double pp = 2.0 * p;
  if (p < 0.5) {
    coef[0] = p * (pp + 1.0);
    coef[1] = (1.0 + pp) * (1.0 - pp);
    coef[2] = -p * (1.0 - pp);
  } else {
    coef[0] = 1.0 / (p * (pp + 1.0));
    coef[1] = (pp - 1.0) / p;
    coef[2] = (1.0 - pp) / (1.0 + pp);
  }
}

// Values read by link k (targets T0, T1, T2 of link_adj).
__device__ __forceinline__ void link_reads(const FusedArgs& a, int k, double v[3]) {
  const int q = a.link_q[k], qb = opp(q);
  const long long x = a.link_cell[k];
  v[0] = xval(a, q, x);
  v[1] = v[2] = 0.0;
  if (!a.ibb) return;
  const long long x1 = a.link_nb1[k];
  if (a.link_p[k] < 0.5) {
    v[1] = xval(a, q, x1);
    v[2] = xval(a, q, a.link_nb2[k]);
  } else {
    v[1] = xval(a, qb, x);
    v[2] = xval(a, qb, x1);
  }
}

// State of special cell s after its first K ops (corner excluded).
__device__ void chain_prefix(const AdjArgs& A, int s, int i, int j, const OpList& o, int K,
                             CellBC<double>& c) {
  const FusedArgs& a = A.f;
  const int nx = a.nx, ny = a.ny;
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    const int si = i - cx(q), sj = j - cy(q);
    c.g[q] = (si >= 0 && si < nx && sj >= 0 && sj < ny) ? xval(a, q, (long long)si * ny + sj) : 0.0;
  }
  c.rho = c.ux = c.uy = 0.0;
  int op = 0;
  for (int l = 0; l < o.nl && op < K; ++l, ++op) {
    const int k = a.special_link_ids[o.l0 + l];
    double coef[3], v[3];
    link_rows(a, k, coef);
    link_reads(a, k, v);
    set_pop<double>(c.g, opp(a.link_q[k]), coef[0] * v[0] + coef[1] * v[1] + coef[2] * v[2]);
  }
  for (int w = 0; w < o.nw && op < K; ++w, ++op) {
    double p[2];
    wall_params(A, o.walls[w], i, j, p);
    apply_wall<double>(o.walls[w], c, p[0], p[1]);
  }
}

// Pulled/link state, the state before each of the first two wall ops and the
// state after all wall ops (corner excluded) of special cell s, in one pass.
__device__ void chain_states(const AdjArgs& A, int s, int i, int j, const OpList& o,
                             CellBC<double> pre_wall[2], CellBC<double>& c) {
  chain_prefix(A, s, i, j, o, o.nl, c);
  for (int w = 0; w < o.nw; ++w) {
    if (w < 2) pre_wall[w] = c;
    double p[2];
    wall_params(A, o.walls[w], i, j, p);
    apply_wall<double>(o.walls[w], c, p[0], p[1]);
  }
}

// Reverse the non-corner part of the chain: adj (adjoint after the last
// wall op) -> adjoint of the pulled values; link reads and BC gradients are
// emitted.  pre_wall: states before the first two wall ops (chain_states).
// Warp-cooperative (one warp per cell, lane 0 writes).
__device__ void reverse_chain(const AdjArgs& A, int s, int i, int j, const OpList& o,
                              const CellBC<double> pre_wall[2], CellBC<double>& adj) {
  const FusedArgs& a = A.f;
  const bool lead = (threadIdx.x & 31) == 0;  // the warp's writer
  for (int w = o.nw - 1; w >= 0; --w) {
    CellBC<double> c;
    if (w < 2) {
      c = pre_wall[w];
    } else {
      chain_prefix(A, s, i, j, o, o.nl + w, c);
    }
    double p[2], ap[2];
    wall_params(A, o.walls[w], i, j, p);
    op_transpose(o.walls[w], c, p, 2, adj, ap);
    int k0, k1;
    wall_param_index(o.walls[w], i, j, a.nx, a.ny, k0, k1);
    const double bs = bc_scale_at(a, A.it - 1);
    if (lead) {
      A.grad_bc_base[k0] += ap[0];
      A.grad_bc_base[k1] += ap[1];
      A.grad_bc_vec[k0] += bs * ap[0];
      A.grad_bc_vec[k1] += bs * ap[1];
    }
  }
  for (int l = o.nl - 1; l >= 0; --l) {
    const int k = a.special_link_ids[o.l0 + l];
    const int qb = opp(a.link_q[k]);
    double coef[3];
    link_rows(a, k, coef);
    const double ag = get_pop<double>(adj.g, qb);
    if (lead) {
      A.link_adj[k] += coef[0] * ag;
      A.link_adj[a.n_links + k] += coef[1] * ag;
      A.link_adj[2 * a.n_links + k] += coef[2] * ag;
    }
    set_pop<double>(adj.g, qb, 0.0);  // overwritten by the link
  }
  const long long cell = (long long)i * a.ny + j;
  if (lead) {
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      const int si = i - cx(q), sj = j - cy(q);
      const bool pulled = si >= 0 && si < a.nx && sj >= 0 && sj < a.ny;
      A.adj_pulled[q * a.N + cell] = pulled ? adj.g[q] : 0.0;
    }
  }
}

// Collision transpose + drag seeds of special cell s, given its post-BC g
// (warp-cooperative; the om_p term is returned by lane 0 only).
__device__ double seed_special(const AdjArgs& A, int s, long long cell, const OpList& o,
                               const CellBC<double>& post, CellBC<double>& adj,
                               bool write = true) {
  const FusedArgs& a = A.f;
  double lam[9], ad[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) lam[q] = A.lam_in[q * a.N + cell];
  const double dom = collide_transpose(post.g, lam, A.k, ad);
#pragma unroll
  for (int q = 0; q < 9; ++q) adj.g[q] = ad[q];
  adj.rho = adj.ux = adj.uy = 0.0;
  // drag/lift of iteration it - 1: (x(n-1)[q, x] + g_post[qb, x]) c_q per link
  const bool lead = (threadIdx.x & 31) == 0;
  for (int l = 0; l < o.nl; ++l) {
    const int k = a.special_link_ids[o.l0 + l];
    double wgt_k = 0.0;
    if (A.in_window) {
      const int q = a.link_q[k];
      int ob = 0;  // obstacle of link k
      while (ob + 1 < a.n_obs && a.obs_start[ob + 1] <= k) ++ob;
      wgt_k = A.obj_w[ob] * (double)cx(q) + A.obj_w[a.n_obs + ob] * (double)cy(q);
      set_pop<double>(adj.g, opp(q), get_pop<double>(adj.g, opp(q)) + wgt_k);
    }
    if (lead && write) {
      A.link_adj[k] = wgt_k;  // the x(n-1)[q, x] term
      A.link_adj[a.n_links + k] = 0.0;
      A.link_adj[2 * a.n_links + k] = 0.0;
    }
  }
  return lead ? dom : 0.0;
}

// Adjoint of corner op cn: the corner cell's collision transpose and drag
// seeds, then the corner op transposed.  Returns in adj the adjoint of the
// corner's state before the corner op (with its pre-wall states and op list
// for reverse_chain) and in ap the adjoint of the x-neighbour's (rho, ux,
// uy) that the corner op reads (nb.py:254-257).  write = false computes the
// same values without writing the corner's link terms (the neighbour's warp
// recomputes the seed it needs instead of waiting for the corner's warp).
__device__ double corner_adjoint(const AdjArgs& A, int cn, bool write, CellBC<double>& adj,
                                 double ap[3], CellBC<double> pre_wall[2], OpList& o) {
  const FusedArgs& a = A.f;
  const int s = a.corner_special[cn];
  const int cell = a.special_cell[s];
  const int i = cell / a.ny, j = cell - i * a.ny;
  o = op_list(a, s, i, j);
  // neighbour state after its own links and walls
  const int snb = a.corner_nb_special[cn];
  const int cnb = a.special_cell[snb];
  const int inb = cnb / a.ny, jnb = cnb - inb * a.ny;
  const OpList onb = op_list(a, snb, inb, jnb);
  CellBC<double> nb;
  chain_prefix(A, snb, inb, jnb, onb, onb.nl + onb.nw, nb);
  const double params[3] = {nb.rho, nb.ux, nb.uy};
  CellBC<double> pre, post;
  chain_states(A, s, i, j, o, pre_wall, pre);
  post = pre;
  zh_corner<double>(cn, post, params[0], params[1], params[2]);
  const double dom = seed_special(A, s, cell, o, post, adj, write);
  op_transpose(5 + cn, pre, params, 3, adj, ap);
  return dom;
}

// Special cell s that is not a corner (warp-cooperative).
__device__ double adj_special_cell(const AdjArgs& A, int s) {
  const FusedArgs& a = A.f;
  const int cell = a.special_cell[s];
  const int i = cell / a.ny, j = cell - i * a.ny;
  const OpList o = op_list(a, s, i, j);
  if (o.corner >= 0) return 0.0;
  CellBC<double> pre_wall[2], post, adj;
  chain_states(A, s, i, j, o, pre_wall, post);
  const double dom = seed_special(A, s, cell, o, post, adj);
  // x-neighbour of a corner: add the adjoint of the rho/u the corner read
  for (int w = 0; w < a.n_corner_ops; ++w) {
    const int cn = a.corner_ops[w];
    if (a.corner_nb_special[cn] == s) {
      CellBC<double> cadj, cpre[2];
      OpList co;
      double ap[3];
      corner_adjoint(A, cn, false, cadj, ap, cpre, co);
      adj.rho += ap[0];
      adj.ux += ap[1];
      adj.uy += ap[2];
    }
  }
  reverse_chain(A, s, i, j, o, pre_wall, adj);
  return dom;
}

// Corner op number w of the program (warp-cooperative).
__device__ double adj_corner(const AdjArgs& A, int w) {
  const FusedArgs& a = A.f;
  const int cn = a.corner_ops[w];
  CellBC<double> adj, pre_wall[2];
  OpList o;
  double ap[3];
  const double dom = corner_adjoint(A, cn, true, adj, ap, pre_wall, o);
  const int s = a.corner_special[cn];
  const int cell = a.special_cell[s];
  const int i = cell / a.ny, j = cell - i * a.ny;
  reverse_chain(A, s, i, j, o, pre_wall, adj);
  return dom;
}

// Every cell of the adjoint step in one launch (128 threads per block):
// blocks [0, nbb) bulk cells, one per thread; blocks [nbb, nbb + nbs) special
// cells other than corners, one per warp; the last block the corner ops,
// one per warp.  Corner chains, special cells and bulk cells run side by
// side; the long special and corner chains are scheduled first (launch
// order rotated by nbb), the bulk blocks fill in behind them.  Each block
// adds its part of d/d om_p to grad_omega[block].
__global__ void __launch_bounds__(128) k_adj_cells(AdjArgs A, int nbb, int nbs) {
  __shared__ double sh[128];
  const FusedArgs& a = A.f;
  double dom = 0.0;
  const int b = (int)((blockIdx.x + (unsigned)nbb) % (unsigned)(nbb + nbs + 1));
  if (b < nbb) {
    dom = adj_bulk_cell(A, (long long)b * blockDim.x + threadIdx.x);
  } else if (b < nbb + nbs) {
    const int s = (b - nbb) * 4 + (int)(threadIdx.x >> 5);
    if (s < a.n_special) dom = adj_special_cell(A, s);
  } else {
    const int w = threadIdx.x >> 5;
    if (w < a.n_corner_ops) dom = adj_corner(A, w);
  }
  const double t = block_sum(dom, sh);
  if (threadIdx.x == 0) A.grad_omega[b] += t;
}

// lambda(n-1)[q, y] = adjoint of the value pulled by cell y + c_q.
__global__ void __launch_bounds__(128) k_adj_gather(AdjArgs A) {
  const FusedArgs& a = A.f;
  const long long N = a.N;
  const long long cell = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= N) return;
  const int i = (int)(cell / a.ny), j = (int)(cell - (long long)i * a.ny);
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    const int di = i + cx(q), dj = j + cy(q);
    double v = 0.0;
    if (di >= 0 && di < a.nx && dj >= 0 && dj < a.ny)
      v = A.adj_pulled[q * N + (long long)di * a.ny + dj];
    A.lam_out[q * N + cell] = v;
  }
}

// IBB/BB reads and drag terms on x(n-1), one thread per link (atomic adds:
// several links may read the same population).
__global__ void __launch_bounds__(256) k_adj_links(AdjArgs A) {
  const FusedArgs& a = A.f;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.n_links) return;
  const int q = a.link_q[k], qb = opp(q);
  const long long N = a.N;
  const long long x = a.link_cell[k];
  atomicAdd(&A.lam_out[q * N + x], A.link_adj[k]);
  if (!a.ibb) return;
  const long long x1 = a.link_nb1[k];
  if (a.link_p[k] < 0.5) {
    atomicAdd(&A.lam_out[q * N + x1], A.link_adj[a.n_links + k]);
    atomicAdd(&A.lam_out[q * N + a.link_nb2[k]], A.link_adj[2 * a.n_links + k]);
  } else {
    atomicAdd(&A.lam_out[qb * N + x], A.link_adj[a.n_links + k]);
    atomicAdd(&A.lam_out[qb * N + x1], A.link_adj[2 * a.n_links + k]);
  }
}

// d(lambda(0) . collide(g0))/d om_p for the first collision (from g).
__global__ void __launch_bounds__(256) k_adj_initial(AdjArgs A, const double* __restrict__ g0) {
  __shared__ double sh[256];
  const long long N = A.f.N;
  const long long cell = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double dom = 0.0;
  if (cell < N) {
    double d[9], lam[9], adj[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      d[q] = g0[q * N + cell];
      lam[q] = A.lam_in[q * N + cell];
    }
    dom = collide_transpose(d, lam, A.k, adj);
#pragma unroll
    for (int q = 0; q < 9; ++q) A.lam_out[q * N + cell] = adj[q];
  }
  const double s = block_sum(dom, sh);
  if (threadIdx.x == 0) A.grad_omega[blockIdx.x] += s;
}

int adjoint_supported(const lbm_problem* p) {
  bool wall_ok[4] = {false, false, false, false};  // left, right, top, bottom
  for (int w = 0; w < p->n_wall_ops; ++w) {
    switch (p->wall_ops[w]) {
      case LBM_WALL_LEFT_VELOCITY: wall_ok[0] = true; break;
      case LBM_WALL_RIGHT_VELOCITY:
      case LBM_WALL_RIGHT_PRESSURE: wall_ok[1] = true; break;
      case LBM_WALL_TOP_VELOCITY: wall_ok[2] = true; break;
      default: wall_ok[3] = true; break;
    }
  }
  return wall_ok[0] && wall_ok[1] && wall_ok[2] && wall_ok[3] && p->n_corner_ops == 4 &&
         p->precision == LBM_PREC_F64 && (p->row_pitch == 0 || p->row_pitch == p->ny);
}

}  // namespace
}  // namespace lbm

using namespace lbm;

extern "C" size_t lbm_adjoint_omega_slots(const lbm_problem* p) {
  if (!p) return 0;
  const long long N = (long long)p->nx * p->ny;
  return (size_t)((N + 127) / 128 + (p->n_special + 3) / 4 + 1);
}

namespace {
int adjoint_args_check(const lbm_problem* p, const lbm_adjoint* adj, const char* fn) {
  if (int rc = problem_check(p, fn)) return rc;
  if (!adjoint_supported(p)) {
    set_error("%s: needs FP64, a Zou-He operation on every wall and all four corners", fn);
    return LBM_ERR_UNSUPPORTED;
  }
  if (!adj || !adj->adj_pulled || !adj->grad_bc_base || !adj->grad_bc_vec || !adj->grad_omega ||
      !adj->is_special || !adj->corner_seed || (p->n_links > 0 && !adj->link_adj) ||
      (p->n_obstacles > 0 && !adj->obj_w) ||
      (size_t)adj->grad_omega_len < lbm_adjoint_omega_slots(p)) {
    set_error("%s: bad arguments", fn);
    return LBM_ERR_ARG;
  }
  return LBM_OK;
}

// Enqueue adjoint step `it` (checked arguments).
// The arguments of the adjoint step that do not change from step to step.
void adjoint_prepare(const lbm_problem* p, const lbm_adjoint* adj, AdjArgs& A) {
  memset(&A, 0, sizeof(A));
  A.f = make_args(p, LBM_MODE_STEP, 0);
  A.k = make_rates(p->om_p, p->om_m, 0.25);
  A.adj_pulled = adj->adj_pulled;
  A.link_adj = adj->link_adj;
  A.corner_seed = adj->corner_seed;
  A.grad_bc_base = adj->grad_bc_base;
  A.grad_bc_vec = adj->grad_bc_vec;
  A.grad_omega = adj->grad_omega;
  A.is_special = adj->is_special;
  A.obj_w = adj->obj_w;
}

// One adjoint step (iteration it) with the prepared arguments.
int adjoint_launch(const lbm_problem* p, const lbm_adjoint* adj, AdjArgs& A, int64_t it,
                   const double* x_prev, const double* lam_in, double* lam_out, cudaStream_t st,
                   const char* fn) {
  if (!x_prev || !lam_in || !lam_out || it < 1) {
    set_error("%s: bad arguments", fn);
    return LBM_ERR_ARG;
  }
  if (p->bc_vec && ((it - 1) - p->bc_scale_it0 < 0 || (it - 1) - p->bc_scale_it0 >= p->bc_scale_len)) {
    set_error("%s: BC scale table does not cover iteration %lld", fn, (long long)it - 1);
    return LBM_ERR_ARG;
  }
  A.f.fin = x_prev;
  A.lam_in = lam_in;
  A.lam_out = lam_out;
  A.it = it;
  A.in_window = (it - 1 >= adj->obj_it_first && it - 1 <= adj->obj_it_last) ? 1 : 0;
  const long long N = (long long)p->nx * p->ny;
  const int nbb = (int)((N + 127) / 128);
  const int nbs = (p->n_special + 3) / 4;  // one warp per special cell
  k_adj_cells<<<nbb + nbs + 1, 128, 0, st>>>(A, nbb, nbs);
  k_adj_gather<<<(unsigned)((N + 127) / 128), 128, 0, st>>>(A);
  if (p->n_links > 0) k_adj_links<<<(p->n_links + 255) / 256, 256, 0, st>>>(A);
  LBM_CUDA_CHECK(cudaGetLastError(), fn);
  return LBM_OK;
}

int adjoint_enqueue(const lbm_problem* p, const lbm_adjoint* adj, int64_t it, const double* x_prev,
                    const double* lam_in, double* lam_out, cudaStream_t st, const char* fn) {
  AdjArgs A;
  adjoint_prepare(p, adj, A);
  return adjoint_launch(p, adj, A, it, x_prev, lam_in, lam_out, st, fn);
}
}  // namespace

extern "C" int lbm_adjoint_step(const lbm_problem* p, const lbm_adjoint* adj, int64_t it,
                                const double* x_prev, const double* lam_in, double* lam_out,
                                void* stream) {
  if (int rc = adjoint_args_check(p, adj, "lbm_adjoint_step")) return rc;
  return adjoint_enqueue(p, adj, it, x_prev, lam_in, lam_out, (cudaStream_t)stream,
                         "lbm_adjoint_step");
}

extern "C" int lbm_adjoint_recompute(const lbm_problem* p, int64_t it_first, int n_steps,
                                     double* states, int64_t stride, void* stream) {
  const char* fn = "lbm_adjoint_recompute";
  if (int rc = problem_check(p, fn)) return rc;
  if (!adjoint_supported(p)) {
    set_error("%s: needs FP64, a Zou-He operation on every wall and all four corners", fn);
    return LBM_ERR_UNSUPPORTED;
  }
  const long long N9 = 9LL * p->nx * p->ny;
  if (!states || n_steps < 1 || it_first < 0 || stride < N9) {
    set_error("%s: bad arguments", fn);
    return LBM_ERR_ARG;
  }
  // Each step reads one slot and writes the next; no drag history (the
  // objective is known from the forward run).
  return fused_enqueue_chain(p, it_first, n_steps, states, stride, (cudaStream_t)stream);
}

extern "C" int lbm_adjoint_sweep(const lbm_problem* p, const lbm_adjoint* adj, int64_t it_first,
                                 int n_steps, const double* states, int64_t stride, double* lam0,
                                 double* lam1, int parity, void* stream) {
  const char* fn = "lbm_adjoint_sweep";
  if (int rc = adjoint_args_check(p, adj, fn)) return rc;
  const long long N9 = 9LL * p->nx * p->ny;
  if (!states || !lam0 || !lam1 || n_steps < 1 || it_first < 0 || stride < N9 ||
      (parity != 0 && parity != 1)) {
    set_error("%s: bad arguments", fn);
    return LBM_ERR_ARG;
  }
  double* lam[2] = {lam0, lam1};
  int cur = parity;
  AdjArgs A;
  adjoint_prepare(p, adj, A);
  for (int64_t n = it_first + n_steps; n > it_first; --n) {
    const double* x_prev = states + (n - 1 - it_first) * stride;
    if (int rc = adjoint_launch(p, adj, A, n, x_prev, lam[cur], lam[cur ^ 1],
                                (cudaStream_t)stream, fn))
      return rc;
    cur ^= 1;
  }
  return LBM_OK;
}

extern "C" int lbm_adjoint_initial(const lbm_problem* p, const lbm_adjoint* adj, const double* g0,
                                   const double* lam_in, double* lam_out, void* stream) {
  if (int rc = problem_check(p, "lbm_adjoint_initial")) return rc;
  if (!adjoint_supported(p) || !adj || !g0 || !lam_in || !lam_out || !adj->grad_omega) {
    set_error("lbm_adjoint_initial: bad arguments");
    return LBM_ERR_ARG;
  }
  AdjArgs A;
  memset(&A, 0, sizeof(A));
  A.f = make_args(p, LBM_MODE_STEP, 0);
  A.k = make_rates(p->om_p, p->om_m, 0.25);
  A.lam_in = lam_in;
  A.lam_out = lam_out;
  A.grad_omega = adj->grad_omega;
  const long long N = (long long)p->nx * p->ny;
  k_adj_initial<<<(unsigned)((N + 255) / 256), 256, 0, (cudaStream_t)stream>>>(A, g0);
  LBM_CUDA_CHECK(cudaGetLastError(), "lbm_adjoint_initial");
  return LBM_OK;
}
