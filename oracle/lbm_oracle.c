/*
 * CPU oracle for the D2Q9 TRT lattice update -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference kernels in jviquerat/lbm
 * (lbm/src/core/nb.py and lattice.macro in lbm/src/core/lattice.py), used by
 * the tests and by the CPU-baseline leg of the benchmark as the checker.  It is
 * never linked into, loaded by or called from the product library.
 *
 * Layout follows the reference: distributions g[q][i][j] (q = 0..8, i = 0..nx-1,
 * j = 0..ny-1, j fastest), rho[i][j], u[d][i][j], BC vectors u_left[d][j],
 * u_right[d][j], u_top[d][i], u_bot[d][i], rho_right[j].
 * D2Q9 order c = (0,0),(1,0),(-1,0),(0,1),(0,-1),(1,1),(-1,-1),(-1,1),(1,-1)
 * (lbm/src/core/lattice.py:135-139), opposite ns = 0,2,1,4,3,6,5,8,7 (:152).
 *
 * Arithmetic is written in the same operation order as the reference
 * expressions and must be compiled without floating-point contraction
 * (-ffp-contract=off) so that x86 and Arm hosts give identical results.
 * Cell loops are split over OpenMP threads (each cell is independent, so the
 * result does not depend on the thread count); link loops stay serial, in
 * the reference's order.
 * Parity with the reference is pinned by the tests/golden/ fixtures, generated from the
 * reference source itself.
 */
#include <stddef.h>
#include <stdlib.h>
#include <stdint.h>

int oracle_threads(void) {
#ifdef _OPENMP
  extern int omp_get_max_threads(void);
  return omp_get_max_threads();
#else
  return 1;
#endif
}

static const int CX[9] = {0, 1, -1, 0, 0, 1, -1, -1, 1};
static const int CY[9] = {0, 0, 0, 1, -1, 1, -1, 1, -1};
static const int NS[9] = {0, 2, 1, 4, 3, 6, 5, 8, 7};

#define G(a, q, i, j) (a)[((size_t)(q) * nx + (size_t)(i)) * ny + (size_t)(j)]
#define F2(a, i, j) (a)[(size_t)(i) * ny + (size_t)(j)]
#define U(a, d, i, j) (a)[((size_t)(d) * nx + (size_t)(i)) * ny + (size_t)(j)]

static double weight(int q) { return q == 0 ? 4.0 / 9.0 : (q < 5 ? 1.0 / 9.0 : 1.0 / 36.0); }

/* Per-cell pieces of the bulk update.  Every public function below (the
 * kernel-level ones and the fused loop of oracle_run) evaluates a cell with
 * these, so a cell gets the same bits whichever entry point computes it.
 * N = nx * ny is the plane size; c = i * ny + j the cell. */

/* lattice.macro, lbm/src/core/lattice.py:178-189: rho = sum_q g (sequential
 * over q), u_d = (sum_q c_qd g_q) / rho. */
static inline void macro_cell(const double* g, size_t N, size_t c, double* r_out,
                              double* ux_out, double* uy_out) {
  double r = g[c];
  for (int q = 1; q < 9; ++q) r += g[q * N + c];
  double jx = 0.0, jy = 0.0;
  for (int q = 0; q < 9; ++q) {
    jx += (double)CX[q] * g[q * N + c];
    jy += (double)CY[q] * g[q * N + c];
  }
  *r_out = r;
  *ux_out = jx / r;
  *uy_out = jy / r;
}

/* nb_equilibrium, lbm/src/core/nb.py:7-17. */
static inline void equilibrium_cell(double ux, double uy, double r, double* geq) {
  double v = 1.5 * (ux * ux + uy * uy);
  for (int q = 0; q < 9; ++q) {
    double t = 3.0 * (ux * (double)CX[q] + uy * (double)CY[q]);
    double e = 1.0 + t + 0.5 * (t * t) - v;
    geq[q] = e * (r * weight(q));
  }
}

/* TRT collision of nb_col_str, lbm/src/core/nb.py:21-37 (g_up of one cell
 * from its g and g_eq). */
static inline void collide_cell(const double* gc, const double* geq, double om_p, double om_m,
                                double* up) {
  const double a = 1.0 - 0.5 * (om_p + om_m);
  const double b = 0.5 * (om_p - om_m);
  const double cc = 0.5 * (om_p + om_m);
  up[0] = (1.0 - om_p) * gc[0] + om_p * geq[0];
  for (int q = 1; q < 9; ++q) {
    int qb = NS[q];
    up[q] = a * gc[q] - b * gc[qb] + cc * geq[q] + b * geq[qb];
  }
}

void oracle_macro(const double* g, double* rho, double* u, int nx, int ny) {
  const size_t N = (size_t)nx * ny;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j) {
      const size_t c = (size_t)i * ny + j;
      macro_cell(g, N, c, &rho[c], &u[c], &u[N + c]);
    }
}

void oracle_equilibrium(const double* u, const double* rho, double* g_eq, int nx, int ny) {
  const size_t N = (size_t)nx * ny;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j) {
      const size_t c = (size_t)i * ny + j;
      double geq[9];
      equilibrium_cell(u[c], u[N + c], rho[c], geq);
      for (int q = 0; q < 9; ++q) g_eq[q * N + c] = geq[q];
    }
}

/* Streaming half of nb_col_str, lbm/src/core/nb.py:38-45: shift-copy of
 * g_up into g on interior slices only (edge entries with no source keep
 * their previous value; no periodic wrap). */
static void stream(double* g, const double* g_up, int nx, int ny) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nx; ++i)
    for (int q = 0; q < 9; ++q) {
      const int si = i - CX[q];
      if (si < 0 || si >= nx) continue;
      const int j0 = CY[q] > 0 ? 1 : 0, j1 = CY[q] < 0 ? ny - 1 : ny;
      for (int j = j0; j < j1; ++j) G(g, q, i, j) = G(g_up, q, si, j - CY[q]);
    }
}

/* nb_col_str, lbm/src/core/nb.py:21-45: TRT collision into g_up, then the
 * shift-copy stream into g. */
void oracle_col_str(double* g, const double* g_eq, double* g_up, double om_p, double om_m,
                    int nx, int ny) {
  const size_t N = (size_t)nx * ny;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j) {
      const size_t c = (size_t)i * ny + j;
      double gc[9], geq[9], up[9];
      for (int q = 0; q < 9; ++q) {
        gc[q] = g[q * N + c];
        geq[q] = g_eq[q * N + c];
      }
      collide_cell(gc, geq, om_p, om_m, up);
      for (int q = 0; q < 9; ++q) g_up[q * N + c] = up[q];
    }
  stream(g, g_up, nx, ny);
}

/* macro, equilibrium and col_str in one pass over the lattice rows (each
 * element computed by the expressions of macro_cell, equilibrium_cell and
 * collide_cell, in their order; a row at a time so that the compiler can
 * vectorise along j), then the stream. */
static void macro_eq_col_str(double* g, double* g_eq, double* g_up, double* rho, double* u,
                             double om_p, double om_m, int nx, int ny) {
  const size_t N = (size_t)nx * ny;
  const double a = 1.0 - 0.5 * (om_p + om_m);
  const double b = 0.5 * (om_p - om_m);
  const double cc = 0.5 * (om_p + om_m);
#pragma omp parallel
  {
    double* jx = (double*)malloc(sizeof(double) * 2 * (size_t)ny);
    double* jy = jx + ny;
#pragma omp for schedule(static)
    for (int i = 0; i < nx; ++i) {
      const size_t r0 = (size_t)i * ny;
      double* restrict r = rho + r0;
      double* restrict ux = u + r0;
      double* restrict uy = u + N + r0;
      for (int j = 0; j < ny; ++j) r[j] = g[r0 + j];
      for (int q = 1; q < 9; ++q) {
        const double* restrict gq = g + q * N + r0;
        for (int j = 0; j < ny; ++j) r[j] += gq[j];
      }
      for (int j = 0; j < ny; ++j) jx[j] = jy[j] = 0.0;
      for (int q = 0; q < 9; ++q) {
        const double* restrict gq = g + q * N + r0;
        const double cx = (double)CX[q], cy = (double)CY[q];
        for (int j = 0; j < ny; ++j) {
          jx[j] += cx * gq[j];
          jy[j] += cy * gq[j];
        }
      }
      for (int j = 0; j < ny; ++j) {
        ux[j] = jx[j] / r[j];
        uy[j] = jy[j] / r[j];
      }
      for (int q = 0; q < 9; ++q) {
        double* restrict eq = g_eq + q * N + r0;
        const double cx = (double)CX[q], cy = (double)CY[q], w = weight(q);
        for (int j = 0; j < ny; ++j) {
          double v = 1.5 * (ux[j] * ux[j] + uy[j] * uy[j]);
          double t = 3.0 * (ux[j] * cx + uy[j] * cy);
          double e = 1.0 + t + 0.5 * (t * t) - v;
          eq[j] = e * (r[j] * w);
        }
      }
      {
        const double* restrict g0 = g + r0;
        const double* restrict e0 = g_eq + r0;
        double* restrict u0 = g_up + r0;
        for (int j = 0; j < ny; ++j) u0[j] = (1.0 - om_p) * g0[j] + om_p * e0[j];
      }
      for (int q = 1; q < 9; ++q) {
        const int qb = NS[q];
        const double* restrict gq = g + q * N + r0;
        const double* restrict gb = g + qb * N + r0;
        const double* restrict eq = g_eq + q * N + r0;
        const double* restrict eb = g_eq + qb * N + r0;
        double* restrict up = g_up + q * N + r0;
        for (int j = 0; j < ny; ++j) up[j] = a * gq[j] - b * gb[j] + cc * eq[j] + b * eb[j];
      }
    }
    free(jx);
  }
  stream(g, g_up, nx, ny);
}

/* Python-style index: -n <= k < 0 wraps, k >= n is an error (the reference
 * raises IndexError under NumPy). */
static int wrap_index(long k, int n, int* ok) {
  if (k < 0) k += n;
  if (k < 0 || k >= n) { *ok = 0; return 0; }
  return (int)k;
}

/* Momentum-exchange sums of nb_drag_lift, lbm/src/core/nb.py:49-69
 * (sequential sum over links). */
static int drag_sums(const int64_t* links, int64_t n, const double* g_up, const double* g, int nx,
                     int ny, double* fx_out, double* fy_out) {
  double fx = 0.0, fy = 0.0;
  for (int64_t k = 0; k < n; ++k) {
    int ok = 1;
    int i = wrap_index(links[3 * k], nx, &ok), j = wrap_index(links[3 * k + 1], ny, &ok);
    int q = (int)links[3 * k + 2];
    if (!ok || q < 0 || q > 8) return -1;
    int qb = NS[q];
    double g0 = G(g_up, q, i, j) + G(g, qb, i, j);
    fx += g0 * (double)CX[q];
    fy += g0 * (double)CY[q];
  }
  *fx_out = fx;
  *fy_out = fy;
  return 0;
}

/* nb_drag_lift, lbm/src/core/nb.py:49-73. */
int oracle_drag_lift(const int64_t* links, int64_t n, const double* g_up, const double* g, int nx,
                     int ny, double R_ref, double U_ref, double L_ref, double* out_cx_cy) {
  double fx, fy;
  if (drag_sums(links, n, g_up, g, nx, ny, &fx, &fy)) return -1;
  out_cx_cy[0] = -2.0 * fx / (R_ref * L_ref * (U_ref * U_ref));
  out_cx_cy[1] = -2.0 * fy / (R_ref * L_ref * (U_ref * U_ref));
  return 0;
}

/* nb_bounce_back_obstacle, lbm/src/core/nb.py:77-117: quadratic interpolated
 * bounce-back (ibb != 0) or halfway bounce-back, links applied in order. */
int oracle_bounce_back(int ibb, const int64_t* links, int64_t n, const double* p_ibb,
                       const double* g_up, double* g, int nx, int ny) {
  for (int64_t k = 0; k < n; ++k) {
    int ok = 1;
    long i0 = links[3 * k], j0 = links[3 * k + 1];
    int q = (int)links[3 * k + 2];
    if (q < 0 || q > 8) return -1;
    int qb = NS[q];
    int i = wrap_index(i0, nx, &ok), j = wrap_index(j0, ny, &ok);
    if (!ok) return -1;
    if (ibb) {
      int im = wrap_index(i0 + CX[qb], nx, &ok), jm = wrap_index(j0 + CY[qb], ny, &ok);
      if (!ok) return -1;
      double p = p_ibb[k];
      double pp = 2.0 * p;
      if (p < 0.5) {
        /* x + 2 c_qb is only indexed in this branch (nb.py:98-100) */
        int imm = wrap_index(i0 + 2 * CX[qb], nx, &ok), jmm = wrap_index(j0 + 2 * CY[qb], ny, &ok);
        if (!ok) return -1;
        G(g, qb, i, j) = p * (pp + 1.0) * G(g_up, q, i, j) +
                         (1.0 + pp) * (1.0 - pp) * G(g_up, q, im, jm) -
                         p * (1.0 - pp) * G(g_up, q, imm, jmm);
      } else {
        G(g, qb, i, j) = (1.0 / (p * (pp + 1.0))) * G(g_up, q, i, j) +
                         ((pp - 1.0) / p) * G(g_up, qb, i, j) +
                         ((1.0 - pp) / (1.0 + pp)) * G(g_up, qb, im, jm);
      }
    } else {
      G(g, qb, i, j) = G(g_up, q, i, j);
    }
  }
  return 0;
}

static const double C1 = 2.0 / 3.0, C2 = 1.0 / 6.0, C3 = 1.0 / 2.0;

/* nb_zou_he_left_wall_velocity, lbm/src/core/nb.py:121-143. */
void oracle_zh_left(double* u, const double* u_left, double* rho, double* g, int nx, int ny) {
  for (int j = 0; j < ny; ++j) {
    U(u, 0, 0, j) = u_left[j];
    U(u, 1, 0, j) = u_left[ny + j];
    double ux = U(u, 0, 0, j), uy = U(u, 1, 0, j);
    double r = (G(g, 0, 0, j) + G(g, 3, 0, j) + G(g, 4, 0, j) + 2.0 * G(g, 2, 0, j) +
                2.0 * G(g, 6, 0, j) + 2.0 * G(g, 7, 0, j)) / (1.0 - ux);
    F2(rho, 0, j) = r;
    G(g, 1, 0, j) = G(g, 2, 0, j) + C1 * r * ux;
    G(g, 5, 0, j) = G(g, 6, 0, j) - C3 * (G(g, 3, 0, j) - G(g, 4, 0, j)) + C2 * r * ux + C3 * r * uy;
    G(g, 8, 0, j) = G(g, 7, 0, j) + C3 * (G(g, 3, 0, j) - G(g, 4, 0, j)) + C2 * r * ux - C3 * r * uy;
  }
}

/* nb_zou_he_right_wall_velocity, lbm/src/core/nb.py:147-169. */
void oracle_zh_right(double* u, const double* u_right, double* rho, double* g, int nx, int ny) {
  const int lx = nx - 1;
  for (int j = 0; j < ny; ++j) {
    U(u, 0, lx, j) = u_right[j];
    U(u, 1, lx, j) = u_right[ny + j];
    double ux = U(u, 0, lx, j), uy = U(u, 1, lx, j);
    double r = (G(g, 0, lx, j) + G(g, 3, lx, j) + G(g, 4, lx, j) + 2.0 * G(g, 1, lx, j) +
                2.0 * G(g, 5, lx, j) + 2.0 * G(g, 8, lx, j)) / (1.0 + ux);
    F2(rho, lx, j) = r;
    G(g, 2, lx, j) = G(g, 1, lx, j) - C1 * r * ux;
    G(g, 6, lx, j) = G(g, 5, lx, j) + C3 * (G(g, 3, lx, j) - G(g, 4, lx, j)) - C2 * r * ux - C3 * r * uy;
    G(g, 7, lx, j) = G(g, 8, lx, j) - C3 * (G(g, 3, lx, j) - G(g, 4, lx, j)) - C2 * r * ux + C3 * r * uy;
  }
}

/* nb_zou_he_right_wall_pressure, lbm/src/core/nb.py:173-195. */
void oracle_zh_right_pressure(double* u, const double* rho_right, const double* u_right,
                              double* rho, double* g, int nx, int ny) {
  const int lx = nx - 1;
  for (int j = 0; j < ny; ++j) {
    F2(rho, lx, j) = rho_right[j];
    U(u, 1, lx, j) = u_right[ny + j];
    double r = F2(rho, lx, j);
    U(u, 0, lx, j) = (G(g, 0, lx, j) + G(g, 3, lx, j) + G(g, 4, lx, j) + 2.0 * G(g, 1, lx, j) +
                      2.0 * G(g, 5, lx, j) + 2.0 * G(g, 8, lx, j)) / r - 1.0;
    double ux = U(u, 0, lx, j), uy = U(u, 1, lx, j);
    G(g, 2, lx, j) = G(g, 1, lx, j) - C1 * r * ux;
    G(g, 6, lx, j) = G(g, 5, lx, j) + C3 * (G(g, 3, lx, j) - G(g, 4, lx, j)) - C2 * r * ux - C3 * r * uy;
    G(g, 7, lx, j) = G(g, 8, lx, j) - C3 * (G(g, 3, lx, j) - G(g, 4, lx, j)) - C2 * r * ux + C3 * r * uy;
  }
}

/* nb_zou_he_top_wall_velocity, lbm/src/core/nb.py:199-221. */
void oracle_zh_top(double* u, const double* u_top, double* rho, double* g, int nx, int ny) {
  const int ly = ny - 1;
  for (int i = 0; i < nx; ++i) {
    U(u, 0, i, ly) = u_top[i];
    U(u, 1, i, ly) = u_top[nx + i];
    double ux = U(u, 0, i, ly), uy = U(u, 1, i, ly);
    double r = (G(g, 0, i, ly) + G(g, 1, i, ly) + G(g, 2, i, ly) + 2.0 * G(g, 3, i, ly) +
                2.0 * G(g, 5, i, ly) + 2.0 * G(g, 7, i, ly)) / (1.0 + uy);
    F2(rho, i, ly) = r;
    G(g, 4, i, ly) = G(g, 3, i, ly) - C1 * r * uy;
    G(g, 8, i, ly) = G(g, 7, i, ly) - C3 * (G(g, 1, i, ly) - G(g, 2, i, ly)) + C3 * r * ux - C2 * r * uy;
    G(g, 6, i, ly) = G(g, 5, i, ly) + C3 * (G(g, 1, i, ly) - G(g, 2, i, ly)) - C3 * r * ux - C2 * r * uy;
  }
}

/* nb_zou_he_bottom_wall_velocity, lbm/src/core/nb.py:225-247. */
void oracle_zh_bottom(double* u, const double* u_bot, double* rho, double* g, int nx, int ny) {
  for (int i = 0; i < nx; ++i) {
    U(u, 0, i, 0) = u_bot[i];
    U(u, 1, i, 0) = u_bot[nx + i];
    double ux = U(u, 0, i, 0), uy = U(u, 1, i, 0);
    double r = (G(g, 0, i, 0) + G(g, 1, i, 0) + G(g, 2, i, 0) + 2.0 * G(g, 4, i, 0) +
                2.0 * G(g, 6, i, 0) + 2.0 * G(g, 8, i, 0)) / (1.0 - uy);
    F2(rho, i, 0) = r;
    G(g, 3, i, 0) = G(g, 4, i, 0) + C1 * r * uy;
    G(g, 5, i, 0) = G(g, 6, i, 0) - C3 * (G(g, 1, i, 0) - G(g, 2, i, 0)) + C3 * r * ux + C2 * r * uy;
    G(g, 7, i, 0) = G(g, 8, i, 0) + C3 * (G(g, 1, i, 0) - G(g, 2, i, 0)) - C3 * r * ux + C2 * r * uy;
  }
}

/* Corners, lbm/src/core/nb.py:250-344.  corner: 0 = bottom-left,
 * 1 = top-left, 2 = top-right, 3 = bottom-right. */
void oracle_corner(int corner, double* u, double* rho, double* g, int nx, int ny) {
  const int lx = nx - 1, ly = ny - 1;
  int i, j, in;
  int k1, k2, k3, z1, z2;          /* set, set, set, zeroed, zeroed */
  int s1, s2, s3;                  /* sources of the three set populations */
  double a1, a2, b1, b2;           /* signs: k1 = s1 + a1*2/3 r ux; k2 = s2 + a2*2/3 r uy; k3 = s3 + b1/6 r ux + b2/6 r uy */
  switch (corner) {
    case 0: i = 0; j = 0; in = 1; k1 = 1; s1 = 2; a1 = 1; k2 = 3; s2 = 4; a2 = 1;
            k3 = 5; s3 = 6; b1 = 1; b2 = 1; z1 = 7; z2 = 8; break;
    case 1: i = 0; j = ly; in = 1; k1 = 1; s1 = 2; a1 = 1; k2 = 4; s2 = 3; a2 = -1;
            k3 = 8; s3 = 7; b1 = 1; b2 = -1; z1 = 5; z2 = 6; break;
    case 2: i = lx; j = ly; in = lx - 1; k1 = 2; s1 = 1; a1 = -1; k2 = 4; s2 = 3; a2 = -1;
            k3 = 6; s3 = 5; b1 = -1; b2 = -1; z1 = 7; z2 = 8; break;
    default: i = lx; j = 0; in = lx - 1; k1 = 2; s1 = 1; a1 = -1; k2 = 3; s2 = 4; a2 = 1;
            k3 = 7; s3 = 8; b1 = -1; b2 = 1; z1 = 5; z2 = 6; break;
  }
  U(u, 0, i, j) = U(u, 0, in, j);
  U(u, 1, i, j) = U(u, 1, in, j);
  F2(rho, i, j) = F2(rho, in, j);
  double r = F2(rho, i, j), ux = U(u, 0, i, j), uy = U(u, 1, i, j);
  G(g, k1, i, j) = a1 > 0 ? G(g, s1, i, j) + (2.0 / 3.0) * r * ux : G(g, s1, i, j) - (2.0 / 3.0) * r * ux;
  G(g, k2, i, j) = a2 > 0 ? G(g, s2, i, j) + (2.0 / 3.0) * r * uy : G(g, s2, i, j) - (2.0 / 3.0) * r * uy;
  {
    double t = G(g, s3, i, j);
    t = b1 > 0 ? t + (1.0 / 6.0) * r * ux : t - (1.0 / 6.0) * r * ux;
    t = b2 > 0 ? t + (1.0 / 6.0) * r * uy : t - (1.0 / 6.0) * r * uy;
    G(g, k3, i, j) = t;
  }
  G(g, z1, i, j) = 0.0;
  G(g, z2, i, j) = 0.0;
  G(g, 0, i, j) = r - G(g, 1, i, j) - G(g, 2, i, j) - G(g, 3, i, j) - G(g, 4, i, j) - G(g, 5, i, j) -
                  G(g, 6, i, j) - G(g, 7, i, j) - G(g, 8, i, j);
}

/* The driver loop of lbm/src/core/run.py:24-54 for an app whose outputs hook
 * does nothing, whose set_inlets sets the BC vectors to
 * base + scale(it) * vec (every app's ramp, lbm/src/app/cavity.py:65-76,
 * turek.py:94-109) and whose set_bc is a fixed sequence of lattice calls.
 * Iterations it0 .. it0 + n_iter - 1:
 *
 *   set_inlets(it); macro; equilibrium; col_str; set_bc; drag/lift sums
 *
 * with the kernels above, so every value equals the one the kernel-level
 * entry points give when a host loop calls them in that order.
 *
 * prog: n_prog pairs (kind, arg) in set_bc call order: kind 0 = bounce-back
 * of obstacle arg (links[obs_start[arg] .. obs_start[arg+1]) and the IBB
 * distances p at the same offsets), 1 = Zou-He wall arg (0 left velocity,
 * 1 right velocity, 2 right pressure, 3 top velocity, 4 bottom velocity),
 * 2 = corner arg (0 bottom-left, 1 top-left, 2 top-right, 3 bottom-right).
 * bc_base, bc_vec: packed u_left | u_right | u_top | u_bot | rho_right
 * (bc_vec NULL: constant); scale[k]: the scale of iteration it0 + k.
 * drag (optional): n_iter x n_obs x 2 raw sums (fx, fy) of every obstacle
 * after set_bc, i.e. nb_drag_lift before its -2 / (R L U^2) factor.
 * Returns 0, or -1 when a link or a program entry is out of range. */
int oracle_run(double* g, double* g_eq, double* g_up, double* rho, double* u, double* u_left,
               double* u_right, double* u_top, double* u_bot, double* rho_right, int nx, int ny,
               double om_p, double om_m, int ibb, const int32_t* prog, int n_prog,
               const int64_t* links, const int64_t* obs_start, const double* p, int n_obs,
               const double* bc_base, const double* bc_vec, const double* scale,
               int64_t n_iter, double* drag) {
  const size_t nb = (size_t)4 * ny + (size_t)4 * nx + (size_t)ny;
  for (int k = 0; k < n_prog; ++k) {
    const int kind = prog[2 * k], arg = prog[2 * k + 1];
    if ((kind == 0 && (arg < 0 || arg >= n_obs)) || (kind == 1 && (arg < 0 || arg > 4)) ||
        (kind == 2 && (arg < 0 || arg > 3)) || kind < 0 || kind > 2)
      return -1;
  }
  for (int64_t it = 0; it < n_iter; ++it) {
    /* set_inlets */
    const double s = scale ? scale[it] : 0.0;
    for (size_t e = 0; e < nb; ++e) {
      const double v = bc_vec ? bc_base[e] + s * bc_vec[e] : bc_base[e];
      if (e < (size_t)2 * ny) u_left[e] = v;
      else if (e < (size_t)4 * ny) u_right[e - 2 * (size_t)ny] = v;
      else if (e < (size_t)4 * ny + 2 * (size_t)nx) u_top[e - 4 * (size_t)ny] = v;
      else if (e < (size_t)4 * ny + 4 * (size_t)nx) u_bot[e - 4 * (size_t)ny - 2 * (size_t)nx] = v;
      else rho_right[e - 4 * (size_t)ny - 4 * (size_t)nx] = v;
    }
    /* macro, equilibrium, collision_stream */
    macro_eq_col_str(g, g_eq, g_up, rho, u, om_p, om_m, nx, ny);
    /* set_bc */
    for (int k = 0; k < n_prog; ++k) {
      const int kind = prog[2 * k], arg = prog[2 * k + 1];
      if (kind == 0) {
        const int64_t l0 = obs_start[arg], n = obs_start[arg + 1] - l0;
        if (oracle_bounce_back(ibb, links + 3 * l0, n, ibb ? p + l0 : p, g_up, g, nx, ny))
          return -1;
      } else if (kind == 1) {
        switch (arg) {
          case 0: oracle_zh_left(u, u_left, rho, g, nx, ny); break;
          case 1: oracle_zh_right(u, u_right, rho, g, nx, ny); break;
          case 2: oracle_zh_right_pressure(u, rho_right, u_right, rho, g, nx, ny); break;
          case 3: oracle_zh_top(u, u_top, rho, g, nx, ny); break;
          default: oracle_zh_bottom(u, u_bot, rho, g, nx, ny); break;
        }
      } else {
        oracle_corner(arg, u, rho, g, nx, ny);
      }
    }
    /* observables */
    if (drag)
      for (int o = 0; o < n_obs; ++o) {
        const int64_t l0 = obs_start[o], n = obs_start[o + 1] - l0;
        double* d = drag + ((size_t)it * n_obs + o) * 2;
        if (drag_sums(links + 3 * l0, n, g_up, g, nx, ny, &d[0], &d[1])) return -1;
      }
  }
  return 0;
}
