// Device-side building blocks of the D2Q9 TRT lattice update.
//
// D2Q9 order c = (0,0),(1,0),(-1,0),(0,1),(0,-1),(1,1),(-1,-1),(-1,1),(1,-1),
// opposite ns = 0,2,1,4,3,6,5,8,7 and weights 4/9, 1/9 x4, 1/36 x4, as in the
// reference (lbm/src/core/lattice.py:135-152).  Distributions are stored
// q-major, g[q][i][j] with j fastest (lattice.py:155-157): plane q of a
// lattice with N = nx*ny cells starts at q*N and cell (i, j) is i*ny + j.
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <stdint.h>

namespace lbm {

__host__ __device__ constexpr int cx(int q) {
  return q == 1 || q == 5 || q == 8 ? 1 : (q == 2 || q == 6 || q == 7 ? -1 : 0);
}
__host__ __device__ constexpr int cy(int q) {
  return q == 3 || q == 5 || q == 7 ? 1 : (q == 4 || q == 6 || q == 8 ? -1 : 0);
}
__host__ __device__ constexpr int opp(int q) {
  return q == 0 ? 0 : (q & 1 ? q + 1 : q - 1);
}
__host__ __device__ constexpr double wgt(int q) {
  return q == 0 ? 4.0 / 9.0 : (q < 5 ? 1.0 / 9.0 : 1.0 / 36.0);
}

// ---------------------------------------------------------------------------
// Reciprocal.  FP64: hardware approximation (PTX rcp.approx.ftz.f64) refined
// by one third-order Householder step r <- r + r*(e + e^2), e = 1 - x*r
// (Householder, "The Numerical Treatment of a Single Nonlinear Equation",
// 1970); the error after the step is about 1 ulp for the density range of a
// lattice (|rho - 1| << 1).  FP32: plain IEEE division by the compiler.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double recip(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  double e = fma(-x, r, 1.0);
  double e2 = fma(e, e, e);
  return fma(r, e2, r);
}
__device__ __forceinline__ float recip(float x) { return 1.0f / x; }

// ---------------------------------------------------------------------------
// Storage forms.  Full-precision values are T (double for F64, float for the
// reduced forms); shifted forms store d = kScale (f - w_q * rho0).  FP16
// stores the deviations times 2^10: FP16's normal range [2^-14, 65504] then
// covers |f - w rho0| in [6e-8, 64], so the small deviations of a slowly
// starting flow keep 11 significant bits instead of falling into FP16's
// subnormals (and its overflow bound stays far above any deviation of a
// stable lattice).  The scale is exact (a power of two) and folds into the
// moments (moments(): rho = rho0 + drho / kScale, u = j / (kScale rho)); the
// collision is linear in (d, drho, j) at fixed u.
// ---------------------------------------------------------------------------
// store_r(p, v, r): the store of a kernel's update, given 32 random bits r;
// only the stochastic-rounding forms use r.
#ifndef LBM_F16_SCALE_LOG2
#define LBM_F16_SCALE_LOG2 10
#endif
struct StoreF64 {
  using S = double;
  using T = double;
  static constexpr bool kShift = false;
  static constexpr bool kFixed = false;
  static constexpr bool kStochastic = false;
  static constexpr T kScale = 1, kInvScale = 1;
  __device__ static T load(const S* p) { return *p; }
  __device__ static void store(S* p, T v) { *p = v; }
  __device__ static void store_r(S* p, T v, unsigned) { *p = v; }
  __device__ static void store_pair(S* p, T v0, T v1, unsigned) { p[0] = v0; p[1] = v1; }
};
struct StoreF32 {
  using S = float;
  using T = float;
  static constexpr bool kShift = true;
  static constexpr bool kFixed = false;
  static constexpr bool kStochastic = false;
  static constexpr T kScale = 1, kInvScale = 1;
  __device__ static T load(const S* p) { return *p; }
  __device__ static void store(S* p, T v) { *p = v; }
  __device__ static void store_r(S* p, T v, unsigned) { *p = v; }
  __device__ static void store_pair(S* p, T v0, T v1, unsigned) { p[0] = v0; p[1] = v1; }
};
struct StoreF16 {
  using S = __half;
  using T = float;
  static constexpr bool kShift = true;
  static constexpr bool kFixed = false;
  static constexpr bool kStochastic = false;
  static constexpr T kScale = (T)(1 << LBM_F16_SCALE_LOG2), kInvScale = T(1) / kScale;
  __device__ static T load(const S* p) { return __half2float(*p); }
  __device__ static void store(S* p, T v) { *p = __float2half_rn(v); }
  __device__ static void store_r(S* p, T v, unsigned) { *p = __float2half_rn(v); }
  // p[0] = v0, p[1] = v1 (p 4-byte aligned), one packed conversion.
  __device__ static void store_pair(S* p, T v0, T v1, unsigned) {
    *reinterpret_cast<__half2*>(p) = __floats2half2_rn(v0, v1);
  }
};
struct StoreBF16 {
  using S = __nv_bfloat16;
  using T = float;
  static constexpr bool kShift = true;
  static constexpr bool kFixed = false;
  static constexpr bool kStochastic = false;
  static constexpr T kScale = 1, kInvScale = 1;
  __device__ static T load(const S* p) { return __bfloat162float(*p); }
  __device__ static void store(S* p, T v) { *p = __float2bfloat16_rn(v); }
  __device__ static void store_r(S* p, T v, unsigned) { *p = __float2bfloat16_rn(v); }
  __device__ static void store_pair(S* p, T v0, T v1, unsigned) {
    *reinterpret_cast<__nv_bfloat162*>(p) = __floats2bfloat162_rn(v0, v1);
  }
};

// ---------------------------------------------------------------------------
// Stochastic rounding for the 16-bit forms.  Round-to-nearest storage loses
// every per-iteration change of a population smaller than half an ulp of its
// deviation, which damps slow dynamics (vortex shedding amplitude in a
// cylinder wake); rounding up with probability equal to the discarded
// fraction keeps those changes in expectation.  FP32 -> FP16: add 13 random
// bits below the 10 kept mantissa bits and truncate; FP32 -> BF16: 16 bits
// below 7.  Values below the FP16 normal range (|v| < 2^-14) or near its top
// round to nearest.  The random bits come from a deterministic hash of
// (cell, iteration) advanced by xorshift32 per store, so runs are repeatable.
// ---------------------------------------------------------------------------
// 32-bit integer hash "lowbias32" (C. Wellons, hash-prospector, public domain).
__device__ __forceinline__ unsigned hash32(unsigned x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}
// xorshift32 (G. Marsaglia, "Xorshift RNGs", J. Stat. Softw. 8(14), 2003).
__device__ __forceinline__ unsigned xorshift32(unsigned x) {
  x ^= x << 13;
  x ^= x >> 17;
  x ^= x << 5;
  return x;
}
// Random state of one cell at one iteration (never zero): sr_cell of the
// cell's storage index and sr_iter of the iteration.
__device__ __forceinline__ unsigned sr_iter(long long it) {
  return hash32((unsigned)it * 0x9e3779b9u + 0x632be5abu);
}
__device__ __forceinline__ unsigned sr_cell(long long cell, unsigned it_hash) {
  return hash32((unsigned)cell ^ it_hash) | 1u;
}
__device__ __forceinline__ unsigned sr_seed(long long cell, long long it) {
  return sr_cell(cell, sr_iter(it));
}
__device__ __forceinline__ __half half_sr(float v, unsigned r) {
  const unsigned b = __float_as_uint(v), mag = b & 0x7fffffffu;
  if (mag < 0x38800000u || mag >= 0x477fe000u) return __float2half_rn(v);
  return __float2half_rz(__uint_as_float(b + (r & 0x1fffu)));
}
__device__ __forceinline__ __nv_bfloat16 bf16_sr(float v, unsigned r) {
  const unsigned b = __float_as_uint(v), mag = b & 0x7fffffffu;
  if (mag < 0x00800000u || mag >= 0x7f7f0000u) return __float2bfloat16_rn(v);
  return __float2bfloat16_rz(__uint_as_float(b + (r & 0xffffu)));
}
// Linear congruential step (constants of Numerical Recipes, 2nd ed., 7.1).
__device__ __forceinline__ unsigned lcg32(unsigned x) { return x * 1664525u + 1013904223u; }

// Packed stochastic rounding in one instruction (cvt.rs, sm_100 and later):
// the random bits rbits are added below the kept mantissa bits before
// truncation, as the dither above, bits 0..12 for the low element and
// 16..28 for the high one (FP16), 0..15 and 16..31 (BF16) -- the layout of
// the instruction, confirmed on the GB300 with one bit set at a time on
// values halfway between two neighbours.  The FP16 pair stores pass the LCG
// state itself: the high element takes bits 16..28, the low one bits
// 0..12, whose lowest bits repeat with short periods (bit k with period
// 2^(k+1) along the state sequence).  The hashed (cell, iteration) seed has
// bit 0 set and uniform bits 1..31, so every state has uniform bits 1..31
// and a bit 0 fixed by its position in the sequence: each rounding is
// unbiased to within 2^-13 of an ulp, and the regular low bits only
// correlate the least significant dither bits (below 2^-8 of an ulp) of one
// cell pair's planes.
// Tempering the state first (r ^ r >> 15) cost 4 % of the FP16 bulk kernel.
__device__ __forceinline__ unsigned f16x2_rs(float lo, float hi, unsigned rbits) {
  unsigned d;
  asm("cvt.rs.f16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(hi), "f"(lo), "r"(rbits));
  return d;
}

struct StoreF16SR : StoreF16 {
  static constexpr bool kStochastic = true;
  __device__ static void store_r(S* p, T v, unsigned r) { *p = half_sr(v, r); }
  __device__ static void store_pair(S* p, T v0, T v1, unsigned r) {
    *reinterpret_cast<unsigned*>(p) = f16x2_rs(v0, v1, r);
  }
};
// BF16 pairs keep the dither: 16 random bits below the 7 kept mantissa bits
// of each value (bits 16..31 of the state and of one more LCG step), then a
// truncating packed conversion.  Measured on 8192x2048: 111.5 us per bulk
// launch, against 127.1 us with bf16x2_rs.
__device__ __forceinline__ unsigned bf16x2_rz(float lo, float hi) {
  unsigned d;
  asm("cvt.rz.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
  return d;
}
struct StoreBF16SR : StoreBF16 {
  static constexpr bool kStochastic = true;
  __device__ static void store_r(S* p, T v, unsigned r) { *p = bf16_sr(v, r); }
  __device__ static void store_pair(S* p, T v0, T v1, unsigned r) {
    const unsigned r2 = lcg32(r);
    const float a = __uint_as_float(__float_as_uint(v0) + (r >> 16));
    const float b = __uint_as_float(__float_as_uint(v1) + (r2 >> 16));
    *reinterpret_cast<unsigned*>(p) = bf16x2_rz(a, b);
  }
};

// ---------------------------------------------------------------------------
// 64-bit fixed point, Q3.60: a population f is held as the signed integer
// X = round(f * 2^60), |f| < 8.  Resolution 2^-60 = 8.7e-19, finer than half
// an FP64 ulp for every |f| >= 2^-7; sums of populations are exact.  The
// bulk collision of this form runs on the integer pipes (collide_q60), which
// on GB300 issue 64-bit high multiplies several times faster than the FP64
// pipe issues DFMA.  Cells that need FP64 (walls, obstacle links) convert on
// load and store.  kQ60Bad marks a value outside the range (NaN, Inf or
// |f| >= 8); it converts back to NaN.
// ---------------------------------------------------------------------------
constexpr long long kQ60Bad = (long long)0x8000000000000000ULL;

// Conversions on the integer pipes (the FP64 <-> int64 conversion
// instructions issue at the FP64 rate on GB300).  Both round to nearest,
// ties to even, like cvt.rni.s64.f64 of v 2^60 and cvt.rn.f64.s64 of x
// scaled by 2^-60; double -> Q3.60 is exact for |v| >= 2^-8.
__device__ __forceinline__ long long q60_from_double(double v) {
  typedef unsigned long long ull;
  const ull b = (ull)__double_as_longlong(v);
  const int e = (int)((b >> 52) & 0x7ff);
  if (e > 1025) return kQ60Bad;  // |v| >= 8, Inf or NaN
  const ull m = (b & 0xfffffffffffffULL) | (1ULL << 52);
  const int sh = e - 1015;  // X = m 2^(e - 1075 + 60)
  ull X = 0;
  if (sh >= 0) {
    X = m << sh;
  } else if (sh > -54) {
    const int r = -sh;
    const ull q = m >> r, rem = m & ((1ULL << r) - 1), half = 1ULL << (r - 1);
    X = q + (ull)((rem > half) | ((rem == half) & (q & 1)));
  }  // else below 2^-61: zero (zeros and subnormals included)
  return (b >> 63) ? -(long long)X : (long long)X;
}
__device__ __forceinline__ double q60_to_double(long long x) {
  typedef unsigned long long ull;
  if (x == kQ60Bad) return __longlong_as_double(0x7ff8000000000000LL);
  if (x == 0) return 0.0;
  const ull sgn = (ull)x & (1ULL << 63);
  const ull a = x < 0 ? (ull)(-x) : (ull)x;
  const int lz = __clzll((long long)a);  // >= 1
  const ull n = a << lz;                  // leading one at bit 63
  ull m = n >> 11;                        // 53 bits, leading one at bit 52
  const ull rem = n & 0x7ff;
  m += (ull)((rem > 0x400) | ((rem == 0x400) & (m & 1)));
  // a 2^-60 has biased exponent 1026 - lz; m carries the leading one (and a
  // rounding carry) into the exponent field.
  return __longlong_as_double((long long)((((ull)(1025 - lz)) << 52) + m) | (long long)sgn);
}

struct StoreQ60 {
  using S = long long;
  using T = double;
  static constexpr bool kShift = false;
  static constexpr bool kFixed = true;
  static constexpr bool kStochastic = false;
  static constexpr T kScale = 1, kInvScale = 1;
  __device__ static T load(const S* p) { return q60_to_double(*p); }
  __device__ static void store(S* p, T v) { *p = q60_from_double(v); }
  __device__ static void store_r(S* p, T v, unsigned) { *p = q60_from_double(v); }
  __device__ static void store_pair(S* p, T v0, T v1, unsigned) {
    p[0] = q60_from_double(v0);
    p[1] = q60_from_double(v1);
  }
};

// Signed 64 x 64 -> high 64 multiply from three 32 x 32 -> 64 products.
// x = h 2^32 + l with both halves signed 32-bit (split); then
//   x y / 2^64 = xh yh + (xh yl + xl yh) / 2^32 + xl yl / 2^64,
// and mul_hi drops the last term and floors the middle one: the result is
// within (-1/4, 5/4) of x y / 2^64 for |x|, |y| < 2^62.  Three IMAD.WIDE
// instead of the longer unsigned-product-plus-sign-correction sequence of
// mul.hi.s64.
struct Split {
  int h, l;
};
__host__ __device__ __forceinline__ Split split(long long x) {
  Split s;
  s.l = (int)(unsigned)x;
  s.h = (int)(x >> 32) + (int)((unsigned)x >> 31);
  return s;
}
__device__ __forceinline__ long long mul_hi(Split x, Split y) {
  const long long cross = (long long)x.h * y.l + (long long)x.l * y.h;
  return (long long)x.h * y.h + (cross >> 32);
}

// TRT coefficients of the Q3.60 collision as split integers (host:
// make_coef_q60).  A constant c with |c| < 1/2 is stored as round(c 2^64)
// and applied as mul_hi(x, C); |c| < 1 as round(c 2^63) applied to x << 1.
struct CoefQ60 {
  Split alpha;   // (1 - om_p) / 2   * 2^64
  Split beta;    // (1 - om_m) / 2   * 2^64
  Split a0;      // (1 - om_p)       * 2^63
  Split wp;      // om_p w1 = om_p/9 * 2^64
  Split wm;      // 3 om_m w1 = om_m/3 * 2^63
  Split c1;      // 4.5 om_p w1 = om_p/2 * 2^63
  Split third;   // 1/3 * 2^64
};

// Moments and TRT collision of one cell in Q3.60, in place on x[0..8].
// Same update as collide() above (pair form), with
//   A_q = alpha s_q + om_p w_q P_q,  B_q = beta t_q + 3 om_m w_q c_q.j,
//   g_up_q = A_q + B_q,  g_up_qb = A_q - B_q,  s = g_q + g_qb, t = g_q - g_qb,
//   P_q = rho + 4.5 (c_q.j)^2/rho - 1.5 |j|^2/rho,
// where 1/rho comes from an FP32 seed refined by one cubic step in integer
// arithmetic.  Every product is a mul_hi (error below 1.25 units of 2^-60).
// Returns false, leaving x undefined, when the state is outside the range of
// the form: rho not in (9/16, 15/4), a momentum component |j| >= 3/2, or a
// velocity component |u| >= 3 / om_p.  (rho, jx, jy) are returned in
// Q3.60 for the macro output.
__device__ __forceinline__ bool collide_q60(long long x[9], const CoefQ60& k, long long& rho,
                                            long long& jx, long long& jy) {
  typedef long long ll;
  typedef unsigned long long ull;
  const ll s12 = x[1] + x[2], t12 = x[1] - x[2];
  const ll s34 = x[3] + x[4], t34 = x[3] - x[4];
  const ll s56 = x[5] + x[6], t56 = x[5] - x[6];
  const ll s78 = x[7] + x[8], t78 = x[7] - x[8];
  rho = (((x[0] + s12) + s34) + s56) + s78;
  jx = (t12 + t56) - t78;
  jy = (t34 + t56) + t78;
  // Range of the form (keeps every operand of mul_hi below 2^63 - 2^32).
  const ll kRhoLo = 9LL << 56, kRhoHi = 15LL << 58, kJ = 3LL << 59;
  bool ok = (ull)(rho - kRhoLo - 1) < (ull)(kRhoHi - kRhoLo - 1);
  ok &= (ull)(jx + kJ - 1) < (ull)(2 * kJ - 1);
  ok &= (ull)(jy + kJ - 1) < (ull)(2 * kJ - 1);
  if (!ok) return false;

  // 1/rho in Q61 (K in (2^59, 2^62)): FP32 reciprocal of the top 32 bits of
  // rho as the seed (about 23 bits), then K <- K (1 + e + e^2), e = 1 - rho K
  // (Householder's third-order step), e in Q59.
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"((float)(int)(rho >> 32)));
  const unsigned K0 = __float2uint_rn(r * 0x1p57f);  // 1/rho in Q29
  // rho K0 in Q59: (rho << 2) K0 / 2^32 as a 64 x 32 product, low word floored
  const ull rho2 = (ull)rho << 2;
  const ll rK = (ll)((rho2 >> 32) * K0 + (((rho2 & 0xffffffffULL) * K0) >> 32));
  const ll E = (1LL << 59) - rK;
  const ll Eh = E >> 18;
  const ll C = E + (((ll)(int)Eh * (ll)(int)Eh) >> 23);
  const ll K = ((ll)K0 << 32) + mul_hi(split((ll)K0 << 33), split(C << 4));

  // c1 u = c1 j / rho (Q60), c1 = om_p / 2
  const Split jx2 = split(jx << 2), jy2 = split(jy << 2);
  const Split Kc = split(mul_hi(split(K << 1), k.c1) << 1);  // c1 / rho, Q62
  const ll Ux = mul_hi(jx2, Kc);
  const ll Uy = mul_hi(jy2, Kc);
  ok = (ull)(Ux + kJ - 1) < (ull)(2 * kJ - 1);
  ok &= (ull)(Uy + kJ - 1) < (ull)(2 * kJ - 1);
  if (!ok) return false;
  // c1 Qx, c1 Qy, c1 jx uy with Q = (c.j)(c.u)
  const Split Uy2 = split(Uy << 2);
  const ll Tx = mul_hi(jx2, split(Ux << 2));
  const ll Ty = mul_hi(jy2, Uy2);
  const ll Txy = mul_hi(jx2, Uy2);
  // om_p w1 R, R = rho - 1.5 |j|^2 / rho   (1.5 om_p w1 = c1 / 3)
  const ll WR = mul_hi(split(rho), k.wp) - mul_hi(split(Tx + Ty), k.third);
  // om_p w q P_q: axis pairs w1, diagonal pairs w2 = w1 / 4
  const ll P1 = WR + Tx, P3 = WR + Ty;
  const ll Pd = WR + Tx + Ty;
  const ll P5 = (Pd + 2 * Txy) >> 2, P7 = (Pd - 2 * Txy) >> 2;
  // 3 om_m w_q c_q.j
  const ll M1 = mul_hi(split(jx << 1), k.wm), M3 = mul_hi(split(jy << 1), k.wm);
  const ll M5 = (M1 + M3) >> 2, M7 = (M3 - M1) >> 2;
  x[0] = mul_hi(split(x[0] << 1), k.a0) + (WR << 2);
#define LBM_PAIR_Q(q, qb, s, t, P, M)                   \
  {                                                     \
    const ll A = mul_hi(split(s), k.alpha) + (P);       \
    const ll B = mul_hi(split(t), k.beta) + (M);        \
    x[q] = A + B;                                       \
    x[qb] = A - B;                                      \
  }
  LBM_PAIR_Q(1, 2, s12, t12, P1, M1)
  LBM_PAIR_Q(3, 4, s34, t34, P3, M3)
  LBM_PAIR_Q(5, 6, s56, t56, P5, M5)
  LBM_PAIR_Q(7, 8, s78, t78, P7, M7)
#undef LBM_PAIR_Q
  return true;
}

// ---------------------------------------------------------------------------
// TRT collision coefficients (lattice.py:127-131; nb.py:32-35 rewritten in the
// symmetric/antisymmetric pair form).  With a = 1 - (om_p + om_m)/2 and
// b = (om_p - om_m)/2 the reference update
//   g_up_q = a g_q - b g_qb + (a' g_eq_q + b g_eq_qb),  a' = (om_p + om_m)/2
// equals, for the pair (q, qb) with t = 3 c_q.u,
//   g_up_q  = a d_q  - b d_qb + w om_p (drho + rho(t^2/2 - v)) + w om_m rho t
//   g_up_qb = a d_qb - b d_q  + w om_p (drho + rho(t^2/2 - v)) - w om_m rho t
// where d = g - w rho0 and drho = rho - rho0 (rho0 = 0 for the plain form).
// ---------------------------------------------------------------------------
template <typename T>
struct Coef {
  T a, mb;          // a, -b
  T a0, p0;         // q = 0: 1 - om_p, om_p * w0
  T wp1, wm1;       // om_p * w1, 3 * om_m * w1  (axis pairs)
  T wp2, wm2;       // om_p * w2, 3 * om_m * w2  (diagonal pairs)
  T rho0;
  T w[9];           // weights * rho0 (shift of each population)
};

template <typename T>
__host__ __device__ inline Coef<T> make_coef(double om_p, double om_m, double rho0) {
  Coef<T> k;
  double a = 1.0 - 0.5 * (om_p + om_m);
  double b = 0.5 * (om_p - om_m);
  k.a = (T)a;
  k.mb = (T)(-b);
  k.a0 = (T)(1.0 - om_p);
  k.p0 = (T)(om_p * (4.0 / 9.0));
  k.wp1 = (T)(om_p * (1.0 / 9.0));
  k.wm1 = (T)(3.0 * om_m * (1.0 / 9.0));
  k.wp2 = (T)(om_p * (1.0 / 36.0));
  k.wm2 = (T)(3.0 * om_m * (1.0 / 36.0));
  k.rho0 = (T)rho0;
  for (int q = 0; q < 9; ++q) k.w[q] = (T)(wgt(q) * rho0);
  return k;
}

// Moments of the (shifted) populations d[0..8]: drho = sum d, j = sum c d,
// rho = rho0 + drho, u = j / rho.
template <typename T, bool SHIFT>
struct Moments {
  T drho, rho, jx, jy, ux, uy;
};

template <typename T, bool SHIFT>
// inv_scale: 1 / the storage form's kScale (drho and j stay scaled, rho and
// u are the physical values).
__device__ __forceinline__ Moments<T, SHIFT> moments(const T d[9], T rho0, T inv_scale = T(1)) {
  Moments<T, SHIFT> m;
  T s12 = d[1] + d[2], s34 = d[3] + d[4], s56 = d[5] + d[6], s78 = d[7] + d[8];
  T d12 = d[1] - d[2], d34 = d[3] - d[4], d56 = d[5] - d[6], d87 = d[8] - d[7];
  m.drho = (((d[0] + s12) + s34) + s56) + s78;
  m.rho = SHIFT ? rho0 + m.drho * inv_scale : m.drho;
  m.jx = (d12 + d56) + d87;
  m.jy = (d34 + d56) - d87;
  T r = recip(m.rho) * inv_scale;
  m.ux = m.jx * r;
  m.uy = m.jy * r;
  return m;
}

// In-place TRT collision of d[0..8] given its moments.
template <typename T, bool SHIFT>
__device__ __forceinline__ void collide(T d[9], const Moments<T, SHIFT>& m, const Coef<T>& k) {
  const T jx = m.jx, jy = m.jy, ux = m.ux, uy = m.uy;
  const T Qx = jx * ux, Qy = jy * uy;
  const T j5 = jx + jy, u5 = ux + uy, Q5 = j5 * u5;
  const T j7 = jy - jx, u7 = uy - ux, Q7 = j7 * u7;
  // R = drho - rho*v  with rho*v = 1.5 (jx ux + jy uy)
  const T R = fma(T(-1.5), Qx + Qy, m.drho);
  d[0] = fma(k.a0, d[0], k.p0 * R);
#define LBM_PAIR(q, qb, Q, cj, wp, wm)             \
  {                                                \
    const T P = fma(T(4.5), Q, R);                 \
    const T M = (wm) * (cj);                       \
    const T base = (wp) * P;                       \
    const T dq = d[q], dqb = d[qb];                \
    d[q] = fma(k.a, dq, fma(k.mb, dqb, base + M)); \
    d[qb] = fma(k.a, dqb, fma(k.mb, dq, base - M)); \
  }
  LBM_PAIR(1, 2, Qx, jx, k.wp1, k.wm1)
  LBM_PAIR(3, 4, Qy, jy, k.wp1, k.wm1)
  LBM_PAIR(5, 6, Q5, j5, k.wp2, k.wm2)
  LBM_PAIR(7, 8, Q7, j7, k.wp2, k.wm2)
#undef LBM_PAIR
}

// ---------------------------------------------------------------------------
// Two cells at once in packed FP32 (the FADD2 / FMUL2 / FFMA2 instructions of
// sm_100 and later: one instruction for both elements of a float2).  Each
// element goes through the arithmetic of moments() and collide() on float,
// with w+ P +- M fused into one multiply-add; the bulk kernels of the
// reduced forms, which update cells in pairs anyway (packed conversions on
// store), use these to halve their FP32 instruction count.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 f2(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
// a - b: b * -1 is exact, so the fused multiply-add rounds a - b once.
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, f2(-1.0f), a); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

struct Moments2 {
  float2 drho, rho, jx, jy, ux, uy;
};

// moments<float, SHIFT>() of two cells (d[q].x: first cell, .y: second).
template <bool SHIFT>
__device__ __forceinline__ Moments2 moments2(const float2 d[9], float rho0, float inv_scale) {
  Moments2 m;
  const float2 s12 = add2(d[1], d[2]), s34 = add2(d[3], d[4]), s56 = add2(d[5], d[6]),
               s78 = add2(d[7], d[8]);
  const float2 d12 = sub2(d[1], d[2]), d34 = sub2(d[3], d[4]), d56 = sub2(d[5], d[6]),
               d87 = sub2(d[8], d[7]);
  m.drho = add2(add2(add2(add2(d[0], s12), s34), s56), s78);
  m.rho = SHIFT ? fma2(m.drho, f2(inv_scale), f2(rho0)) : m.drho;
  m.jx = add2(add2(d12, d56), d87);
  m.jy = sub2(add2(d34, d56), d87);
  const float2 r = mul2(make_float2(recip(m.rho.x), recip(m.rho.y)), f2(inv_scale));
  m.ux = mul2(m.jx, r);
  m.uy = mul2(m.jy, r);
  return m;
}

// collide<float, SHIFT>() of two cells.
__device__ __forceinline__ void collide2(float2 d[9], const Moments2& m, const Coef<float>& k) {
  const float2 jx = m.jx, jy = m.jy, ux = m.ux, uy = m.uy;
  const float2 Qx = mul2(jx, ux), Qy = mul2(jy, uy);
  const float2 j5 = add2(jx, jy), u5 = add2(ux, uy), Q5 = mul2(j5, u5);
  const float2 j7 = sub2(jy, jx), u7 = sub2(uy, ux), Q7 = mul2(j7, u7);
  const float2 R = fma2(f2(-1.5f), add2(Qx, Qy), m.drho);
  d[0] = fma2(f2(k.a0), d[0], mul2(f2(k.p0), R));
#define LBM_PAIR2(q, qb, Q, cj, wp, wm)                                  \
  {                                                                      \
    const float2 P = fma2(f2(4.5f), Q, R);                               \
    const float2 M = mul2(f2(wm), cj), Mn = mul2(f2(-(wm)), cj);         \
    const float2 dq = d[q], dqb = d[qb];                                 \
    d[q] = fma2(f2(k.a), dq, fma2(f2(k.mb), dqb, fma2(f2(wp), P, M)));   \
    d[qb] = fma2(f2(k.a), dqb, fma2(f2(k.mb), dq, fma2(f2(wp), P, Mn))); \
  }
  LBM_PAIR2(1, 2, Qx, jx, k.wp1, k.wm1)
  LBM_PAIR2(3, 4, Qy, jy, k.wp1, k.wm1)
  LBM_PAIR2(5, 6, Q5, j5, k.wp2, k.wm2)
  LBM_PAIR2(7, 8, Q7, j7, k.wp2, k.wm2)
#undef LBM_PAIR2
}

// ---------------------------------------------------------------------------
// Boundary operations on full (unshifted) populations of one cell, written in
// the operation order of the reference expressions.
// ---------------------------------------------------------------------------
template <typename T>
struct CellBC {
  T g[9];
  T rho, ux, uy;
};

// nb_zou_he_left_wall_velocity, nb.py:121-143.
template <typename T>
__device__ __forceinline__ void zh_left(CellBC<T>& c, T ubx, T uby) {
  const T C1 = T(2.0 / 3.0), C2 = T(1.0 / 6.0), C3 = T(0.5);
  c.ux = ubx;
  c.uy = uby;
  T r = (c.g[0] + c.g[3] + c.g[4] + T(2) * c.g[2] + T(2) * c.g[6] + T(2) * c.g[7]) / (T(1) - c.ux);
  c.rho = r;
  c.g[1] = c.g[2] + C1 * r * c.ux;
  c.g[5] = c.g[6] - C3 * (c.g[3] - c.g[4]) + C2 * r * c.ux + C3 * r * c.uy;
  c.g[8] = c.g[7] + C3 * (c.g[3] - c.g[4]) + C2 * r * c.ux - C3 * r * c.uy;
}
// nb_zou_he_right_wall_velocity, nb.py:147-169.
template <typename T>
__device__ __forceinline__ void zh_right(CellBC<T>& c, T ubx, T uby) {
  const T C1 = T(2.0 / 3.0), C2 = T(1.0 / 6.0), C3 = T(0.5);
  c.ux = ubx;
  c.uy = uby;
  T r = (c.g[0] + c.g[3] + c.g[4] + T(2) * c.g[1] + T(2) * c.g[5] + T(2) * c.g[8]) / (T(1) + c.ux);
  c.rho = r;
  c.g[2] = c.g[1] - C1 * r * c.ux;
  c.g[6] = c.g[5] + C3 * (c.g[3] - c.g[4]) - C2 * r * c.ux - C3 * r * c.uy;
  c.g[7] = c.g[8] - C3 * (c.g[3] - c.g[4]) - C2 * r * c.ux + C3 * r * c.uy;
}
// nb_zou_he_right_wall_pressure, nb.py:173-195.
template <typename T>
__device__ __forceinline__ void zh_right_pressure(CellBC<T>& c, T rho_b, T uby) {
  const T C1 = T(2.0 / 3.0), C2 = T(1.0 / 6.0), C3 = T(0.5);
  c.rho = rho_b;
  c.uy = uby;
  T r = c.rho;
  c.ux = (c.g[0] + c.g[3] + c.g[4] + T(2) * c.g[1] + T(2) * c.g[5] + T(2) * c.g[8]) / r - T(1);
  c.g[2] = c.g[1] - C1 * r * c.ux;
  c.g[6] = c.g[5] + C3 * (c.g[3] - c.g[4]) - C2 * r * c.ux - C3 * r * c.uy;
  c.g[7] = c.g[8] - C3 * (c.g[3] - c.g[4]) - C2 * r * c.ux + C3 * r * c.uy;
}
// nb_zou_he_top_wall_velocity, nb.py:199-221.
template <typename T>
__device__ __forceinline__ void zh_top(CellBC<T>& c, T ubx, T uby) {
  const T C1 = T(2.0 / 3.0), C2 = T(1.0 / 6.0), C3 = T(0.5);
  c.ux = ubx;
  c.uy = uby;
  T r = (c.g[0] + c.g[1] + c.g[2] + T(2) * c.g[3] + T(2) * c.g[5] + T(2) * c.g[7]) / (T(1) + c.uy);
  c.rho = r;
  c.g[4] = c.g[3] - C1 * r * c.uy;
  c.g[8] = c.g[7] - C3 * (c.g[1] - c.g[2]) + C3 * r * c.ux - C2 * r * c.uy;
  c.g[6] = c.g[5] + C3 * (c.g[1] - c.g[2]) - C3 * r * c.ux - C2 * r * c.uy;
}
// nb_zou_he_bottom_wall_velocity, nb.py:225-247.
template <typename T>
__device__ __forceinline__ void zh_bottom(CellBC<T>& c, T ubx, T uby) {
  const T C1 = T(2.0 / 3.0), C2 = T(1.0 / 6.0), C3 = T(0.5);
  c.ux = ubx;
  c.uy = uby;
  T r = (c.g[0] + c.g[1] + c.g[2] + T(2) * c.g[4] + T(2) * c.g[6] + T(2) * c.g[8]) / (T(1) - c.uy);
  c.rho = r;
  c.g[3] = c.g[4] + C1 * r * c.uy;
  c.g[5] = c.g[6] - C3 * (c.g[1] - c.g[2]) + C3 * r * c.ux + C2 * r * c.uy;
  c.g[7] = c.g[8] + C3 * (c.g[1] - c.g[2]) - C3 * r * c.ux + C2 * r * c.uy;
}

// Corners, nb.py:250-344.  rho/u are first copied from the x-neighbour.
template <typename T>
__device__ __forceinline__ void zh_corner(int corner, CellBC<T>& c, T rho_nb, T ux_nb, T uy_nb) {
  const T C23 = T(2.0 / 3.0), C16 = T(1.0 / 6.0);
  c.ux = ux_nb;
  c.uy = uy_nb;
  c.rho = rho_nb;
  const T r = c.rho, ux = c.ux, uy = c.uy;
  switch (corner) {
    case 0:  // bottom-left, nb.py:251-271
      c.g[1] = c.g[2] + C23 * r * ux;
      c.g[3] = c.g[4] + C23 * r * uy;
      c.g[5] = c.g[6] + C16 * r * ux + C16 * r * uy;
      c.g[7] = T(0);
      c.g[8] = T(0);
      break;
    case 1:  // top-left, nb.py:275-296
      c.g[1] = c.g[2] + C23 * r * ux;
      c.g[4] = c.g[3] - C23 * r * uy;
      c.g[8] = c.g[7] + C16 * r * ux - C16 * r * uy;
      c.g[5] = T(0);
      c.g[6] = T(0);
      break;
    case 2:  // top-right, nb.py:300-320
      c.g[2] = c.g[1] - C23 * r * ux;
      c.g[4] = c.g[3] - C23 * r * uy;
      c.g[6] = c.g[5] - C16 * r * ux - C16 * r * uy;
      c.g[7] = T(0);
      c.g[8] = T(0);
      break;
    default:  // bottom-right, nb.py:324-344
      c.g[2] = c.g[1] - C23 * r * ux;
      c.g[3] = c.g[4] + C23 * r * uy;
      c.g[7] = c.g[8] - C16 * r * ux + C16 * r * uy;
      c.g[5] = T(0);
      c.g[6] = T(0);
      break;
  }
  c.g[0] = r - c.g[1] - c.g[2] - c.g[3] - c.g[4] - c.g[5] - c.g[6] - c.g[7] - c.g[8];
}

// Interpolated bounce-back of one link, nb.py:77-117, as three coefficients
// of the link's distance p (the parenthesised factors of the reference
// expressions, evaluated in the same order):
//   p <  1/2: g[qb] = c1 up_q_x + c2 up_q_1 - c3 up_q_2
//   p >= 1/2: g[qb] = c1 up_q_x + c2 up_qb_x + c3 up_qb_1
// with up_q_x = g_up[q, x], up_q_1 = g_up[q, x + c_qb], up_q_2 =
// g_up[q, x + 2 c_qb], up_qb_x = g_up[qb, x], up_qb_1 = g_up[qb, x + c_qb].
// The host computes the same coefficients once per link (link_coef).
template <typename T>
__host__ __device__ __forceinline__ void ibb_coefs(T p, T& c1, T& c2, T& c3) {
  const T pp = T(2) * p;
  if (p < T(0.5)) {
    c1 = p * (pp + T(1));
    c2 = (T(1) + pp) * (T(1) - pp);
    c3 = p * (T(1) - pp);
  } else {
    c1 = T(1) / (p * (pp + T(1)));
    c2 = (pp - T(1)) / p;
    c3 = (T(1) - pp) / (T(1) + pp);
  }
}

// g[q] = v / g[q] for a run-time q in 1..8 without dynamic register indexing.
template <typename T>
__device__ __forceinline__ void set_pop(T g[9], int q, T v) {
#pragma unroll
  for (int k = 1; k < 9; ++k)
    if (k == q) g[k] = v;
}
template <typename T>
__device__ __forceinline__ T get_pop(const T g[9], int q) {
  T v = g[0];
#pragma unroll
  for (int k = 1; k < 9; ++k)
    if (k == q) v = g[k];
  return v;
}

}  // namespace lbm
