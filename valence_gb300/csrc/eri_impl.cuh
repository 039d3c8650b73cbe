/*
 * eri_impl.cuh -- shell-quartet electron-repulsion integrals fused with the
 * LCAO-weight contraction of VALENCE's int2e (valence.F90:3184-3438),
 * templated on the arithmetic of the 2D tables and component sums.
 *
 * int2e contracts every shell quartet of four orbital bases with the weight
 * products dij(ab) dkl(cd) (valence.F90:3372-3412).  Here each unique AO shell
 * quartet (AB|CD) is evaluated once and transformed straight into the
 * orbital-pair matrix
 *     U[(i,k)][(j,l)] += sum_ab sum_cd X_ik(ab) (ab|cd) X_jl(cd),
 * X_ik(ab) = angn_a angn_b (C_i(a) C_k(b) + C_k(a) C_i(b)); T = U + U^T then
 * holds every (i k | j l) that vsvb_energy asks int2e for (valence.F90:1256,
 * 1264) and the Schwarz table (:1516).  No AO integral is written to HBM.
 *
 * Integrals: Rys quadrature (Rys, Dupuis & King, J. Comput. Chem. 4, 154
 * (1983)); per primitive quartet only the 2D recurrence tables G(i, k) of the
 * (e0|f0) integrals (e on centre A, |e| = la..la+lb; f on C).  The horizontal
 * transfer (ab| = sum_e M(ab, e) (e0| depends on the pair geometry alone, so
 * with X' = X M (xhrr_kernel) the transform reads
 *     U += X'_P (e0|f0) X'_Q^T
 * and the transfer costs nothing per primitive.  Roots and weights come from
 * project-generated Chebyshev tables (gen_rys_tables.py).
 *
 * Work split.  Per primitive quartet, 3*n_r lanes build the x/y/z 2D tables
 * of the n_r roots in shared memory (G2 primitive quartets at once per
 * warp).  Then, in line mode, a lane owns one function of the larger side
 * (e or f) and accumulates its whole line of components, the function's
 * table rows held in registers and the line's exponents compile-time
 * constants; lines of up to 16 run two or more primitive quartets side by
 * side.  Small blocks take one warp per shell quartet; blocks of >= 80
 * components put a whole CTA on one shell quartet, its warps splitting the
 * primitive quartets.  After the primitive loop the block is staged in
 * shared memory and transformed with the X' tables; U is updated with FP64
 * atomics.
 *
 * Arithmetic.  R = double: everything FP64.  R = double-float (df64, an
 * unevaluated sum of two FP32 numbers, ~48-bit significand): the Boys
 * argument T, 1/(p+q), the prefactor and the Chebyshev evaluation of the Rys
 * roots and weights run in double-float (the small high-order Chebyshev
 * terms in FP32) with no FP64 instruction, so roots and weights keep ~1e-14
 * relative accuracy on the FP32 pipes; tables and component sums in df64;
 * the transform in FP64.  R = float (quartets, or primitive quartets, whose
 * Schwarz bound is below the mixed threshold): everything in FP32, including
 * the roots and the transform, with FP64 atomics into U.
 */
#ifndef VSVB_ERI_IMPL_CUH
#define VSVB_ERI_IMPL_CUH
#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>
#include <utility>

#include "eri.cuh"
#include "vsvb_internal.h"

namespace {

/* Cartesian exponents of function k of the list l0, l0+1, ... (each
 * angular momentum in CCA order: x-power descending, then y-power) */
__device__ __forceinline__ void list_exp(int l0, int k, int e[3]) {
  for (int l = l0;; ++l) {
    const int n = (l + 1) * (l + 2) / 2;
    if (k < n) {
      for (int lx = l; lx >= 0; --lx) {
        const int m = l - lx + 1;
        if (k < m) {
          e[0] = lx;
          e[1] = l - lx - k;
          e[2] = k;
          return;
        }
        k -= m;
      }
    }
    k -= n;
  }
}

/* list_exp at compile time: exponent d (0: x, 1: y, 2: z) of function k */
__host__ __device__ constexpr int cexp(int l0, int k, int d) {
  for (int l = l0;; ++l) {
    const int n = (l + 1) * (l + 2) / 2;
    if (k < n) {
      for (int lx = l; lx >= 0; --lx) {
        const int m = l - lx + 1;
        if (k < m) return d == 0 ? lx : (d == 1 ? l - lx - k : k);
        k -= m;
      }
    }
    k -= n;
  }
}

/* the inverse: index of exponents (x, y, z) in the list l0, l0+1, ... */
__host__ __device__ constexpr int kindex(int l0, int x, int y, int z) {
  int k = 0;
  const int l = x + y + z;
  for (int m = l0; m < l; ++m) k += (m + 1) * (m + 2) / 2;
  for (int lx = l; lx > x; --lx) k += l - lx + 1;
  return k + z;
}

/* warp shuffle down in each arithmetic type */
__device__ __forceinline__ float shfl_down_r(float v, int d) { return __shfl_down_sync(0xffffffffu, v, d); }
__device__ __forceinline__ double shfl_down_r(double v, int d) { return __shfl_down_sync(0xffffffffu, v, d); }
__device__ __forceinline__ df64 shfl_down_r(df64 v, int d) {
  return df64(__shfl_down_sync(0xffffffffu, v.hi, d), __shfl_down_sync(0xffffffffu, v.lo, d));
}

/* f(integral_constant<int, 0>), ..., f(integral_constant<int, N-1>) */
template <typename F, int... I>
__device__ __forceinline__ void static_for_impl(F &&f, std::integer_sequence<int, I...>) {
  (f(std::integral_constant<int, I>{}), ...);
}
template <int N, typename F>
__device__ __forceinline__ void static_for(F &&f) {
  static_for_impl(f, std::make_integer_sequence<int, N>{});
}

constexpr int RYS_NCHEB_D = 12;
constexpr double RYS_TMAX_D = 64.0;
constexpr double RYS_H_D = 0.5;
constexpr int RYS_DF_SPLIT = 5; /* Chebyshev terms >= this index are summed in FP32 */

/* ---- double-float arithmetic -------------------------------------------- */

/* df_quick, +, -, * and += on df64: vsvb_internal.h */

/* reciprocal, square root and inverse square root in double-float: an
 * FP32 first guess refined by one Newton step in df64 (~2^-46 relative) */
__device__ __forceinline__ df64 df_recip(df64 a) {
  const float r0 = 1.0f / a.hi;
  const df64 e = df64(1.f) - a * df64(r0);
  return df64(r0) + df64(r0) * e;
}
__device__ __forceinline__ df64 df_sqrt(df64 a) {
  if (a.hi <= 0.f) return df64(0.f);
  const float s0 = sqrtf(a.hi);
  const df64 d = a - df64(s0) * df64(s0);
  return df64(s0) + d * df64(0.5f / s0);
}
__device__ __forceinline__ df64 df_rsqrt(df64 a) { return df_recip(df_sqrt(a)); }

/* acc += x*y*z.  For df64 the accumulator is kept unnormalised (hi, lo) and
 * the two products skip their intermediate renormalisation. */
__device__ __forceinline__ void acc3(double &acc, double x, double y, double z) { acc = fma(x * y, z, acc); }
__device__ __forceinline__ void acc3(float &acc, float x, float y, float z) { acc = fmaf(x * y, z, acc); }
__device__ __forceinline__ void acc3(df64 &acc, df64 x, df64 y, df64 z) {
  const float p = x.hi * y.hi;
  float e = fmaf(x.hi, y.hi, -p);
  e = fmaf(x.hi, y.lo, e);
  e = fmaf(x.lo, y.hi, e);
  const float q = p * z.hi;
  float f = fmaf(p, z.hi, -q);
  f = fmaf(p, z.lo, f);
  f = fmaf(e, z.hi, f);
  const float s = acc.hi + q;
  const float v = s - acc.hi;
  const float err = (acc.hi - (s - v)) + (q - v);
  acc.lo += err + f;
  acc.hi = s;
}
/* the same with the x*y product shared by several z: mul_xy once, then
 * acc_xyz per component (the arithmetic of acc3, split in two) */
template <typename R>
struct XYProd {
  R v;
};
template <>
struct XYProd<df64> {
  float p, e; /* unnormalised product hi + error */
};
__device__ __forceinline__ XYProd<double> mul_xy(double x, double y) { return {x * y}; }
__device__ __forceinline__ XYProd<float> mul_xy(float x, float y) { return {x * y}; }
__device__ __forceinline__ XYProd<df64> mul_xy(df64 x, df64 y) {
  XYProd<df64> r;
  r.p = x.hi * y.hi;
  float e = fmaf(x.hi, y.hi, -r.p);
  e = fmaf(x.hi, y.lo, e);
  r.e = fmaf(x.lo, y.hi, e);
  return r;
}
__device__ __forceinline__ void acc_xyz(double &acc, const XYProd<double> &xy, double z) { acc = fma(xy.v, z, acc); }
__device__ __forceinline__ void acc_xyz(float &acc, const XYProd<float> &xy, float z) { acc = fmaf(xy.v, z, acc); }
__device__ __forceinline__ void acc_xyz(df64 &acc, const XYProd<df64> &xy, df64 z) {
  const float q = xy.p * z.hi;
  float f = fmaf(xy.p, z.hi, -q);
  f = fmaf(xy.p, z.lo, f);
  f = fmaf(xy.e, z.hi, f);
  const float s = acc.hi + q;
  const float v = s - acc.hi;
  const float err = (acc.hi - (s - v)) + (q - v);
  acc.lo += err + f;
  acc.hi = s;
}
__device__ __forceinline__ double to_double(double v) { return v; }
__device__ __forceinline__ double to_double(float v) { return (double)v; }
__device__ __forceinline__ double to_double(df64 v) { return (double)v.hi + (double)v.lo; }

/* s += a*b and read-only loads in the transform arithmetic (FP64 or FP32) */
__device__ __forceinline__ void mad(double &s, double a, double b) { s = fma(a, b, s); }
__device__ __forceinline__ void mad(float &s, float a, float b) { s = fmaf(a, b, s); }
__device__ __forceinline__ double ldt(const double *p) { return __ldg(p); }
__device__ __forceinline__ float ldt(const float *p) { return __ldg(p); }

/* ---- Rys roots ------------------------------------------------------------ */

__device__ __forceinline__ double clenshaw12(const double *__restrict__ c, double t) {
  double b1 = 0.0, b2 = 0.0;
#pragma unroll
  for (int k = RYS_NCHEB_D - 1; k > 0; --k) {
    double b0 = fma(2.0 * t, b1, c[k] - b2);
    b2 = b1;
    b1 = b0;
  }
  return fma(t, b1, c[0] - b2);
}

/* root r of the n-point rule in FP64: x (= t^2) and weight */
__device__ __forceinline__ void rys_root(int n, int r, double T, const double *__restrict__ tab, const RysConst &rc,
                                         double &x, double &w) {
  if (T < RYS_TMAX_D) {
    int j = (int)(T * (1.0 / RYS_H_D));
    double t = (T - j * RYS_H_D) * (2.0 / RYS_H_D) - 1.0;
    const double *c = tab + rc.off[n - 1] + (size_t)j * (2 * n) * RYS_NCHEB_D;
    double fx = clenshaw12(c + r * RYS_NCHEB_D, t);
    double fw = clenshaw12(c + (n + r) * RYS_NCHEB_D, t);
    const double s = rsqrt(1.0 + T);
    x = fx * s * s;
    w = fw * s;
  } else {
    const double s = rsqrt(T);
    x = rc.ax[n - 1][r] * s * s;
    w = rc.aw[n - 1][r] * s;
  }
}

/* Chebyshev sum in double-float: the high-order terms (below the FP32 noise
 * of the result) in FP32, the rest in df64.  c: (hi, lo) coefficient pairs. */
__device__ __forceinline__ df64 clenshaw12_df(const float2 *__restrict__ c, df64 t) {
  /* the 12 (hi, lo) pairs are 96 contiguous, 16-byte aligned bytes: six
   * vector loads */
  float2 k[RYS_NCHEB_D];
#pragma unroll
  for (int i = 0; i < RYS_NCHEB_D / 2; ++i) {
    const float4 v = __ldg(reinterpret_cast<const float4 *>(c) + i);
    k[2 * i] = make_float2(v.x, v.y);
    k[2 * i + 1] = make_float2(v.z, v.w);
  }
  float b1f = 0.f, b2f = 0.f;
  const float t2f = 2.f * t.hi;
#pragma unroll
  for (int i = RYS_NCHEB_D - 1; i >= RYS_DF_SPLIT; --i) {
    const float b0 = fmaf(t2f, b1f, k[i].x - b2f);
    b2f = b1f;
    b1f = b0;
  }
  df64 b1(b1f), b2(b2f);
  const df64 t2 = t + t;
#pragma unroll
  for (int i = RYS_DF_SPLIT - 1; i > 0; --i) {
    const df64 b0 = t2 * b1 - b2 + df64(k[i].x, k[i].y);
    b2 = b1;
    b1 = b0;
  }
  return t * b1 - b2 + df64(k[0].x, k[0].y);
}

/* root r in double-float; interval j, Chebyshev variable t and
 * s = (1+T)^(-1/2) (or T^(-1/2) beyond the tables) given */
__device__ __forceinline__ void rys_root_df(int n, int r, int j, bool in_table, df64 t, df64 s,
                                            const float2 *__restrict__ tab, const RysConst &rc, df64 &x, df64 &w) {
  if (in_table) {
    const float2 *c = tab + rc.off[n - 1] + (size_t)j * (2 * n) * RYS_NCHEB_D;
    const df64 fx = clenshaw12_df(c + r * RYS_NCHEB_D, t);
    const df64 fw = clenshaw12_df(c + (n + r) * RYS_NCHEB_D, t);
    x = fx * s * s;
    w = fw * s;
  } else {
    x = df64(rc.axf[n - 1][r].x, rc.axf[n - 1][r].y) * s * s;
    w = df64(rc.awf[n - 1][r].x, rc.awf[n - 1][r].y) * s;
  }
}

/* FP32 Chebyshev sum for the FP32 kernels (their integrals carry FP32
 * rounding anyway), from the FP32 roundings of the same tables.  Only the
 * first 8 of the 12 coefficients of one (interval, root): the dropped tail
 * is below 1.3e-9 of the value for the weights and 5e-13 for the roots on
 * every interval of the 1-5 root rules, far under FP32 rounding (6e-8).
 * They are 32 contiguous, 16-byte aligned bytes (each 12-coefficient block
 * starts on a 48-byte boundary), read as two vectors. */
constexpr int RYS_NCHEB_F = 8;
__device__ __forceinline__ float clenshaw8_f4(const float *__restrict__ c, float t) {
  const float4 a = __ldg(reinterpret_cast<const float4 *>(c));
  const float4 b = __ldg(reinterpret_cast<const float4 *>(c) + 1);
  const float k[RYS_NCHEB_F] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
  float b1 = 0.f, b2 = 0.f;
  const float t2 = 2.f * t;
#pragma unroll
  for (int i = RYS_NCHEB_F - 1; i > 0; --i) {
    const float b0 = fmaf(t2, b1, k[i] - b2);
    b2 = b1;
    b1 = b0;
  }
  return fmaf(t, b1, k[0] - b2);
}

__device__ __forceinline__ const PrimT<df64> *args_primdf(const EriArgs &a) {
  return static_cast<const PrimT<df64> *>(a.primdf);
}

/* per-precision views of the primitive-pair and pair-geometry arrays */
template <typename R>
struct prec_data;
template <>
struct prec_data<double> {
  static __device__ const void *prim(const EriArgs &a) { return a.prim64; }
  static __device__ const void *geom(const EriArgs &a) { return a.geom64; }
};
template <>
struct prec_data<float> {
  static __device__ const void *prim(const EriArgs &a) { return a.prim32; }
  static __device__ const void *geom(const EriArgs &a) { return a.geom32; }
};
template <>
struct prec_data<df64> {
  static __device__ const void *prim(const EriArgs &a) { return a.primdf; }
  static __device__ const void *geom(const EriArgs &a) { return a.geomdf; }
};

template <typename R>
__device__ __forceinline__ R from_df(df64 v);
template <>
__device__ __forceinline__ float from_df<float>(df64 v) {
  return v.hi + v.lo;
}
template <>
__device__ __forceinline__ df64 from_df<df64>(df64 v) {
  return v;
}

template <int L>
struct NC {
  static constexpr int v = (L + 1) * (L + 2) / 2;
};
/* functions of angular momentum la .. la+lb: the (e0| list of a pair */
constexpr int ne_c(int la, int lb) {
  int n = 0;
  for (int l = la; l <= la + lb; ++l) n += (l + 1) * (l + 2) / 2;
  return n;
}

/* x (or y, z) 2D factor for one root: G(i, k), i <= LAB on the bra centre
 * A, k <= LCD on the ket centre C, by the Rys recurrences.  The horizontal
 * transfers to the second centres are not done here: they are folded into
 * the weight tables (X' = X M), so the components contracted are (e0|f0). */
/* a*b + c in R: FMA for float/double; for df64 the product's error terms
 * come from FMAs and are added with c under one TwoSum and one final
 * renormalisation (15 FP32 operations against 18 for a product then a sum) */
__device__ __forceinline__ float mad_r(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double mad_r(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ df64 mad_r(df64 a, df64 b, df64 c) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  const float s = p + c.hi;
  const float v = s - p;
  const float t = ((p - (s - v)) + (c.hi - v)) + (e + c.lo);
  return df_quick(s, t);
}

template <int LAB, int LCD, typename R, int STRIDE, int ROWSTRIDE>
__device__ __forceinline__ void rys_g(R g00, R c00, R d00, R b00, R b10, R b01, R *__restrict__ out) {
  /* integer multiples of the coefficients, formed once */
  R ib10[LAB > 1 ? LAB : 1], ib00[LAB + 1], kb01[LCD > 1 ? LCD : 1];
#pragma unroll
  for (int i = 1; i < LAB; ++i) ib10[i] = R(i) * b10;
#pragma unroll
  for (int i = 1; i <= LAB; ++i) ib00[i] = R(i) * b00;
#pragma unroll
  for (int k = 1; k < LCD; ++k) kb01[k] = R(k) * b01;
  R G[LAB + 1][LCD + 1];
  G[0][0] = g00;
#pragma unroll
  for (int i = 0; i < LAB; ++i)
    G[i + 1][0] = i > 0 ? mad_r(c00, G[i][0], ib10[i > 0 ? i : 0] * G[i > 0 ? i - 1 : 0][0]) : c00 * G[0][0];
#pragma unroll
  for (int k = 0; k < LCD; ++k) {
#pragma unroll
    for (int i = 0; i <= LAB; ++i) {
      R t;
      if (k > 0 && i > 0)
        t = mad_r(kb01[k > 0 ? k : 0], G[i][k > 0 ? k - 1 : 0], ib00[i] * G[i > 0 ? i - 1 : 0][k]);
      else if (k > 0)
        t = kb01[k > 0 ? k : 0] * G[i][k > 0 ? k - 1 : 0];
      else if (i > 0)
        t = ib00[i] * G[i > 0 ? i - 1 : 0][k];
      G[i][k + 1] = (k > 0 || i > 0) ? mad_r(d00, G[i][k], t) : d00 * G[i][k];
    }
  }
#pragma unroll
  for (int i = 0; i <= LAB; ++i)
#pragma unroll
    for (int k = 0; k <= LCD; ++k) out[i * ROWSTRIDE + k * STRIDE] = G[i][k];
}

/* vector load of V consecutive table entries (V * sizeof(R) bytes, aligned) */
template <int V>
__device__ __forceinline__ void ldv(const float *p, float (&o)[V]) {
  if constexpr (V == 4) {
    const float4 f = *reinterpret_cast<const float4 *>(p);
    o[0] = f.x; o[1] = f.y; o[2] = f.z; o[3] = f.w;
  } else if constexpr (V == 2) {
    const float2 f = *reinterpret_cast<const float2 *>(p);
    o[0] = f.x; o[1] = f.y;
  } else {
    o[0] = *p;
  }
}
template <int V>
__device__ __forceinline__ void ldv(const double *p, double (&o)[V]) {
  if constexpr (V == 2) {
    const double2 f = *reinterpret_cast<const double2 *>(p);
    o[0] = f.x; o[1] = f.y;
  } else {
    o[0] = *p;
  }
}
template <int V>
__device__ __forceinline__ void ldv(const df64 *p, df64 (&o)[V]) {
  if constexpr (V == 2) {
    const float4 f = *reinterpret_cast<const float4 *>(p);
    o[0] = df64(f.x, f.y);
    o[1] = df64(f.z, f.w);
  } else {
    o[0] = *p;
  }
}

constexpr int WARPS = 4;

/* block mode: the places of pair function (a of shell A, b of shell B) in
 * its atom pair's rows, row = f1 * nf2 + f2 with f1 a function of the pair's
 * first atom and f2 of its second (bp: off A, off B, flags, nf2) */
__device__ __forceinline__ int blk_places(int4 bp, int a, int b, int *pos) {
  const int fa = bp.x + a, fb = bp.y + b;
  if (bp.z & 2) {
    pos[0] = fa * bp.w + fb;
    if (bp.z & 4) return 1;
    pos[1] = fb * bp.w + fa;
    return 2;
  }
  pos[0] = (bp.z & 1) ? fb * bp.w + fa : fa * bp.w + fb;
  return 1;
}

/* RB: bytes of one element of the arithmetic type (2D tables, roots) */
template <int LA, int LB, int LC, int LD, int RB = 8>
struct QuartetShape {
  static constexpr int NAB = NC<LA>::v * NC<LB>::v; /* transferred bra functions (Schwarz) */
  static constexpr int LAB = LA + LB, LCD = LC + LD;
  static constexpr int NEA = ne_c(LA, LB), NEC = ne_c(LC, LD); /* (e0| and |f0) functions */
  static constexpr int NCOMP = NEA * NEC;
  static constexpr int NR = (LAB + LCD) / 2 + 1;
  static constexpr int N2D = (LAB + 1) * (LCD + 1);
  /* primitive quartets processed side by side per warp iteration: each takes
   * 3*NR lanes for its 2D tables (G2 slots).  Large blocks (CTA mode) put the
   * CTA's warps on one shell quartet, each with its own partial block */
  static constexpr int G0 = 32 / (3 * NR) < 1 ? 1 : 32 / (3 * NR);
  static constexpr bool CTA = NCOMP >= 80;
  static constexpr int G2 = G0;
  static constexpr int JCH = 8; /* ket orbital pairs per transform chunk */
  static constexpr int NMAX = NEA > NEC ? NEA : NEC;
  /* 2D tables are stored root-innermost, [slot][dir][entry][root], each
   * entry padded to NRP roots so that VEC roots load as one 8/16-byte
   * vector: NGF full vector groups and REM roots loaded one by one */
  static constexpr int VEC = RB == 4 ? (NR >= 4 ? 4 : (NR >= 2 ? 2 : 1)) : (NR >= 2 ? 2 : 1);
  static constexpr int NRP = (NR + VEC - 1) / VEC * VEC;
  static constexpr int NGF = NR / VEC, REM = NR % VEC;
  /* row stride RS of a direction's table (entries (i, k) at i*RS + k*NRP):
   * padded by one vector when the rows would otherwise start 32-byte
   * aligned, so that the lanes of line mode, which read different rows of
   * 16-byte vectors, spread over the shared-memory banks */
  static constexpr int RS0 = (LCD + 1) * NRP;
  static constexpr int RS = (VEC * RB == 16 && ((RS0 * RB / 16) % 2 == 0)) ? RS0 + VEC : RS0;
  static constexpr int DS = (LAB + 1) * RS; /* one direction's table */
  static constexpr int SM_2D = (G2 * 3 * DS * RB + 15) / 16 * 2; /* per warp, in doubles (16-byte multiple) */
  /* per warp: roots, weights, 1/(p+q) of 32 primitive quartets, and their indices */
  static constexpr int SM_ROOT = (((2 * 32 * NR + 32) * RB + 7) / 8 + 16 + 1) / 2 * 2;
  /* staging: E[NCOMP] + a transform chunk; per warp in warp mode, one per
   * CTA in CTA mode */
  static constexpr int SM_TR = NCOMP + JCH * NMAX;
  static constexpr int PER_WARP0 = CTA ? SM_2D + SM_ROOT : (SM_2D + SM_ROOT > SM_TR ? SM_2D + SM_ROOT : SM_TR);
  static constexpr int PER_WARP = (PER_WARP0 + 1) / 2 * 2;
  static constexpr int SHARED = CTA ? SM_TR : 0;
  /* FP32 and double-float kernels, line mode: a lane owns one function of
   * the larger side (e for ROWM, else f) and accumulates the whole line of
   * components it spans, with that function's 2D table entries in registers
   * -- three shared-memory vectors per table row instead of three per
   * component, which is what bounds the component loop in FP32.  SL slots
   * side by side when a line takes at most half a warp. */
  static constexpr bool ROWM = NEA >= NEC;
  static constexpr int NL = ROWM ? NEA : NEC, NK = ROWM ? NEC : NEA;
  static constexpr int KD = ROWM ? LCD + 1 : LAB + 1; /* table rows a lane loads per direction */
  static constexpr int SL0 = 32 / NL > G2 ? G2 : 32 / NL;
  static constexpr int SL = SL0 < 1 ? 1 : SL0;
  /* CTA mode stages each warp's partial block in that warp's table area */
  static_assert(!CTA || PER_WARP * 8 >= NCOMP * (RB == 4 ? 4 : 8), "per-warp area too small for the partial block");
};

/* Rys roots rx and scaled weights rw (2 pi^(5/2) Kp Kq / sqrt(p+q) folded
 * in) of the primitive quartet of primitive pairs pi, qi, and 1/(p+q), in
 * the kernel arithmetic R: FP64 from the FP64 tables; FP32 from their FP32
 * roundings; double-float with no FP64 instruction.  UR: unroll count of the
 * loops over roots (1 keeps the code small where rx, rw live in shared
 * memory; full unrolling keeps them in registers). */
template <typename R, int NR, int UR>
__device__ __forceinline__ void prim_roots(const EriArgs &args, const PrimT<R> *__restrict__ primR, int pi, int qi,
                                           R *rx, R *rw, R &ripq) {
  if constexpr (std::is_same<R, double>::value) {
    const double two_pi_25 = 34.98683665524972; /* 2 pi^(5/2) */
    const PrimPair &pp = args.prims[pi];
    const PrimPair &qq = args.prims[qi];
    const double p = pp.p, q = qq.p;
    const double ipq = 1.0 / (p + q);
    const double dx = pp.P[0] - qq.P[0], dy = pp.P[1] - qq.P[1], dz = pp.P[2] - qq.P[2];
    const double Tb = p * q * ipq * (dx * dx + dy * dy + dz * dz);
    const double pref = two_pi_25 * pp.Kp * qq.Kp * sqrt(ipq);
#pragma unroll UR
    for (int rr = 0; rr < NR; ++rr) {
      double u, w;
      rys_root(NR, rr, Tb, args.rys, args.rc, u, w);
      rx[rr] = R(u);
      rw[rr] = R(w * pref);
    }
    ripq = R(ipq);
  } else if constexpr (std::is_same<R, float>::value) {
    /* FP32 kernels: roots, weights and prefactor in FP32 */
    const PrimT<float> &pp = primR[pi];
    const PrimT<float> &qq = primR[qi];
    const float ipq = 1.f / (pp.p + qq.p);
    const float dx = pp.P[0] - qq.P[0], dy = pp.P[1] - qq.P[1], dz = pp.P[2] - qq.P[2];
    const float Tb = pp.p * qq.p * ipq * (dx * dx + dy * dy + dz * dz);
    const float pref = 34.98683665f /* 2 pi^(5/2) */ * pp.Kp * qq.Kp * sqrtf(ipq);
    if (Tb < (float)RYS_TMAX_D) {
      const int j = max(0, min((int)(Tb * (float)(1.0 / RYS_H_D)), (int)(RYS_TMAX_D / RYS_H_D) - 1));
      const float t = (Tb - (float)(j * RYS_H_D)) * (float)(2.0 / RYS_H_D) - 1.f;
      const float sc = rsqrtf(1.f + Tb);
      const float *c = args.rys32 + args.rc.off[NR - 1] + (size_t)j * (2 * NR) * RYS_NCHEB_D;
#pragma unroll UR
      for (int rr = 0; rr < NR; ++rr) {
        rx[rr] = clenshaw8_f4(c + rr * RYS_NCHEB_D, t) * sc * sc;
        rw[rr] = clenshaw8_f4(c + (NR + rr) * RYS_NCHEB_D, t) * sc * pref;
      }
    } else {
      const float sc = rsqrtf(Tb);
#pragma unroll UR
      for (int rr = 0; rr < NR; ++rr) {
        rx[rr] = args.rc.axf[NR - 1][rr].x * sc * sc;
        rw[rr] = args.rc.awf[NR - 1][rr].x * sc * pref;
      }
    }
    ripq = ipq;
  } else {
    /* double-float throughout: no FP64 instruction on this path */
    const PrimT<df64> &pp = args_primdf(args)[pi];
    const PrimT<df64> &qq = args_primdf(args)[qi];
    const df64 pq = pp.p + qq.p;
    const df64 ipq = df_recip(pq);
    const df64 dx = pp.P[0] - qq.P[0], dy = pp.P[1] - qq.P[1], dz = pp.P[2] - qq.P[2];
    const df64 Tb = pp.p * qq.p * ipq * (dx * dx + dy * dy + dz * dz);
    const df64 pref = df64(34.98683547973633f, 1.1755134e-06f) /* 2 pi^(5/2) */ * pp.Kp * qq.Kp * df_sqrt(ipq);
    const float Tf = Tb.hi;
    df64 t(0.f), sc(0.f);
    int j = 0;
    if (Tf < (float)RYS_TMAX_D) {
      j = (int)(Tf * (float)(1.0 / RYS_H_D));
      /* guard the interval choice against hi-part rounding at its edge */
      const df64 tj = Tb - df64((float)(j * RYS_H_D));
      if (tj.hi < 0.f) {
        --j;
      } else if (tj.hi >= (float)RYS_H_D) {
        ++j;
      }
      j = max(0, min(j, (int)(RYS_TMAX_D / RYS_H_D) - 1));
      t = (Tb - df64((float)(j * RYS_H_D))) * df64((float)(2.0 / RYS_H_D)) - df64(1.f);
      sc = df_rsqrt(Tb + df64(1.f));
    } else {
      sc = df_rsqrt(Tb);
    }
#pragma unroll UR
    for (int rr = 0; rr < NR; ++rr) {
      df64 x, w;
      rys_root_df(NR, rr, j, Tf < (float)RYS_TMAX_D, t, sc, args.rysdf, args.rc, x, w);
      rx[rr] = from_df<R>(x);
      rw[rr] = from_df<R>(w * pref);
    }
    ripq = from_df<R>(ipq);
  }
}

/*
 * MODE 0: forward transform into U.
 * MODE 1: Schwarz diagonal -- qmax_out[P] = sqrt(max_ab |(ab|ab)|).
 * MODE 2: adjoint -- accumulate dE/dX for both pairs from Tbar.
 * MODE 3: forward and adjoint from one evaluation of each quartet.
 */
/* TAB: a batch launch over the quartets of many molecules -- item i of the
 * work list belongs to molecule wmol[i], whose arguments are tab[wmol[i]];
 * the launch's own arguments give only the primitive window */
template <int LA, int LB, int LC, int LD, typename R, int MODE, bool TAB = false>
__global__ void __launch_bounds__(WARPS * 32) eri_kernel(EriArgs args0, const int4 *__restrict__ work, int nwork,
                                                         const EriArgs *__restrict__ tab, const int *__restrict__ wmol) {
  using S = QuartetShape<LA, LB, LC, LD, sizeof(R)>;
  constexpr bool CTA = S::CTA;
  extern __shared__ double smem[];
  double *wbase = smem;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double *ws = wbase + (size_t)warp * S::PER_WARP;
  /* staging area: per warp (warp mode) or shared by the CTA */
  double *stage = CTA ? wbase + (size_t)WARPS * S::PER_WARP : ws;
  const int tid = CTA ? (int)threadIdx.x : lane;
  const int nthr = CTA ? (int)blockDim.x : 32;

  /* line mode: the lane's own function (e for ROWM, else f) and its slot */
  const int lslot = lane / S::NL, lfun = lane - lslot * S::NL;
  int lexp[3];
  list_exp(S::ROWM ? LA : LC, lfun, lexp);
  R *h2d = reinterpret_cast<R *>(ws);

  const int item0 = CTA ? (int)blockIdx.x : (int)blockIdx.x * WARPS + warp;
  const int istep = CTA ? (int)gridDim.x : (int)gridDim.x * WARPS;
  for (int item = item0; item < nwork; item += istep) {
    const EriArgs &args = TAB ? tab[wmol[item]] : args0;
    const PrimT<R> *__restrict__ primR = static_cast<const PrimT<R> *>(prec_data<R>::prim(args));
    const GeomT<R> *__restrict__ geomR = static_cast<const GeomT<R> *>(prec_data<R>::geom(args));
    const int4 pq = work[item];
    const ShellPair &P = args.pairs[pq.x];
    const ShellPair &Q = args.pairs[pq.y];
    R acc[S::NK];
#pragma unroll
    for (int m = 0; m < S::NK; ++m) acc[m] = R(0);
    /* primitive screen: pairs' primitives are sorted by their bound q0, so
     * rows ip whose q0_p q0_q(first) falls below eps end the contraction */
    const float eps = args0.prim_lo, eps_hi = args0.prim_hi;
    int nrow = P.nprim;
    if (eps > 0.f) {
      const float qtop = args.prim_q0[Q.prim0];
      for (int base = 0; base < P.nprim; base += 32) {
        const int ip = base + lane;
        const unsigned fail = __ballot_sync(0xffffffffu, ip < P.nprim && args.prim_q0[P.prim0 + ip] * qtop < eps);
        if (fail) {
          nrow = base + __ffs(fail) - 1;
          break;
        }
      }
    }
    /* this item's rows of P's primitive pairs (block-mode items carry their
     * staging place instead: every row) */
    const int row0 = MODE == 4 ? 0 : pq.z, rowe = MODE == 4 ? nrow : pq.w;
    const int r1 = min(rowe, nrow), pq_begin = row0 * Q.nprim;
    const int npq = r1 > row0 ? (r1 - row0) * Q.nprim : 0;
    /* lane roles in the 2D phase: slot g, root r, direction dir */
    const int g = lane / (3 * S::NR), rem = lane - g * (3 * S::NR);
    const int r = rem / 3, dir = rem - 3 * (rem / 3);
    const bool lane_a = g < S::G2;
    /* rounds of 32 candidate primitive quartets per warp; in CTA mode a
     * round covers 32*WARPS consecutive candidates interleaved over the warps
     * (stride WARPS), so that the survivors -- concentrated at low indices by
     * the sorted primitives -- spread evenly over the warps */
    const int cstep = CTA ? WARPS * 32 : 32;
    R *rx = reinterpret_cast<R *>(ws + S::SM_2D); /* [32][NR] roots */
    R *rw = rx + 32 * S::NR;                      /* [32][NR] scaled weights */
    R *ripq = rw + 32 * S::NR;                    /* [32] 1/(p+q) */
    int *plist = reinterpret_cast<int *>(ws + S::SM_2D + S::SM_ROOT - 16); /* [32] kept quartets */

    /* FP32 sums are taken smallest first: the chunks (and the quartets in a
     * chunk) in reverse, against the descending order of the bounds */
    constexpr bool ASC = std::is_same<R, float>::value;
    const int nchunk = (npq + cstep - 1) / cstep;
    for (int kc = 0; kc < nchunk; ++kc) {
      const int round = ASC ? nchunk - 1 - kc : kc;
      const int cand = CTA ? round * cstep + lane * WARPS + warp : round * cstep + lane;
      /* compaction: the chunk's primitive quartets that pass the screen */
      int nch;
      {
        const int pqi = pq_begin + cand;
        bool keep = cand < npq;
        if (keep && (eps > 0.f || eps_hi < INFINITY)) {
          const int ip = pqi / Q.nprim, iq = pqi - ip * Q.nprim;
          const float b = args.prim_q0[P.prim0 + ip] * args.prim_q0[Q.prim0 + iq];
          keep = b >= eps && b < eps_hi;
        }
        const unsigned bal = __ballot_sync(0xffffffffu, keep);
        nch = __popc(bal);
        if (keep) {
          const int pos = __popc(bal & ((1u << lane) - 1u));
          plist[ASC ? nch - 1 - pos : pos] = pqi;
        }
      }
      __syncwarp();
      if (nch == 0) continue;
      /* phase R: one primitive quartet per lane -- Boys argument, 1/(p+q),
       * prefactor and the n_r Rys roots/weights */
      {
        if (lane < nch) {
          const int pqi = plist[lane];
          const int ip = pqi / Q.nprim, iq = pqi - ip * Q.nprim;
          prim_roots<R, S::NR, 1>(args, primR, P.prim0 + ip, Q.prim0 + iq, rx + lane * S::NR, rw + lane * S::NR,
                                  ripq[lane]);
        }
      }
      __syncwarp();
      for (int sub = 0; sub < nch; sub += S::G2) {
        const int li = sub + g; /* local index of this slot's primitive quartet */
        const bool act = lane_a && li < nch;
        if (act) {
          const int pqi = plist[li];
          const int ip = pqi / Q.nprim, iq = pqi - ip * Q.nprim;
          const R uR = rx[li * S::NR + r], wR = rw[li * S::NR + r], ipqR = ripq[li];
          /* 2D recurrence coefficients in R, from the primitive-pair and
           * pair-geometry data stored in R */
          const PrimT<R> &pr = primR[P.prim0 + ip], &qr = primR[Q.prim0 + iq];
          const R Ad = geomR[pq.x].A[dir], Cd = geomR[pq.y].A[dir];
          const R Pd = pr.P[dir], Qd = qr.P[dir];
          const R PQ = Pd - Qd, uq = uR * ipqR;
          const R b00 = R(0.5f) * uq;
          const R b10 = R(0.5f) * pr.inv_p * (R(1) - qr.p * uq);
          const R b01 = R(0.5f) * qr.inv_p * (R(1) - pr.p * uq);
          const R c00 = (Pd - Ad) - qr.p * uq * PQ;
          const R d00 = (Qd - Cd) + pr.p * uq * PQ;
          const R g00 = dir == 2 ? wR : R(1);
          rys_g<S::LAB, S::LCD, R, S::NRP, S::RS>(g00, c00, d00, b00, b10, b01, h2d + (size_t)(g * 3 + dir) * S::DS + r);
        }
        __syncwarp();
        const int nact = min(S::G2, nch - sub);
        constexpr int DS = S::DS; /* one direction's table */
        {
          /* lane (slot lslot, function lfun): the table rows of its function
           * (one per exponent of the other side), then its line of NK
           * components, exponents known at compile time */
          constexpr int KB = S::ROWM ? S::RS : S::NRP; /* the lane's own exponent: rows (e) or columns (f) */
          constexpr int KS = S::ROWM ? S::NRP : S::RS; /* and the stride of the other side's exponent */
          const int sx = lexp[0] * KB, sy = lexp[1] * KB, sz = lexp[2] * KB;
#pragma unroll 1
          for (int gs = 0; gs < nact; gs += S::SL) {
            const int gg = gs + lslot;
            if (lslot < S::SL && gg < nact) {
              const R *hx = h2d + (size_t)gg * 3 * DS;
#pragma unroll 1
              for (int rg = 0; rg < S::NGF; ++rg) {
                R X[S::KD][S::VEC], Yv[S::KD][S::VEC], Z[S::KD][S::VEC];
#pragma unroll
                for (int kk = 0; kk < S::KD; ++kk) {
                  ldv<S::VEC>(hx + sx + kk * KS + rg * S::VEC, X[kk]);
                  ldv<S::VEC>(hx + DS + sy + kk * KS + rg * S::VEC, Yv[kk]);
                  ldv<S::VEC>(hx + 2 * DS + sz + kk * KS + rg * S::VEC, Z[kk]);
                }
                /* the line's components by (x, y) exponent pair: the x*y
                 * product once, then one z per angular momentum */
                constexpr int l0 = S::ROWM ? LC : LA, l1 = S::ROWM ? S::LCD : S::LAB;
                static_for<l1 + 1>([&](auto kxc) {
                  constexpr int kx = decltype(kxc)::value;
                  static_for<l1 + 1 - kx>([&](auto kyc) {
                    constexpr int ky = decltype(kyc)::value;
                    XYProd<R> xy[S::VEC];
#pragma unroll
                    for (int v = 0; v < S::VEC; ++v) xy[v] = mul_xy(X[kx][v], Yv[ky][v]);
                    static_for<l1 - l0 + 1>([&](auto lc) {
                      constexpr int kz = l0 + decltype(lc)::value - kx - ky;
                      if constexpr (kz >= 0) {
                        constexpr int k = kindex(l0, kx, ky, kz);
#pragma unroll
                        for (int v = 0; v < S::VEC; ++v) acc_xyz(acc[k], xy[v], Z[kz][v]);
                      }
                    });
                  });
                });
              }
              if constexpr (S::REM > 0) {
#pragma unroll 1
                for (int rr = S::NGF * S::VEC; rr < S::NR; ++rr) {
                  R X1[S::KD], Y1[S::KD], Z1[S::KD];
#pragma unroll
                  for (int kk = 0; kk < S::KD; ++kk) {
                    X1[kk] = hx[sx + kk * KS + rr];
                    Y1[kk] = hx[DS + sy + kk * KS + rr];
                    Z1[kk] = hx[2 * DS + sz + kk * KS + rr];
                  }
                  static_for<S::NK>([&](auto kc) {
                    constexpr int k = decltype(kc)::value;
                    constexpr int l0 = S::ROWM ? LC : LA;
                    acc3(acc[k], X1[cexp(l0, k, 0)], Y1[cexp(l0, k, 1)], Z1[cexp(l0, k, 2)]);
                  });
                }
              }
            }
          }
        }
        __syncwarp();
      }
    }

    /* stage the block E[c] in the transform arithmetic TT: FP32 for the
     * FP32 kernels (small quartets, or the small-primitive tail of large
     * ones); FP64 otherwise -- for the double-float kernels too, whose FP64
     * transform runs on the otherwise idle FP64 pipe beside the other warps'
     * FP32 work (a double-float transform measured slower) */
    using TT = typename std::conditional<std::is_same<R, float>::value, float, double>::type;
    auto tt = [](R v) -> TT {
      if constexpr (std::is_same<R, float>::value) return v;
      else return to_double(v);
    };
    TT *E = reinterpret_cast<TT *>(stage);
    /* the slots' partial lines to slot 0 (shuffles), then one line per lane */
#pragma unroll
    for (int k = 0; k < S::NK; ++k) {
      R v = acc[k];
#pragma unroll
      for (int s2 = 1; s2 < S::SL; ++s2) v += shfl_down_r(acc[k], s2 * S::NL);
      acc[k] = v;
    }
    if (CTA) {
      /* per-warp partial blocks (in the warps' own, now idle, table
       * areas), summed in warp order: deterministic */
      TT *part = reinterpret_cast<TT *>(ws);
      if (lslot == 0)
#pragma unroll
        for (int k = 0; k < S::NK; ++k) part[S::ROWM ? lfun * S::NEC + k : k * S::NEC + lfun] = tt(acc[k]);
      __syncthreads();
      for (int c = tid; c < S::NCOMP; c += nthr) {
        TT sum = reinterpret_cast<const TT *>(wbase)[c];
        for (int w = 1; w < WARPS; ++w) sum += reinterpret_cast<const TT *>(wbase + (size_t)w * S::PER_WARP)[c];
        E[c] = sum;
      }
      __syncthreads();
    } else {
      if (lslot == 0)
#pragma unroll
        for (int k = 0; k < S::NK; ++k) E[S::ROWM ? lfun * S::NEC + k : k * S::NEC + lfun] = tt(acc[k]);
      __syncwarp();
    }
    if (MODE == 1) {
      /* Schwarz: max over the diagonal (ab|ab) = M_ab E M_ab^T (P == Q), by
       * the first warp */
      if (!CTA || warp == 0) {
        const double *M = args.hrr + P.m0;
        double mx = 0.0;
        /* and sqrt(max_e |(e0|e0)|), the size of the untransferred block */
        double mx0 = 0.0;
        for (int e = lane; e < S::NEA; e += 32) mx0 = fmax(mx0, fabs((double)E[e * S::NEC + e]));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx0 = fmax(mx0, __shfl_xor_sync(0xffffffffu, mx0, o));
        if (lane == 0) args.q0max_out[pq.x] = sqrt(mx0);
        for (int ab = lane; ab < S::NAB; ab += 32) {
          const double *m = M + (size_t)ab * S::NEA;
          double v = 0.0;
          for (int e = 0; e < S::NEA; ++e) {
            const double me = m[e];
            if (me == 0.0) continue;
            double t = 0.0;
            for (int f = 0; f < S::NEC; ++f) t = fma((double)E[e * S::NEC + f], m[f], t);
            v = fma(me, t, v);
          }
          mx = fmax(mx, fabs(v));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (lane == 0) args.qmax_out[pq.x] = sqrt(mx);
      }
      if (CTA) __syncthreads();
      else __syncwarp();
      continue;
    }

    if constexpr (MODE == 4) {
      /* block mode: (ab|cd) = M_P E M_Q^T (the sparse transfer rows) added
       * into the atom quartet's staging block at every place the pair
       * functions take there: both orders of two shells on one atom, and the
       * transposed block when bra and ket are the same atom pair */
      constexpr int NCB = NC<LB>::v, NDD = NC<LD>::v, NCDF = NC<LC>::v * NC<LD>::v;
      const int4 bp = __ldg(args.pair_blk + pq.x), bq = __ldg(args.pair_blk + pq.y);
      const int ncol = pq.w & 0xFFFFF;
      const bool swp = (pq.w >> 20) & 1, dg = ((pq.w >> 21) & 1) && pq.x != pq.y;
      double *Gq = args.G + (unsigned)pq.z;
      const double *MP = args.hrr + P.m0, *MQ = args.hrr + Q.m0;
      /* the ket transfer first, Y[e][cd] = sum_f E[e][f] M_Q[cd][f], in the
       * idle table area (warp 1's in CTA mode, past E in warp mode) */
      constexpr int EW = (S::NCOMP * (int)sizeof(TT) + 7) / 8; /* E's doubles in warp mode */
      static_assert(CTA ? S::NEA * NCDF <= S::PER_WARP : EW + S::NEA * NCDF <= S::PER_WARP,
                    "block-mode transfer area too small");
      double *Yt = CTA ? wbase + S::PER_WARP : ws + EW;
      for (int o = tid; o < S::NEA * NCDF; o += nthr) {
        const int e = o / NCDF, cd = o - e * NCDF;
        double t = 0.0;
        for (int f = 0; f < S::NEC; ++f) {
          const double mq = __ldg(MQ + cd * S::NEC + f);
          if (mq != 0.0) t = fma((double)E[e * S::NEC + f], mq, t);
        }
        Yt[o] = t;
      }
      if (CTA) __syncthreads();
      else __syncwarp();
      for (int o = tid; o < S::NAB * NCDF; o += nthr) {
        const int ab = o / NCDF, cd = o - ab * NCDF;
        double v = 0.0;
        for (int e = 0; e < S::NEA; ++e) {
          const double mp = __ldg(MP + ab * S::NEA + e);
          if (mp != 0.0) v = fma(mp, Yt[e * NCDF + cd], v);
        }
        int rows[2], cols[2];
        const int nr = blk_places(bp, ab / NCB, ab - (ab / NCB) * NCB, rows);
        const int nc = blk_places(bq, cd / NDD, cd - (cd / NDD) * NDD, cols);
        /* (P|Q) at [P's place][Q's place] when P is on the bra atom pair of
         * the quartet, else transposed; and the other orientation too when
         * bra and ket are the same atom pair */
        for (int i = 0; i < nr; ++i)
          for (int j = 0; j < nc; ++j) {
            const size_t pq_at = (size_t)rows[i] * ncol + cols[j], qp_at = (size_t)cols[j] * ncol + rows[i];
            atomicAdd(Gq + (swp ? qp_at : pq_at), v);
            if (dg) atomicAdd(Gq + (swp ? pq_at : qp_at), v);
          }
      }
      if (CTA) __syncthreads();
      else __syncwarp();
      continue;
    }

    TT *Y = E + S::NCOMP;
    const TT *xtT;
    const TT *TbarT;
    if constexpr (std::is_same<TT, float>::value) {
      xtT = args.xtab32;
      TbarT = args.Tbar32;
    } else {
      xtT = args.xtab;
      TbarT = args.Tbar;
    }
    const TT *XP = xtT + P.xh0;
    const TT *XQ = xtT + Q.xh0;
    const int *opP = args.pair_opid + P.op0;
    const int *opQ = args.pair_opid + Q.op0;
    const bool same = pq.x == pq.y;
    auto sync = [&]() {
      if (CTA) __syncthreads();
      else __syncwarp();
    };
    /* adjoint of one ket chunk (with Y[jl][ab] = (E X_Q^T)[ab][jl] staged):
     * dX_P[ik][ab] += sum_jl W(ik,jl) Y[jl][ab], W(ik,jl) = Tbar[ik][jl]
     * (+ Tbar[jl][ik] when the pairs differ).  A thread takes BA components
     * of one bra orbital pair, so each W element is gathered once per BA
     * components; every output keeps its jl order. */
    constexpr int BA = S::NEA < 8 ? S::NEA : 8, NBA = (S::NEA + BA - 1) / BA;
    auto adj_bra = [&](int j0, int nj) {
      double *XPb = args.xbar + P.xh0;
      for (int o = tid; o < P.nop * NBA; o += nthr) {
        const int ik = o / NBA, ab0 = (o - ik * NBA) * BA;
        const int a = __ldg(opP + ik);
        TT acc[BA];
#pragma unroll
        for (int u = 0; u < BA; ++u) acc[u] = TT(0);
        for (int jl = 0; jl < nj; ++jl) {
          const int b = __ldg(opQ + j0 + jl);
          TT wv = ldt(TbarT + (size_t)a * args.np + b);
          if (!same) wv += ldt(TbarT + (size_t)b * args.np + a);
          const TT *y = Y + jl * S::NEA + ab0;
#pragma unroll
          for (int u = 0; u < BA; ++u)
            if (ab0 + u < S::NEA) mad(acc[u], wv, y[u]);
        }
#pragma unroll
        for (int u = 0; u < BA; ++u)
          if (ab0 + u < S::NEA) atomicAdd(XPb + (size_t)ik * S::NEA + ab0 + u, (double)acc[u]);
      }
    };
    if (MODE == 0 || MODE == 3) {
      for (int j0 = 0; j0 < Q.nop; j0 += S::JCH) {
        const int nj = min(S::JCH, Q.nop - j0);
        /* Y[jl][ab] = sum_cd E[ab][cd] X_Q[jl][cd] */
        for (int o = tid; o < nj * S::NEA; o += nthr) {
          const int jl = o / S::NEA, abi = o - jl * S::NEA;
          const TT *xq = XQ + (size_t)(j0 + jl) * S::NEC;
          const TT *e = E + abi * S::NEC;
          TT s = TT(0);
#pragma unroll
          for (int c = 0; c < S::NEC; ++c) mad(s, e[c], ldt(xq + c));
          Y[o] = s;
        }
        sync();
        /* Z[ik][jl] = sum_ab X_P[ik][ab] Y[jl][ab] -> U (one orientation) */
        for (int o = tid; o < P.nop * nj; o += nthr) {
          const int ik = o / nj, jl = o - ik * nj;
          const TT *xp = XP + (size_t)ik * S::NEA;
          const TT *y = Y + jl * S::NEA;
          TT s = TT(0);
#pragma unroll
          for (int c = 0; c < S::NEA; ++c) mad(s, ldt(xp + c), y[c]);
          const int a = __ldg(opP + ik), b = __ldg(opQ + j0 + jl);
          atomicAdd(args.T + (size_t)a * args.np + b, same ? 0.5 * (double)s : (double)s);
        }
        if (MODE == 3) adj_bra(j0, nj); /* the same Y serves the bra adjoint */
        sync();
      }
    }
    if (MODE == 2 || MODE == 3) {
      /* adjoint.  With Z(ik,jl) = X_P E X_Q^T and W = dE/dZ
       * (Tbar[ik][jl] (+ Tbar[jl][ik] when the pairs differ)):
       * dX_P[ik][ab] += sum_jl W(ik,jl) (E X_Q^T)[ab][jl] and
       * dX_Q[jl][cd] += sum_ik W(ik,jl) (X_P E)[ik][cd] */
      double *XQb = args.xbar + Q.xh0;
      for (int j0 = 0; MODE == 2 && j0 < Q.nop; j0 += S::JCH) {
        const int nj = min(S::JCH, Q.nop - j0);
        for (int o = tid; o < nj * S::NEA; o += nthr) {
          const int jl = o / S::NEA, abi = o - jl * S::NEA;
          const TT *xq = XQ + (size_t)(j0 + jl) * S::NEC;
          const TT *e = E + abi * S::NEC;
          TT s = TT(0);
#pragma unroll
          for (int c = 0; c < S::NEC; ++c) mad(s, e[c], ldt(xq + c));
          Y[o] = s;
        }
        sync();
        adj_bra(j0, nj);
        sync();
      }
      constexpr int ICH = S::JCH;
      for (int i0 = 0; i0 < P.nop; i0 += ICH) {
        const int ni = min(ICH, P.nop - i0);
        for (int o = tid; o < ni * S::NEC; o += nthr) {
          const int ik = o / S::NEC, cdi = o - ik * S::NEC;
          const TT *xp = XP + (size_t)(i0 + ik) * S::NEA;
          TT s = TT(0);
#pragma unroll
          for (int c = 0; c < S::NEA; ++c) mad(s, ldt(xp + c), E[c * S::NEC + cdi]);
          Y[o] = s;
        }
        sync();
        /* dX_Q[jl][cd] += sum_ik W(ik,jl) Y[ik][cd], BC components of one
         * ket orbital pair per thread */
        constexpr int BC = S::NEC < 8 ? S::NEC : 8, NBC = (S::NEC + BC - 1) / BC;
        for (int o = tid; o < Q.nop * NBC; o += nthr) {
          const int jl = o / NBC, cd0 = (o - jl * NBC) * BC;
          const int b = __ldg(opQ + jl);
          TT acc[BC];
#pragma unroll
          for (int u = 0; u < BC; ++u) acc[u] = TT(0);
          for (int ik = 0; ik < ni; ++ik) {
            const int a = __ldg(opP + i0 + ik);
            TT wv = ldt(TbarT + (size_t)a * args.np + b);
            if (!same) wv += ldt(TbarT + (size_t)b * args.np + a);
            const TT *y = Y + ik * S::NEC + cd0;
#pragma unroll
            for (int u = 0; u < BC; ++u)
              if (cd0 + u < S::NEC) mad(acc[u], wv, y[u]);
          }
#pragma unroll
          for (int u = 0; u < BC; ++u)
            if (cd0 + u < S::NEC) atomicAdd(XQb + (size_t)jl * S::NEC + cd0 + u, (double)acc[u]);
        }
        sync();
      }
    }
    if (CTA) __syncthreads();
  }
}


/*
 * Block mode, low classes (s and p pairs with at most 27 (e0|f0)
 * components): one lane per shell quartet.  The lane walks the quartet's
 * primitive quartets inside [prim_lo, prim_hi) of the primitive bound
 * (smallest bounds first in FP32), with roots, 2D tables and the component
 * sums in registers; then the transfer to (ab|cd) in closed form for s and
 * p, (a b| = (a+b, 0| + (A-B)_b (a 0| (Head-Gordon & Pople), and the block
 * is added into the atom quartet's staging block as mode 4 does.  Against
 * the warp kernels this drops the shared-memory tables, the compaction
 * ballots and the warp synchronisation that dominate these small classes.
 */
template <int LA, int LB>
struct LanePair {
  static constexpr int NE = ne_c(LA, LB);
};

/* (ab| from the (e0| list of a pair (la >= lb, both <= 1): e indexes the
 * functions of angular momentum la .. la+lb in CCA order */
template <int LA, int LB, typename TT>
__device__ __forceinline__ TT lane_hrr(int a, int b, const TT *e, const TT AB[3]) {
  if constexpr (LB == 0) {
    return e[a];
  } else {
    /* la = lb = 1: (a b| = (a+b, 0| + AB_b (a 0|, the 6 d functions after the 3 p */
    constexpr int dix[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    return e[3 + dix[a][b]] + AB[b] * e[a];
  }
}

template <int LA, int LB, int LC, int LD, typename R>
__global__ void __launch_bounds__(128) eri_lane_kernel(EriArgs args, const int4 *__restrict__ work, int nwork) {
  constexpr int LAB = LA + LB, LCD = LC + LD, NR = (LAB + LCD) / 2 + 1;
  constexpr int NEA = LanePair<LA, LB>::NE, NEC = LanePair<LC, LD>::NE;
  constexpr bool ASC = std::is_same<R, float>::value;
  const PrimT<R> *__restrict__ primR = static_cast<const PrimT<R> *>(prec_data<R>::prim(args));
  const GeomT<R> *__restrict__ geomR = static_cast<const GeomT<R> *>(prec_data<R>::geom(args));
  const float eps = args.prim_lo, eps_hi = args.prim_hi;
  for (int item = blockIdx.x * blockDim.x + threadIdx.x; item < nwork; item += gridDim.x * blockDim.x) {
    const int4 pq = work[item];
    const ShellPair &P = args.pairs[pq.x];
    const ShellPair &Q = args.pairs[pq.y];
    const int np_ = P.nprim, nq_ = Q.nprim;
    const float *q0p = args.prim_q0 + P.prim0, *q0q = args.prim_q0 + Q.prim0;
    R acc[NEA][NEC];
#pragma unroll
    for (int e = 0; e < NEA; ++e)
#pragma unroll
      for (int f = 0; f < NEC; ++f) acc[e][f] = R(0);
    R Ad[3], Cd[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      Ad[k] = geomR[pq.x].A[k];
      Cd[k] = geomR[pq.y].A[k];
    }
    /* the window's primitive quartets only: the primitives of both pairs are
     * sorted by bound, descending, so row ip keeps the columns [jhi, jlo)
     * with q0_p q0_q >= eps for iq < jlo and < eps_hi from jhi on, both ends
     * monotone over the rows */
    auto body = [&](int ip, int iq) {
      R rx[NR], rw[NR], ipq;
      prim_roots<R, NR, NR>(args, primR, P.prim0 + ip, Q.prim0 + iq, rx, rw, ipq);
      const PrimT<R> &pr = primR[P.prim0 + ip], &qr = primR[Q.prim0 + iq];
#pragma unroll
      for (int r = 0; r < NR; ++r) {
        const R uq = rx[r] * ipq;
        const R b00 = R(0.5f) * uq;
        const R b10 = R(0.5f) * pr.inv_p * (R(1) - qr.p * uq);
        const R b01 = R(0.5f) * qr.inv_p * (R(1) - pr.p * uq);
        R G[3][(LAB + 1) * (LCD + 1)];
#pragma unroll
        for (int dir = 0; dir < 3; ++dir) {
          const R Pd = pr.P[dir], Qd = qr.P[dir], PQ = Pd - Qd;
          const R c00 = (Pd - Ad[dir]) - qr.p * uq * PQ;
          const R d00 = (Qd - Cd[dir]) + pr.p * uq * PQ;
          rys_g<LAB, LCD, R, 1, LCD + 1>(dir == 2 ? rw[r] : R(1), c00, d00, b00, b10, b01, G[dir]);
        }
        static_for<NEA>([&](auto ec) {
          constexpr int e = decltype(ec)::value;
          constexpr int ex = cexp(LA, e, 0), ey = cexp(LA, e, 1), ez = cexp(LA, e, 2);
          static_for<NEC>([&](auto fc) {
            constexpr int f = decltype(fc)::value;
            constexpr int fx = cexp(LC, f, 0), fy = cexp(LC, f, 1), fz = cexp(LC, f, 2);
            acc3(acc[e][f], G[0][ex * (LCD + 1) + fx], G[1][ey * (LCD + 1) + fy], G[2][ez * (LCD + 1) + fz]);
          });
        });
      }
    };
    int nrow = 0;
    while (nrow < np_ && q0p[nrow] * q0q[0] >= eps) ++nrow;
    if constexpr (ASC) {
      /* FP32: smallest bounds first -- rows from the last, columns down */
      int jlo = 0, jhi = 0;
      for (int ip = nrow - 1; ip >= 0; --ip) {
        while (jlo < nq_ && q0p[ip] * q0q[jlo] >= eps) ++jlo;
        while (jhi < nq_ && q0p[ip] * q0q[jhi] >= eps_hi) ++jhi;
        for (int iq = jlo - 1; iq >= jhi; --iq) body(ip, iq);
      }
    } else {
      int jlo = nq_, jhi = nq_;
      for (int ip = 0; ip < nrow; ++ip) {
        while (jlo > 0 && !(q0p[ip] * q0q[jlo - 1] >= eps)) --jlo;
        while (jhi > 0 && !(q0p[ip] * q0q[jhi - 1] >= eps_hi)) --jhi;
        for (int iq = jhi; iq < jlo; ++iq) body(ip, iq);
      }
    }
    /* transfer to (ab|cd) and the staging block (mode 4 places): in FP32
     * for the FP32 quartets (whose integrals carry FP32 rounding anyway),
     * in FP64 otherwise */
    using TT = typename std::conditional<std::is_same<R, float>::value, float, double>::type;
    TT E[NEA * NEC];
#pragma unroll
    for (int e = 0; e < NEA; ++e)
#pragma unroll
      for (int f = 0; f < NEC; ++f) {
        if constexpr (std::is_same<R, float>::value) E[e * NEC + f] = acc[e][f];
        else E[e * NEC + f] = to_double(acc[e][f]);
      }
    TT ABp[3], ABq[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if constexpr (std::is_same<R, float>::value) {
        ABp[k] = geomR[pq.x].AB[k];
        ABq[k] = geomR[pq.y].AB[k];
      } else {
        ABp[k] = P.A[k] - P.B[k];
        ABq[k] = Q.A[k] - Q.B[k];
      }
    }
    const int4 bp = __ldg(args.pair_blk + pq.x), bq = __ldg(args.pair_blk + pq.y);
    const int ncol = pq.w & 0xFFFFF;
    const bool swp = (pq.w >> 20) & 1, dg = ((pq.w >> 21) & 1) && pq.x != pq.y;
    double *Gq = args.G + (unsigned)pq.z;
#pragma unroll
    for (int c = 0; c < NC<LC>::v; ++c)
#pragma unroll
      for (int d = 0; d < NC<LD>::v; ++d) {
        /* the ket transfer: Y[e] = (e0|cd) */
        TT Y[NEA];
#pragma unroll
        for (int e = 0; e < NEA; ++e) Y[e] = lane_hrr<LC, LD, TT>(c, d, E + e * NEC, ABq);
        int cols[2];
        const int nc = blk_places(bq, c, d, cols);
#pragma unroll
        for (int a = 0; a < NC<LA>::v; ++a)
#pragma unroll
          for (int bb = 0; bb < NC<LB>::v; ++bb) {
            const double v = (double)lane_hrr<LA, LB, TT>(a, bb, Y, ABp);
            int rows[2];
            const int nr = blk_places(bp, a, bb, rows);
            for (int i = 0; i < nr; ++i)
              for (int j = 0; j < nc; ++j) {
                const size_t pq_at = (size_t)rows[i] * ncol + cols[j], qp_at = (size_t)cols[j] * ncol + rows[i];
                atomicAdd(Gq + (swp ? qp_at : pq_at), v);
                if (dg) atomicAdd(Gq + (swp ? pq_at : qp_at), v);
              }
          }
      }
  }
}

template <int LA, int LB, int LC, int LD, typename R>
int launch_lane(const EriArgs &args, const int4 *work, int nwork, int max_blocks, cudaStream_t st) {
  if (nwork <= 0) return 0;
  int blocks = (nwork + 127) / 128;
  if (blocks > max_blocks) blocks = max_blocks;
  eri_lane_kernel<LA, LB, LC, LD, R><<<blocks, 128, 0, st>>>(args, work, nwork);
  return cudaGetLastError() != cudaSuccess;
}

template <int LA, int LB, int LC, int LD, typename R, int MODE, bool TAB = false>
int launch_one(const EriArgs &args, const int4 *work, int nwork, int max_blocks, cudaStream_t st,
               const EriArgs *tab = nullptr, const int *wmol = nullptr) {
  if (nwork <= 0) return 0;
  using S = QuartetShape<LA, LB, LC, LD, sizeof(R)>;
  size_t shm = sizeof(double) * ((size_t)WARPS * S::PER_WARP + S::SHARED);
  auto kfn = eri_kernel<LA, LB, LC, LD, R, MODE, TAB>;
  static bool attr_done = false;
  if (!attr_done) {
    if (cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm) != cudaSuccess) return 1;
    attr_done = true;
  }
  const int per_block = S::CTA ? 1 : WARPS;
  int blocks = (nwork + per_block - 1) / per_block;
  if (blocks > max_blocks) blocks = max_blocks; /* grid-stride beyond this */
  kfn<<<blocks, WARPS * 32, shm, st>>>(args, work, nwork, tab, wmol);
  return cudaGetLastError() != cudaSuccess;
}

/* class id of a pair (la>=lb): 00->0 10->1 11->2 20->3 21->4 22->5 */
template <int C>
struct ClsL;
template <> struct ClsL<0> { static constexpr int a = 0, b = 0; };
template <> struct ClsL<1> { static constexpr int a = 1, b = 0; };
template <> struct ClsL<2> { static constexpr int a = 1, b = 1; };
template <> struct ClsL<3> { static constexpr int a = 2, b = 0; };
template <> struct ClsL<4> { static constexpr int a = 2, b = 1; };
template <> struct ClsL<5> { static constexpr int a = 2, b = 2; };

template <int CP, int CQ, typename R, int MODE, bool TAB = false>
int launch_cls(const EriArgs &a, const int4 *w, int n, int max_blocks, cudaStream_t st, const EriArgs *tab = nullptr,
               const int *wmol = nullptr) {
  return launch_one<ClsL<CP>::a, ClsL<CP>::b, ClsL<CQ>::a, ClsL<CQ>::b, R, MODE, TAB>(a, w, n, max_blocks, st, tab,
                                                                                     wmol);
}

/* batch launches (forward + adjoint, mode 3) over the quartets of many
 * molecules, per-item arguments from tab[wmol[item]] */
template <typename R>
int dispatch_tab(int cp, int cq, const EriArgs &a, const int4 *w, int n, int max_blocks, cudaStream_t st,
                 const EriArgs *tab, const int *wmol) {
#define CASE(X, Y) \
  if (cp == X && cq == Y) return launch_cls<X, Y, R, 3, true>(a, w, n, max_blocks, st, tab, wmol);
  CASE(0, 0) CASE(1, 0) CASE(1, 1) CASE(2, 0) CASE(2, 1) CASE(2, 2)
  CASE(3, 0) CASE(3, 1) CASE(3, 2) CASE(3, 3) CASE(4, 0) CASE(4, 1) CASE(4, 2) CASE(4, 3) CASE(4, 4)
  CASE(5, 0) CASE(5, 1) CASE(5, 2) CASE(5, 3) CASE(5, 4) CASE(5, 5)
#undef CASE
  return 2;
}

/* block mode: s and p pair classes only; up to 27 (e0|f0) components one
 * lane per shell quartet, (pp|pp) on the CTA kernel */
template <typename R>
int dispatch_blk(int cp, int cq, const EriArgs &a, const int4 *w, int n, int max_blocks, cudaStream_t st) {
  if (cp == 0 && cq == 0) return launch_lane<0, 0, 0, 0, R>(a, w, n, max_blocks, st);
  if (cp == 1 && cq == 0) return launch_lane<1, 0, 0, 0, R>(a, w, n, max_blocks, st);
  if (cp == 1 && cq == 1) return launch_lane<1, 0, 1, 0, R>(a, w, n, max_blocks, st);
  if (cp == 2 && cq == 0) return launch_lane<1, 1, 0, 0, R>(a, w, n, max_blocks, st);
  if (cp == 2 && cq == 1) return launch_lane<1, 1, 1, 0, R>(a, w, n, max_blocks, st);
  if (cp == 2 && cq == 2) {
    /* (pp|pp): 81 components -- in registers one lane per quartet in FP32,
     * the CTA kernel in the wider arithmetics */
    if constexpr (std::is_same<R, float>::value) return launch_lane<1, 1, 1, 1, R>(a, w, n, max_blocks, st);
    else return launch_cls<2, 2, R, 4>(a, w, n, max_blocks, st);
  }
  return 2;
}

template <typename R, int MODE>
int dispatch(int cp, int cq, const EriArgs &a, const int4 *w, int n, int max_blocks, cudaStream_t st) {
#define CASE(X, Y) \
  if (cp == X && cq == Y) return launch_cls<X, Y, R, MODE>(a, w, n, max_blocks, st);
  CASE(0, 0) CASE(1, 0) CASE(1, 1) CASE(2, 0) CASE(2, 1) CASE(2, 2)
  CASE(3, 0) CASE(3, 1) CASE(3, 2) CASE(3, 3) CASE(4, 0) CASE(4, 1) CASE(4, 2) CASE(4, 3) CASE(4, 4)
  CASE(5, 0) CASE(5, 1) CASE(5, 2) CASE(5, 3) CASE(5, 4) CASE(5, 5)
#undef CASE
  return 2;
}

}  // namespace
#endif
