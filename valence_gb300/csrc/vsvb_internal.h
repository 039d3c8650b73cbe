/*
 * vsvb_internal.h -- device data layout of the GB300 VSVB energy path.
 *
 * HBM layout (all per handle, built once by vsvb_gpu_create unless noted):
 *   shells      GShell[nshell]       global Cartesian shells (atom-ordered)
 *   prims       PrimPair[nprimpair]  primitive pairs of every kept shell pair
 *   pairs       ShellPair[npair]     unique shell pairs (A>=B), first shell has
 *                                    the higher angular momentum
 *   pair_ops    int[]                orbital pairs (i,k) touching each shell pair
 *   xtab        double[]             per evaluation: X_op(a,b) = angn_a angn_b
 *                                    (C_i(a) C_k(b) + C_k(a) C_i(b)) on that pair
 *   work        int2[] per class     screened shell-quartet schedule
 *   S_ao,H_ao   double[nao*nao]      AO overlap and core Hamiltonian
 *   C_obs       double[norb*maxobs]  per evaluation: normalised orbital weights
 *   T           double[np*np]        per evaluation: orbital-pair ERIs
 *                                    (i k | j l), np = n(n+1)/2
 *   det data    per determinant pair q: det, inverse (n x n) per spin; a
 *               block flagged singular keeps det(A + delta I) and that
 *               matrix's inverse for the adjoint, and its pair takes a slot
 *               of the exact-minor pool: inverse and det of A + k P, k = 1..3
 */
#ifndef VSVB_INTERNAL_H
#define VSVB_INTERNAL_H

#include <cstdint>

#define VSVB_LMAX 2     /* highest angular momentum on the GPU */
#define VSVB_NCLS 6     /* shell-pair classes (la>=lb): 00 10 11 20 21 22 */

struct GShell {
  int l, nprim, prim0, atom; /* prim0 indexes the global exponent/coef arrays */
  int ao0;                   /* first global AO (Cartesian) function */
  int pad;
  double xyz[3];
};

struct PrimPair {
  double P[3];
  double p;      /* alpha + beta */
  double inv_p;  /* 1 / p */
  double Kp;     /* c_a c_b exp(-alpha beta / p |AB|^2) / p */
};

#ifdef __CUDACC__
#define VSVB_HD __host__ __device__
#else
#define VSVB_HD
#endif

/* double-float: an unevaluated sum hi + lo of two FP32 numbers (about 48
 * significant bits), used on the mixed path for quartets that need
 * FP64-class accuracy while running on the FP32 pipes */
struct df64 {
  float hi, lo;
  df64() = default;
  VSVB_HD df64(float h, float l) : hi(h), lo(l) {}
  VSVB_HD df64(float h) : hi(h), lo(0.0f) {}
  VSVB_HD df64(int i) : hi((float)i), lo(0.0f) {}
  VSVB_HD explicit df64(double d) {
    hi = (float)d;
    lo = (float)(d - (double)hi);
  }
  VSVB_HD explicit operator double() const { return (double)hi + (double)lo; }
};

#ifdef __CUDACC__
/* double-float arithmetic: Knuth's TwoSum and an FMA-based TwoProduct
 * (Dekker), renormalised by a quick two-sum */
__device__ __forceinline__ df64 df_quick(float s, float e) {
  const float r = s + e;
  return df64(r, e - (r - s));
}
__device__ __forceinline__ df64 operator+(df64 a, df64 b) {
  const float s = a.hi + b.hi;
  const float v = s - a.hi;
  float e = (a.hi - (s - v)) + (b.hi - v);
  e += a.lo + b.lo;
  return df_quick(s, e);
}
__device__ __forceinline__ df64 operator-(df64 a) { return df64(-a.hi, -a.lo); }
__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + (-b); }
__device__ __forceinline__ df64 operator*(df64 a, df64 b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return df_quick(p, e);
}
__device__ __forceinline__ df64 &operator+=(df64 &a, df64 b) {
  a = a + b;
  return a;
}

/* double -> double-float without FP64 arithmetic (whose rate is 1/58 of
 * FP32 on this part): hi takes the sign, exponent and top 23 mantissa bits
 * (a truncation, exact in FP32), lo the remaining 29 mantissa bits scaled by
 * their weight (rounded to 24 bits: ~48 significant bits in all).  Values
 * below the FP32 normal range (2^-126) become zero. */
__device__ __forceinline__ df64 df64_split(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7ff);
  if (e <= 1023 - 127) return df64(0.f, 0.f);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const float hi = __uint_as_float(sign | ((unsigned)(e - 1023 + 127) << 23) | (unsigned)((b >> 29) & 0x7fffffu));
  const float lo = ldexpf(__uint2float_rn((unsigned)(b & 0x1fffffffu)), e - 1075);
  return df64(hi, sign ? -lo : lo);
}
#endif

/* primitive-pair and pair-geometry data in the arithmetic type R of a kernel */
template <typename R>
struct PrimT {
  R P[3];
  R p, inv_p;
  R Kp; /* c_a c_b exp(-alpha beta / p |AB|^2) / p */
};
template <typename R>
struct GeomT {
  R A[3];   /* first centre */
  R AB[3];  /* A - B */
};

struct ShellPair {
  int shA, shB;      /* global shells; l(shA) >= l(shB) */
  int cls;           /* pair class 0..5 */
  int prim0, nprim;  /* into prims */
  int op0, nop;      /* into pair_ops / orbital-pair lists */
  int x0;            /* into xtab: nop * n_a * n_b doubles */
  int xh0;           /* into the transferred table X' = X M: nop * ne doubles */
  int m0;            /* into hrr: the n_a n_b x ne transfer matrix M */
  double A[3], B[3];
  double qmax;       /* sqrt(max (ab|ab)) */
  double pad;
};

/* one orbital-pair term of a shell pair: orbital i on shell A, k on shell B
 * (or the reverse), flattened for the X-table kernel */
struct PairOp {
  int op;       /* global orbital-pair index i*(i+1)/2+k, i>=k */
  int oi, ok;   /* orbitals (0-based) */
  int pad;
};

struct DetSetup {
  int nelec, nalpha, nbeta, npair, nunpd, ndocc, nnd, nsp;
  /* non-DOCC spatial orbitals of the task loop (num_non_docc of vsvb_energy):
   * nnd, or nnd + 2 when a DOCC orbital's alpha and beta slots hold
   * different orbitals (first_order_opt, valence.F90:578-603) */
  int nsd;
  int nsc;          /* number of spin couplings used (>=1) */
  long long nq;     /* determinant pairs */
};

#endif
