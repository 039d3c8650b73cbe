/*
 * eri.cu -- shell-quartet electron-repulsion integrals fused with the
 * LCAO-weight contraction of VALENCE's int2e (valence.F90:3184-3438).
 *
 * int2e contracts every shell quartet of four orbital bases with the weight
 * products dij(ab) dkl(cd) (valence.F90:3372-3412).  Here each unique AO shell
 * quartet (AB|CD) is evaluated once and transformed straight into the
 * orbital-pair matrix
 *     T[(i,k)][(j,l)] += sum_ab sum_cd X_ik(ab) (ab|cd) X_jl(cd),
 * X_ik(ab) = angn_a angn_b (C_i(a) C_k(b) + C_k(a) C_i(b)), so T holds every
 * (i k | j l) that vsvb_energy asks int2e for (valence.F90:1256,1264) and
 * the Schwarz table (:1516).  No AO integral is ever written to HBM.
 *
 * Integrals: Rys quadrature (Rys, Dupuis & King, J. Comput. Chem. 4, 154
 * (1983)) with the 2D recurrences for the x, y, z factors and horizontal
 * transfer to the second centre of each pair; roots and weights come from
 * project-generated Chebyshev tables (gen_rys_tables.py).
 *
 * Work split: one warp per shell quartet.  Per primitive quartet, lanes
 * 0..n_roots-1 evaluate the roots, lanes (root, direction) build the 2D
 * tables in shared memory, then all 32 lanes accumulate their share of the
 * Cartesian components in registers.  After the primitive loop the block is
 * staged in shared memory and transformed with the X tables; the result is
 * added to T with FP64 atomics.  R is the arithmetic type of the 2D tables
 * and the component accumulation (double, or float on the mixed path); the
 * roots, prefactors and the transform stay FP64.
 */
#include <cuda_runtime.h>

#include <cstdint>

#include "vsvb_internal.h"
#include "eri.cuh"

namespace {

__constant__ int c_rys_off[5];
__constant__ double c_rys_ax[5][5];
__constant__ double c_rys_aw[5][5];
/* Cartesian exponents in CCA order, l = 0..2: [l][k][xyz] */
__constant__ int c_cart[3][6][3] = {
    {{0, 0, 0}},
    {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}},
    {{2, 0, 0}, {1, 1, 0}, {1, 0, 1}, {0, 2, 0}, {0, 1, 1}, {0, 0, 2}}};

constexpr int RYS_NCHEB_D = 12;
constexpr double RYS_TMAX_D = 64.0;
constexpr double RYS_H_D = 0.5;

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

/* root r of the n-point rule: x (= t^2) and weight */
__device__ __forceinline__ void rys_root(int n, int r, double T, const double *__restrict__ tab, double &x,
                                         double &w) {
  if (T < RYS_TMAX_D) {
    int j = (int)(T * (1.0 / RYS_H_D));
    double t = (T - j * RYS_H_D) * (2.0 / RYS_H_D) - 1.0;
    const double *c = tab + c_rys_off[n - 1] + (size_t)j * (2 * n) * RYS_NCHEB_D;
    double fx = clenshaw12(c + r * RYS_NCHEB_D, t);
    double fw = clenshaw12(c + (n + r) * RYS_NCHEB_D, t);
    const double s = rsqrt(1.0 + T);
    x = fx * s * s;
    w = fw * s;
  } else {
    const double s = rsqrt(T);
    x = c_rys_ax[n - 1][r] * s * s;
    w = c_rys_aw[n - 1][r] * s;
  }
}

template <int L>
struct NC {
  static constexpr int v = (L + 1) * (L + 2) / 2;
};

/* x (or y, z) 2D factor for one root: G(i,k) by the Rys recurrences, then
 * horizontal transfer to (ia, ib, kc, kd) */
template <int LA, int LB, int LC, int LD, typename R>
__device__ __forceinline__ void rys_2d(R g00, R c00, R d00, R b00, R b10, R b01, R ab, R cd, R *__restrict__ out) {
  constexpr int LAB = LA + LB, LCD = LC + LD;
  R G[LAB + 1][LCD + 1];
  G[0][0] = g00;
#pragma unroll
  for (int i = 0; i < LAB; ++i) G[i + 1][0] = c00 * G[i][0] + (i > 0 ? R(i) * b10 * G[i > 0 ? i - 1 : 0][0] : R(0));
#pragma unroll
  for (int k = 0; k < LCD; ++k) {
#pragma unroll
    for (int i = 0; i <= LAB; ++i) {
      R v = d00 * G[i][k];
      if (k > 0) v += R(k) * b01 * G[i][k > 0 ? k - 1 : 0];
      if (i > 0) v += R(i) * b00 * G[i > 0 ? i - 1 : 0][k];
      G[i][k + 1] = v;
    }
  }
  /* ket transfer: K[i][c][d] = G(i, c+d) reduced to (c,d) */
  R K[LAB + 1][LC + 1][LD + 1];
#pragma unroll
  for (int i = 0; i <= LAB; ++i) {
    R W[LCD + 1][LD + 1];
#pragma unroll
    for (int c = 0; c <= LCD; ++c) W[c][0] = G[i][c];
#pragma unroll
    for (int d = 1; d <= LD; ++d)
#pragma unroll
      for (int c = 0; c <= LCD - d; ++c) W[c][d] = W[c + 1][d - 1] + cd * W[c][d - 1];
#pragma unroll
    for (int c = 0; c <= LC; ++c)
#pragma unroll
      for (int d = 0; d <= LD; ++d) K[i][c][d] = W[c][d];
  }
  /* bra transfer */
#pragma unroll
  for (int c = 0; c <= LC; ++c)
#pragma unroll
    for (int d = 0; d <= LD; ++d) {
      R V[LAB + 1][LB + 1];
#pragma unroll
      for (int a = 0; a <= LAB; ++a) V[a][0] = K[a][c][d];
#pragma unroll
      for (int b = 1; b <= LB; ++b)
#pragma unroll
        for (int a = 0; a <= LAB - b; ++a) V[a][b] = V[a + 1][b - 1] + ab * V[a][b - 1];
#pragma unroll
      for (int a = 0; a <= LA; ++a)
#pragma unroll
        for (int b = 0; b <= LB; ++b) out[((a * (LB + 1) + b) * (LC + 1) + c) * (LD + 1) + d] = V[a][b];
    }
}

template <int LA, int LB, int LC, int LD>
struct QuartetShape {
  static constexpr int NA = NC<LA>::v, NB = NC<LB>::v, NCc = NC<LC>::v, ND = NC<LD>::v;
  static constexpr int NAB = NA * NB, NCD = NCc * ND, NCOMP = NAB * NCD;
  static constexpr int NR = (LA + LB + LC + LD) / 2 + 1;
  static constexpr int N2D = (LA + 1) * (LB + 1) * (LC + 1) * (LD + 1);
  /* primitive quartets processed side by side per warp iteration: each takes
   * 3*NR lanes for its 2D tables; large blocks keep one slot so that the
   * per-lane accumulators stay in registers */
  static constexpr int G0 = 32 / (3 * NR);
  static constexpr int G = NCOMP >= 200 ? 1 : (G0 < 1 ? 1 : G0);
  static constexpr int NITEM = G * NCOMP;
  static constexpr int PER_LANE = (NITEM + 31) / 32;
  static constexpr int JCH = 8; /* ket orbital pairs per transform chunk */
  /* per-warp shared memory in doubles: 2D tables (phase 1) and block + Y
   * chunk (phase 2) share storage */
  static constexpr int SM_2D = G * 3 * NR * N2D;
  static constexpr int SM_TR = NCOMP + (NITEM > JCH * (NAB > NCD ? NAB : NCD) ? NITEM : JCH * (NAB > NCD ? NAB : NCD));
  static constexpr int PER_WARP = (SM_2D > SM_TR ? SM_2D : SM_TR);
};

constexpr int WARPS = 4;

/*
 * MODE 0: forward transform into T.
 * MODE 1: Schwarz diagonal -- pairs[P].qmax = sqrt(max_ab |(ab|ab)|).
 * MODE 2: adjoint -- accumulate dE/dX for both pairs from Tbar.
 * MODE 3: forward and adjoint from one evaluation of each quartet.
 */
template <int LA, int LB, int LC, int LD, typename R, int MODE>
__global__ void __launch_bounds__(WARPS * 32) eri_kernel(EriArgs args, const int2 *__restrict__ work, int nwork) {
  using S = QuartetShape<LA, LB, LC, LD>;
  extern __shared__ double smem[];
  int *idx = reinterpret_cast<int *>(smem);
  double *wbase = smem + (S::NCOMP + 1) / 2 + 1;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double *ws = wbase + (size_t)warp * S::PER_WARP;

  for (int c = threadIdx.x; c < S::NCOMP; c += blockDim.x) {
    int a = c / (S::NB * S::NCD), b = (c / S::NCD) % S::NB, cc = (c / S::ND) % S::NCc, d = c % S::ND;
    int ix = 0, iy = 0, iz = 0;
    int pw[4][3];
#pragma unroll
    for (int t = 0; t < 3; ++t) {
      pw[0][t] = c_cart[LA][a][t];
      pw[1][t] = c_cart[LB][b][t];
      pw[2][t] = c_cart[LC][cc][t];
      pw[3][t] = c_cart[LD][d][t];
    }
    ix = ((pw[0][0] * (LB + 1) + pw[1][0]) * (LC + 1) + pw[2][0]) * (LD + 1) + pw[3][0];
    iy = ((pw[0][1] * (LB + 1) + pw[1][1]) * (LC + 1) + pw[2][1]) * (LD + 1) + pw[3][1];
    iz = ((pw[0][2] * (LB + 1) + pw[1][2]) * (LC + 1) + pw[2][2]) * (LD + 1) + pw[3][2];
    idx[c] = ix | (iy << 10) | (iz << 20);
  }
  __syncthreads();

  R *h2d = reinterpret_cast<R *>(ws);
  const double two_pi_25 = 34.98683665524972; /* 2 pi^(5/2) */

  for (int item = blockIdx.x * WARPS + warp; item < nwork; item += gridDim.x * WARPS) {
    const int2 pq = work[item];
    const ShellPair &P = args.pairs[pq.x];
    const ShellPair &Q = args.pairs[pq.y];
    R acc[S::PER_LANE];
#pragma unroll
    for (int m = 0; m < S::PER_LANE; ++m) acc[m] = R(0);
    const int npq = P.nprim * Q.nprim;
    /* lane roles in phase A: slot g, root r, direction dir */
    const int g = lane / (3 * S::NR), rem = lane - g * (3 * S::NR);
    const int r = rem / 3, dir = rem - 3 * (rem / 3);
    const bool lane_a = g < S::G;

    for (int base = 0; base < npq; base += S::G) {
      const int pqi = base + g;
      const bool act = lane_a && pqi < npq;
      const unsigned amask = __ballot_sync(0xffffffffu, act);
      double u = 0.0, w = 0.0, ipq = 0.0;
      if (act) {
        const int ip = pqi / Q.nprim, iq = pqi - ip * Q.nprim;
        const PrimPair &pp = args.prims[P.prim0 + ip];
        const PrimPair &qq = args.prims[Q.prim0 + iq];
        /* FP64: reciprocal of p+q, Boys argument, Rys root and scaled weight */
        if (dir == 0) {
          const double p = pp.p, q = qq.p;
          ipq = 1.0 / (p + q);
          const double dx = pp.P[0] - qq.P[0], dy = pp.P[1] - qq.P[1], dz = pp.P[2] - qq.P[2];
          const double Tb = p * q * ipq * (dx * dx + dy * dy + dz * dz);
          rys_root(S::NR, r, Tb, args.rys, u, w);
          w *= two_pi_25 * pp.Kp * qq.Kp * sqrt(ipq);
        }
        u = __shfl_sync(amask, u, lane - dir);
        w = __shfl_sync(amask, w, lane - dir);
        ipq = __shfl_sync(amask, ipq, lane - dir);
        /* 2D recurrence coefficients in the kernel's precision */
        const R uR = R(u), ipqR = R(ipq);
        const R pR = R(pp.p), qR = R(qq.p), ipR = R(pp.inv_p), iqR = R(qq.inv_p);
        const R Pd = R(pp.P[dir]), Qd = R(qq.P[dir]);
        const R PQ = Pd - Qd, uq = uR * ipqR;
        const R b00 = R(0.5) * uq;
        const R b10 = R(0.5) * ipR * (R(1) - qR * uq);
        const R b01 = R(0.5) * iqR * (R(1) - pR * uq);
        const R c00 = (Pd - R(P.A[dir])) - qR * uq * PQ;
        const R d00 = (Qd - R(Q.A[dir])) + pR * uq * PQ;
        const R g00 = dir == 2 ? R(w) : R(1);
        rys_2d<LA, LB, LC, LD, R>(g00, c00, d00, b00, b10, b01, R(P.A[dir] - P.B[dir]), R(Q.A[dir] - Q.B[dir]),
                                  h2d + (size_t)((g * 3 + dir) * S::NR + r) * S::N2D);
      }
      __syncwarp();
      const int nact = min(S::G, npq - base);
#pragma unroll
      for (int m = 0; m < S::PER_LANE; ++m) {
        const int it = lane + 32 * m;
        if (it < S::NITEM) {
          const int gg = it / S::NCOMP, c = it - gg * S::NCOMP;
          if (gg < nact) {
            const int id = idx[c];
            const int ix = id & 1023, iy = (id >> 10) & 1023, iz = id >> 20;
            const R *hx = h2d + (size_t)(gg * 3 + 0) * S::NR * S::N2D;
            const R *hy = hx + S::NR * S::N2D, *hz = hy + S::NR * S::N2D;
            R sacc = acc[m];
#pragma unroll
            for (int rr = 0; rr < S::NR; ++rr)
              sacc += hx[rr * S::N2D + ix] * hy[rr * S::N2D + iy] * hz[rr * S::N2D + iz];
            acc[m] = sacc;
          }
        }
      }
      __syncwarp();
    }

    /* stage the block: sum the slots into E[c] (double) */
    double *E = ws;
    double *E2 = ws + S::NCOMP;
    if (S::G == 1) {
#pragma unroll
      for (int m = 0; m < S::PER_LANE; ++m) {
        const int c = lane + 32 * m;
        if (c < S::NCOMP) E[c] = (double)acc[m];
      }
    } else {
#pragma unroll
      for (int m = 0; m < S::PER_LANE; ++m) {
        const int it = lane + 32 * m;
        if (it < S::NITEM) E2[it] = (double)acc[m];
      }
      __syncwarp();
      for (int c = lane; c < S::NCOMP; c += 32) {
        double sum = 0.0;
        for (int gg = 0; gg < S::G; ++gg) sum += E2[gg * S::NCOMP + c];
        E[c] = sum;
      }
    }
    __syncwarp();
    if (MODE == 1) {
      /* Schwarz: max over diagonal components (ab|ab) */
      double mx = 0.0;
      for (int c = lane; c < S::NCOMP; c += 32)
        if ((c / S::NCD) == (c % S::NCD)) mx = fmax(mx, fabs(E[c]));
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      if (lane == 0) args.qmax_out[pq.x] = sqrt(mx);
      __syncwarp();
      continue;
    }
    double *Y = ws + S::NCOMP; /* reuses the slot buffer */
    const double *XP = args.xtab + P.x0;
    const double *XQ = args.xtab + Q.x0;
    const int *opP = args.pair_opid + P.op0;
    const int *opQ = args.pair_opid + Q.op0;
    const bool same = pq.x == pq.y;
    if (MODE == 0 || MODE == 3) {
      for (int j0 = 0; j0 < Q.nop; j0 += S::JCH) {
        const int nj = min(S::JCH, Q.nop - j0);
        /* Y[jl][ab] = sum_cd E[ab][cd] X_Q[jl][cd] */
        for (int o = lane; o < nj * S::NAB; o += 32) {
          const int jl = o / S::NAB, abi = o - jl * S::NAB;
          const double *xq = XQ + (size_t)(j0 + jl) * S::NCD;
          const double *e = E + abi * S::NCD;
          double s = 0.0;
#pragma unroll
          for (int c = 0; c < S::NCD; ++c) s = fma(e[c], __ldg(xq + c), s);
          Y[o] = s;
        }
        __syncwarp();
        /* Z[ik][jl] = sum_ab X_P[ik][ab] Y[jl][ab] */
        for (int o = lane; o < P.nop * nj; o += 32) {
          const int ik = o / nj, jl = o - ik * nj;
          const double *xp = XP + (size_t)ik * S::NAB;
          const double *y = Y + jl * S::NAB;
          double s = 0.0;
#pragma unroll
          for (int c = 0; c < S::NAB; ++c) s = fma(__ldg(xp + c), y[c], s);
          const int a = __ldg(opP + ik), b = __ldg(opQ + j0 + jl);
          atomicAdd(args.T + (size_t)a * args.np + b, same ? 0.5 * s : s);
        }
        __syncwarp();
      }
    }
    if (MODE == 2 || MODE == 3) {
      /* MODE 2/3: adjoint.  With Tbar symmetric and Z(ik,jl) = X_P E X_Q^T,
       * dE/dX_P[ik][ab] += sum_jl W(ik,jl) (E X_Q^T)[ab][jl] and
       * dE/dX_Q[jl][cd] += sum_ik W(ik,jl) (X_P E)[ik][cd], where
       * W = Tbar[ik][jl] (+ Tbar[jl][ik] when the pairs differ). */
      double *XPb = args.xbar + P.x0;
      double *XQb = args.xbar + Q.x0;
      for (int j0 = 0; j0 < Q.nop; j0 += S::JCH) {
        const int nj = min(S::JCH, Q.nop - j0);
        for (int o = lane; o < nj * S::NAB; o += 32) {
          const int jl = o / S::NAB, abi = o - jl * S::NAB;
          const double *xq = XQ + (size_t)(j0 + jl) * S::NCD;
          const double *e = E + abi * S::NCD;
          double s = 0.0;
#pragma unroll
          for (int c = 0; c < S::NCD; ++c) s = fma(e[c], __ldg(xq + c), s);
          Y[o] = s;
        }
        __syncwarp();
        /* dX_P[ik][ab] += sum_jl W(ik,jl) Y[jl][ab] */
        for (int o = lane; o < P.nop * S::NAB; o += 32) {
          const int ik = o / S::NAB, abi = o - ik * S::NAB;
          const int a = __ldg(opP + ik);
          double s = 0.0;
          for (int jl = 0; jl < nj; ++jl) {
            const int b = __ldg(opQ + j0 + jl);
            double wv = args.Tbar[(size_t)a * args.np + b];
            if (!same) wv += args.Tbar[(size_t)b * args.np + a];
            s = fma(wv, Y[jl * S::NAB + abi], s);
          }
          atomicAdd(XPb + (size_t)ik * S::NAB + abi, s);
        }
        __syncwarp();
      }
      /* dX_Q[jl][cd] += sum_ik W(ik,jl) (X_P E)[ik][cd]; Y holds an
       * (ik-chunk x NCD) block (sized JCH x max(NAB, NCD)) */
      constexpr int ICH = S::JCH;
      for (int i0 = 0; i0 < P.nop; i0 += ICH) {
        const int ni = min(ICH, P.nop - i0);
        for (int o = lane; o < ni * S::NCD; o += 32) {
          const int ik = o / S::NCD, cdi = o - ik * S::NCD;
          const double *xp = XP + (size_t)(i0 + ik) * S::NAB;
          double s = 0.0;
#pragma unroll
          for (int c = 0; c < S::NAB; ++c) s = fma(__ldg(xp + c), E[c * S::NCD + cdi], s);
          Y[o] = s;
        }
        __syncwarp();
        for (int o = lane; o < Q.nop * S::NCD; o += 32) {
          const int jl = o / S::NCD, cdi = o - jl * S::NCD;
          const int b = __ldg(opQ + jl);
          double s = 0.0;
          for (int ik = 0; ik < ni; ++ik) {
            const int a = __ldg(opP + i0 + ik);
            double wv = args.Tbar[(size_t)a * args.np + b];
            if (!same) wv += args.Tbar[(size_t)b * args.np + a];
            s = fma(wv, Y[ik * S::NCD + cdi], s);
          }
          atomicAdd(XQb + (size_t)jl * S::NCD + cdi, s);
        }
        __syncwarp();
      }
    }
  }
}

template <int LA, int LB, int LC, int LD, typename R, int MODE>
int launch_one(const EriArgs &args, const int2 *work, int nwork, int nsm, cudaStream_t st) {
  if (nwork <= 0) return 0;
  using S = QuartetShape<LA, LB, LC, LD>;
  size_t shm = sizeof(double) * ((S::NCOMP + 1) / 2 + 1 + (size_t)WARPS * S::PER_WARP);
  auto kfn = eri_kernel<LA, LB, LC, LD, R, MODE>;
  static bool attr_done = false;
  if (!attr_done) {
    if (cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm) != cudaSuccess) return 1;
    attr_done = true;
  }
  int blocks = (nwork + WARPS - 1) / WARPS;
  int cap = nsm * 16;
  if (blocks > cap) blocks = cap;
  kfn<<<blocks, WARPS * 32, shm, st>>>(args, work, nwork);
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

template <int CP, int CQ, typename R, int MODE>
int launch_cls(const EriArgs &a, const int2 *w, int n, int nsm, cudaStream_t st) {
  return launch_one<ClsL<CP>::a, ClsL<CP>::b, ClsL<CQ>::a, ClsL<CQ>::b, R, MODE>(a, w, n, nsm, st);
}

template <typename R, int MODE>
int dispatch(int cp, int cq, const EriArgs &a, const int2 *w, int n, int nsm, cudaStream_t st) {
#define CASE(X, Y) \
  if (cp == X && cq == Y) return launch_cls<X, Y, R, MODE>(a, w, n, nsm, st);
  CASE(0, 0) CASE(1, 0) CASE(1, 1) CASE(2, 0) CASE(2, 1) CASE(2, 2)
  CASE(3, 0) CASE(3, 1) CASE(3, 2) CASE(3, 3) CASE(4, 0) CASE(4, 1) CASE(4, 2) CASE(4, 3) CASE(4, 4)
  CASE(5, 0) CASE(5, 1) CASE(5, 2) CASE(5, 3) CASE(5, 4) CASE(5, 5)
#undef CASE
  return 2;
}

__global__ void symmetrize_kernel(double *T, int np) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long n = (long long)np * (np + 1) / 2;
  if (t >= n) return;
  long long i = (long long)((sqrt(8.0 * t + 1.0) - 1.0) / 2.0);
  while ((i + 1) * (i + 2) / 2 <= t) ++i;
  while (i * (i + 1) / 2 > t) --i;
  long long j = t - i * (i + 1) / 2;
  double *a = T + i * np + j, *b = T + j * np + i;
  double v = *a + *b;
  if (i == j) v = 2.0 * (*a);
  *a = v;
  *b = v;
}

}  // namespace

/* T = U + U^T after the forward pass (the kernels accumulate one orientation) */
int eri_symmetrize(double *T, int np, cudaStream_t st) {
  long long n = (long long)np * (np + 1) / 2;
  if (n == 0) return 0;
  symmetrize_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(T, np);
  return cudaGetLastError() != cudaSuccess;
}

/* algorithmic FLOPs of one shell quartet of class (cp, cq) in this
 * formulation: per primitive quartet the n_r roots (two 12-term Clenshaw sums
 * each), the 3 n_r 2D tables (recurrence + transfers) and the component sums
 * (3 flops per component and root); per quartet the two transform GEMVs. */
double eri_flops(int cp, int cq, int nprimP, int nprimQ, int nopP, int nopQ) {
  static const int la_[6] = {0, 1, 1, 2, 2, 2}, lb_[6] = {0, 0, 1, 0, 1, 2};
  int la = la_[cp], lb = lb_[cp], lc = la_[cq], ld = lb_[cq];
  auto nc = [](int l) { return (l + 1) * (l + 2) / 2; };
  int nab = nc(la) * nc(lb), ncd = nc(lc) * nc(ld), ncomp = nab * ncd;
  int nr = (la + lb + lc + ld) / 2 + 1;
  int n2d = (la + 1) * (lb + 1) * (lc + 1) * (ld + 1);
  double roots = nr * 2.0 * 24.0;
  double twod = 3.0 * nr * (5.0 * (la + lb + 1) * (lc + ld + 1) + 2.0 * n2d);
  double comp = 3.0 * nr * (double)ncomp;
  double prim = 30.0 + roots + twod + comp;
  double tr = 2.0 * nopQ * (double)nab * ncd + 2.0 * nopP * (double)nopQ * nab;
  return (double)nprimP * nprimQ * prim + tr;
}

int eri_set_tables(const int *off, const double *ax, const double *aw) {
  if (cudaMemcpyToSymbol(c_rys_off, off, sizeof(int) * 5) != cudaSuccess) return 1;
  if (cudaMemcpyToSymbol(c_rys_ax, ax, sizeof(double) * 25) != cudaSuccess) return 1;
  if (cudaMemcpyToSymbol(c_rys_aw, aw, sizeof(double) * 25) != cudaSuccess) return 1;
  return 0;
}

int eri_launch(int mode, int fp32, int cp, int cq, const EriArgs &a, const int2 *work, int nwork, int nsm,
               cudaStream_t st) {
  if (mode == 1) return dispatch<double, 1>(cp, cq, a, work, nwork, nsm, st);
  if (mode == 3) return fp32 ? dispatch<float, 3>(cp, cq, a, work, nwork, nsm, st)
                             : dispatch<double, 3>(cp, cq, a, work, nwork, nsm, st);
  if (mode == 2) return fp32 ? dispatch<float, 2>(cp, cq, a, work, nwork, nsm, st)
                             : dispatch<double, 2>(cp, cq, a, work, nwork, nsm, st);
  return fp32 ? dispatch<float, 0>(cp, cq, a, work, nwork, nsm, st) : dispatch<double, 0>(cp, cq, a, work, nwork, nsm, st);
}
