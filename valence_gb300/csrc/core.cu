/*
 * core.cu -- the VSVB energy summed over determinant pairs that share a
 * doubly occupied core, in closed form (valence.F90:1010-1434 with
 * density/dbra/dket/det, :1535-2056, and givdr, :2067-2144).
 *
 * Every determinant of a spin-coupled wave function without unpaired
 * orbitals holds, per spin, the nD doubly occupied (core) orbitals D and one
 * orbital of each of the P coupled pairs; the determinant pair (K, L) of
 * spin s has the overlap block S[K_s, L_s] with the core rows and columns
 * shared by all pairs.  With G = S_DD^-1 and the Schur complement
 *   M = S_CC - S_CD G S_DC      (C: the 2P coupled orbitals)
 * the block of pair (K, L) factorises as
 *   det S[K_s, L_s] = det S_DD * det M_s,   M_s = M[k_s, l_s]  (P x P)
 * and its transition density (bra orbital i, ket orbital j) is
 *   P_s = P0 + U N_s U^T,   P0 = G on the core block,
 *   U = (e_c - G S_Dc)_c,   N_s[a][b] = (M_s^-1)[pos b][pos a].
 * So every determinant pair is one P x P factorisation per spin, and the
 * energy needs the pair sums
 *   A0 = sum_q w d_a d_b,  A1 = sum_q w (d_b L_a + d_a L_b),
 *   A2 = sum_q w (d_b Q_a + d_a Q_b + (L_a (x) L_b + L_b (x) L_a) / 2)
 * over the C-space first cofactors L_s = d_s N_s and second cofactors
 *   Q_s[abcd] = d_s (N_ab N_cd - N_ad N_cb) / 2.
 * The pair-summed first- and second-order densities are then
 *   gamma = 2 A0 P0 + R1,   R1 = U A1 U^T,
 *   Gamma[ik][jl] = 2 A0 P0_ik P0_jl + P0_ik R1_jl + R1_ik P0_jl
 *                 - A0 P0_il P0_jk - (P0_il R1_jk + R1_il P0_jk) / 2
 *                 + sum_abcd U_ia U_kb U_jc U_ld A2[abcd],
 * and with the orbital-pair ERI matrix T masked by the reference's screens
 * (the Schwarz product of its two pairs and |ERI| above itol, :1189-1190,
 * :1286-1287 -- both functions of the T element alone)
 *   e1 = <h, gamma>,  wfnorm = <S, gamma> / nelec,  e2 = <T_masked, Gamma>
 * over ordered orbital indices: the same sums as the task loop's (its DOCC
 * parity skips and the i = j skips of coupled orbitals are exact zeros of
 * these densities).  The orbital-pair form of the U-part of Gamma is one
 * GEMM, Wv A2x Wv^T, whose epilogue adds the exchange terms of the core.
 * For an energy it contracts with T on the fly and Gamma is never stored;
 * for a gradient Gamma is stored before the ERI sweep as its dE_num/dT and
 * contracted with T after it.
 *
 * A spin block whose pivots fall below 1e-7 of max(its largest entry, 1)
 * (exact rank deficiency from molecular symmetry, or an orbital far from
 * the rest: the Schur complement of normalised orbitals has entries of at
 * most 1) takes the exact path of the
 * per-pair kernels: with Pert a fixed rank-2 matrix, every determinant,
 * first and second cofactor of the block is a polynomial of degree <= 2 in
 * k over block + k Pert, so its value at k = 0 is 3 f(1) - 3 f(2) + f(3);
 * the three perturbed factorisations are kept in a pool slot for the
 * second cofactors.  The core block itself must be regular (status 8).
 */
#include <cuda_runtime.h>

#include <cmath>

#include "core.cuh"
#include "vsvb_internal.h"

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int WLD = 33; /* row stride of a warp's P x 2P elimination tile */

__device__ __forceinline__ double pert_entry(int r, int c, double s) {
  const double w1 = sin(1.0 + 0.7548776662466927 * r), w2 = sin(2.0 + 0.5698402909980532 * r);
  const double z1 = cos(0.5 + 0.6180339887498949 * c), z2 = cos(1.5 + 0.4142135623730950 * c);
  return s * (w1 * z1 + w2 * z2);
}

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  return v;
}

/* block-wide sum in a fixed order (every thread gets it) */
__device__ double block_sum(double v, double *red) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  for (int k = 0; k < nw; ++k) s += red[k];
  return s;
}

__device__ __forceinline__ long long pair_of(const CoreArgs &a, int bd, int kd) {
  const int P = a.P;
  const int m = (1 << P) - 1;
  return ((long long)((bd >> P) * a.nsc + (kd >> P)) << (2 * P)) | ((long long)(bd & m) << P) | (kd & m);
}

__device__ __forceinline__ double weight_of(const CoreArgs &a, int bd, int kd) {
  return a.csc[bd >> a.P] * a.csc[kd >> a.P];
}

/* unordered pair index u -> (x, y), x >= y, u = x (x + 1) / 2 + y */
__device__ __forceinline__ void unpair(int u, int &x, int &y) {
  x = (int)((sqrt(8.0 * u + 1.0) - 1.0) * 0.5);
  while (x * (x + 1) / 2 > u) --x;
  while ((x + 1) * (x + 2) / 2 <= u) ++x;
  y = u - x * (x + 1) / 2;
}

/* Gauss-Jordan with partial pivoting of the warp's tile W = [A | I]
 * (P x 2P, P <= 16, lane = column): W becomes [. | A^-1]; returns det A,
 * ok = false when a pivot is not above pmin */
__device__ double warp_gj(double *W, int P, int lane, double pmin, bool &ok) {
  double det = 1.0;
  const int n2 = 2 * P;
  for (int k = 0; k < P; ++k) {
    double v = (lane >= k && lane < P) ? fabs(W[lane * WLD + k]) : -1.0;
    int idx = lane;
    for (int o = 16; o > 0; o >>= 1) {
      const double ov = __shfl_xor_sync(FULL, v, o);
      const int oi = __shfl_xor_sync(FULL, idx, o);
      if (ov > v || (ov == v && oi < idx)) {
        v = ov;
        idx = oi;
      }
    }
    if (!(v > pmin)) {
      ok = false;
      return 0.0;
    }
    const double piv = W[idx * WLD + k];
    det *= idx != k ? -piv : piv;
    __syncwarp();
    if (idx != k && lane < n2) {
      const double t = W[k * WLD + lane];
      W[k * WLD + lane] = W[idx * WLD + lane];
      W[idx * WLD + lane] = t;
    }
    __syncwarp();
    const double rk = lane < n2 ? W[k * WLD + lane] / piv : 0.0;
    /* column k is read by every lane and left alone by its own lane */
    if (lane < n2 && lane != k) {
      for (int i = 0; i < P; ++i)
        if (i != k) W[i * WLD + lane] -= W[i * WLD + k] * rk;
      W[k * WLD + lane] = rk;
    }
    __syncwarp();
  }
  ok = true;
  return det;
}

/* Q_s[abcd] of pair q from its block positions (ra, rc bra; cb, cd ket) */
__device__ __forceinline__ double second_cof(const CoreArgs &a, long long q, int s, int ra, int rc, int cb, int cd) {
  const int P = a.P, P2 = P * P;
  const int ps = a.pslot[q];
  if (ps >= 0 && ((ps >> s) & 1)) {
    const double *e = a.pool + (size_t)(ps >> 2) * 6 * (1 + P2);
    const double cf[3] = {3.0, -3.0, 1.0};
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double *v = e + (size_t)(2 * k + s) * (1 + P2);
      const double dk = v[0];
      if (dk != 0.0) {
        const double *Lk = v + 1;
        acc += cf[k] * 0.5 * (Lk[ra * P + cb] * Lk[rc * P + cd] - Lk[ra * P + cd] * Lk[rc * P + cb]) / dk;
      }
    }
    return acc;
  }
  const double ds = a.dd[2 * q + s];
  if (ds == 0.0) return 0.0;
  const double *Ls = a.L + ((size_t)q * 2 + s) * P2;
  return 0.5 * (Ls[ra * P + cb] * Ls[rc * P + cd] - Ls[ra * P + cd] * Ls[rc * P + cb]) / ds;
}

/* the core block: G = S_DD^-1, Y = G S_DC, det S_DD, then M, U and P0 */
__global__ void __launch_bounds__(1024) core_factor_kernel(CoreArgs a) {
  __shared__ double red[32];
  __shared__ int redi[32];
  __shared__ double sdet, samax;
  __shared__ int spiv, sbad;
  const int nD = a.nD, nC = a.nC, nsp = a.nsp, ld = 2 * nD + nC;
  const int tid = threadIdx.x, nt = blockDim.x;
  double *W = a.fw;
  double mx = 0.0;
  for (long long t = tid; t < (long long)nD * ld; t += nt) {
    const int r = (int)(t / ld), c = (int)(t - (long long)r * ld);
    double v;
    if (c < nD) {
      v = a.So[(size_t)(nC + r) * nsp + nC + c];
      mx = fmax(mx, fabs(v));
    } else if (c < nD + nC) {
      v = a.So[(size_t)(nC + r) * nsp + (c - nD)];
    } else {
      v = (c - nD - nC == r) ? 1.0 : 0.0;
    }
    W[t] = v;
  }
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(FULL, mx, o));
  if ((tid & 31) == 0) red[tid >> 5] = mx;
  __syncthreads();
  if (tid == 0) {
    double m = 0.0;
    for (int w = 0; w < (nt >> 5); ++w) m = fmax(m, red[w]);
    samax = m;
    sdet = 1.0;
    sbad = 0;
  }
  __syncthreads();
  for (int k = 0; k < nD; ++k) {
    double best = -1.0;
    int bi = k;
    for (int i = k + tid; i < nD; i += nt) {
      const double v = fabs(W[(size_t)i * ld + k]);
      if (v > best) {
        best = v;
        bi = i;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double ob = __shfl_xor_sync(FULL, best, o);
      const int oi = __shfl_xor_sync(FULL, bi, o);
      if (ob > best || (ob == best && oi < bi)) {
        best = ob;
        bi = oi;
      }
    }
    if ((tid & 31) == 0) {
      red[tid >> 5] = best;
      redi[tid >> 5] = bi;
    }
    __syncthreads();
    if (tid == 0) {
      double b = -1.0;
      int p = k;
      for (int w = 0; w < (nt >> 5); ++w)
        if (red[w] > b || (red[w] == b && redi[w] < p)) {
          b = red[w];
          p = redi[w];
        }
      spiv = p;
      if (!(b > 1e-13 * samax)) sbad = 1;
      const double pv = W[(size_t)p * ld + k];
      sdet *= p != k ? -pv : pv;
    }
    __syncthreads();
    if (sbad) break;
    const int p = spiv;
    if (p != k)
      for (int c = tid; c < ld; c += nt) {
        const double t = W[(size_t)k * ld + c];
        W[(size_t)k * ld + c] = W[(size_t)p * ld + c];
        W[(size_t)p * ld + c] = t;
      }
    __syncthreads();
    const double piv = W[(size_t)k * ld + k];
    __syncthreads();
    for (int c = k + 1 + tid; c < ld; c += nt) W[(size_t)k * ld + c] /= piv;
    __syncthreads();
    const int w = ld - k - 1;
    for (long long t = tid; t < (long long)nD * w; t += nt) {
      const int i = (int)(t / w), c = k + 1 + (int)(t - (long long)i * w);
      if (i != k) W[(size_t)i * ld + c] -= W[(size_t)i * ld + k] * W[(size_t)k * ld + c];
    }
    __syncthreads();
  }
  if (sbad) {
    if (tid == 0) {
      atomicOr(a.status, 8);
      *a.s0 = 0.0;
    }
    return;
  }
  if (tid == 0) *a.s0 = sdet;
  for (int t = tid; t < nD * nD; t += nt) {
    const int r = t / nD, c = t - r * nD;
    a.G[t] = W[(size_t)r * ld + nD + nC + c];
  }
  for (int t = tid; t < nD * nC; t += nt) {
    const int r = t / nC, c = t - r * nC;
    a.Y[t] = W[(size_t)r * ld + nD + c];
  }
  __syncthreads();
  for (int t = tid; t < nC * nC; t += nt) {
    const int x = t / nC, y = t - x * nC;
    double v = a.So[(size_t)x * nsp + y];
    for (int r = 0; r < nD; ++r) v -= a.So[(size_t)x * nsp + nC + r] * a.Y[r * nC + y];
    a.M[t] = v;
  }
  for (int t = tid; t < nsp * nC; t += nt) {
    const int i = t / nC, c = t - i * nC;
    a.U[t] = i < nC ? (i == c ? 1.0 : 0.0) : -a.Y[(i - nC) * nC + c];
  }
  for (int t = tid; t < nsp * nsp; t += nt) {
    const int i = t / nsp, j = t - i * nsp;
    a.P0[t] = (i >= nC && j >= nC) ? a.G[(i - nC) * nD + (j - nC)] : 0.0;
  }
}

/* one warp per determinant pair: per spin the P x P block of M, its
 * determinant (times det S_DD) and first cofactors; flagged blocks through
 * three perturbed factorisations kept in the pool */
__global__ void __launch_bounds__(256) core_pairs_kernel(CoreArgs a) {
  __shared__ double Wsh[8][16 * WLD];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long q = (long long)blockIdx.x * 8 + warp;
  if (q >= a.nq) return;
  const int P = a.P, P2 = P * P, nC = a.nC;
  const int m = (1 << P) - 1;
  const int kb = (int)(q & m), bb = (int)((q >> P) & m);
  const long long sp = q >> (2 * P);
  const int isc = (int)(sp / a.nsc), jsc = (int)(sp % a.nsc);
  const unsigned char *ob = a.detorb + (size_t)((isc << P) | bb) * 2 * P;
  const unsigned char *ok = a.detorb + (size_t)((jsc << P) | kb) * 2 * P;
  double *W = Wsh[warp];
  const double s0 = *a.s0;
  int slot = -1, flags = 0;
  for (int s = 0; s < 2; ++s) {
    const unsigned char *ro = ob + s * P, *co = ok + s * P;
    /* W = [M_s + kp Pert | I]; returns the largest |M_s| entry */
    auto fill = [&](double kp) -> double {
      double mx = 0.0;
      if (lane < 2 * P)
        for (int r = 0; r < P; ++r) {
          double v;
          if (lane < P) {
            v = a.M[ro[r] * nC + co[lane]];
            mx = fmax(mx, fabs(v));
            if (kp != 0.0) v += pert_entry(r, lane, kp);
          } else {
            v = (lane - P == r) ? 1.0 : 0.0;
          }
          W[r * WLD + lane] = v;
        }
      for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(FULL, mx, o));
      __syncwarp();
      return mx;
    };
    double *Lq = a.L + ((size_t)q * 2 + s) * P2;
    /* the Schur complement of normalised orbitals has entries of at most 1:
     * pivot floor and perturbation on that scale, so that the near-zero
     * block of an orbital far from the rest is flagged and perturbed */
    const double scl = fmax(fill(0.0), 1.0);
    bool good;
    const double det = warp_gj(W, P, lane, 1e-7 * scl, good);
    if (good) {
      const double d = s0 * det;
      for (int t = lane; t < P2; t += 32) {
        const int r = t / P, c = t - r * P;
        Lq[t] = d * W[c * WLD + P + r];
      }
      if (lane == 0) a.dd[2 * q + s] = d;
      __syncwarp();
      continue;
    }
    if (slot < 0) {
      int sl = 0;
      if (lane == 0) sl = atomicAdd(a.pcount, 1);
      slot = __shfl_sync(FULL, sl, 0);
    }
    flags |= 1 << s;
    const bool room = slot < a.cap;
    if (!room && lane == 0) atomicOr(a.status, 4);
    const double scale = 0.1 * scl / sqrt((double)P);
    const double cf[3] = {3.0, -3.0, 1.0};
    double lacc[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) lacc[j] = 0.0;
    double dsum = 0.0;
    bool zero = false;
    for (int k = 1; k <= 3 && !zero; ++k) {
      fill(k * scale);
      bool g2;
      const double det2 = warp_gj(W, P, lane, 1e-7 * scl, g2);
      if (!g2) {
        zero = true;
        break;
      }
      const double d = s0 * det2;
      double *e = room ? a.pool + ((size_t)slot * 6 + (size_t)(2 * (k - 1) + s)) * (1 + P2) : nullptr;
      if (e && lane == 0) e[0] = d;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int t = lane + 32 * j;
        if (t < P2) {
          const int r = t / P, c = t - r * P;
          const double v = d * W[c * WLD + P + r];
          if (e) e[1 + t] = v;
          lacc[j] += cf[k - 1] * v;
        }
      }
      dsum += cf[k - 1] * d;
      __syncwarp();
    }
    if (zero) {
      /* rank deficiency of 3 or more: every cofactor with at most two
       * strikes vanishes */
      dsum = 0.0;
#pragma unroll
      for (int j = 0; j < 8; ++j) lacc[j] = 0.0;
      if (room && lane < 3) a.pool[((size_t)slot * 6 + (size_t)(2 * lane + s)) * (1 + P2)] = 0.0;
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int t = lane + 32 * j;
      if (t < P2) Lq[t] = lacc[j];
    }
    if (lane == 0) a.dd[2 * q + s] = dsum;
    __syncwarp();
  }
  if (lane == 0) {
    a.pslot[q] = (slot >= 0 && slot < a.cap) ? slot * 4 + flags : -1;
    const double w = a.csc[isc] * a.csc[jsc], d0 = a.dd[2 * q], d1 = a.dd[2 * q + 1];
    a.qf[2 * q] = d0 != 0.0 ? 0.5 * w * d1 / d0 : 0.0;
    a.qf[2 * q + 1] = d1 != 0.0 ? 0.5 * w * d0 / d1 : 0.0;
  }
}

/* A0 = sum_q w d_a d_b, fixed order; the flagged pair count */
__global__ void __launch_bounds__(1024) core_a0_kernel(CoreArgs a) {
  __shared__ double red[32];
  const int P = a.P;
  double s = 0.0;
  for (long long q = threadIdx.x; q < a.nq; q += blockDim.x) {
    const long long sp = q >> (2 * P);
    const int isc = (int)(sp / a.nsc), jsc = (int)(sp % a.nsc);
    s += a.csc[isc] * a.csc[jsc] * a.dd[2 * q] * a.dd[2 * q + 1];
  }
  s = block_sum(s, red);
  if (threadIdx.x == 0) {
    *a.A0 = s;
    *a.nsing = *a.pcount;
  }
}

/* A1[a][b] = sum_q w (d_b L_a + d_a L_b)[a][b]: one warp per (a, b) over
 * the determinant pairs holding a and b in the same spin */
__global__ void __launch_bounds__(256) core_a1_kernel(CoreArgs a) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int e = blockIdx.x * 8 + warp, nC = a.nC, P = a.P;
  if (e >= nC * nC) return;
  const int x = e / nC, y = e - x * nC;
  double acc = 0.0;
  for (int s = 0; s < 2; ++s) {
    const int *Bl = a.lst1 + a.off1[2 * x + s], *Kl = a.lst1 + a.off1[2 * y + s];
    const int nb = a.off1[2 * x + s + 1] - a.off1[2 * x + s], nk = a.off1[2 * y + s + 1] - a.off1[2 * y + s];
    for (int ib = 0; ib < nb; ++ib) {
      const int bd = Bl[ib];
      const int ra = a.detpos[(size_t)bd * nC + x] & 31;
      for (int ik = lane; ik < nk; ik += 32) {
        const int kd = Kl[ik];
        const long long q = pair_of(a, bd, kd);
        const int cb = a.detpos[(size_t)kd * nC + y] & 31;
        acc += weight_of(a, bd, kd) * a.dd[2 * q + 1 - s] * a.L[((size_t)q * 2 + s) * P * P + ra * P + cb];
      }
    }
  }
  acc = warp_sum(acc);
  if (lane == 0) a.A1[e] = acc;
}

/* A2[abcd]: one warp per entry over the determinant pairs holding a, c in
 * the bra and b, d in the ket with the spins of each term */
__global__ void __launch_bounds__(256) core_a2_kernel(CoreArgs a) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nC = a.nC, P = a.P, P2 = P * P;
  const long long e = (long long)blockIdx.x * 8 + warp;
  if (e >= (long long)nC * nC * nC * nC) return;
  const int d4 = (int)(e % nC), c4 = (int)((e / nC) % nC), b4 = (int)((e / nC / nC) % nC), a4 = (int)(e / nC / nC / nC);
  double acc = 0.0;
  /* g = 2 spin(a) + spin(c) on the bra, 2 spin(b) + spin(d) on the ket */
  for (int g = 0; g < 4; ++g) {
    const bool same = g == 0 || g == 3;
    if (same && (a4 == c4 || b4 == d4)) continue;
    const int ib = 4 * (a4 * nC + c4) + g, ik = 4 * (b4 * nC + d4) + g;
    const int *Bl = a.lst2 + a.off2[ib], *Kl = a.lst2 + a.off2[ik];
    const int nb = a.off2[ib + 1] - a.off2[ib], nk = a.off2[ik + 1] - a.off2[ik];
    for (int jb = 0; jb < nb; ++jb) {
      const int bd = Bl[jb];
      const int ra = a.detpos[(size_t)bd * nC + a4] & 31, rc = a.detpos[(size_t)bd * nC + c4] & 31;
      for (int jk = lane; jk < nk; jk += 32) {
        const int kd = Kl[jk];
        const long long q = pair_of(a, bd, kd);
        const double w = weight_of(a, bd, kd);
        const int cb = a.detpos[(size_t)kd * nC + b4] & 31, cd = a.detpos[(size_t)kd * nC + d4] & 31;
        if (same) {
          const int s = g == 0 ? 0 : 1;
          const int ps = a.pslot[q];
          if (ps >= 0 && ((ps >> s) & 1)) {
            acc += w * a.dd[2 * q + 1 - s] * second_cof(a, q, s, ra, rc, cb, cd);
          } else {
            const double *Ls = a.L + ((size_t)q * 2 + s) * P2;
            acc += a.qf[2 * q + s] * (Ls[ra * P + cb] * Ls[rc * P + cd] - Ls[ra * P + cd] * Ls[rc * P + cb]);
          }
        } else {
          /* g = 1: a, b alpha and c, d beta; g = 2: the reverse */
          const int s1 = g == 1 ? 0 : 1;
          const double *L1 = a.L + ((size_t)q * 2 + s1) * P2, *L2 = a.L + ((size_t)q * 2 + 1 - s1) * P2;
          acc += 0.5 * w * L1[ra * P + cb] * L2[rc * P + cd];
        }
      }
    }
  }
  acc = warp_sum(acc);
  if (lane == 0) a.A2[e] = acc;
}

/* A2x: A2 summed over the orderings of each coupled-orbital pair, with the
 * 2 x 2 block [[2 A0, 1], [1, 0]] of the core's direct terms appended */
__global__ void core_a2x_kernel(CoreArgs a) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int kx = a.kx, ncp = a.ncp, nC = a.nC;
  if (t >= kx * kx) return;
  const int u = t / kx, v = t - u * kx;
  double r = 0.0;
  if (u < ncp && v < ncp) {
    int x, y, z, w;
    unpair(u, x, y);
    unpair(v, z, w);
    for (int o1 = 0; o1 < (x != y ? 2 : 1); ++o1)
      for (int o2 = 0; o2 < (z != w ? 2 : 1); ++o2) {
        const int i = o1 ? y : x, k = o1 ? x : y, j = o2 ? w : z, l = o2 ? z : w;
        r += a.A2[(((size_t)i * nC + k) * nC + j) * nC + l];
      }
  } else if (u == ncp && v == ncp) {
    r = 2.0 * *a.A0;
  } else if ((u == ncp && v == ncp + 1) || (u == ncp + 1 && v == ncp)) {
    r = 1.0;
  }
  a.A2x[t] = r;
}

/* R1 = U A1 U^T */
__global__ void core_r1_kernel(CoreArgs a) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = a.nsp, nC = a.nC;
  if (t >= n * n) return;
  const int i = t / n, j = t - i * n;
  double r = 0.0;
  for (int x = 0; x < nC; ++x) {
    const double ux = a.U[i * nC + x];
    if (ux == 0.0) continue;
    double s = 0.0;
    for (int y = 0; y < nC; ++y) s += a.A1[x * nC + y] * a.U[j * nC + y];
    r += ux * s;
  }
  a.R1[t] = r;
}

/* Wv[p][u]: orbital pair p = (i, k) against coupled-orbital pair u = (x, y),
 * summed over the orderings of p; the last two columns carry the core's
 * P0 and R1 over the orderings of p */
__global__ void core_wv_kernel(CoreArgs a) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int kx = a.kx, ncp = a.ncp, nC = a.nC, n = a.nsp;
  if (t >= (long long)a.np * kx) return;
  const int p = (int)(t / kx), u = (int)(t - (long long)p * kx);
  const int2 ik = a.pik[p];
  const int i = ik.x, k = ik.y;
  double r;
  if (u < ncp) {
    int x, y;
    unpair(u, x, y);
    r = a.U[i * nC + x] * a.U[k * nC + y];
    if (i != k) r += a.U[k * nC + x] * a.U[i * nC + y];
  } else {
    const double *Z = u == ncp ? a.P0 : a.R1;
    r = Z[i * n + k];
    if (i != k) r += Z[k * n + i];
  }
  a.Wv[t] = r;
}

/* X = Wv A2x */
__global__ void core_x_kernel(CoreArgs a) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int kx = a.kx;
  if (t >= (long long)a.np * kx) return;
  const int p = (int)(t / kx), v = (int)(t - (long long)p * kx);
  const double *w = a.Wv + (size_t)p * kx;
  double r = 0.0;
  for (int u = 0; u < kx; ++u) r += w[u] * a.A2x[u * kx + v];
  a.X[t] = r;
}

/* the core's exchange terms of Gamma over the orderings of (i, k) and (j, l) */
__device__ __forceinline__ double core_exch(const CoreArgs &a, double A0, int i, int k, int j, int l) {
  const int n = a.nsp;
  double s = 0.0;
  for (int o1 = 0; o1 < (i != k ? 2 : 1); ++o1)
    for (int o2 = 0; o2 < (j != l ? 2 : 1); ++o2) {
      const int i1 = o1 ? k : i, k1 = o1 ? i : k, j1 = o2 ? l : j, l1 = o2 ? j : l;
      const double pil = a.P0[i1 * n + l1], pjk = a.P0[j1 * n + k1];
      const double ril = a.R1[i1 * n + l1], rjk = a.R1[j1 * n + k1];
      s += -A0 * pil * pjk - 0.5 * (pil * rjk + ril * pjk);
    }
  return s;
}

constexpr int GT = 64, GK = 16;

/* the GEMMs' arithmetic AT: FP64, or double-float (48-bit, on the FP32
 * pipe, whose rate is 58x the FP64 rate here) for the mixed path */
template <typename AT>
__device__ __forceinline__ AT to_at(double v);
template <>
__device__ __forceinline__ double to_at<double>(double v) { return v; }
template <>
__device__ __forceinline__ df64 to_at<df64>(double v) { return df64_split(v); }
__device__ __forceinline__ void fmad(double &acc, double x, double y) { acc = fma(x, y, acc); }
__device__ __forceinline__ void fmad(df64 &acc, df64 x, df64 y) { acc += x * y; }
__device__ __forceinline__ double as_d(double v) { return v; }
__device__ __forceinline__ double as_d(df64 v) { return (double)v.hi + (double)v.lo; }

/* Gamma tile (I, J), I <= J, of X Wv^T plus the core's exchange terms:
 * contracted with the masked T tile (off-diagonal tiles count twice), or
 * with STORE written to Gam with its mirror tile */
template <bool STORE, typename AT>
__global__ void __launch_bounds__(256) core_gemm_kernel(CoreArgs a, double *Gam) {
  const int I = blockIdx.y, J = blockIdx.x;
  double *part = a.part + (size_t)I * a.ntile + J;
  if (I > J) {
    if (!STORE && threadIdx.x == 0) *part = 0.0;
    return;
  }
  __shared__ AT As[GK][GT + 1], Bs[GK][GT + 1];
  __shared__ double red[8];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int p0 = I * GT, q0 = J * GT, np = a.np, kx = a.kx;
  AT acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = to_at<AT>(0.0);
  for (int k0 = 0; k0 < kx; k0 += GK) {
    for (int e = tid; e < GT * GK; e += 256) {
      const int m = e / GK, kk = e - m * GK, k = k0 + kk;
      const int p = p0 + m, q = q0 + m;
      As[kk][m] = to_at<AT>((p < np && k < kx) ? a.X[(size_t)p * kx + k] : 0.0);
      Bs[kk][m] = to_at<AT>((q < np && k < kx) ? a.Wv[(size_t)q * kx + k] : 0.0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GK; ++kk) {
      AT av[4], bv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) av[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) bv[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) fmad(acc[i][j], av[i], bv[j]);
    }
    __syncthreads();
  }
  const double A0 = *a.A0, itol = a.itol;
  double e = 0.0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int p = p0 + ty + 16 * i;
    if (p >= np) continue;
    const int2 ik = a.pik[p];
    const double sp = STORE ? 0.0 : a.sq[p];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int q = q0 + tx + 16 * j;
      if (q >= np) continue;
      const int2 jl = a.pik[q];
      if (STORE) {
        const double gv = as_d(acc[i][j]) + core_exch(a, A0, ik.x, ik.y, jl.x, jl.y);
        Gam[(size_t)p * np + q] = gv;
        Gam[(size_t)q * np + p] = gv;
        continue;
      }
      const double t = a.T[(size_t)p * np + q];
      if (!(sp * a.sq[q] > itol && fabs(t) > itol)) continue;
      e += t * (as_d(acc[i][j]) + core_exch(a, A0, ik.x, ik.y, jl.x, jl.y));
    }
  }
  if (STORE) return;
  e = block_sum(e, red);
  if (tid == 0) *part = I == J ? e : 2.0 * e;
}

/* e2 partials from a stored Gamma: the masked T against it, one chunk of
 * the np x np elements per block */
__global__ void __launch_bounds__(256) core_e2_kernel(CoreArgs a, const double *Gam) {
  __shared__ double red[8];
  const long long n = (long long)a.np * a.np, nb = (long long)gridDim.x;
  const long long c0 = n * blockIdx.x / nb, c1 = n * (blockIdx.x + 1) / nb;
  double e = 0.0;
  for (long long t = c0 + threadIdx.x; t < c1; t += blockDim.x) {
    const int p = (int)(t / a.np), q = (int)(t - (long long)p * a.np);
    const double tv = a.T[t];
    if (a.sq[p] * a.sq[q] > a.itol && fabs(tv) > a.itol) e += tv * Gam[t];
  }
  e = block_sum(e, red);
  if (threadIdx.x == 0) a.part[blockIdx.x] = e;
}

/* e2 from the tiles, e1 and wfnorm from gamma = 2 A0 P0 + R1, the energy */
__global__ void __launch_bounds__(1024) core_result_kernel(CoreArgs a) {
  __shared__ double red[32];
  const int n = a.nsp;
  const double A0 = *a.A0;
  double e2 = 0.0, e1 = 0.0, wf = 0.0;
  for (int t = threadIdx.x; t < a.ntile * a.ntile; t += blockDim.x) e2 += a.part[t];
  for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
    const double g = 2.0 * A0 * a.P0[t] + a.R1[t];
    e1 += a.Ho[t] * g;
    wf += a.So[t] * g;
  }
  e2 = block_sum(e2, red);
  e1 = block_sum(e1, red);
  wf = block_sum(wf, red);
  if (threadIdx.x == 0) {
    const double w = wf / (double)a.nelec;
    a.out[0] = (e1 + e2) / w + a.enuc;
    a.out[1] = e1 + e2;
    a.out[2] = e1;
    a.out[3] = e2;
    a.out[4] = w;
  }
}


/* ---- adjoint ----
 * With W = wfnorm, e_num = e1 + e2 and E = e_num / W + E_nuc:
 *   dE/dh = gamma / W,  dE/dGamma = T_masked / W,
 *   dE/dgamma = h / W - e_num S / (nelec W^2) =: Hb,
 *   explicit dE/dS = -e_num gamma / (nelec W^2).
 * Through Gamma_pair = Wv A2x Wv^T + (core exchange terms) and gamma:
 *   Yg = (T_masked / W) Wv,  A2x-bar = Wv^T Yg,  Wv-bar = 2 Yg A2x,
 *   R1-bar = Hb + Wv-bar[., r1] - KP,
 *   P0-bar = 2 A0 Hb + Wv-bar[., v0] - 2 A0 KP - KR,
 *   A0-bar = 2 <Hb, P0> + 2 A2x-bar[v0][v0] - <KP, P0>,
 * with the exchange builds KP, KR of T_masked / W (KX[j][k] = sum_il
 * T[(ik)][(jl)] X[i][l]); A1-bar = U^T R1-bar U; U-bar from Wv-bar and R1;
 * per pair the derivative of its share of <A-bar, A> with respect to its
 * blocks M_s (closed forms in M_s^-1; flagged blocks extrapolated over the
 * three perturbed factorisations like the forward values); then
 *   dE/dS = U M-bar U^T - P0 P0-bar P0 - P0 U-bar U^T + 2 Lambda P0 + explicit,
 * from dM = U^T dS U, dU = -P0 dS U, dP0 = -P0 dS P0, d det S_DD = det S_DD
 * <P0, dS> and every pair sum being proportional to (det S_DD)^2. */

__device__ __forceinline__ int opair(int i, int k) { return i >= k ? i * (i + 1) / 2 + k : k * (k + 1) / 2 + i; }

__device__ __forceinline__ double masked_t(const CoreArgs &a, int p, int q) {
  const double t = a.T[(size_t)p * a.np + q];
  return (a.sq[p] * a.sq[q] > a.itol && fabs(t) > a.itol) ? t : 0.0;
}

/* Yg = (T_masked / W) Wv: tiles of 64 orbital pairs x 64 columns */
template <typename AT>
__global__ void __launch_bounds__(256) core_ygemm_kernel(CoreArgs a, CoreGrad g) {
  __shared__ AT As[GK][GT + 1], Bs[GK][GT + 1];
  const int vt = blockIdx.x, I = blockIdx.y;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int p0 = I * GT, v0 = vt * GT, np = a.np, kx = a.kx;
  AT acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = to_at<AT>(0.0);
  for (int q0 = 0; q0 < np; q0 += GK) {
    for (int e = tid; e < GT * GK; e += 256) {
      const int m = e / GK, kk = e - m * GK;
      const int p = p0 + m, q = q0 + kk;
      As[kk][m] = to_at<AT>((p < np && q < np) ? masked_t(a, p, q) : 0.0);
    }
    for (int e = tid; e < GK * GT; e += 256) {
      const int kk = e / GT, n = e - kk * GT;
      const int q = q0 + kk, v = v0 + n;
      Bs[kk][n] = to_at<AT>((q < np && v < kx) ? a.Wv[(size_t)q * kx + v] : 0.0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GK; ++kk) {
      AT av[4], bv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) av[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) bv[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) fmad(acc[i][j], av[i], bv[j]);
    }
    __syncthreads();
  }
  const double iw = 1.0 / a.out[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int p = p0 + ty + 16 * i;
    if (p >= np) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int v = v0 + tx + 16 * j;
      if (v < kx) g.Yg[(size_t)p * kx + v] = as_d(acc[i][j]) * iw;
    }
  }
}

/* partial Wv^T Yg over a chunk of orbital pairs: block (u, chunk), threads over v */
__global__ void core_axp_kernel(CoreArgs a, CoreGrad g) {
  const int u = blockIdx.x, ch = blockIdx.y, kx = a.kx, np = a.np;
  const int pa = (int)((long long)np * ch / g.nchunk), pb = (int)((long long)np * (ch + 1) / g.nchunk);
  for (int v = threadIdx.x; v < kx; v += blockDim.x) {
    double s = 0.0;
    for (int p = pa; p < pb; ++p) s += a.Wv[(size_t)p * kx + u] * g.Yg[(size_t)p * kx + v];
    g.Axp[((size_t)ch * kx + u) * kx + v] = s;
  }
}

__global__ void core_axr_kernel(CoreArgs a, CoreGrad g) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x, kx = a.kx;
  if (t >= kx * kx) return;
  double s = 0.0;
  for (int c = 0; c < g.nchunk; ++c) s += g.Axp[(size_t)c * kx * kx + t];
  g.Ax[t] = s;
}

/* out = scale * in M over rows of kx columns (M kx x kx) */
__global__ void core_rowmat_kernel(const double *in, const double *M, double *out, int rows, int kx, double scale) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)rows * kx) return;
  const int p = (int)(t / kx), v = (int)(t - (long long)p * kx);
  const double *w = in + (size_t)p * kx;
  double r = 0.0;
  for (int u = 0; u < kx; ++u) r += w[u] * M[u * kx + v];
  out[t] = scale * r;
}

/* KP[j][k], KR[j][k] = sum_il (T_masked / W)[(ik)][(jl)] {P0, R1}[i][l]: one block per (j, k) */
__global__ void __launch_bounds__(256) core_kbuild_kernel(CoreArgs a, CoreGrad g) {
  __shared__ double red[8];
  const int n = a.nsp, j = blockIdx.x / n, k = blockIdx.x - j * n;
  double s1 = 0.0, s2 = 0.0;
  for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
    const int i = t / n, l = t - i * n;
    const double tv = masked_t(a, opair(i, k), opair(j, l));
    if (tv != 0.0) {
      s1 += tv * a.P0[t];
      s2 += tv * a.R1[t];
    }
  }
  s1 = block_sum(s1, red);
  s2 = block_sum(s2, red);
  if (threadIdx.x == 0) {
    const double iw = 1.0 / a.out[4];
    g.KP[blockIdx.x] = s1 * iw;
    g.KR[blockIdx.x] = s2 * iw;
  }
}

/* R1-bar and P0-bar, elementwise */
__global__ void core_bar_kernel(CoreArgs a, CoreGrad g) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x, n = a.nsp;
  if (t >= n * n) return;
  const int i = t / n, k = t - i * n;
  const double W = a.out[4], en = a.out[1], A0 = *a.A0;
  const double hb = a.Ho[t] / W - en / (W * W) * a.So[t] / a.nelec;
  const double *wb = g.Wvb + (size_t)opair(i, k) * a.kx;
  g.R1b[t] = hb + wb[a.ncp + 1] - g.KP[t];
  g.P0b[t] = 2.0 * A0 * hb + wb[a.ncp] - 2.0 * A0 * g.KP[t] - g.KR[t];
}

/* A0-bar */
__global__ void __launch_bounds__(1024) core_bar0_kernel(CoreArgs a, CoreGrad g) {
  __shared__ double red[32];
  const int n = a.nsp;
  const double W = a.out[4], en = a.out[1];
  double s = 0.0;
  for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
    const double hb = a.Ho[t] / W - en / (W * W) * a.So[t] / a.nelec;
    s += (2.0 * hb - g.KP[t]) * a.P0[t];
  }
  s = block_sum(s, red);
  if (threadIdx.x == 0) g.sc[0] = s + 2.0 * g.Ax[(size_t)a.ncp * a.kx + a.ncp];
}

/* A1-bar = U^T R1-bar U: one block per entry */
__global__ void __launch_bounds__(256) core_a1b_kernel(CoreArgs a, CoreGrad g) {
  __shared__ double red[8];
  const int nC = a.nC, n = a.nsp, x = blockIdx.x / nC, y = blockIdx.x - x * nC;
  double s = 0.0;
  for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
    const int i = t / n, k = t - i * n;
    s += a.U[i * nC + x] * g.R1b[t] * a.U[k * nC + y];
  }
  s = block_sum(s, red);
  if (threadIdx.x == 0) g.A1b[blockIdx.x] = s;
}

/* A2-bar[abcd] from the coupled-pair layout of A2x-bar */
__device__ __forceinline__ double a2bar(const CoreArgs &a, const CoreGrad &g, int x, int y, int z, int w) {
  return g.Ax[(size_t)opair(x, y) * a.kx + opair(z, w)];
}

/* one warp per determinant pair: dE/dM_s of its share of <A-bar, A> per
 * spin block, and the share itself */
__global__ void __launch_bounds__(256) core_pair_adj_kernel(CoreArgs a, CoreGrad g) {
  extern __shared__ double sm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long q = (long long)blockIdx.x * 8 + warp;
  if (q >= a.nq) return;
  const int P = a.P, P2 = P * P, nC = a.nC;
  const int m = (1 << P) - 1;
  const int kb = (int)(q & m), bb = (int)((q >> P) & m);
  const long long spp = q >> (2 * P);
  const int isc = (int)(spp / a.nsc), jsc = (int)(spp % a.nsc);
  const unsigned char *obr = a.detorb + (size_t)((isc << P) | bb) * 2 * P;
  const unsigned char *okr = a.detorb + (size_t)((jsc << P) | kb) * 2 * P;
  const double w = a.csc[isc] * a.csc[jsc];
  double *Zs = sm + (size_t)warp * 5 * P2, *Ph = Zs + P2, *Om = Ph + P2, *PZ = Om + P2, *Bs = PZ + P2;
  const double A0b = g.sc[0];
  const double d2[2] = {a.dd[2 * q], a.dd[2 * q + 1]};
  const double *L2[2] = {a.L + (size_t)q * 2 * P2, a.L + ((size_t)q * 2 + 1) * P2};
  /* f_s = <A1-bar, L_s> + <A2-bar, Q_s> */
  double f[2];
  for (int s = 0; s < 2; ++s) {
    const unsigned char *ob = obr + s * P, *ok = okr + s * P;
    double acc = 0.0;
    for (int t = lane; t < P2; t += 32) {
      const int r = t / P, c = t - r * P;
      acc += g.A1b[ob[r] * nC + ok[c]] * L2[s][t];
    }
    /* <A2-bar, Q_s>: per factorisation sum Psi (L L - L L), then / (2 d) */
    const int ps0 = a.pslot[q];
    const bool fl = ps0 >= 0 && ((ps0 >> s) & 1);
    for (int k = 0; k < (fl ? 3 : 1); ++k) {
      double dk;
      const double *Lk;
      if (fl) {
        const double *e = a.pool + ((size_t)(ps0 >> 2) * 6 + (size_t)(2 * k + s)) * (1 + P2);
        dk = e[0];
        Lk = e + 1;
      } else {
        dk = d2[s];
        Lk = L2[s];
      }
      if (dk == 0.0) continue;
      double hs = 0.0;
      for (int t = lane; t < P2 * P2; t += 32) {
        const int r1 = t / (P * P2), c1 = (t / P2) % P, r2 = (t / P) % P, c2 = t % P;
        if (r1 == r2 || c1 == c2) continue;
        hs += a2bar(a, g, ob[r1], ok[c1], ob[r2], ok[c2]) *
              (Lk[r1 * P + c1] * Lk[r2 * P + c2] - Lk[r1 * P + c2] * Lk[r2 * P + c1]);
      }
      acc += (fl ? (k == 0 ? 3.0 : (k == 1 ? -3.0 : 1.0)) : 1.0) * 0.5 * hs / dk;
    }
    f[s] = warp_sum(acc);
  }
  double cross = 0.0;
  const int ps = a.pslot[q];
  for (int s = 0; s < 2; ++s) {
    const unsigned char *ob = obr + s * P, *ok = okr + s * P;
    const unsigned char *ob0 = obr, *ok0 = okr, *ob1 = obr + P, *ok1 = okr + P;
    const double dso = d2[1 - s];
    const double *Lo = L2[1 - s];
    /* B_s = the cross term's weight of L_s; Phi' = d_other A1-bar_s + B_s */
    for (int t = lane; t < P2; t += 32) {
      const int r = t / P, c = t - r * P;
      double b = 0.0;
      for (int u = 0; u < P2; ++u) {
        const int r2 = u / P, c2 = u - r2 * P;
        const double xi = s == 0 ? a2bar(a, g, ob0[r], ok0[c], ob1[r2], ok1[c2])
                                 : a2bar(a, g, ob0[r2], ok0[c2], ob1[r], ok1[c]);
        b += xi * Lo[u];
      }
      Bs[t] = b;
      Ph[t] = dso * g.A1b[ob[r] * nC + ok[c]] + b;
    }
    __syncwarp();
    if (s == 0) {
      double cc = 0.0;
      for (int t = lane; t < P2; t += 32) cc += Bs[t] * L2[0][t];
      cross = warp_sum(cc);
    }
    const double aco = A0b * dso + f[1 - s];
    const bool flagged = ps >= 0 && ((ps >> s) & 1);
    const int nver = flagged ? 3 : 1;
    double macc[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) macc[j] = 0.0;
    for (int k = 0; k < nver; ++k) {
      const double cf = flagged ? (k == 0 ? 3.0 : (k == 1 ? -3.0 : 1.0)) : 1.0;
      double dk;
      const double *Lk;
      if (flagged) {
        const double *e = a.pool + ((size_t)(ps >> 2) * 6 + (size_t)(2 * k + s)) * (1 + P2);
        dk = e[0];
        Lk = e + 1;
      } else {
        dk = d2[s];
        Lk = L2[s];
      }
      if (dk == 0.0) {
        /* rank deficiency of 3 or more: third cofactors need not vanish */
        if (lane == 0 && (flagged || d2[s] == 0.0)) atomicOr(a.status, 2);
        continue;
      }
      const double idk = 1.0 / dk;
      for (int t = lane; t < P2; t += 32) {
        const int r = t / P, c = t - r * P;
        Zs[c * P + r] = Lk[t] * idk;
      }
      __syncwarp();
      /* Omega[r1][c1] = 2 sum Z[c2][r2] (Psi[r1 c1 r2 c2] - Psi[r1 c2 r2 c1]) */
      double tp = 0.0, hz = 0.0;
      for (int t = lane; t < P2; t += 32) {
        const int r1 = t / P, c1 = t - r1 * P;
        double o = 0.0;
        for (int u = 0; u < P2; ++u) {
          const int r2 = u / P, c2 = u - r2 * P;
          if (r2 == r1) continue;
          o += Zs[c2 * P + r2] *
               (a2bar(a, g, ob[r1], ok[c1], ob[r2], ok[c2]) - a2bar(a, g, ob[r1], ok[c2], ob[r2], ok[c1]));
        }
        Om[t] = 2.0 * o;
        tp += Ph[t] * Zs[c1 * P + r1];
        hz += Zs[c1 * P + r1] * 2.0 * o;
      }
      tp = warp_sum(tp);
      const double h = 0.25 * dk * warp_sum(hz);
      __syncwarp();
      /* PZ = Phi' Z and Bs = Omega Z (B_s no longer needed) */
      double pz[8], oz[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int t = lane + 32 * j;
        pz[j] = oz[j] = 0.0;
        if (t < P2) {
          const int x = t / P, r = t - x * P;
          for (int y = 0; y < P; ++y) {
            pz[j] += Ph[x * P + y] * Zs[y * P + r];
            oz[j] += Om[x * P + y] * Zs[y * P + r];
          }
        }
      }
      __syncwarp();
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int t = lane + 32 * j;
        if (t < P2) {
          PZ[t] = pz[j];
          Bs[t] = oz[j];
        }
      }
      __syncwarp();
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int t = lane + 32 * j;
        if (t < P2) {
          const int r = t / P, c = t - r * P;
          double zpz = 0.0, zoz = 0.0;
          for (int x = 0; x < P; ++x) {
            zpz += Zs[c * P + x] * PZ[x * P + r];
            zoz += Zs[c * P + x] * Bs[x * P + r];
          }
          const double zt = Zs[c * P + r];
          macc[j] += cf * w * (aco * dk * zt + dk * (tp * zt - zpz) + dso * (h * zt - 0.5 * dk * zoz));
        }
      }
      __syncwarp();
    }
    double *Mo = g.Mbp + ((size_t)q * 2 + s) * P2;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int t = lane + 32 * j;
      if (t < P2) Mo[t] = macc[j];
    }
    __syncwarp();
  }
  if (lane == 0) g.lam[q] = w * (A0b * d2[0] * d2[1] + d2[1] * f[0] + d2[0] * f[1] + cross);
}

/* M-bar[a][b] = sum over the pairs holding a, b in one spin: one warp per entry */
__global__ void __launch_bounds__(256) core_mbar_kernel(CoreArgs a, CoreGrad g) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int e = blockIdx.x * 8 + warp, nC = a.nC, P = a.P;
  if (e >= nC * nC) return;
  const int x = e / nC, y = e - x * nC;
  double acc = 0.0;
  for (int s = 0; s < 2; ++s) {
    const int *Bl = a.lst1 + a.off1[2 * x + s], *Kl = a.lst1 + a.off1[2 * y + s];
    const int nb = a.off1[2 * x + s + 1] - a.off1[2 * x + s], nk = a.off1[2 * y + s + 1] - a.off1[2 * y + s];
    for (int ib = 0; ib < nb; ++ib) {
      const int bd = Bl[ib];
      const int ra = a.detpos[(size_t)bd * nC + x] & 31;
      for (int ik = lane; ik < nk; ik += 32) {
        const int kd = Kl[ik];
        const long long q = pair_of(a, bd, kd);
        const int cb = a.detpos[(size_t)kd * nC + y] & 31;
        acc += g.Mbp[((size_t)q * 2 + s) * P * P + ra * P + cb];
      }
    }
  }
  acc = warp_sum(acc);
  if (lane == 0) g.Mb[e] = acc;
}

/* Lambda = sum_q of the pairs' shares, fixed order */
__global__ void __launch_bounds__(1024) core_lam_kernel(CoreArgs a, CoreGrad g) {
  __shared__ double red[32];
  double s = 0.0;
  for (long long q = threadIdx.x; q < a.nq; q += blockDim.x) s += g.lam[q];
  s = block_sum(s, red);
  if (threadIdx.x == 0) g.sc[1] = s;
}

/* U-bar[m][c] = sum_n sum_z Wv-bar[(mn)][(cz)] U[n][z] (2 when z = c)
 *             + (R1-bar U A1^T + R1-bar^T U A1)[m][c] */
__global__ void core_ub_kernel(CoreArgs a, CoreGrad g) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x, nC = a.nC, n = a.nsp, kx = a.kx;
  if (t >= n * nC) return;
  const int mm = t / nC, c = t - mm * nC;
  double s = 0.0;
  for (int nn = 0; nn < n; ++nn) {
    const double *wb = g.Wvb + (size_t)opair(mm, nn) * kx;
    const double r1 = g.R1b[mm * n + nn], r2 = g.R1b[nn * n + mm];
    for (int z = 0; z < nC; ++z) {
      const double u = a.U[nn * nC + z];
      if (u == 0.0) continue;
      s += wb[opair(c, z)] * u * (z == c ? 2.0 : 1.0) + (r1 * a.A1[c * nC + z] + r2 * a.A1[z * nC + c]) * u;
    }
  }
  g.Ub[t] = s;
}

/* C = beta C + alpha op(A) op(B), m x n with inner dimension kk */
__global__ void core_mm_kernel(const double *A, int lda, int ta, const double *B, int ldb, int tb, double *C, int ldc,
                               int mr, int nc, int kk, double alpha, double beta) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= mr * nc) return;
  const int i = t / nc, j = t - i * nc;
  double s = 0.0;
  for (int k = 0; k < kk; ++k) s += (ta ? A[k * lda + i] : A[i * lda + k]) * (tb ? B[j * ldb + k] : B[k * ldb + j]);
  C[i * ldc + j] = (beta != 0.0 ? beta * C[i * ldc + j] : 0.0) + alpha * s;
}

/* dE/dS += 2 Lambda P0 - e_num gamma / (nelec W^2); dE/dh = gamma / W */
__global__ void core_sbar_final_kernel(CoreArgs a, CoreGrad g) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x, n = a.nsp;
  if (t >= n * n) return;
  const double W = a.out[4], en = a.out[1];
  const double gam = 2.0 * *a.A0 * a.P0[t] + a.R1[t];
  g.Sbar[t] += 2.0 * g.sc[1] * a.P0[t] - en / (W * W) * gam / a.nelec;
  g.Hbar[t] = gam / W;
}

unsigned nblk(long long n, int b) { return (unsigned)((n + b - 1) / b); }

}  // namespace

int core_pre(const CoreArgs &a, cudaStream_t st) {
  if (cudaMemsetAsync(a.pcount, 0, sizeof(int), st) != cudaSuccess) return -1;
  core_factor_kernel<<<1, 1024, 0, st>>>(a);
  core_pairs_kernel<<<nblk(a.nq, 8), 256, 0, st>>>(a);
  core_a0_kernel<<<1, 1024, 0, st>>>(a);
  core_a1_kernel<<<nblk((long long)a.nC * a.nC, 8), 256, 0, st>>>(a);
  core_a2_kernel<<<nblk((long long)a.nC * a.nC * a.nC * a.nC, 8), 256, 0, st>>>(a);
  core_a2x_kernel<<<nblk((long long)a.kx * a.kx, 256), 256, 0, st>>>(a);
  core_r1_kernel<<<nblk((long long)a.nsp * a.nsp, 256), 256, 0, st>>>(a);
  core_wv_kernel<<<nblk((long long)a.np * a.kx, 256), 256, 0, st>>>(a);
  core_x_kernel<<<nblk((long long)a.np * a.kx, 256), 256, 0, st>>>(a);
  return cudaGetLastError() == cudaSuccess ? 9 : -1;
}

int core_gamma(const CoreArgs &a, double *Gam, cudaStream_t st) {
  if (a.df)
    core_gemm_kernel<true, df64><<<dim3(a.ntile, a.ntile), 256, 0, st>>>(a, Gam);
  else
    core_gemm_kernel<true, double><<<dim3(a.ntile, a.ntile), 256, 0, st>>>(a, Gam);
  return cudaGetLastError() == cudaSuccess ? 1 : -1;
}

int core_post(const CoreArgs &a, const double *Gam, cudaStream_t st) {
  if (Gam)
    core_e2_kernel<<<a.ntile * a.ntile, 256, 0, st>>>(a, Gam);
  else
    core_gemm_kernel<false, double><<<dim3(a.ntile, a.ntile), 256, 0, st>>>(a, nullptr);
  core_result_kernel<<<1, 1024, 0, st>>>(a);
  return cudaGetLastError() == cudaSuccess ? 2 : -1;
}


int core_adjoint(const CoreArgs &a, const CoreGrad &g, cudaStream_t st) {
  const int n = a.nsp, nC = a.nC, kx = a.kx;
  const int nn = n * n;
  if (a.df)
    core_ygemm_kernel<df64><<<dim3((kx + GT - 1) / GT, a.ntile), 256, 0, st>>>(a, g);
  else
    core_ygemm_kernel<double><<<dim3((kx + GT - 1) / GT, a.ntile), 256, 0, st>>>(a, g);
  core_axp_kernel<<<dim3(kx, g.nchunk), 256, 0, st>>>(a, g);
  core_axr_kernel<<<nblk((long long)kx * kx, 256), 256, 0, st>>>(a, g);
  core_rowmat_kernel<<<nblk((long long)a.np * kx, 256), 256, 0, st>>>(g.Yg, a.A2x, g.Wvb, a.np, kx, 2.0);
  core_kbuild_kernel<<<nn, 256, 0, st>>>(a, g);
  core_bar_kernel<<<nblk(nn, 256), 256, 0, st>>>(a, g);
  core_bar0_kernel<<<1, 1024, 0, st>>>(a, g);
  core_a1b_kernel<<<nC * nC, 256, 0, st>>>(a, g);
  const size_t psm = sizeof(double) * 8 * 5 * a.P * a.P;
  core_pair_adj_kernel<<<nblk(a.nq, 8), 256, psm, st>>>(a, g);
  core_mbar_kernel<<<nblk((long long)nC * nC, 8), 256, 0, st>>>(a, g);
  core_lam_kernel<<<1, 1024, 0, st>>>(a, g);
  core_ub_kernel<<<nblk((long long)n * nC, 256), 256, 0, st>>>(a, g);
  /* Sbar = -P0 (P0-bar P0) - P0 (U-bar U^T) + (U M-bar) U^T, then the rest */
  core_mm_kernel<<<nblk(nn, 256), 256, 0, st>>>(g.P0b, n, 0, a.P0, n, 0, g.t1, n, n, n, n, 1.0, 0.0);
  core_mm_kernel<<<nblk(nn, 256), 256, 0, st>>>(g.Ub, nC, 0, a.U, nC, 1, g.t2, n, n, n, nC, 1.0, 0.0);
  core_mm_kernel<<<nblk(nn, 256), 256, 0, st>>>(a.P0, n, 0, g.t1, n, 0, g.Sbar, n, n, n, n, -1.0, 0.0);
  core_mm_kernel<<<nblk(nn, 256), 256, 0, st>>>(a.P0, n, 0, g.t2, n, 0, g.Sbar, n, n, n, n, -1.0, 1.0);
  core_mm_kernel<<<nblk((long long)n * nC, 256), 256, 0, st>>>(a.U, nC, 0, g.Mb, nC, 0, g.t1, nC, n, nC, nC, 1.0, 0.0);
  core_mm_kernel<<<nblk(nn, 256), 256, 0, st>>>(g.t1, nC, 0, a.U, nC, 1, g.Sbar, n, n, n, nC, 1.0, 1.0);
  core_sbar_final_kernel<<<nblk(nn, 256), 256, 0, st>>>(a, g);
  return cudaGetLastError() == cudaSuccess ? 19 : -1;
}

double core_gemm_fma(const CoreArgs &a) {
  const double nt = a.ntile;
  return nt * (nt + 1) * 0.5 * GT * GT * (double)a.kx;
}
