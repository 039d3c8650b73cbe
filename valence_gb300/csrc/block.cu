/*
 * block.cu -- block mode of the orbital-pair ERI matrix, for large systems
 * of s and p shells (the 4x4x4 Li/F cluster: 320 shells, 304 orbitals,
 * 4.8e8 screened shell quartets).
 *
 * int2e (valence.F90:3184-3438) contracts, for every orbital quartet, the
 * shell quartets of the four orbital basis sets with the weight products.
 * The per-quartet path (eri_impl.cuh, modes 0/3) evaluates each AO shell
 * quartet once and transforms it at once into every orbital pair touching
 * its two shell pairs: with orbitals on one or two atoms that is ~45 x 45
 * orbital pairs per shell quartet, about 1e12 FP64 atomics for the cluster.
 * Block mode instead gathers the shell quartets of one atom quartet
 * (AB|CD) -- every shell pair of atoms A, B against every one of C, D --
 * into a staging block G[(a,b)][(c,d)] over the atoms' functions (mode 4 of
 * the ERI kernels adds each transferred (ab|cd) block there), and transforms
 * the block once, index by index:
 *     Y1[ab][c][v] = sum_d G[ab][cd] C_v(d)          v on atom D
 *     Z [ab][u][v] = sum_c C_u(c) Y1[ab][c][v]        u on atom C
 *     Y3[a][t][uv] = sum_b C_t(b) Z[ab][uv]           t on atom B
 *     W [s][t][uv] = sum_a C_s(a) Y3[a][t][uv]        s on atom A
 * W[s][t][u][v] is the atom quartet's share of (s t | u v); it is added into
 * U at the orbital pairs (s,t), (u,v) (an orbital pair on one atom once, in
 * the order i >= k; across two atoms both orders add, and an orbital paired
 * with itself there counts twice), with weight 1/2 when bra and ket are the
 * same atom pair, and T = U + U^T as on the other path.
 * C_o(f) carries angn_f and int2e's per-shell LCAO screen sum(c^2) > dtol
 * (valence.F90:3296-3348), as the per-quartet weight tables do.
 *
 * Staging: the atom quartets are processed in chunks whose blocks fit a
 * fixed buffer (two buffers alternate, so the integrals of one chunk run
 * while the previous chunk is transformed); the transform clears the block
 * it has read.  Nothing beyond one chunk of blocks exists at a time.
 */
#include <cuda_runtime.h>

#include "block.cuh"
#include "vsvb_internal.h"

namespace {

/* arithmetic of the transform: FP64, FP32, or double-float (an unevaluated
 * sum of two FP32 numbers, ~48-bit significand, on the FP32 pipes: the
 * FP64-class transforms of the double-float path).  Double-float products
 * and sums are the error-free TwoProduct (by FMA) and TwoSum of Dekker and
 * Knuth. */
__device__ __forceinline__ void to_t(double x, double &y) { y = x; }
__device__ __forceinline__ void to_t(double x, float &y) { y = (float)x; }
__device__ __forceinline__ void to_t(double x, df64 &y) { y = df64_split(x); }
__device__ __forceinline__ double dbl(double v) { return v; }
__device__ __forceinline__ double dbl(float v) { return (double)v; }
__device__ __forceinline__ double dbl(df64 v) { return (double)v.hi + (double)v.lo; }
__device__ __forceinline__ void zero_t(double &v) { v = 0.0; }
__device__ __forceinline__ void zero_t(float &v) { v = 0.f; }
__device__ __forceinline__ void zero_t(df64 &v) { v = df64(0.f, 0.f); }
__device__ __forceinline__ bool nonzero_t(double v) { return v != 0.0; }
__device__ __forceinline__ bool nonzero_t(float v) { return v != 0.f; }
__device__ __forceinline__ bool nonzero_t(df64 v) { return v.hi != 0.f || v.lo != 0.f; }
/* s += a b */
__device__ __forceinline__ void mac(double &s, double a, double b) { s = fma(a, b, s); }
__device__ __forceinline__ void mac(float &s, float a, float b) { s = fmaf(a, b, s); }
__device__ __forceinline__ void mac(df64 &s, df64 a, df64 b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  const float t = s.hi + p;
  const float v = t - s.hi;
  const float err = (s.hi - (t - v)) + (p - v);
  const float lo = s.lo + (e + err);
  const float hi = t + lo;
  s = df64(hi, lo - (hi - t));
}

__device__ __forceinline__ int opidx_b(int i, int k) { return i >= k ? i * (i + 1) / 2 + k : k * (k + 1) / 2 + i; }

__global__ void blk_coef_kernel(BlkCoefArgs a) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a.n) return;
  const int4 s = a.src[e];
  double v = 0.0;
  if (s.y >= 0) {
    const double *c = a.C + (size_t)s.x * a.maxobs;
    double w = 0.0;
    for (int k = 0; k < s.w; ++k) w += c[s.z + k] * c[s.z + k];
    if (w > a.dtol) v = c[s.y] * a.angn[a.ao[e]];
  }
  a.catom[e] = v;
}

constexpr int OB = 8; /* output orbitals per thread pass: independent accumulators */

template <typename TT>
__global__ void __launch_bounds__(256) blk_transform_kernel(BlkArgs a, int aq0) {
  extern __shared__ double sm_raw[];
  TT *sm = reinterpret_cast<TT *>(sm_raw);
  const int4 q = a.aq[aq0 + blockIdx.x];
  const int4 p1 = a.ap[q.x], p2 = a.ap[q.y];
  const int XA = p1.x, XB = p1.y, XC = p2.x, XD = p2.y;
  const int nfA = a.atom_nf[XA], nfB = a.atom_nf[XB], nfC = a.atom_nf[XC], nfD = a.atom_nf[XD];
  const int2 oA = a.atom_orb[XA], oB = a.atom_orb[XB], oC = a.atom_orb[XC], oD = a.atom_orb[XD];
  const int nA = oA.y, nB = oB.y, nC = oC.y, nD = oD.y;
  /* weight blocks [orbital][function], orbital rows zero-padded to a
   * multiple of OB so that the blocked passes need no guards */
  const int cw = a.nomaxp * a.nfmax;
  TT *CA = sm, *CB = CA + cw, *CC = CB + cw, *CD = CC + cw;
  TT *R1 = CD + cw;
  TT *R2 = R1 + a.r1n;
  const int tid = threadIdx.x, nt = blockDim.x;
  auto load_c = [&](TT *dst, int atom, int n, int nf) {
    for (int t = tid; t < a.nomaxp * nf; t += nt) {
      if (t < n * nf) to_t(a.catom[a.atom_c0[atom] + t], dst[t]);
      else zero_t(dst[t]);
    }
  };
  load_c(CA, XA, nA, nfA);
  load_c(CB, XB, nB, nfB);
  load_c(CC, XC, nC, nfC);
  load_c(CD, XD, nD, nfD);
  __syncthreads();
  const int nAB = nfA * nfB, ncol = nfC * nfD, nCD = nC * nD;
  const double *G = a.G + (unsigned)q.z;
  /* 1: the d index -- item (ab, c), outputs v */
  for (int it = tid; it < nAB * nfC; it += nt) {
    const double *g = G + (size_t)(it / nfC) * ncol + (it % nfC) * nfD;
    for (int v0 = 0; v0 < nD; v0 += OB) {
      TT acc[OB];
#pragma unroll
      for (int k = 0; k < OB; ++k) zero_t(acc[k]);
      for (int d = 0; d < nfD; ++d) {
        TT x;
        to_t(g[d], x);
        const TT *cd = CD + v0 * nfD + d;
#pragma unroll
        for (int k = 0; k < OB; ++k) mac(acc[k], x, cd[k * nfD]);
      }
#pragma unroll
      for (int k = 0; k < OB; ++k)
        if (v0 + k < nD) R1[(size_t)it * nD + v0 + k] = acc[k];
    }
  }
  __syncthreads();
  /* the block has been read: clear it for the chunk that reuses the buffer */
  for (int idx = tid; idx < nAB * ncol; idx += nt) a.G_clear[(unsigned)q.z + idx] = 0.0;
  /* 2: the c index -- item (ab, v), outputs u */
  for (int it = tid; it < nAB * nD; it += nt) {
    const int ab = it / nD, v = it - ab * nD;
    const TT *y = R1 + (size_t)ab * nfC * nD + v;
    for (int u0 = 0; u0 < nC; u0 += OB) {
      TT acc[OB];
#pragma unroll
      for (int k = 0; k < OB; ++k) zero_t(acc[k]);
      for (int c = 0; c < nfC; ++c) {
        const TT x = y[c * nD];
        const TT *cc = CC + u0 * nfC + c;
#pragma unroll
        for (int k = 0; k < OB; ++k) mac(acc[k], x, cc[k * nfC]);
      }
#pragma unroll
      for (int k = 0; k < OB; ++k)
        if (u0 + k < nC) R2[((size_t)ab * nC + u0 + k) * nD + v] = acc[k];
    }
  }
  __syncthreads();
  /* 3: the b index -- item (a, uv), outputs t */
  for (int it = tid; it < nfA * nCD; it += nt) {
    const int aa = it / nCD, uv = it - aa * nCD;
    const TT *z = R2 + (size_t)aa * nfB * nCD + uv;
    for (int t0 = 0; t0 < nB; t0 += OB) {
      TT acc[OB];
#pragma unroll
      for (int k = 0; k < OB; ++k) zero_t(acc[k]);
      for (int b = 0; b < nfB; ++b) {
        const TT x = z[(size_t)b * nCD];
        const TT *cb = CB + t0 * nfB + b;
#pragma unroll
        for (int k = 0; k < OB; ++k) mac(acc[k], x, cb[k * nfB]);
      }
#pragma unroll
      for (int k = 0; k < OB; ++k)
        if (t0 + k < nB) R1[((size_t)aa * nB + t0 + k) * nCD + uv] = acc[k];
    }
  }
  __syncthreads();
  /* 4: the a index -- item (t, uv), outputs s -- and the orbital-pair scatter */
  const double wgt = q.w & 1 ? 0.5 : 1.0;
  for (int it = tid; it < nB * nCD; it += nt) {
    const int t = it / nCD, uv = it - t * nCD;
    const int u = uv / nD, v = uv - u * nD;
    const int ot = a.orb[oB.x + t], ou = a.orb[oC.x + u], ov = a.orb[oD.x + v];
    if (XC == XD && ou < ov) continue;
    const int qcol = opidx_b(ou, ov);
    const double wq = wgt * (XC != XD && ou == ov ? 2.0 : 1.0);
    const TT *y = R1 + (size_t)t * nCD + uv;
    for (int s0 = 0; s0 < nA; s0 += OB) {
      TT acc[OB];
#pragma unroll
      for (int k = 0; k < OB; ++k) zero_t(acc[k]);
      for (int aa = 0; aa < nfA; ++aa) {
        const TT x = y[(size_t)aa * nB * nCD];
        const TT *ca = CA + s0 * nfA + aa;
#pragma unroll
        for (int k = 0; k < OB; ++k) mac(acc[k], x, ca[k * nfA]);
      }
#pragma unroll
      for (int k = 0; k < OB; ++k) {
        if (s0 + k >= nA) continue;
        const int os = a.orb[oA.x + s0 + k];
        if (XA == XB && os < ot) continue;
        /* across two atoms an orbital paired with itself takes both orders
         * of its weight product, C_i(a) C_i(b) + C_i(b) C_i(a): weight 2 */
        const double w2 = wq * (XA != XB && os == ot ? 2.0 : 1.0);
        if (nonzero_t(acc[k])) atomicAdd(a.U + (size_t)opidx_b(os, ot) * a.np + qcol, w2 * dbl(acc[k]));
      }
    }
  }
}

}  // namespace

int blk_coef(const BlkCoefArgs &a, cudaStream_t st) {
  if (a.n <= 0) return 0;
  blk_coef_kernel<<<(a.n + 255) / 256, 256, 0, st>>>(a);
  return cudaGetLastError() != cudaSuccess;
}

int blk_r1(int nfmax, int nomax) {
  const int nf3 = nfmax * nfmax * nfmax, no3 = nomax * nomax * nomax;
  return nf3 * nomax > nfmax * no3 ? nf3 * nomax : nfmax * no3;
}

size_t blk_transform_smem(int nfmax, int nomax, int tt) {
  const size_t r1 = (size_t)blk_r1(nfmax, nomax);
  const size_t r2 = (size_t)nfmax * nfmax * nomax * nomax;
  const size_t nomaxp = (size_t)(nomax + 7) / 8 * 8;
  const size_t n = 4 * nomaxp * nfmax + r1 + r2;
  return n * (tt == 1 ? sizeof(float) : sizeof(double)); /* double-float: two FP32 */
}

template <typename TT>
int launch_transform(const BlkArgs &a, int aq0, int n, size_t smem_bytes, cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(blk_transform_kernel<TT>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024) !=
        cudaSuccess)
      return 1;
    attr = true;
  }
  blk_transform_kernel<TT><<<n, 256, smem_bytes, st>>>(a, aq0);
  return cudaGetLastError() != cudaSuccess;
}

int blk_transform(const BlkArgs &a, int aq0, int n, int tt, size_t smem_bytes, cudaStream_t st) {
  if (n <= 0) return 0;
  if (tt == 1) return launch_transform<float>(a, aq0, n, smem_bytes, st);
  if (tt == 2) return launch_transform<df64>(a, aq0, n, smem_bytes, st);
  return launch_transform<double>(a, aq0, n, smem_bytes, st);
}

double blk_transform_flops(int nfa, int nfb, int nfc, int nfd, int na, int nb, int nc, int nd) {
  const double nab = (double)nfa * nfb;
  return 2.0 * (nab * nfc * nd * nfd + nab * nc * nd * nfc + (double)nfa * nb * nc * nd * nfb +
                (double)na * nb * nc * nd * nfa);
}
