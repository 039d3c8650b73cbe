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
__device__ __forceinline__ void to_t(double x, df64 &y) {
  const float h = (float)x;
  y = df64(h, (float)(x - (double)h));
}
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
  const int cw = a.nomax * a.nfmax;
  TT *CA = sm, *CB = CA + cw, *CC = CB + cw, *CD = CC + cw;
  TT *R1 = CD + cw;
  TT *R2 = R1 + a.r1n;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int t = tid; t < nA * nfA; t += nt) to_t(a.catom[a.atom_c0[XA] + t], CA[t]);
  for (int t = tid; t < nB * nfB; t += nt) to_t(a.catom[a.atom_c0[XB] + t], CB[t]);
  for (int t = tid; t < nC * nfC; t += nt) to_t(a.catom[a.atom_c0[XC] + t], CC[t]);
  for (int t = tid; t < nD * nfD; t += nt) to_t(a.catom[a.atom_c0[XD] + t], CD[t]);
  __syncthreads();
  const int nAB = nfA * nfB, ncol = nfC * nfD, nCD = nC * nD;
  const double *G = a.G + (unsigned)q.z;
  /* 1: the d index */
  for (int idx = tid; idx < nAB * nfC * nD; idx += nt) {
    const int v = idx % nD, t = idx / nD, c = t % nfC, ab = t / nfC;
    const double *g = G + (size_t)ab * ncol + c * nfD;
    const TT *cd = CD + v * nfD;
    TT s;
    zero_t(s);
    for (int d = 0; d < nfD; ++d) {
      TT gv;
      to_t(g[d], gv);
      mac(s, gv, cd[d]);
    }
    R1[idx] = s;
  }
  __syncthreads();
  /* the block has been read: clear it for the chunk that reuses the buffer */
  for (int idx = tid; idx < nAB * ncol; idx += nt) a.G_clear[(unsigned)q.z + idx] = 0.0;
  /* 2: the c index */
  for (int idx = tid; idx < nAB * nCD; idx += nt) {
    const int v = idx % nD, t = idx / nD, u = t % nC, ab = t / nC;
    const TT *y = R1 + (size_t)ab * nfC * nD + v;
    const TT *cc = CC + u * nfC;
    TT s;
    zero_t(s);
    for (int c = 0; c < nfC; ++c) mac(s, cc[c], y[c * nD]);
    R2[idx] = s;
  }
  __syncthreads();
  /* 3: the b index */
  for (int idx = tid; idx < nfA * nB * nCD; idx += nt) {
    const int uv = idx % nCD, t2 = idx / nCD, t = t2 % nB, aa = t2 / nB;
    const TT *z = R2 + (size_t)aa * nfB * nCD + uv;
    const TT *cb = CB + t * nfB;
    TT s;
    zero_t(s);
    for (int b = 0; b < nfB; ++b) mac(s, cb[b], z[(size_t)b * nCD]);
    R1[idx] = s;
  }
  __syncthreads();
  /* 4: the a index, and the orbital-pair scatter */
  const double wgt = q.w & 1 ? 0.5 : 1.0;
  for (int idx = tid; idx < nA * nB * nCD; idx += nt) {
    const int uv = idx % nCD, t2 = idx / nCD, t = t2 % nB, s = t2 / nB;
    const int u = uv / nD, v = uv - u * nD;
    const int os = a.orb[oA.x + s], ot = a.orb[oB.x + t], ou = a.orb[oC.x + u], ov = a.orb[oD.x + v];
    if (XA == XB && os < ot) continue;
    if (XC == XD && ou < ov) continue;
    /* across two atoms an orbital paired with itself takes both orders of
     * its weight product, C_i(a) C_i(b) + C_i(b) C_i(a): weight 2 */
    const double w2 = (XA != XB && os == ot ? 2.0 : 1.0) * (XC != XD && ou == ov ? 2.0 : 1.0);
    const TT *y = R1 + (size_t)t * nCD + uv;
    const TT *ca = CA + s * nfA;
    TT acc;
    zero_t(acc);
    for (int aa = 0; aa < nfA; ++aa) mac(acc, ca[aa], y[(size_t)aa * nB * nCD]);
    if (nonzero_t(acc)) atomicAdd(a.U + (size_t)opidx_b(os, ot) * a.np + opidx_b(ou, ov), wgt * w2 * dbl(acc));
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
  const size_t n = 4 * (size_t)nomax * nfmax + r1 + r2;
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
