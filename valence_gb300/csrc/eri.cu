/*
 * eri.cu / eri_impl.cuh / eri_{f64,f32,df64}.cu -- shell-quartet
 * electron-repulsion integrals fused with the
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
 * (1983)): per primitive quartet the 2D recurrences G(i, k) for x, y, z give
 * the (e0|f0) integrals on the bra and ket centres A and C; the horizontal
 * transfer to B and D (Head-Gordon & Pople, J. Chem. Phys. 89, 5777 (1988))
 * is linear in the contracted (e0|f0) block, (ab|cd) = M_P (e0|f0) M_Q^T
 * with M fixed by the pair geometry, so it is folded into the weight tables
 * (X' = X M, one small product per evaluation) and never runs per
 * primitive.  Roots and weights come from project-generated Chebyshev tables
 * (gen_rys_tables.py).  Kernel structure and arithmetic kinds: eri_impl.cuh.
 */
#include <cuda_runtime.h>

#include <algorithm>

#include "eri.cuh"

namespace {

/* T = U + U^T in 32 x 32 tiles (i-tile >= j-tile), the transposed tile
 * staged in shared memory so that both reads and both writes are coalesced;
 * the diagonal tiles also store the Schwarz factors sqrt(T[p][p]) of
 * schwarz_ints (valence.F90:1516) */
__global__ void symmetrize_kernel(double *T, int np, double *sq) {
  __shared__ double tl[32][33];
  const long long tile = blockIdx.x;
  long long ti = (long long)((sqrtf(8.0f * (float)tile + 1.0f) - 1.0f) * 0.5f);
  while ((ti + 1) * (ti + 2) / 2 <= tile) ++ti;
  while (ti * (ti + 1) / 2 > tile) --ti;
  const long long tj = tile - ti * (ti + 1) / 2;
  const int tx = threadIdx.x, ty = threadIdx.y; /* 32 x 8 */
  /* the mirror tile (rows of tile j, columns of tile i), read coalesced */
  for (int r = ty; r < 32; r += 8) {
    const long long row = tj * 32 + r, col = ti * 32 + tx;
    tl[r][tx] = row < np && col < np ? T[row * np + col] : 0.0;
  }
  __syncthreads();
  double v[4];
  for (int k = 0, r = ty; r < 32; r += 8, ++k) {
    const long long row = ti * 32 + r, col = tj * 32 + tx;
    v[k] = row < np && col < np ? T[row * np + col] + tl[tx][r] : 0.0;
  }
  __syncthreads();
  for (int k = 0, r = ty; r < 32; r += 8, ++k) {
    const long long row = ti * 32 + r, col = tj * 32 + tx;
    if (row < np && col < np) {
      T[row * np + col] = v[k];
      if (row == col) sq[row] = sqrt(fmax(v[k], 0.0));
    }
    tl[r][tx] = v[k];
  }
  __syncthreads();
  if (ti != tj)
    for (int r = ty; r < 32; r += 8) {
      const long long row = tj * 32 + r, col = ti * 32 + tx;
      if (row < np && col < np) T[row * np + col] = tl[tx][r];
    }
}

__global__ void to_float_kernel(const double *in, float *out, size_t n) {
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
    out[t] = (float)in[t];
}

}  // namespace

int eri_to_float(const double *in, float *out, size_t n, cudaStream_t st) {
  if (n == 0) return 0;
  const size_t blocks = std::min<size_t>((n + 255) / 256, 152 * 16);
  to_float_kernel<<<(unsigned)blocks, 256, 0, st>>>(in, out, n);
  return cudaGetLastError() != cudaSuccess;
}

/* T = U + U^T after the forward pass (the kernels accumulate one
 * orientation); sq[p] = sqrt(max(T[p][p], 0)) */
int eri_symmetrize(double *T, int np, double *sq, cudaStream_t st) {
  if (np == 0) return 0;
  const long long nt = (np + 31) / 32;
  symmetrize_kernel<<<(unsigned)(nt * (nt + 1) / 2), dim3(32, 8), 0, st>>>(T, np, sq);
  return cudaGetLastError() != cudaSuccess;
}

/* algorithmic FLOPs of one shell quartet of class (cp, cq) in this
 * formulation: per primitive quartet the n_r roots (two 12-term Clenshaw sums
 * each), the 3 n_r 2D recurrence tables G(i, k) and the (e0|f0) component
 * sums (3 flops per component and root); per quartet the two transform
 * GEMVs with the transferred weights X' (ne_P x ne_Q block), and in modes 2
 * and 3 the four GEMVs of the adjoint (dX'_P and dX'_Q).  nprimq: the
 * primitive quartets evaluated (after the primitive screen). */
double eri_flops(int mode, int cp, int cq, double nprimq, int nopP, int nopQ) {
  static const int la_[6] = {0, 1, 1, 2, 2, 2}, lb_[6] = {0, 0, 1, 0, 1, 2};
  const int la = la_[cp], lb = lb_[cp], lc = la_[cq], ld = lb_[cq];
  auto nc = [](int l) { return (l + 1) * (l + 2) / 2; };
  auto ne = [&](int l0, int l1) {
    int n = 0;
    for (int l = l0; l <= l0 + l1; ++l) n += nc(l);
    return n;
  };
  const int nea = ne(la, lb), nec = ne(lc, ld);
  const int nr = (la + lb + lc + ld) / 2 + 1;
  const double roots = nr * 2.0 * 24.0;
  const double twod = 3.0 * nr * 5.0 * (la + lb + 1) * (lc + ld + 1);
  const double comp = 3.0 * nr * (double)nea * nec;
  const double prim = 30.0 + roots + twod + comp;
  const double fwd = 2.0 * nopQ * (double)nea * nec + 2.0 * nopP * (double)nopQ * nea;
  const double adj = 2.0 * nopQ * (double)nea * nec + 2.0 * nopP * (double)nopQ * nea +
                     2.0 * nopP * (double)nea * nec + 2.0 * nopQ * (double)nopP * nec;
  const double tr = (mode == 0 ? fwd : 0.0) + (mode == 2 ? adj : 0.0) + (mode == 3 ? fwd + adj : 0.0);
  return nprimq * prim + tr;
}

double eri_block_hrr_flops(int cp, int cq) {
  /* (ab| = sum_e M(ab, e) (e0|: one term per function pair of an s or p
   * pair without a p on B, two with one (the transfer adds A-B times the
   * lower function); per block element the product of the two counts, 2
   * flops each */
  static const int nab_[3] = {1, 3, 9}, nt_[3] = {1, 1, 2};
  if (cp > 2 || cq > 2) return 0.0;
  return 2.0 * nab_[cp] * nab_[cq] * nt_[cp] * nt_[cq];
}

int eri_launch(int mode, int kind, int cp, int cq, const EriArgs &a, const int4 *work, int nwork, int max_blocks,
               cudaStream_t st) {
  /* the Schwarz pass and the separate adjoint sweep (grad_mode 1) always run
   * in FP64; the FP32 / double-float kinds instantiate modes 0 and 3 only */
  if (mode == 1 || mode == 2 || kind == ERI_F64) return eri_dispatch_f64(mode, cp, cq, a, work, nwork, max_blocks, st);
  if (kind == ERI_F32) return eri_dispatch_f32(mode, cp, cq, a, work, nwork, max_blocks, st);
  return eri_dispatch_df64(mode, cp, cq, a, work, nwork, max_blocks, st);
}

int eri_launch_tab(int kind, int cp, int cq, const EriArgs &a, const int4 *work, int nwork, int max_blocks,
                   cudaStream_t st, const EriArgs *tab, const int *wmol) {
  if (kind == ERI_F64) return eri_dispatch_tab_f64(cp, cq, a, work, nwork, max_blocks, st, tab, wmol);
  if (kind == ERI_F32) return eri_dispatch_tab_f32(cp, cq, a, work, nwork, max_blocks, st, tab, wmol);
  return eri_dispatch_tab_df64(cp, cq, a, work, nwork, max_blocks, st, tab, wmol);
}
