/*
 * onee.cu -- one-electron and orbital-weight kernels.
 *
 *   ao_1e_kernel    AO overlap, kinetic and nuclear-attraction matrices with
 *                   VALENCE's per-component angn factors (what ovint/int1e
 *                   contract, valence.F90:2891-3176; simint_compute_overlap,
 *                   _ke, _potential).  Obara-Saika recursions; geometry only,
 *                   run once per handle.
 *   ndf_norm / orb_norm
 *                   the weight scatter of ovint/int1e/int2e (with derived
 *                   basis functions mapped through ndf2obs, valence.F90:
 *                   2191-2247) and normal() (valence.F90:2157-2182): NDFs first,
 *                   then the orbitals, each scaled to unit self-overlap.
 *   orb_1e_kernel   orbital overlap S_ij (wfndet, valence.F90:1440-1480) and
 *                   core Hamiltonian h_ij (int1e) as C_i^T S_AO C_j.
 *   xtab_kernel     per shell pair and orbital pair the weight products
 *                   X(a,b) of int2e (dij/dkl, valence.F90:3372-3396) with its
 *                   per-shell LCAO screen sum(c^2) > dtol (:3296-3348).
 *   xhrr_kernel     the horizontal transfer of each shell pair folded into
 *                   its weights: X' = X M (M from the pair geometry), so the
 *                   ERI kernels contract (e0|f0) integrals.
 *   orb_grad kernels  the adjoints of the above for the weight gradient.
 */
#include <cuda_runtime.h>

#include "onee.cuh"

namespace {

__constant__ int k_cart[3][6][3] = {
    {{0, 0, 0}},
    {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}},
    {{2, 0, 0}, {1, 1, 0}, {1, 0, 1}, {0, 2, 0}, {0, 1, 1}, {0, 0, 2}}};

__device__ __forceinline__ int ncart(int l) { return (l + 1) * (l + 2) / 2; }
__device__ __forceinline__ int ncart_upto(int l) { return (l + 1) * (l + 2) * (l + 3) / 6; }
__device__ __forceinline__ int cidx(int x, int y, int z) {
  int l = x + y + z, i = l - x;
  return l * (l + 1) * (l + 2) / 6 + i * (i + 1) / 2 + z;
}

/* Boys function F_0..F_mmax (mmax <= 8): series plus downward recursion
 * below T = 30, F_0 from erf and upward recursion above. */
__device__ void boys_dev(int mmax, double t, double *f) {
  if (t < 30.0) {
    double et = exp(-t);
    double term = 1.0 / (2 * mmax + 1), sum = term;
    for (int k = 1; k < 400; ++k) {
      term *= 2.0 * t / (2 * mmax + 2 * k + 1);
      sum += term;
      if (term < sum * 1e-17) break;
    }
    f[mmax] = et * sum;
    for (int m = mmax - 1; m >= 0; --m) f[m] = (2.0 * t * f[m + 1] + et) / (2 * m + 1);
  } else {
    double et = exp(-t), st = sqrt(t);
    f[0] = 0.886226925452758014 / st * erf(st); /* sqrt(pi)/2 */
    for (int m = 0; m < mmax; ++m) f[m + 1] = ((2 * m + 1) * f[m] - et) / (2.0 * t);
  }
}

/* 1D Obara-Saika overlap table s[i][j], i<=imax, j<=jmax (<= 3) */
__device__ void os1d(double a, double b, double xa, double xb, int imax, int jmax, double s[4][4]) {
  double p = a + b, xp = (a * xa + b * xb) / p, xpa = xp - xa, xpb = xp - xb, oo2p = 0.5 / p;
  double d = xa - xb;
  s[0][0] = sqrt(3.14159265358979323846 / p) * exp(-a * b / p * d * d);
  for (int i = 0; i <= imax; ++i) {
    if (i > 0) s[i][0] = xpa * s[i - 1][0] + (i > 1 ? oo2p * (i - 1) * s[i - 2][0] : 0.0);
    for (int j = 1; j <= jmax; ++j) {
      double v = xpb * s[i][j - 1];
      if (i > 0) v += oo2p * i * s[i - 1][j - 1];
      if (j > 1) v += oo2p * (j - 1) * s[i][j - 2];
      s[i][j] = v;
    }
  }
}

}  // namespace

/* one thread per unique shell pair (A >= B); writes both triangles */
/* one warp per shell pair: overlap and kinetic in every lane, the nuclear
 * attraction split over the nuclei by lane and summed over the warp in a
 * fixed order */
__global__ void ao_1e_kernel(Ao1eArgs a) {
  const int t = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  int ns = a.nshell;
  if (t >= ns * (ns + 1) / 2) return;
  int A = (int)((sqrt(8.0 * t + 1.0) - 1.0) / 2.0);
  while ((A + 1) * (A + 2) / 2 <= t) ++A;
  while (A * (A + 1) / 2 > t) --A;
  int B = t - A * (A + 1) / 2;
  const GShell sa = a.shells[A], sb = a.shells[B];
  const int la = sa.l, lb = sb.l, na = ncart(la), nb = ncart(lb);
  double S[36], Tk[36], V[36];
  for (int i = 0; i < na * nb; ++i) S[i] = Tk[i] = V[i] = 0.0;
  double ab[3];
  for (int d = 0; d < 3; ++d) ab[d] = sa.xyz[d] - sb.xyz[d];
  const double ab2 = ab[0] * ab[0] + ab[1] * ab[1] + ab[2] * ab[2];
  const int L = la + lb;
  for (int ia = 0; ia < sa.nprim; ++ia)
    for (int ib = 0; ib < sb.nprim; ++ib) {
      const double al = a.exps[sa.prim0 + ia], be = a.exps[sb.prim0 + ib];
      const double cc = a.coefs[sa.prim0 + ia] * a.coefs[sb.prim0 + ib];
      double sx[4][4], sy[4][4], sz[4][4];
      os1d(al, be, sa.xyz[0], sb.xyz[0], la + 1, lb + 1, sx);
      os1d(al, be, sa.xyz[1], sb.xyz[1], la + 1, lb + 1, sy);
      os1d(al, be, sa.xyz[2], sb.xyz[2], la + 1, lb + 1, sz);
      for (int i = 0; i < na; ++i) {
        const int *pa = k_cart[la][i];
        for (int j = 0; j < nb; ++j) {
          const int *pb = k_cart[lb][j];
          double Sx = sx[pa[0]][pb[0]], Sy = sy[pa[1]][pb[1]], Sz = sz[pa[2]][pb[2]];
          S[i * nb + j] += cc * Sx * Sy * Sz;
          double tt[3];
          double (*ss[3])[4] = {sx, sy, sz};
          for (int d = 0; d < 3; ++d) {
            int ii = pa[d], jj = pb[d];
            double (*s)[4] = ss[d];
            double v = 4.0 * al * be * s[ii + 1][jj + 1];
            if (ii > 0 && jj > 0) v += (double)ii * jj * s[ii - 1][jj - 1];
            if (ii > 0) v -= 2.0 * be * ii * s[ii - 1][jj + 1];
            if (jj > 0) v -= 2.0 * al * jj * s[ii + 1][jj - 1];
            tt[d] = 0.5 * v;
          }
          Tk[i * nb + j] += cc * (tt[0] * Sy * Sz + Sx * tt[1] * Sz + Sx * Sy * tt[2]);
        }
      }
      /* nuclear attraction: (e|A^(m)|0) for |e| <= L, then transfer to B */
      const double p = al + be;
      double P[3], PA[3];
      for (int d = 0; d < 3; ++d) {
        P[d] = (al * sa.xyz[d] + be * sb.xyz[d]) / p;
        PA[d] = P[d] - sa.xyz[d];
      }
      const double base = 2.0 * 3.14159265358979323846 / p * exp(-al * be / p * ab2) * cc;
      /* a primitive pair with a prefactor below 1e-40 adds below 1e-32 to
       * any element (Boys values <= 1, distance factors up to ~1e8) */
      if (fabs(base) < 1e-40) continue;
      for (int c = lane; c < a.natom; c += 32) {
        const double zc = a.charge[c];
        if (fabs(zc) <= 1e-12) continue;
        double PC[3];
        for (int d = 0; d < 3; ++d) PC[d] = P[d] - a.atom_xyz[3 * c + d];
        double fm[9];
        boys_dev(L, p * (PC[0] * PC[0] + PC[1] * PC[1] + PC[2] * PC[2]), fm);
        double v[5][35];
        for (int m = 0; m <= L; ++m) v[m][0] = base * fm[m];
        for (int el = 1; el <= L; ++el)
          for (int i = 0; i <= el; ++i)
            for (int j = 0; j <= i; ++j) {
              int e[3] = {el - i, i - j, j};
              int d = e[0] ? 0 : (e[1] ? 1 : 2);
              int e1[3] = {e[0], e[1], e[2]};
              e1[d]--;
              int i1 = cidx(e1[0], e1[1], e1[2]), i2 = -1;
              if (e1[d] > 0) i2 = cidx(e1[0] - (d == 0), e1[1] - (d == 1), e1[2] - (d == 2));
              int ie = cidx(e[0], e[1], e[2]);
              for (int m = 0; m <= L - el; ++m) {
                double val = PA[d] * v[m][i1] - PC[d] * v[m + 1][i1];
                if (i2 >= 0) val += e1[d] / (2.0 * p) * (v[m][i2] - v[m + 1][i2]);
                v[m][ie] = val;
              }
            }
        /* transfer to B: h[a][b] */
        double h[35][10];
        const int nall = ncart_upto(L), nball = ncart_upto(lb);
        for (int k = 0; k < nall; ++k) h[k][0] = v[0][k];
        for (int bl = 1; bl <= lb; ++bl)
          for (int i = 0; i <= bl; ++i)
            for (int j = 0; j <= i; ++j) {
              int bb[3] = {bl - i, i - j, j};
              int d = bb[0] ? 0 : (bb[1] ? 1 : 2);
              int b1[3] = {bb[0], bb[1], bb[2]};
              b1[d]--;
              int ibb = cidx(bb[0], bb[1], bb[2]), ib1 = cidx(b1[0], b1[1], b1[2]);
              for (int al2 = la; al2 <= L - bl; ++al2)
                for (int ii = 0; ii <= al2; ++ii)
                  for (int jj = 0; jj <= ii; ++jj) {
                    int aa[3] = {al2 - ii, ii - jj, jj};
                    int iap = cidx(aa[0] + (d == 0), aa[1] + (d == 1), aa[2] + (d == 2));
                    int iaa = cidx(aa[0], aa[1], aa[2]);
                    h[iaa][ibb] = h[iap][ib1] + ab[d] * h[iaa][ib1];
                  }
            }
        (void)nball;
        for (int i = 0; i < na; ++i) {
          const int *pa = k_cart[la][i];
          for (int j = 0; j < nb; ++j) {
            const int *pb = k_cart[lb][j];
            V[i * nb + j] -= zc * h[cidx(pa[0], pa[1], pa[2])][cidx(pb[0], pb[1], pb[2])];
          }
        }
      }
    }
  for (int k = 0; k < na * nb; ++k)
    for (int o = 16; o > 0; o >>= 1) V[k] += __shfl_xor_sync(0xffffffffu, V[k], o);
  if (lane != 0) return;
  const int nao = a.nao;
  for (int i = 0; i < na; ++i)
    for (int j = 0; j < nb; ++j) {
      double f = a.angn[sa.ao0 + i] * a.angn[sb.ao0 + j];
      double s = S[i * nb + j] * f, hh = (Tk[i * nb + j] + V[i * nb + j]) * f;
      size_t r = sa.ao0 + i, c = sb.ao0 + j;
      a.S[r * nao + c] = s;
      a.S[c * nao + r] = s;
      a.H[r * nao + c] = hh;
      a.H[c * nao + r] = hh;
    }
}

/* ---- orbital weights -------------------------------------------------- */

/* block reduce helper (blockDim.x == 128) */
__device__ double block_sum(double v, double *red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
  __syncthreads();
  if (threadIdx.x == 0) red[0] = s;
  __syncthreads();
  s = red[0];
  __syncthreads();
  return s;
}

/* v^T S_AO v over an orbital's OBS slots */
__device__ double obs_quad(const double *v, const int *ao, int n, const double *S, int nao, double *red) {
  double s = 0.0;
  for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
    int k = t / n, l = t - k * n;
    s += v[k] * S[(size_t)ao[k] * nao + ao[l]] * v[l];
  }
  return block_sum(s, red);
}

/* one block per NDF: scale = (v^T S v)^(-1/2) */
__global__ void ndf_norm_kernel(OrbArgs a) {
  __shared__ double red[8];
  extern __shared__ double v[];
  int f = blockIdx.x, o = a.ndf_orb[f];
  int n = a.obs_n[o];
  const int *ao = a.obs_ao + (size_t)o * a.maxobs;
  for (int k = threadIdx.x; k < n; k += blockDim.x) v[k] = 0.0;
  __syncthreads();
  if (threadIdx.x == 0)
    for (int t = a.term0[o]; t < a.term0[o + 1]; ++t) v[a.term_slot[t]] += a.coeff[a.term_j[t]];
  __syncthreads();
  double s = obs_quad(v, ao, n, a.S, a.nao, red);
  if (threadIdx.x == 0) {
    a.ndf_scale[f] = s > 0.0 ? rsqrt(s) : 0.0;
    if (!(s > 0.0)) atomicOr(a.status, 1);
  }
}

/* one block per orbital (non-NDF): raw vector, self overlap, normalised C */
__global__ void orb_norm_kernel(OrbArgs a) {
  __shared__ double red[8];
  extern __shared__ double v[];
  int o = blockIdx.x;
  int n = a.obs_n[o];
  const int *ao = a.obs_ao + (size_t)o * a.maxobs;
  for (int k = threadIdx.x; k < n; k += blockDim.x) v[k] = 0.0;
  __syncthreads();
  if (threadIdx.x == 0)
    for (int t = a.term0[o]; t < a.term0[o + 1]; ++t) {
      double c = a.coeff[a.term_j[t]];
      if (a.term_m[t] >= 0) c *= a.coeff[a.term_m[t]] * a.ndf_scale[a.term_f[t]];
      v[a.term_slot[t]] += c;
    }
  __syncthreads();
  double s = obs_quad(v, ao, n, a.S, a.nao, red);
  double sc = s > 0.0 ? rsqrt(s) : 0.0;
  if (o == a.fixed_orb) sc = 1.0; /* first_order_opt's dummy orbitals keep weight 1 */
  if (threadIdx.x == 0) {
    a.orb_scale[o] = sc;
    if (!(s > 0.0)) atomicOr(a.status, 1);
  }
  for (int k = threadIdx.x; k < a.maxobs; k += blockDim.x) {
    a.Craw[(size_t)o * a.maxobs + k] = k < n ? v[k] : 0.0;
    a.C[(size_t)o * a.maxobs + k] = k < n ? v[k] * sc : 0.0;
  }
}

/* one block per (i, j), i, j < nsp: S_ij = C_i^T S_AO C_j, h_ij likewise */
__global__ void orb_1e_kernel(OrbArgs a, double *So, double *Ho) {
  __shared__ double red[8];
  int i = blockIdx.x, j = blockIdx.y;
  int ni = a.obs_n[i], nj = a.obs_n[j];
  const int *aoi = a.obs_ao + (size_t)i * a.maxobs, *aoj = a.obs_ao + (size_t)j * a.maxobs;
  const double *ci = a.C + (size_t)i * a.maxobs, *cj = a.C + (size_t)j * a.maxobs;
  double s = 0.0, h = 0.0;
  for (int t = threadIdx.x; t < ni * nj; t += blockDim.x) {
    int k = t / nj, l = t - k * nj;
    size_t off = (size_t)aoi[k] * a.nao + aoj[l];
    double w = ci[k] * cj[l];
    s += w * a.S[off];
    h += w * a.H[off];
  }
  s = block_sum(s, red);
  h = block_sum(h, red);
  if (threadIdx.x == 0) {
    So[i * gridDim.y + j] = s;
    Ho[i * gridDim.y + j] = h;
  }
}

/* LCAO shell weight of orbital o on the shell starting at OBS slot s0 */
__device__ __forceinline__ bool shell_kept(const double *c, int s0, int n, double dtol) {
  double w = 0.0;
  for (int k = 0; k < n; ++k) w += c[s0 + k] * c[s0 + k];
  return w > dtol;
}

/* one thread per (pair term, a, b) */
__global__ void xtab_kernel(XtabArgs x) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= x.nelem) return;
  /* locate the pair term by binary search over elem0 */
  int lo = 0, hi = x.nterm - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (x.elem0[mid] <= t) lo = mid;
    else hi = mid - 1;
  }
  const XTerm &tm = x.terms[lo];
  int e = (int)(t - x.elem0[lo]);
  int na = ncart(tm.la), nb = ncart(tm.lb);
  int ia = e / nb, ib = e - ia * nb;
  const double *ci = x.C + (size_t)tm.oi * x.maxobs, *ck = x.C + (size_t)tm.ok * x.maxobs;
  /* the orbital keep_orb is never screened (a negative tolerance keeps every shell) */
  const double dti = tm.oi == x.keep_orb ? -1.0 : x.dtol, dtk = tm.ok == x.keep_orb ? -1.0 : x.dtol;
  auto val = [&](const double *c, int s0, int n, int comp, double dt) -> double {
    if (s0 < 0) return 0.0;
    if (!shell_kept(c, s0, n, dt)) return 0.0;
    return c[s0 + comp];
  };
  double ciA = val(ci, tm.sAi, na, ia, dti), ckB = val(ck, tm.sBk, nb, ib, dtk);
  double v = ciA * ckB;
  if (!tm.same_shell) {
    double ckA = val(ck, tm.sAk, na, ia, dtk), ciB = val(ci, tm.sBi, nb, ib, dti);
    v += ckA * ciB;
  }
  x.xtab[t] = v * x.angn[tm.aoA + ia] * x.angn[tm.aoB + ib];
}

/* adjoint of xtab_kernel: dE/dC from dE/dX (same thread layout) */
__global__ void xtab_adjoint_kernel(XtabArgs x, const double *xbar, double *Cbar) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= x.nelem) return;
  int lo = 0, hi = x.nterm - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (x.elem0[mid] <= t) lo = mid;
    else hi = mid - 1;
  }
  const XTerm &tm = x.terms[lo];
  int e = (int)(t - x.elem0[lo]);
  int na = ncart(tm.la), nb = ncart(tm.lb);
  int ia = e / nb, ib = e - ia * nb;
  const double *ci = x.C + (size_t)tm.oi * x.maxobs, *ck = x.C + (size_t)tm.ok * x.maxobs;
  const double scale = x.wres ? x.xbar_scale / x.wres[4] : x.xbar_scale;
  double g = xbar[t] * scale * x.angn[tm.aoA + ia] * x.angn[tm.aoB + ib];
  if (g == 0.0) return;
  const double dti = tm.oi == x.keep_orb ? -1.0 : x.dtol, dtk = tm.ok == x.keep_orb ? -1.0 : x.dtol;
  auto kept = [&](const double *c, int s0, int n, double dt) -> bool { return s0 >= 0 && shell_kept(c, s0, n, dt); };
  double *gi = Cbar + (size_t)tm.oi * x.maxobs, *gk = Cbar + (size_t)tm.ok * x.maxobs;
  if (kept(ci, tm.sAi, na, dti) && kept(ck, tm.sBk, nb, dtk)) {
    atomicAdd(gi + tm.sAi + ia, g * ck[tm.sBk + ib]);
    atomicAdd(gk + tm.sBk + ib, g * ci[tm.sAi + ia]);
  }
  if (!tm.same_shell && kept(ck, tm.sAk, na, dtk) && kept(ci, tm.sBi, nb, dti)) {
    atomicAdd(gk + tm.sAk + ia, g * ci[tm.sBi + ib]);
    atomicAdd(gi + tm.sBi + ib, g * ck[tm.sAk + ia]);
  }
}

/* number of Cartesian functions (a+k, 0) the transfer of an (la, lb) pair
 * starts from: l = la .. la+lb */
__device__ __forceinline__ int ne_of(int la, int lb) { return ncart_upto(la + lb) - (la > 0 ? ncart_upto(la - 1) : 0); }

__device__ __forceinline__ int term_of(const long long *e0, int n, long long t) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (e0[mid] <= t) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

/* X'(op, e) = sum_ab X(op, ab) M(ab, e): the horizontal transfer
 * (ab| = sum_e M(ab, e) (e0| of the pair, folded into its weights so the ERI
 * kernels contract (e0|f0) integrals directly.  One thread per X' element. */
__global__ void xhrr_kernel(XtabArgs x) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= x.nxh) return;
  const int k = term_of(x.xh_elem0, x.nterm, t);
  const XTerm &tm = x.terms[k];
  const int e = (int)(t - x.xh_elem0[k]);
  const int nab = ncart(tm.la) * ncart(tm.lb), ne = ne_of(tm.la, tm.lb);
  const double *X = x.xtab + x.elem0[k];
  const double *M = x.hrr + tm.m0;
  double s = 0.0;
  for (int ab = 0; ab < nab; ++ab) s = fma(X[ab], M[ab * ne + e], s);
  x.xtabh[t] = s;
  x.xtabh32[t] = (float)s;
}

/* adjoint: dE/dX(op, ab) = sum_e dE/dX'(op, e) M(ab, e); one thread per X element */
__global__ void xhrr_adjoint_kernel(XtabArgs x, const double *xbarh, double *xbar) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= x.nelem) return;
  const int k = term_of(x.elem0, x.nterm, t);
  const XTerm &tm = x.terms[k];
  const int ab = (int)(t - x.elem0[k]);
  const int ne = ne_of(tm.la, tm.lb);
  const double *Xb = xbarh + x.xh_elem0[k];
  const double *M = x.hrr + tm.m0 + (size_t)ab * ne;
  double s = 0.0;
  for (int e = 0; e < ne; ++e) s = fma(Xb[e], M[e], s);
  xbar[t] = s;
}

/* adjoint of orb_1e_kernel: Cbar_i(k) += sum_j (Sbar_ij + Sbar_ji) (S C_j)(k)
 * and the same with H; one block per orbital i, threads over its slots */
__global__ void orb_1e_adjoint_kernel(OrbArgs a, const double *Sbar, const double *Hbar, int nsp, double *Cbar) {
  int i = blockIdx.x;
  int ni = a.obs_n[i];
  const int *aoi = a.obs_ao + (size_t)i * a.maxobs;
  for (int k = threadIdx.x; k < ni; k += blockDim.x) {
    double g = 0.0;
    for (int j = 0; j < nsp; ++j) {
      double ws = Sbar[i * nsp + j] + Sbar[j * nsp + i];
      double wh = Hbar[i * nsp + j] + Hbar[j * nsp + i];
      if (ws == 0.0 && wh == 0.0) continue;
      int nj = a.obs_n[j];
      const int *aoj = a.obs_ao + (size_t)j * a.maxobs;
      const double *cj = a.C + (size_t)j * a.maxobs;
      double ss = 0.0, hh = 0.0;
      for (int l = 0; l < nj; ++l) {
        size_t off = (size_t)aoi[k] * a.nao + aoj[l];
        ss += a.S[off] * cj[l];
        hh += a.H[off] * cj[l];
      }
      g += ws * ss + wh * hh;
    }
    Cbar[(size_t)i * a.maxobs + k] += g;
  }
}

/* adjoint of orb_norm_kernel:
 * C = s Craw, s = (Craw^T S Craw)^(-1/2)
 * => Craw_bar = s Cbar - s^3 (Cbar . Craw) S Craw; then over the orbital's
 * weight terms: coeff_bar of its own weight, and for a term through a
 * derived basis function f (Craw[slot] += c_j c_m s_f) also the NDF's weight
 * c_m and the adjoint of its scale s_f (ndf_bar, finished by
 * ndf_norm_adjoint_kernel).  One block per orbital. */
__global__ void orb_norm_adjoint_kernel(OrbArgs a, const double *Cbar, double *coeff_bar, double *ndf_bar) {
  __shared__ double red[8];
  extern __shared__ double sh[];
  int o = blockIdx.x;
  int n = a.obs_n[o];
  const int *ao = a.obs_ao + (size_t)o * a.maxobs;
  const double *cr = a.Craw + (size_t)o * a.maxobs, *cb = Cbar + (size_t)o * a.maxobs;
  double s = a.orb_scale[o];
  double dot = 0.0;
  for (int k = threadIdx.x; k < n; k += blockDim.x) dot += cb[k] * cr[k];
  dot = block_sum(dot, red);
  double *g = sh;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    double scr = 0.0;
    for (int l = 0; l < n; ++l) scr += a.S[(size_t)ao[k] * a.nao + ao[l]] * cr[l];
    g[k] = s * cb[k] - s * s * s * dot * scr;
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int t = a.term0[o]; t < a.term0[o + 1]; ++t) {
      const double gk = g[a.term_slot[t]];
      if (a.term_m[t] < 0) {
        coeff_bar[a.term_j[t]] += gk;
      } else {
        const int m = a.term_m[t], f = a.term_f[t];
        const double cj = a.coeff[a.term_j[t]], cm = a.coeff[m], sf = a.ndf_scale[f];
        coeff_bar[a.term_j[t]] += gk * cm * sf;
        atomicAdd(coeff_bar + m, gk * cj * sf);
        atomicAdd(ndf_bar + f, gk * cj * cm);
      }
    }
}

/* adjoint of ndf_norm_kernel: s_f = (u^T S u)^(-1/2) over the NDF's raw
 * vector u, so dE/dc_m += ndf_bar[f] * (-s_f^3) (S u)[slot of m].  One block
 * per NDF, after orb_norm_adjoint_kernel. */
__global__ void ndf_norm_adjoint_kernel(OrbArgs a, const double *ndf_bar, double *coeff_bar) {
  extern __shared__ double u[];
  const int f = blockIdx.x, o = a.ndf_orb[f];
  const int n = a.obs_n[o];
  const int *ao = a.obs_ao + (size_t)o * a.maxobs;
  double *su = u + a.maxobs;
  for (int k = threadIdx.x; k < n; k += blockDim.x) u[k] = 0.0;
  __syncthreads();
  if (threadIdx.x == 0)
    for (int t = a.term0[o]; t < a.term0[o + 1]; ++t) u[a.term_slot[t]] += a.coeff[a.term_j[t]];
  __syncthreads();
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    double v = 0.0;
    for (int l = 0; l < n; ++l) v += a.S[(size_t)ao[k] * a.nao + ao[l]] * u[l];
    su[k] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const double sf = a.ndf_scale[f], w = -ndf_bar[f] * sf * sf * sf;
    for (int t = a.term0[o]; t < a.term0[o + 1]; ++t) coeff_bar[a.term_j[t]] += w * su[a.term_slot[t]];
  }
}

/* dE/d(weights) of orbital o before normal(): the weight scatter's adjoint
 * over the orbital's terms (an entry through a derived basis function picks
 * up that function's normalised expansion), scaled, into out[0..nent) for
 * the entries j0..j0+nent of the weight array.  One thread, fixed order.
 * flag (optional) collects the evaluation's status bits. */
__global__ void entry_adjoint_kernel(OrbArgs a, int o, int j0, int nent, const double *Cbar, double *out, double scale,
                                     int *flag) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (flag) *flag |= *a.status; /* the evaluation's status bits, kept over the columns */
  for (int e = 0; e < nent; ++e) out[e] = 0.0;
  const double *cb = Cbar + (size_t)o * a.maxobs;
  for (int t = a.term0[o]; t < a.term0[o + 1]; ++t) {
    double f = 1.0;
    if (a.term_m[t] >= 0) f = a.coeff[a.term_m[t]] * a.ndf_scale[a.term_f[t]];
    out[a.term_j[t] - j0] += scale * f * cb[a.term_slot[t]];
  }
}

/* the weight array of a first_order_opt evaluation: entry t takes w[src[t]]
 * from the caller's weights, or (src[t] < 0: the substituted orbital's
 * entries j0, j0+1, ...) 1 at entry j0 + nu and 0 elsewhere */
__global__ void hs_weights_kernel(double *coeff, const double *w, const int *src, int n, int j0, int nu) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  coeff[t] = src[t] >= 0 ? w[src[t]] : (t - j0 == nu ? 1.0 : 0.0);
}
