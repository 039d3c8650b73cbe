/*
 * density.cu -- nonorthogonal cofactor densities and the VSVB energy
 * assembly (valence.F90:1010-1434 with density/density_sc/dbra/dket/det,
 * :1535-2056, and givdr/givens_single, :2067-2144, givens.F90:230-262).
 *
 * The reference re-factorises a struck overlap matrix with Givens rotations
 * for every (orbital quartet x spin term x determinant pair).  Here every
 * determinant pair q of the spin-coupled expansion (dbra x dket over the
 * 2^npair alpha/beta exchanges of each coupling pair, weight
 * coeff_sc(isc) coeff_sc(jsc)) is factorised once (Gauss-Jordan with
 * partial pivoting per spin block), and any struck determinant follows from
 * Jacobi's identity:
 *   det(A with row r -> e_c)               = det A * T[c][r]
 *   det(A with rows r1 -> e_c1, r2 -> e_c2) = det A * (T[c1][r1] T[c2][r2]
 *                                                      - T[c1][r2] T[c2][r1])
 * with T = A^-1.  Blocks whose pivots fall below 1e-7 of their largest entry
 * (exact rank deficiency from molecular symmetry, e.g. pi pairs) take the
 * exact path, which gives what the reference's givdr computes for any rank
 * of A: with P a fixed rank-2 matrix, every struck determinant of A + t P
 * (at most two strikes) is a polynomial of degree <= 2 in t -- the strikes
 * replace rows, so the struck matrix is A_struck + t P' with P' of rank <= 2
 * -- whose value at t = 0 is the struck determinant of A:
 *   f(0) = 3 f(1) - 3 f(2) + f(3),  f(k) = det(A + kP) J_k,
 * J_k from the inverse of A + kP by Jacobi's identity as above.  A + kP is
 * well conditioned for rank deficiency up to 2; at 3 or more it stays
 * singular and every struck determinant with at most two strikes is exactly
 * zero.  Three extra factorisations per flagged block make each struck
 * determinant O(1) at any block size.  For the adjoint such a
 * block also keeps det and inverse of A + delta I (delta = 1e-8 of its
 * largest entry): every struck determinant is a polynomial in A, so the
 * derivative taken through the shifted pair is within about 5 delta
 * (relative) of the exact one at any rank deficiency, where det(A) A^-1
 * itself does not exist.
 *
 * The task loop keeps the reference's arithmetic: the same triangular task
 * enumeration (xm_dtriang8, xm_module.F90:969-991), the Schwarz screens on
 * the orbital-pair table (:1189-1190), the post-hoc |ERI| > itol screen
 * (:1286-1287), the DOCC spin-parity skips (:1352-1375), the sign rule of
 * det() for the exchanged density (:2041-2054) and the factor 2 of the
 * ijkl symmetry (:1420-1428).  Grid: (determinant pair, task split); each
 * thread walks tasks, partial sums are reduced in a fixed order.
 *
 * With GRAD set the same walk also accumulates the adjoints: dE/dT on the
 * orbital-pair ERI matrix, dE/dS_orb and dE/dh_orb directly, and per
 * determinant pair the quantities that give dE/dA for each spin block:
 *   dv/dA = v T^T - det_a det_b J_other T^T (dJ/dT) T^T.
 */
#include <cuda_runtime.h>

#include "density.cuh"

namespace {

/* spin-orbital slot -> spatial orbital (the electron lists of vsvb_energy's
 * callers: bra(i) = i below num_non_docc, then two slots per DOCC orbital) */
__device__ __forceinline__ int spat(const DetCtx &d, int s) { return s < d.ds.nsd ? s : d.ds.nsd + (s - d.ds.nsd) / 2; }

__device__ __forceinline__ void slot_loc(const DetCtx &d, int sc, unsigned bits, int s, int &spin, int &pos) {
  const int np = d.ds.npair;
  if (s < 2 * np) {
    int k = d.slot_pair[sc * 2 * np + s];
    int wh = d.slot_which[sc * 2 * np + s];
    spin = wh ^ ((bits >> k) & 1);
    pos = k;
  } else if (s < d.ds.nnd) {
    spin = 0;
    pos = np + (s - 2 * np);
  } else {
    int dd = s - d.ds.nnd;
    if ((dd & 1) == 0) {
      spin = 0;
      pos = np + d.ds.nunpd + dd / 2;
    } else {
      spin = 1;
      pos = np + dd / 2;
    }
  }
}

__device__ __forceinline__ int pos_slot(const DetCtx &d, int sc, unsigned bits, int spin, int pos) {
  const int np = d.ds.npair;
  if (pos < np) {
    int bit = (bits >> pos) & 1;
    return d.pair_slot[(sc * np + pos) * 2 + (spin ^ bit)];
  }
  if (spin == 0) {
    if (pos < np + d.ds.nunpd) return 2 * np + (pos - np);
    return d.ds.nnd + 2 * (pos - np - d.ds.nunpd);
  }
  return d.ds.nnd + 2 * (pos - np) + 1;
}

struct QInfo {
  int isc, jsc;
  unsigned bb, kb;
  double w;
  /* after the determinant pairs are factorised (load_dets) */
  double da, db; /* det of the alpha / beta block */
  double wdd;    /* w * da * db */
  double wddr;   /* w * det(A + delta I) per block: wdd unless a block is flagged */
  int sing;      /* exact-minor flags per spin block */
  int abeq;      /* the beta block equals the alpha block (DetCtx.abeq) */
};

__device__ __forceinline__ QInfo decode_q(const DetCtx &d, long long q) {
  QInfo r;
  const int np = d.ds.npair;
  const unsigned mask = np > 0 ? ((1u << np) - 1u) : 0u;
  r.kb = (unsigned)(q & mask);
  r.bb = (unsigned)((q >> np) & mask);
  long long sp = q >> (2 * np);
  r.isc = (int)(sp / d.ds.nsc);
  r.jsc = (int)(sp % d.ds.nsc);
  r.w = d.coeff_sc[r.isc] * d.coeff_sc[r.jsc];
  r.da = r.db = r.wdd = r.wddr = 0.0;
  r.sing = 0;
  r.abeq = 0;
  return r;
}

__device__ __forceinline__ void load_dets(const DetCtx &d, long long q, QInfo &qi) {
  qi.da = d.det_a[q];
  qi.db = d.det_b[q];
  qi.wdd = qi.w * qi.da * qi.db;
  qi.sing = d.sing[q];
  qi.wddr = qi.sing ? qi.w * d.detr_a[q] * d.detr_b[q] : qi.wdd;
  qi.abeq = d.abeq ? d.abeq[q] : 0;
}

/* exact determinant of spin block sp of pair q with up to two strikes, from
 * the three perturbed factorisations of its slot (detpair_kernel) */
__device__ __noinline__ double struck_det_exact(const DetCtx &d, long long q, int sp, int ns, const int *rr,
                                                const int *cc) {
  const int slot = d.xslot[q];
  if (slot < 0 || slot >= d.xcap) return 0.0;
  const int na = d.ds.nalpha, nb = d.ds.nbeta, n = sp == 0 ? na : nb;
  const double *X = d.xinv + (size_t)slot * 3 * (na * na + nb * nb) + (sp == 0 ? 0 : 3 * (size_t)na * na);
  const double *dk = d.xdet + (size_t)slot * 6 + sp * 3;
  double f[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double *T = X + (size_t)k * n * n;
    double J = 1.0;
    if (ns == 1) J = T[cc[0] * n + rr[0]];
    else if (ns == 2) J = T[cc[0] * n + rr[0]] * T[cc[1] * n + rr[1]] - T[cc[0] * n + rr[1]] * T[cc[1] * n + rr[0]];
    f[k] = dk[k] * J;
  }
  return 3.0 * f[0] - 3.0 * f[1] + f[2];
}

struct Cof {
  bool ok;        /* spin integration non-zero */
  double v;       /* w * det_a * det_b * J_a * J_b */
  double vr;      /* the same from A + delta I on a flagged block (the
                   * adjoint's value; v elsewhere) */
  int na_s, nb_s; /* strikes per spin */
  int ra[2], ca[2], rb[2], cb[2];
  double Ja, Jb;  /* reduced factors */
};

/* spin and block position of a spin-orbital slot in the bra / ket determinant */
struct Loc {
  int spin, pos;
};

/* cofactor of determinant pair q for up to two strikes (bra slot -> ket
 * slot), given their locations */
__device__ Cof cofactor_loc(const DetCtx &d, long long q, const QInfo &qi, int nst, const Loc *lb, const Loc *lk) {
  Cof c;
  c.ok = false;
  c.v = c.vr = 0.0;
  c.na_s = c.nb_s = 0;
  c.Ja = c.Jb = 1.0;
  for (int t = 0; t < nst; ++t) {
    const int s1 = lb[t].spin, p1 = lb[t].pos, s2 = lk[t].spin, p2 = lk[t].pos;
    if (s1 != s2) return c;
    if (s1 == 0) {
      c.ra[c.na_s] = p1;
      c.ca[c.na_s] = p2;
      c.na_s++;
    } else {
      c.rb[c.nb_s] = p1;
      c.cb[c.nb_s] = p2;
      c.nb_s++;
    }
  }
  c.ok = true;
  const int na = d.ds.nalpha, nb = d.ds.nbeta;
  const int sing = qi.sing;
  /* J from the stored inverse: A^-1, or (A + delta I)^-1 on a flagged block */
  const double *Ta = d.Ta + (size_t)q * na * na;
  if (c.na_s == 1) c.Ja = Ta[c.ca[0] * na + c.ra[0]];
  else if (c.na_s == 2)
    c.Ja = Ta[c.ca[0] * na + c.ra[0]] * Ta[c.ca[1] * na + c.ra[1]] - Ta[c.ca[0] * na + c.ra[1]] * Ta[c.ca[1] * na + c.ra[0]];
  const double *Tb = d.Tb + (size_t)q * nb * nb;
  if (c.nb_s == 1) c.Jb = Tb[c.cb[0] * nb + c.rb[0]];
  else if (c.nb_s == 2)
    c.Jb = Tb[c.cb[0] * nb + c.rb[0]] * Tb[c.cb[1] * nb + c.rb[1]] - Tb[c.cb[0] * nb + c.rb[1]] * Tb[c.cb[1] * nb + c.rb[0]];
  if (!(sing & 3)) {
    c.v = c.vr = qi.wdd * (c.Ja * c.Jb);
    return c;
  }
  /* a flagged block: the value from exact struck determinants */
  const double fa = (sing & 1) && c.na_s > 0 ? struck_det_exact(d, q, 0, c.na_s, c.ra, c.ca) : qi.da * c.Ja;
  const double fb = (sing & 2) && c.nb_s > 0 ? struck_det_exact(d, q, 1, c.nb_s, c.rb, c.cb) : qi.db * c.Jb;
  c.v = qi.w * fa * fb;
  c.vr = qi.wddr * (c.Ja * c.Jb);
  return c;
}

__device__ __forceinline__ Loc loc_bra(const DetCtx &d, const QInfo &qi, int s) {
  Loc l;
  slot_loc(d, qi.isc, qi.bb, s, l.spin, l.pos);
  return l;
}
__device__ __forceinline__ Loc loc_ket(const DetCtx &d, const QInfo &qi, int s) {
  Loc l;
  slot_loc(d, qi.jsc, qi.kb, s, l.spin, l.pos);
  return l;
}

/* cofactor of determinant pair q for up to two (bra slot, ket slot) strikes */
__device__ __forceinline__ Cof cofactor(const DetCtx &d, long long q, const QInfo &qi, int nst, const int *sb,
                                        const int *sk) {
  Loc lb[2], lk[2];
  for (int t = 0; t < nst; ++t) {
    lb[t] = loc_bra(d, qi, sb[t]);
    lk[t] = loc_ket(d, qi, sk[t]);
  }
  return cofactor_loc(d, q, qi, nst, lb, lk);
}

/* dJ/dT accumulation for one cofactor with coefficient coef on v */
__device__ void accum_G(const DetCtx &d, long long q, const QInfo &qi, const Cof &c, double coef, double *Ga, double *Gb,
                        int lda, int ldb) {
  if (!c.ok || coef == 0.0) return;
  const int na = d.ds.nalpha, nb = d.ds.nbeta;
  const double dd = qi.wddr;
  if (c.na_s > 0) {
    const double *Ta = d.Ta + (size_t)q * na * na;
    const double f = coef * dd * c.Jb;
    if (c.na_s == 1) {
      atomicAdd(Ga + c.ca[0] * lda + c.ra[0], f);
    } else {
      atomicAdd(Ga + c.ca[0] * lda + c.ra[0], f * Ta[c.ca[1] * na + c.ra[1]]);
      atomicAdd(Ga + c.ca[1] * lda + c.ra[1], f * Ta[c.ca[0] * na + c.ra[0]]);
      atomicAdd(Ga + c.ca[0] * lda + c.ra[1], -f * Ta[c.ca[1] * na + c.ra[0]]);
      atomicAdd(Ga + c.ca[1] * lda + c.ra[0], -f * Ta[c.ca[0] * na + c.ra[1]]);
    }
  }
  if (c.nb_s > 0) {
    const double *Tb = d.Tb + (size_t)q * nb * nb;
    const double f = coef * dd * c.Ja;
    if (c.nb_s == 1) {
      atomicAdd(Gb + c.cb[0] * ldb + c.rb[0], f);
    } else {
      atomicAdd(Gb + c.cb[0] * ldb + c.rb[0], f * Tb[c.cb[1] * nb + c.rb[1]]);
      atomicAdd(Gb + c.cb[1] * ldb + c.rb[1], f * Tb[c.cb[0] * nb + c.rb[0]]);
      atomicAdd(Gb + c.cb[0] * ldb + c.rb[1], -f * Tb[c.cb[1] * nb + c.rb[0]]);
      atomicAdd(Gb + c.cb[1] * ldb + c.rb[0], -f * Tb[c.cb[0] * nb + c.rb[1]]);
    }
  }
}

__device__ double block_sum_d(double v, double *red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0) {
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
    red[0] = s;
  }
  __syncthreads();
  s = red[0];
  __syncthreads();
  return s;
}

__device__ __forceinline__ int opidx(int i, int k) { return i >= k ? i * (i + 1) / 2 + k : k * (k + 1) / 2 + i; }

/* xm_dtriang / xm_dtriang8: 1-based triangular index -> (i, j), j <= i.
 * An FP32 square root as the first guess (no FP64 on this path), then
 * exact integer correction. */
__device__ __forceinline__ void dtriang(long long ij, int &i, int &j) {
  long long ii = (long long)sqrtf((float)(2 * ij));
  while ((ii * ii + ii) / 2 < ij) ++ii;
  while (ii > 1 && ((ii - 1) * (ii - 1) + (ii - 1)) / 2 >= ij) --ii;
  i = (int)ii;
  j = (int)(ij - (ii * ii - ii) / 2);
}

}  // namespace

/* ---- determinant pairs: one block per q, Gauss-Jordan per spin block ---- */
namespace {
/* the fixed rank-2 matrix of the exact-minor path: P[r][c] = s (w1_r z1_c +
 * w2_r z2_c), entries of w and z from sin / cos of irrational steps */
__device__ __forceinline__ double pert_entry(int r, int c, double s) {
  const double w1 = sin(1.0 + 0.7548776662466927 * r), w2 = sin(2.0 + 0.5698402909980532 * r);
  const double z1 = cos(0.5 + 0.6180339887498949 * c), z2 = cos(1.5 + 0.4142135623730950 * c);
  return s * (w1 * z1 + w2 * z2);
}
}  // namespace

__global__ void __launch_bounds__(512) detpair_kernel(DetCtx d, double *scratch, int ld_scratch) {
  __shared__ double red[32];
  __shared__ int redi[32];
  __shared__ double sdet;
  __shared__ int ssing, spiv, sslot;
  const long long q = blockIdx.x;
  const QInfo qi = decode_q(d, q);
  double *W = scratch + (size_t)blockIdx.x * ld_scratch;
  if (threadIdx.x == 0) {
    sslot = -1;
    if (d.abeq) d.abeq[q] = 0;
  }
  __syncthreads();
  for (int sp = 0; sp < 2; ++sp) {
    const int n = sp == 0 ? d.ds.nalpha : d.ds.nbeta;
    double *Tout = (sp == 0 ? d.Ta : d.Tb) + (size_t)q * n * n;
    if (n == 0) {
      if (threadIdx.x == 0) (sp == 0 ? d.det_a : d.det_b)[q] = (sp == 0 ? d.detr_a : d.detr_b)[q] = 1.0;
      continue;
    }
    const int n2 = 2 * n;
    if (sp == 1 && n == d.ds.nalpha) {
      /* a beta block with the same orbitals as the unflagged alpha block
       * (doubly occupied orbitals only) takes its factorisation */
      int same = !(d.sing[q] & 1);
      for (int r = threadIdx.x; r < n && same; r += blockDim.x)
        same = spat(d, pos_slot(d, qi.isc, qi.bb, 0, r)) == spat(d, pos_slot(d, qi.isc, qi.bb, 1, r)) &&
               spat(d, pos_slot(d, qi.jsc, qi.kb, 0, r)) == spat(d, pos_slot(d, qi.jsc, qi.kb, 1, r));
      if (__syncthreads_and(same)) {
        const double *Ta = d.Ta + (size_t)q * n * n;
        for (int t = threadIdx.x; t < n * n; t += blockDim.x) Tout[t] = Ta[t];
        if (threadIdx.x == 0) {
          d.det_b[q] = d.det_a[q];
          d.detr_b[q] = d.detr_a[q];
          if (d.abeq) d.abeq[q] = d.ds.nunpd == 0;
        }
        __syncthreads();
        continue;
      }
    }
    /* W = [A + shift I + kp P | I]; returns max |A| over the block */
    auto fill = [&](double shift, double kp) -> double {
      double mx = 0.0;
      for (int t = threadIdx.x; t < n * n2; t += blockDim.x) {
        int r = t / n2, c = t - r * n2;
        double v;
        if (c < n) {
          int sb = spat(d, pos_slot(d, qi.isc, qi.bb, sp, r));
          int sk = spat(d, pos_slot(d, qi.jsc, qi.kb, sp, c));
          v = d.So[sb * d.ds.nsp + sk];
          mx = fmax(mx, fabs(v));
          if (c == r) v += shift;
          if (kp != 0.0) v += pert_entry(r, c, kp);
        } else {
          v = (c - n == r) ? 1.0 : 0.0;
        }
        W[t] = v;
      }
      for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
      __syncthreads();
      if (threadIdx.x == 0) {
        double m = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, red[w]);
        red[0] = m;
      }
      __syncthreads();
      const double amax = red[0];
      __syncthreads();
      return amax;
    };
    /* Gauss-Jordan with partial pivoting on W; false (and no inverse) when
     * a pivot is not above pmin; sdet holds the determinant */
    auto gj = [&](double pmin) -> bool {
      if (threadIdx.x == 0) {
        sdet = 1.0;
        ssing = 0;
      }
      __syncthreads();
      for (int k = 0; k < n; ++k) {
        double best = -1.0;
        int bi = k;
        for (int i = k + threadIdx.x; i < n; i += blockDim.x) {
          double v = fabs(W[i * n2 + k]);
          if (v > best) {
            best = v;
            bi = i;
          }
        }
        for (int o = 16; o > 0; o >>= 1) {
          double ob = __shfl_xor_sync(0xffffffffu, best, o);
          int oi = __shfl_xor_sync(0xffffffffu, bi, o);
          if (ob > best || (ob == best && oi < bi)) {
            best = ob;
            bi = oi;
          }
        }
        if ((threadIdx.x & 31) == 0) {
          red[threadIdx.x >> 5] = best;
          redi[threadIdx.x >> 5] = bi;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
          double b = -1.0;
          int p = k;
          for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
            if (red[w] > b || (red[w] == b && redi[w] < p)) {
              b = red[w];
              p = redi[w];
            }
          spiv = p;
          if (!(b > pmin)) ssing = 1;
        }
        __syncthreads();
        if (ssing) break;
        const int p = spiv;
        if (p != k) {
          for (int j = threadIdx.x; j < n2; j += blockDim.x) {
            double t = W[k * n2 + j];
            W[k * n2 + j] = W[p * n2 + j];
            W[p * n2 + j] = t;
          }
        }
        __syncthreads();
        const double piv = W[k * n2 + k];
        if (threadIdx.x == 0) sdet *= (p != k ? -piv : piv);
        __syncthreads();
        for (int j = threadIdx.x; j < n2; j += blockDim.x) W[k * n2 + j] /= piv;
        __syncthreads();
        /* rows to warps, columns to lanes; the pivot column becomes exactly
         * zero (f - f * 1) */
        {
          const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
          const double *prow = W + (size_t)k * n2;
          for (int i = threadIdx.x >> 5; i < n; i += nw) {
            if (i == k) continue;
            double *row = W + (size_t)i * n2;
            const double f = row[k];
            __syncwarp();
            if (f != 0.0)
              for (int j = lane; j < n2; j += 32) row[j] -= f * prow[j];
          }
        }
        __syncthreads();
      }
      const bool ok = !ssing;
      __syncthreads();
      return ok;
    };
    auto store_inverse = [&](double *dst) {
      for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
        int r = t / n, c = t - r * n;
        dst[t] = W[r * n2 + n + c];
      }
    };
    const double amax = fill(0.0, 0.0);
    if (gj(1e-7 * amax)) {
      store_inverse(Tout);
      if (threadIdx.x == 0) (sp == 0 ? d.det_a : d.det_b)[q] = (sp == 0 ? d.detr_a : d.detr_b)[q] = sdet;
      __syncthreads();
      continue;
    }
    /* a flagged block: pivots below 1e-7 of its largest entry */
    if (threadIdx.x == 0) {
      atomicOr(&d.sing[q], 1 << sp);
      if (sslot < 0) {
        const int sl = atomicAdd(d.xcount, 1);
        sslot = sl < d.xcap ? sl : d.xcap;
      }
    }
    __syncthreads();
    const int slot = sslot;
    double det0 = 0.0;
    if (slot < d.xcap) {
      const int na = d.ds.nalpha, nb = d.ds.nbeta;
      double *X = d.xinv + (size_t)slot * 3 * (na * na + nb * nb) + (sp == 0 ? 0 : 3 * (size_t)na * na);
      const double ps = 0.1 * amax * rsqrt((double)n);
      double f[3];
      for (int k = 0; k < 3; ++k) {
        fill(0.0, (k + 1) * ps);
        double *Xk = X + (size_t)k * n * n;
        if (gj(1e-11 * amax)) {
          store_inverse(Xk);
          f[k] = sdet;
        } else {
          /* rank deficiency of 3 or more: every struck determinant with at
           * most two strikes is zero */
          for (int t = threadIdx.x; t < n * n; t += blockDim.x) Xk[t] = 0.0;
          f[k] = 0.0;
        }
        if (threadIdx.x == 0) d.xdet[(size_t)slot * 6 + sp * 3 + k] = f[k];
        __syncthreads();
      }
      det0 = 3.0 * f[0] - 3.0 * f[1] + f[2];
    } else if (threadIdx.x == 0 && d.status) {
      atomicOr(d.status, 4);
    }
    if (threadIdx.x == 0) (sp == 0 ? d.det_a : d.det_b)[q] = det0;
    /* the adjoint's pair: det and inverse of A + delta I (delta = 1e-8 of
     * the largest entry) -- the derivative of every struck determinant of A
     * to about 5 delta relative, whatever the rank deficiency.  Only an
     * exactly zero pivot is reported (status 2): on transition blocks whose
     * left and right null vectors are nearly orthogonal the shifted pivots
     * fall to about 1e-8 of delta, and the derivative taken through det and
     * inverse together still matches central differences there */
    const double shift = 1e-8 * amax;
    fill(shift, 0.0);
    if (gj(0.0)) {
      store_inverse(Tout);
      if (threadIdx.x == 0) (sp == 0 ? d.detr_a : d.detr_b)[q] = sdet;
    } else {
      for (int t = threadIdx.x; t < n * n; t += blockDim.x) Tout[t] = 0.0;
      if (threadIdx.x == 0) {
        (sp == 0 ? d.detr_a : d.detr_b)[q] = 0.0;
        if (d.status) atomicOr(d.status, 2);
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    d.xslot[q] = sslot < d.xcap ? sslot : -1;
    if (d.nsing && d.sing[q]) atomicAdd(d.nsing, 1);
  }
}

/* ---- energy (and adjoint) assembly: grid (nq, nsplit) ---- */
/* MODE 0: energy partial sums (screened as the reference).
 * MODE 1: adjoint walk: dE/dS_orb, dE/dh_orb, per-pair dJ/dT; dE/dT as well
 *         unless a.skip_tbar.
 * MODE 2: unscreened density walk: Tbar += fac*dd at (ik,jl) and -fac*xd at
 *         (il,jk), unscaled by 1/W, for the single-sweep adjoint.
 * MODE 4: MODE 0 and MODE 1 (without dE/dT) in one walk, for the fused
 *         energy + gradient: the adjoint quantities are accumulated without
 *         1/W and E_num/W^2 -- those come later from the reduced energy
 *         (grad_scale_kernel) -- so the walk need not wait for it. */
template <int MODE>
__global__ void assemble_kernel(DetCtx d, AsmArgs a) {
  constexpr bool UNSC = MODE == 4;
  constexpr bool GRAD = MODE == 1 || UNSC;
  constexpr bool DENS = MODE == 2;
  __shared__ double red[8];
  extern __shared__ double gsh[];
  const long long q = blockIdx.x;
  const int split = blockIdx.y, nsplit = gridDim.y;
  QInfo qi = decode_q(d, q);
  load_dets(d, q, qi);
  /* nnd: num_non_docc of the task loop (spatial level); the spin structure
   * of the slots (slot_loc) keeps ds.nnd */
  const int nelec = d.ds.nelec, nnd = d.ds.nsd, nsp = d.ds.nsp;
  const int na = d.ds.nalpha, nb = d.ds.nbeta;
  double *Ga = nullptr, *Gb = nullptr;
  int lda = na, ldb = nb;
  if (GRAD) {
    if (a.g_in_smem) {
      /* g_in_smem = number of copies: one per warp (less atomic contention)
       * or one per block */
      const int ng = na * na + nb * nb;
      const int copy = a.g_in_smem > 1 ? (int)(threadIdx.x >> 5) % a.g_in_smem : 0;
      Ga = gsh + (size_t)copy * ng;
      Gb = Ga + na * na;
      for (int t = threadIdx.x; t < ng * a.g_in_smem; t += blockDim.x) gsh[t] = 0.0;
      __syncthreads();
    } else {
      Ga = a.Gglob + (size_t)q * (na * na + nb * nb);
      Gb = Ga + na * na;
    }
  }
  double e1 = 0.0, wf = 0.0, e2 = 0.0, vtot = 0.0, vtot_s = 0.0;
  double inv_w = UNSC ? 1.0 : a.inv_w, dw_coef = UNSC ? 0.0 : a.dw_coef;
  if (MODE == 1 && a.res) {
    const double W = a.res[4];
    inv_w = 1.0 / W;
    dw_coef = -a.res[1] / (W * W * (double)nelec);
  }
  const long long stride = (long long)nsplit * blockDim.x;
  /* one-electron part (valence.F90:1072-1101) */
  for (long long t = (long long)split * blockDim.x + threadIdx.x; !DENS && t < (long long)nelec * nelec; t += stride) {
    const int i = (int)(t / nelec), j = (int)(t % nelec);
    const bool idocc = i >= nnd, jdocc = j >= nnd;
    /* 1-based parity as in the reference: slots i+1, j+1 */
    if (idocc && jdocc && ((i + 1) & 1) != ((j + 1) & 1)) continue;
    int sb[1] = {i}, sk[1] = {j};
    Cof c = cofactor(d, q, qi, 1, sb, sk);
    if (!c.ok) continue;
    const int si = spat(d, i), sj = spat(d, j);
    const double h = d.Ho[si * nsp + sj], s = d.So[si * nsp + sj];
    e1 += h * c.v;
    wf += s * c.v;
    if (UNSC) {
      /* dE/dh part (scaled by 1/W later) and dE/dS part (scaled by
       * -E_num/(W^2 nelec) later) kept apart */
      vtot += h * c.vr;
      vtot_s += s * c.vr;
      accum_G(d, q, qi, c, h, Ga, Gb, lda, ldb);
      double *Gsa = a.Gs + (size_t)q * (na * na + nb * nb);
      accum_G(d, q, qi, c, s, Gsa, Gsa + na * na, na, nb);
      atomicAdd(a.D1 + si * nsp + sj, c.v);
    } else if (GRAD) {
      const double coef = h * inv_w + dw_coef * s;
      vtot += coef * c.vr;
      accum_G(d, q, qi, c, coef, Ga, Gb, lda, ldb);
      atomicAdd(a.Hbar + si * nsp + sj, c.v * inv_w);
      atomicAdd(a.Sbar + si * nsp + sj, c.v * dw_coef);
    }
  }
  /* two-electron tasks (valence.F90:1153-1433) */
  const int np = a.np;
  const double itol = a.itol;
  for (long long task = (long long)split * blockDim.x + threadIdx.x; task < a.ntasks; task += stride) {
    int ijorb, klorb, io, jo, ko, lo;
    dtriang(task + 1, ijorb, klorb);
    dtriang(ijorb, io, jo);
    dtriang(klorb, ko, lo);
    --io;
    --jo;
    --ko;
    --lo; /* 0-based orbitals */
    if ((io == jo && io < nnd) || (ko == lo && ko < nnd)) continue;
    const int pik = opidx(io, ko), pjl = opidx(jo, lo), pil = opidx(io, lo), pjk = opidx(jo, ko);
    double sik = 0.0, sjl = 0.0, sil = 0.0, sjk = 0.0;
    if (!DENS) {
      sik = a.sq[pik];
      sjl = a.sq[pjl];
      sil = a.sq[pil];
      sjk = a.sq[pjk];
    }
    bool es = sik * sjl > itol, xs = sil * sjk > itol;
    double eint = 0.0, xint = 0.0;
    const bool diag = io == jo && ko == lo;
    if (DENS) {
      es = xs = true;
    } else {
      if (es || xs) {
        if (diag) {
          eint = sik * sik;
          xint = eint;
        } else {
          if (es) eint = a.T[(size_t)pik * np + pjl];
          if (xs) xint = a.T[(size_t)pil * np + pjk];
        }
      }
      es = fabs(eint) > itol;
      xs = fabs(xint) > itol;
      if (!(es || xs)) continue;
    }
    const double fac = (ko == io && lo == jo) ? 1.0 : 2.0;
    const double fw = fac * inv_w;
    const bool id = io >= nnd, jd = jo >= nnd, kd = ko >= nnd, ld = lo >= nnd;
    const int iso = id ? 2 : 1, jso = jd ? 2 : 1, kso = kd ? 2 : 1, lso = ld ? 2 : 1;
    double esum = 0.0, xsum = 0.0, dsum_e = 0.0, dsum_x = 0.0;
    if (MODE == 0 && qi.abeq && id && jd && kd && ld) {
      /* four doubly occupied orbitals and one factorisation for both spin
       * blocks: every cofactor of the 16 spin terms comes from the four
       * inverse entries T[k][i], T[l][j], T[l][i], T[k][j] (block positions
       * do not depend on the spin without unpaired electrons) */
      const int ia = 2 * (io + 1) - nnd - 2, ja = 2 * (jo + 1) - nnd - 2;
      const int ka = 2 * (ko + 1) - nnd - 2, la = 2 * (lo + 1) - nnd - 2;
      const int pi_ = loc_bra(d, qi, ia).pos, pj_ = loc_bra(d, qi, ja).pos;
      const int pk_ = loc_ket(d, qi, ka).pos, pl_ = loc_ket(d, qi, la).pos;
      const double *Tq = d.Ta + (size_t)q * na * na;
      const double tki = Tq[pk_ * na + pi_], tlj = Tq[pl_ * na + pj_];
      const double tli = Tq[pl_ * na + pi_], tkj = Tq[pk_ * na + pj_];
      /* The 16 spin terms in closed form.  Slot parity is spin, so the
       * DOCC parity skips (:1352-1375) keep the terms whose strikes stay in
       * one spin block; with the slot orders j < i, l < k of the task loop:
       *   io > jo, ko > lo: (aa|aa), (bb|bb) give J2 direct and exchanged
       *     (the column-swap rule of det(), :2041-2054), (ab|ab), (ba|ba)
       *     t_ki t_lj direct, (ab|ba), (ba|ab) -t_li t_kj exchanged;
       *   one of io = jo, ko = lo: one direct t_ki t_lj, one exchanged
       *     -t_li t_kj;  both: one direct t_ki t_lj,
       * J2 = t_ki t_lj - t_kj t_li, each term times w det_a det_b. */
      const double a = tki * tlj, x = tli * tkj, j2 = a - tkj * tli;
      double de, dx;
      if (io != jo && ko != lo) {
        de = 2.0 * qi.wdd * (j2 + a);
        dx = 2.0 * qi.wdd * (j2 - x);
      } else if (io != jo || ko != lo) {
        de = qi.wdd * a;
        dx = -qi.wdd * x;
      } else {
        de = qi.wdd * a;
        dx = 0.0;
      }
      if (es) dsum_e = de;
      if (xs) dsum_x = dx;
    } else
    for (int is = 0; is < iso; ++is) {
      /* 0-based slot; 1-based formula 2*io - nnd + is - 2 with 1-based io */
      const int i = id ? 2 * (io + 1) - nnd + (is + 1) - 2 - 1 : io;
      const Loc Li = loc_bra(d, qi, i);
      for (int js = 0; js < jso; ++js) {
        const int j = jd ? 2 * (jo + 1) - nnd + (js + 1) - 2 - 1 : jo;
        if (!(j < i)) continue;
        const Loc Lb[2] = {Li, loc_bra(d, qi, j)};
        for (int ks = 0; ks < kso; ++ks) {
          const int k = kd ? 2 * (ko + 1) - nnd + (ks + 1) - 2 - 1 : ko;
          const Loc Lk = loc_ket(d, qi, k);
          for (int ls = 0; ls < lso; ++ls) {
            const int l = ld ? 2 * (lo + 1) - nnd + (ls + 1) - 2 - 1 : lo;
            if (!(l < k)) continue;
            const Loc Ll = loc_ket(d, qi, l);
            /* 1-based parity for the DOCC spin integration */
            const bool ik0 = id && kd && ((i + 1) & 1) != ((k + 1) & 1);
            const bool jl0 = jd && ld && ((j + 1) & 1) != ((l + 1) & 1);
            const bool il0 = id && ld && ((i + 1) & 1) != ((l + 1) & 1);
            const bool jk0 = jd && kd && ((j + 1) & 1) != ((k + 1) & 1);
            const bool ce = !(ik0 || jl0), cx = !(il0 || jk0);
            if (!((ce && es) || (cx && xs))) continue;
            Cof ce_c, cx_c;
            ce_c.ok = false;
            cx_c.ok = false;
            if (es) {
              const Loc lk[2] = {Lk, Ll};
              ce_c = cofactor_loc(d, q, qi, 2, Lb, lk);
            }
            if (xs) {
              if (es && ce_c.ok) {
                /* both strikes of the direct cofactor in one spin block: the
                 * exchanged one is its column swap, -v exactly, and only
                 * whether it is allowed matters below (det()'s sign rule) */
                cx_c.ok = Lb[0].spin == Ll.spin && Lb[1].spin == Lk.spin;
              } else {
                const Loc lk[2] = {Ll, Lk};
                cx_c = cofactor_loc(d, q, qi, 2, Lb, lk);
              }
            }
            double dd = 0.0, xd = 0.0;
            if (es && ce_c.ok) dd = ce_c.v;
            if (xs && cx_c.ok) xd = (es && ce_c.ok) ? ce_c.v : -cx_c.v;
            /* the task's integrals are common to its spin terms: the sums
             * take the densities, the integrals multiply once below */
            if (es) dsum_e += dd;
            if (xs) dsum_x += xd;
            if (GRAD) {
              /* coefficients of the two cofactors in fac*(dd*eint - xd*xint)/W */
              double cve = 0.0, cvx = 0.0;
              if (es && ce_c.ok) {
                cve = eint;
                if (xs && cx_c.ok) cve -= xint;
              } else if (xs && cx_c.ok) {
                cvx = xint;
              }
              cve *= fw;
              cvx *= fw;
              if (ce_c.ok && cve != 0.0) {
                vtot += cve * ce_c.vr;
                accum_G(d, q, qi, ce_c, cve, Ga, Gb, lda, ldb);
              }
              if (cx_c.ok && cvx != 0.0) {
                vtot += cvx * cx_c.vr;
                accum_G(d, q, qi, cx_c, cvx, Ga, Gb, lda, ldb);
              }
            }
          }
        }
      }
    }
    esum = dsum_e * eint;
    xsum = dsum_x * xint;
    e2 += fac * (esum - xsum);
    if (DENS) {
      if (diag) {
        atomicAdd(a.Tbar + (size_t)pik * np + pik, fac * (dsum_e - dsum_x));
      } else {
        if (dsum_e != 0.0) atomicAdd(a.Tbar + (size_t)pik * np + pjl, fac * dsum_e);
        if (dsum_x != 0.0) atomicAdd(a.Tbar + (size_t)pil * np + pjk, -fac * dsum_x);
      }
    }
    if (GRAD && !a.skip_tbar) {
      const double ge = fac * inv_w * dsum_e, gx = -fac * inv_w * dsum_x;
      if (diag) {
        if (es || xs) atomicAdd(a.Tbar + (size_t)pik * np + pik, (es ? ge : 0.0) + (xs ? gx : 0.0));
      } else {
        if (es && ge != 0.0) atomicAdd(a.Tbar + (size_t)pik * np + pjl, ge);
        if (xs && gx != 0.0) atomicAdd(a.Tbar + (size_t)pil * np + pjk, gx);
      }
    }
  }
  e1 = block_sum_d(e1, red);
  wf = block_sum_d(wf, red);
  e2 = block_sum_d(e2, red);
  const size_t slot = (size_t)q * nsplit + split;
  if (UNSC) {
    vtot_s = block_sum_d(vtot_s, red);
    if (threadIdx.x == 0) {
      a.vtot_s[slot] = vtot_s;
      a.part_e1[slot] = e1;
      a.part_wf[slot] = wf;
      a.part_e2[slot] = e2;
    }
  }
  if (GRAD) {
    vtot = block_sum_d(vtot, red);
    if (threadIdx.x == 0) a.vtot[slot] = vtot;
    if (a.g_in_smem) {
      __syncthreads();
      const int ng = na * na + nb * nb;
      double *Gq = a.Gglob + (size_t)q * ng;
      for (int t = threadIdx.x; t < ng; t += blockDim.x) {
        double v = 0.0;
        for (int c = 0; c < a.g_in_smem; ++c) v += gsh[(size_t)c * ng + t];
        if (v != 0.0) atomicAdd(Gq + t, v);
      }
    }
  } else if (!DENS && threadIdx.x == 0) {
    a.part_e1[slot] = e1;
    a.part_wf[slot] = wf;
    a.part_e2[slot] = e2;
  }
}

/* fixed-order reduction of the partial sums (one block) */
__global__ void energy_reduce_kernel(AsmArgs a, long long nslot, int nelec, double enuc, double *out) {
  __shared__ double red[8];
  double e1 = 0.0, wf = 0.0, e2 = 0.0;
  for (long long t = threadIdx.x; t < nslot; t += blockDim.x) {
    e1 += a.part_e1[t];
    wf += a.part_wf[t];
    e2 += a.part_e2[t];
  }
  e1 = block_sum_d(e1, red);
  wf = block_sum_d(wf, red);
  e2 = block_sum_d(e2, red);
  if (threadIdx.x == 0) {
    double w = wf / (double)nelec;
    out[0] = (e1 + e2) / w + enuc; /* energy */
    out[1] = e1 + e2;
    out[2] = e1;
    out[3] = e2;
    out[4] = w;
  }
}

/* per determinant pair: dE/dA = vtot T^T - T^T G T^T for each spin block,
 * scattered onto dE/dS_orb */
__global__ void detpair_adjoint_kernel(DetCtx d, AsmArgs a, int nsplit) {
  __shared__ double red[8];
  const long long q = blockIdx.x;
  const QInfo qi = decode_q(d, q);
  double vt = 0.0;
  for (int s = threadIdx.x; s < nsplit; s += blockDim.x) vt += a.vtot[(size_t)q * nsplit + s];
  vt = block_sum_d(vt, red);
  const int na = d.ds.nalpha, nb = d.ds.nbeta, nsp = d.ds.nsp;
  const double *Gq = a.Gglob + (size_t)q * (na * na + nb * nb);
  for (int sp = 0; sp < 2; ++sp) {
    const int n = sp == 0 ? na : nb;
    if (n == 0) continue;
    const double *T = (sp == 0 ? d.Ta : d.Tb) + (size_t)q * n * n;
    const double *G = Gq + (sp == 0 ? 0 : na * na);
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
      const int ar = t / n, bc = t - ar * n; /* dE/dA[ar][bc] */
      /* (T^T G T^T)[ar][bc] = sum_xy T[x][ar] G[x][y] T[bc][y] */
      double s = 0.0;
      for (int x = 0; x < n; ++x) {
        const double tx = T[x * n + ar];
        if (tx == 0.0) continue;
        double inner = 0.0;
        for (int y = 0; y < n; ++y) inner += G[x * n + y] * T[bc * n + y];
        s += tx * inner;
      }
      const double abar = vt * T[bc * n + ar] - s;
      const int sb = spat(d, pos_slot(d, qi.isc, qi.bb, sp, ar));
      const int sk = spat(d, pos_slot(d, qi.jsc, qi.kb, sp, bc));
      atomicAdd(a.Sbar + sb * nsp + sk, abar);
    }
  }
}

/* after the MODE 4 walk and the energy reduction: dJ/dT, vtot, dE/dh and
 * dE/dS with 1/W and -E_num/(W^2 nelec) applied (one block per determinant
 * pair; block 0 also writes Hbar and Sbar over the orbital pairs) */
__global__ void grad_scale_kernel(DetCtx d, AsmArgs a, int nsplit) {
  const long long q = blockIdx.x;
  const double W = a.res[4];
  const double inv_w = 1.0 / W, dw = -a.res[1] / (W * W * (double)d.ds.nelec);
  const int ng = d.ds.nalpha * d.ds.nalpha + d.ds.nbeta * d.ds.nbeta;
  double *G = a.Gglob + (size_t)q * ng;
  const double *Gs = a.Gs + (size_t)q * ng;
  for (int t = threadIdx.x; t < ng; t += blockDim.x) G[t] = inv_w * G[t] + dw * Gs[t];
  for (int s = threadIdx.x; s < nsplit; s += blockDim.x) {
    const size_t slot = (size_t)q * nsplit + s;
    a.vtot[slot] = inv_w * a.vtot[slot] + dw * a.vtot_s[slot];
  }
  if (q == 0) {
    const int n2 = d.ds.nsp * d.ds.nsp;
    for (int t = threadIdx.x; t < n2; t += blockDim.x) {
      a.Hbar[t] = inv_w * a.D1[t];
      a.Sbar[t] = dw * a.D1[t];
    }
  }
}

/* the MODE 4 accumulators combined for the derivative of alpha * E_num +
 * beta * W * nelec instead of E = E_num / W: (1, 0) gives dE_num, (0,
 * 1/nelec) dW -- the two first_order_opt matrices come from these (one
 * block per determinant pair; block 0 also writes Hbar and Sbar) */
__global__ void hs_scale_kernel(DetCtx d, AsmArgs a, int nsplit, double alpha, double beta) {
  const long long q = blockIdx.x;
  const int ng = d.ds.nalpha * d.ds.nalpha + d.ds.nbeta * d.ds.nbeta;
  double *G = a.Gglob + (size_t)q * ng;
  const double *Gs = a.Gs + (size_t)q * ng;
  for (int t = threadIdx.x; t < ng; t += blockDim.x) G[t] = alpha * G[t] + beta * Gs[t];
  for (int s = threadIdx.x; s < nsplit; s += blockDim.x) {
    const size_t slot = (size_t)q * nsplit + s;
    a.vtot[slot] = alpha * a.vtot[slot] + beta * a.vtot_s[slot];
  }
  if (q == 0) {
    const int n2 = d.ds.nsp * d.ds.nsp;
    for (int t = threadIdx.x; t < n2; t += blockDim.x) {
      a.Hbar[t] = alpha * a.D1[t];
      a.Sbar[t] = beta * a.D1[t];
    }
  }
}

/* spin_opt's matrices (valence.F90:850-897) from the partial sums of one
 * walk with every coupling weight 1: block (isc, jsc) sums the energy
 * numerator and the norm of its determinant pairs in a fixed order.  One
 * block per (isc, jsc). */
__global__ void spin_block_kernel(DetCtx d, AsmArgs a, int nsplit, double *BH, double *BS) {
  __shared__ double red[8];
  const int blk = blockIdx.x; /* isc * nsc + jsc */
  const long long per = 1LL << (2 * d.ds.npair);
  const long long s0 = (long long)blk * per * nsplit, n = per * nsplit;
  double h = 0.0, w = 0.0;
  for (long long t = threadIdx.x; t < n; t += blockDim.x) {
    h += a.part_e1[s0 + t] + a.part_e2[s0 + t];
    w += a.part_wf[s0 + t];
  }
  h = block_sum_d(h, red);
  w = block_sum_d(w, red);
  if (threadIdx.x == 0) {
    BH[blk] = h;
    BS[blk] = w / (double)d.ds.nelec;
  }
}

cudaError_t launch_assemble(int mode, dim3 grid, int threads, size_t smem, cudaStream_t st, const DetCtx &d,
                            const AsmArgs &a) {
  if (mode == 1) {
    if (smem > 48 * 1024) cudaFuncSetAttribute(assemble_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    assemble_kernel<1><<<grid, threads, smem, st>>>(d, a);
  } else if (mode == 4) {
    if (smem > 48 * 1024) cudaFuncSetAttribute(assemble_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    assemble_kernel<4><<<grid, threads, smem, st>>>(d, a);
  } else if (mode == 2) {
    assemble_kernel<2><<<grid, threads, 0, st>>>(d, a);
  } else {
    assemble_kernel<0><<<grid, threads, 0, st>>>(d, a);
  }
  return cudaGetLastError();
}
