/*
 * ints.c -- ORACLE (test infrastructure): Gaussian integrals over Cartesian
 * shells, restating what VALENCE obtains from simint
 * (simint_compute_overlap / _ke / _potential / _eri, call sites
 * valence.F90:2988, 3132, 3151, 3398).  simint itself is an un-vendored,
 * unpinned third-party dependency (install-simint.sh:4), so the arithmetic
 * here follows the published methods:
 *   Boys function: Taylor-free series  F_m(T) = e^{-T} sum_k (2T)^k /
 *     ((2m+1)(2m+3)...(2m+2k+1)) for T < 30 with downward recursion, and
 *     F_0 = sqrt(pi/T) erf(sqrt T)/2 with upward recursion above.
 *   Overlap / kinetic: Obara & Saika (J. Chem. Phys. 84, 3963 (1986)) 1D
 *     recursions; kinetic as (1/2)<grad a|grad b>.
 *   Nuclear attraction: Obara-Saika auxiliary recursion, then horizontal
 *     transfer to the second centre.
 *   ERI: Head-Gordon & Pople (J. Chem. Phys. 89, 5777 (1988)) vertical
 *     recursion [e0|f0]^(m), primitive contraction, then horizontal
 *     recursions on both sides.
 * Component order within a shell is CCA (valence.F90:2364-2378):
 *   for i=0..l, j=0..i: (l-i, i-j, j).
 * Primitives are the plain x^a y^b z^c exp(-alpha r^2) times the shell's
 * contraction coefficient; VALENCE applies its own norm_prim coefficients and
 * per-component angn factors outside the integral call.
 */
#include "oracle_internal.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define PI 3.14159265358979323846

void vo_boys(int mmax, double t, double *f) {
  if (t < 30.0) {
    /* series for the top order, then downward recursion */
    double et = exp(-t);
    double term = 1.0 / (2 * mmax + 1);
    double sum = term;
    for (int k = 1; k < 400; ++k) {
      term *= 2.0 * t / (2 * mmax + 2 * k + 1);
      sum += term;
      if (term < sum * 1e-17) break;
    }
    f[mmax] = et * sum;
    for (int m = mmax - 1; m >= 0; --m) f[m] = (2.0 * t * f[m + 1] + et) / (2 * m + 1);
  } else {
    double et = exp(-t);
    double st = sqrt(t);
    f[0] = 0.5 * sqrt(PI) / st * erf(st);
    for (int m = 0; m < mmax; ++m) f[m + 1] = ((2 * m + 1) * f[m] - et) / (2.0 * t);
  }
}

/* --- Cartesian indexing ------------------------------------------------ */

int vo_ncart(int l) { return (l + 1) * (l + 2) / 2; }
static int ncart_upto(int l) { return (l + 1) * (l + 2) * (l + 3) / 6; }
/* index of (x,y,z) among all Cartesians of total order <= L */
static int cidx(int x, int y, int z) {
  int l = x + y + z;
  int i = l - x;
  (void)y;
  return l * (l + 1) * (l + 2) / 6 + i * (i + 1) / 2 + z;
}
void vo_cart_comp(int l, int k, int *x, int *y, int *z) {
  int n = 0;
  for (int i = 0; i <= l; ++i)
    for (int j = 0; j <= i; ++j) {
      if (n == k) {
        *x = l - i;
        *y = i - j;
        *z = j;
        return;
      }
      ++n;
    }
}

/* --- one-electron --------------------------------------------------------- */

static void os1d(double a, double b, double xa, double xb, int imax, int jmax, double *s, int ld) {
  /* s[i*ld + j] for i<=imax, j<=jmax : 1D overlap of x^i e^{-a(x-xa)^2}, x^j e^{-b(x-xb)^2} */
  double p = a + b;
  double xp = (a * xa + b * xb) / p;
  double xpa = xp - xa, xpb = xp - xb, oo2p = 0.5 / p;
  double mu = a * b / p;
  double d = xa - xb;
  s[0] = sqrt(PI / p) * exp(-mu * d * d);
  for (int i = 0; i <= imax; ++i) {
    if (i > 0) {
      /* build column j=0 from i-1 */
      double v = xpa * s[(i - 1) * ld + 0];
      if (i > 1) v += oo2p * (i - 1) * s[(i - 2) * ld + 0];
      s[i * ld + 0] = v;
    }
    for (int j = 1; j <= jmax; ++j) {
      double v = xpb * s[i * ld + j - 1];
      if (i > 0) v += oo2p * i * s[(i - 1) * ld + j - 1];
      if (j > 1) v += oo2p * (j - 1) * s[i * ld + j - 2];
      s[i * ld + j] = v;
    }
  }
}

void vo_shell_overlap_kinetic(const vo_shell *A, const vo_shell *B, double *ov, double *ke) {
  int na = vo_ncart(A->l), nb = vo_ncart(B->l);
  int la = A->l, lb = B->l;
  for (int i = 0; i < na * nb; ++i) {
    if (ov) ov[i] = 0.0;
    if (ke) ke[i] = 0.0;
  }
  enum { LD = 8 };
  double sx[LD * LD], sy[LD * LD], sz[LD * LD];
  for (int pa = 0; pa < A->nprim; ++pa)
    for (int pb = 0; pb < B->nprim; ++pb) {
      double a = A->alpha[pa], b = B->alpha[pb];
      double c = A->coef[pa] * B->coef[pb];
      os1d(a, b, A->xyz[0], B->xyz[0], la + 1, lb + 1, sx, LD);
      os1d(a, b, A->xyz[1], B->xyz[1], la + 1, lb + 1, sy, LD);
      os1d(a, b, A->xyz[2], B->xyz[2], la + 1, lb + 1, sz, LD);
      for (int ia = 0; ia < na; ++ia) {
        int ax, ay, az;
        vo_cart_comp(la, ia, &ax, &ay, &az);
        for (int ib = 0; ib < nb; ++ib) {
          int bx, by, bz;
          vo_cart_comp(lb, ib, &bx, &by, &bz);
          double Sx = sx[ax * LD + bx], Sy = sy[ay * LD + by], Sz = sz[az * LD + bz];
          if (ov) ov[ia * nb + ib] += c * Sx * Sy * Sz;
          if (ke) {
            /* T_1d(i,j) = 1/2 <d/dx a | d/dx b> */
#define TK(s, i, j)                                                                       \
  (0.5 * (((i) > 0 && (j) > 0 ? (double)(i) * (j) * s[((i)-1) * LD + (j)-1] : 0.0) -      \
          ((i) > 0 ? 2.0 * b * (i) * s[((i)-1) * LD + (j) + 1] : 0.0) -                   \
          ((j) > 0 ? 2.0 * a * (j) * s[((i) + 1) * LD + (j)-1] : 0.0) +                   \
          4.0 * a * b * s[((i) + 1) * LD + (j) + 1]))
            double Tx = TK(sx, ax, bx), Ty = TK(sy, ay, by), Tz = TK(sz, az, bz);
#undef TK
            ke[ia * nb + ib] += c * (Tx * Sy * Sz + Sx * Ty * Sz + Sx * Sy * Tz);
          }
        }
      }
    }
}

void vo_shell_nuclear(const vo_shell *A, const vo_shell *B, double zc, const double *C, double *out) {
  int la = A->l, lb = B->l, L = la + lb;
  int na = vo_ncart(la), nb = vo_ncart(lb);
  int nall = ncart_upto(L);
  double *acc = (double *)calloc((size_t)nall, sizeof(double));
  double *v = (double *)malloc(sizeof(double) * (size_t)nall * (L + 1));
  double fm[32];
  double ab[3] = {A->xyz[0] - B->xyz[0], A->xyz[1] - B->xyz[1], A->xyz[2] - B->xyz[2]};
  double ab2 = ab[0] * ab[0] + ab[1] * ab[1] + ab[2] * ab[2];
  for (int pa = 0; pa < A->nprim; ++pa)
    for (int pb = 0; pb < B->nprim; ++pb) {
      double a = A->alpha[pa], b = B->alpha[pb], p = a + b;
      double P[3], PA[3], PC[3];
      for (int d = 0; d < 3; ++d) {
        P[d] = (a * A->xyz[d] + b * B->xyz[d]) / p;
        PA[d] = P[d] - A->xyz[d];
        PC[d] = P[d] - C[d];
      }
      double pc2 = PC[0] * PC[0] + PC[1] * PC[1] + PC[2] * PC[2];
      double pref = 2.0 * PI / p * exp(-a * b / p * ab2) * A->coef[pa] * B->coef[pb];
      vo_boys(L, p * pc2, fm);
      /* v[m*nall + idx] = (e|A^(m)|0) */
      for (int m = 0; m <= L; ++m) v[m * nall + 0] = pref * fm[m];
      for (int el = 1; el <= L; ++el)
        for (int i = 0; i <= el; ++i)
          for (int j = 0; j <= i; ++j) {
            int e[3] = {el - i, i - j, j};
            int d = e[0] ? 0 : (e[1] ? 1 : 2);
            int e1[3] = {e[0], e[1], e[2]};
            e1[d]--;
            int i1 = cidx(e1[0], e1[1], e1[2]);
            int i2 = -1;
            if (e1[d] > 0) {
              int e2[3] = {e1[0], e1[1], e1[2]};
              e2[d]--;
              i2 = cidx(e2[0], e2[1], e2[2]);
            }
            int ie = cidx(e[0], e[1], e[2]);
            for (int m = 0; m <= L - el; ++m) {
              double val = PA[d] * v[m * nall + i1] - PC[d] * v[(m + 1) * nall + i1];
              if (i2 >= 0) val += e1[d] / (2.0 * p) * (v[m * nall + i2] - v[(m + 1) * nall + i2]);
              v[m * nall + ie] = val;
            }
          }
      for (int k = 0; k < nall; ++k) acc[k] += v[k];
    }
  /* horizontal transfer to B: (a|b+1_i) = (a+1_i|b) + AB_i (a|b) */
  int nb_all = ncart_upto(lb);
  double *h = (double *)calloc((size_t)nall * nb_all, sizeof(double));
  for (int k = 0; k < nall; ++k) h[k * nb_all + 0] = acc[k];
  for (int bl = 1; bl <= lb; ++bl)
    for (int i = 0; i <= bl; ++i)
      for (int j = 0; j <= i; ++j) {
        int bb[3] = {bl - i, i - j, j};
        int d = bb[0] ? 0 : (bb[1] ? 1 : 2);
        int b1[3] = {bb[0], bb[1], bb[2]};
        b1[d]--;
        int ib = cidx(bb[0], bb[1], bb[2]), ib1 = cidx(b1[0], b1[1], b1[2]);
        for (int al = la; al <= L - bl; ++al)
          for (int ii = 0; ii <= al; ++ii)
            for (int jj = 0; jj <= ii; ++jj) {
              int aa[3] = {al - ii, ii - jj, jj};
              int ap[3] = {aa[0], aa[1], aa[2]};
              ap[d]++;
              int ia = cidx(aa[0], aa[1], aa[2]), iap = cidx(ap[0], ap[1], ap[2]);
              h[ia * nb_all + ib] = h[iap * nb_all + ib1] + ab[d] * h[ia * nb_all + ib1];
            }
      }
  for (int ia = 0; ia < na; ++ia) {
    int ax, ay, az;
    vo_cart_comp(la, ia, &ax, &ay, &az);
    for (int ib = 0; ib < nb; ++ib) {
      int bx, by, bz;
      vo_cart_comp(lb, ib, &bx, &by, &bz);
      out[ia * nb + ib] = -zc * h[cidx(ax, ay, az) * nb_all + cidx(bx, by, bz)];
    }
  }
  free(h);
  free(v);
  free(acc);
}

/* --- two-electron (HGP) --------------------------------------------------- */

void vo_shell_eri(const vo_shell *A, const vo_shell *B, const vo_shell *C, const vo_shell *D, double *out) {
  int la = A->l, lb = B->l, lc = C->l, ld = D->l;
  int le = la + lb, lf = lc + ld, M = le + lf;
  int ne = ncart_upto(le), nf = ncart_upto(lf);
  double *V = (double *)malloc(sizeof(double) * (size_t)(M + 1) * ne * nf);
  double *G = (double *)calloc((size_t)ne * nf, sizeof(double));
  double fm[40];
  double AB[3], CD[3];
  for (int d = 0; d < 3; ++d) {
    AB[d] = A->xyz[d] - B->xyz[d];
    CD[d] = C->xyz[d] - D->xyz[d];
  }
  double ab2 = AB[0] * AB[0] + AB[1] * AB[1] + AB[2] * AB[2];
  double cd2 = CD[0] * CD[0] + CD[1] * CD[1] + CD[2] * CD[2];
#define VV(m, e, f) V[((size_t)(m) * ne + (e)) * nf + (f)]
  for (int pa = 0; pa < A->nprim; ++pa)
    for (int pb = 0; pb < B->nprim; ++pb) {
      double a = A->alpha[pa], b = B->alpha[pb], p = a + b;
      double P[3];
      for (int d = 0; d < 3; ++d) P[d] = (a * A->xyz[d] + b * B->xyz[d]) / p;
      double kab = exp(-a * b / p * ab2) * A->coef[pa] * B->coef[pb];
      for (int pc = 0; pc < C->nprim; ++pc)
        for (int pd = 0; pd < D->nprim; ++pd) {
          double c = C->alpha[pc], dd = D->alpha[pd], q = c + dd;
          double Q[3], W[3], PA[3], WP[3], QC[3], WQ[3];
          for (int d = 0; d < 3; ++d) Q[d] = (c * C->xyz[d] + dd * D->xyz[d]) / q;
          double kcd = exp(-c * dd / q * cd2) * C->coef[pc] * D->coef[pd];
          double rho = p * q / (p + q);
          double pq2 = 0.0;
          for (int d = 0; d < 3; ++d) {
            W[d] = (p * P[d] + q * Q[d]) / (p + q);
            PA[d] = P[d] - A->xyz[d];
            WP[d] = W[d] - P[d];
            QC[d] = Q[d] - C->xyz[d];
            WQ[d] = W[d] - Q[d];
            pq2 += (P[d] - Q[d]) * (P[d] - Q[d]);
          }
          double pref = 2.0 * pow(PI, 2.5) / (p * q * sqrt(p + q)) * kab * kcd;
          vo_boys(M, rho * pq2, fm);
          double oo2p = 0.5 / p, oo2q = 0.5 / q, oo2pq = 0.5 / (p + q), rp = rho / p, rq = rho / q;
          /* f = 0 column: build [e0|00]^(m) */
          for (int m = 0; m <= M; ++m) VV(m, 0, 0) = pref * fm[m];
          for (int el = 1; el <= le; ++el)
            for (int i = 0; i <= el; ++i)
              for (int j = 0; j <= i; ++j) {
                int e[3] = {el - i, i - j, j};
                int d = e[0] ? 0 : (e[1] ? 1 : 2);
                int e1[3] = {e[0], e[1], e[2]};
                e1[d]--;
                int ie = cidx(e[0], e[1], e[2]), i1 = cidx(e1[0], e1[1], e1[2]), i2 = -1;
                if (e1[d] > 0) {
                  int e2[3] = {e1[0], e1[1], e1[2]};
                  e2[d]--;
                  i2 = cidx(e2[0], e2[1], e2[2]);
                }
                for (int m = 0; m <= M - el; ++m) {
                  double v = PA[d] * VV(m, i1, 0) + WP[d] * VV(m + 1, i1, 0);
                  if (i2 >= 0) v += e1[d] * oo2p * (VV(m, i2, 0) - rp * VV(m + 1, i2, 0));
                  VV(m, ie, 0) = v;
                }
              }
          /* ket build */
          for (int fl = 1; fl <= lf; ++fl)
            for (int fi = 0; fi <= fl; ++fi)
              for (int fj = 0; fj <= fi; ++fj) {
                int f[3] = {fl - fi, fi - fj, fj};
                int d = f[0] ? 0 : (f[1] ? 1 : 2);
                int f1[3] = {f[0], f[1], f[2]};
                f1[d]--;
                int jf = cidx(f[0], f[1], f[2]), j1 = cidx(f1[0], f1[1], f1[2]), j2 = -1;
                if (f1[d] > 0) {
                  int f2[3] = {f1[0], f1[1], f1[2]};
                  f2[d]--;
                  j2 = cidx(f2[0], f2[1], f2[2]);
                }
                for (int el = 0; el <= le; ++el)
                  for (int i = 0; i <= el; ++i)
                    for (int j = 0; j <= i; ++j) {
                      int e[3] = {el - i, i - j, j};
                      int ie = cidx(e[0], e[1], e[2]);
                      int ie1 = -1;
                      if (e[d] > 0) {
                        int e1[3] = {e[0], e[1], e[2]};
                        e1[d]--;
                        ie1 = cidx(e1[0], e1[1], e1[2]);
                      }
                      for (int m = 0; m <= M - el - fl; ++m) {
                        double v = QC[d] * VV(m, ie, j1) + WQ[d] * VV(m + 1, ie, j1);
                        if (j2 >= 0) v += f1[d] * oo2q * (VV(m, ie, j2) - rq * VV(m + 1, ie, j2));
                        if (ie1 >= 0) v += e[d] * oo2pq * VV(m + 1, ie1, j1);
                        VV(m, ie, jf) = v;
                      }
                    }
              }
          for (int e = 0; e < ne; ++e)
            for (int f = 0; f < nf; ++f) G[e * nf + f] += VV(0, e, f);
        }
    }
#undef VV
  /* ket HRR: K[e][c][d] for |c|=lc, |d|=ld, built over |d| = 0..ld */
  int ncu = ncart_upto(lf), ndu = ncart_upto(ld);
  double *H = (double *)calloc((size_t)ncu * ndu, sizeof(double));
  int na = vo_ncart(la), nb = vo_ncart(lb), nc = vo_ncart(lc), nd = vo_ncart(ld);
  double *K = (double *)malloc(sizeof(double) * (size_t)ne * nc * nd);
  for (int e = 0; e < ne; ++e) {
    memset(H, 0, sizeof(double) * (size_t)ncu * ndu);
    for (int f = 0; f < nf; ++f) H[f * ndu + 0] = G[e * nf + f];
    for (int dl = 1; dl <= ld; ++dl)
      for (int i = 0; i <= dl; ++i)
        for (int j = 0; j <= i; ++j) {
          int dv[3] = {dl - i, i - j, j};
          int d = dv[0] ? 0 : (dv[1] ? 1 : 2);
          int d1[3] = {dv[0], dv[1], dv[2]};
          d1[d]--;
          int id = cidx(dv[0], dv[1], dv[2]), id1 = cidx(d1[0], d1[1], d1[2]);
          for (int cl = lc; cl <= lf - dl; ++cl)
            for (int ii = 0; ii <= cl; ++ii)
              for (int jj = 0; jj <= ii; ++jj) {
                int cv[3] = {cl - ii, ii - jj, jj};
                int cp[3] = {cv[0], cv[1], cv[2]};
                cp[d]++;
                int ic = cidx(cv[0], cv[1], cv[2]), icp = cidx(cp[0], cp[1], cp[2]);
                H[ic * ndu + id] = H[icp * ndu + id1] + CD[d] * H[ic * ndu + id1];
              }
        }
    for (int ic = 0; ic < nc; ++ic) {
      int cx, cy, cz;
      vo_cart_comp(lc, ic, &cx, &cy, &cz);
      for (int id = 0; id < nd; ++id) {
        int dx, dy, dz;
        vo_cart_comp(ld, id, &dx, &dy, &dz);
        K[(size_t)e * nc * nd + ic * nd + id] = H[cidx(cx, cy, cz) * ndu + cidx(dx, dy, dz)];
      }
    }
  }
  free(H);
  /* bra HRR per (c,d) */
  int nbu = ncart_upto(lb);
  double *Hb = (double *)calloc((size_t)ne * nbu, sizeof(double));
  for (int cd = 0; cd < nc * nd; ++cd) {
    memset(Hb, 0, sizeof(double) * (size_t)ne * nbu);
    for (int e = 0; e < ne; ++e) Hb[e * nbu + 0] = K[(size_t)e * nc * nd + cd];
    for (int bl = 1; bl <= lb; ++bl)
      for (int i = 0; i <= bl; ++i)
        for (int j = 0; j <= i; ++j) {
          int bv[3] = {bl - i, i - j, j};
          int d = bv[0] ? 0 : (bv[1] ? 1 : 2);
          int b1[3] = {bv[0], bv[1], bv[2]};
          b1[d]--;
          int ib = cidx(bv[0], bv[1], bv[2]), ib1 = cidx(b1[0], b1[1], b1[2]);
          for (int al = la; al <= le - bl; ++al)
            for (int ii = 0; ii <= al; ++ii)
              for (int jj = 0; jj <= ii; ++jj) {
                int av[3] = {al - ii, ii - jj, jj};
                int ap[3] = {av[0], av[1], av[2]};
                ap[d]++;
                int ia = cidx(av[0], av[1], av[2]), iap = cidx(ap[0], ap[1], ap[2]);
                Hb[ia * nbu + ib] = Hb[iap * nbu + ib1] + AB[d] * Hb[ia * nbu + ib1];
              }
        }
    for (int ia = 0; ia < na; ++ia) {
      int ax, ay, az;
      vo_cart_comp(la, ia, &ax, &ay, &az);
      for (int ib = 0; ib < nb; ++ib) {
        int bx, by, bz;
        vo_cart_comp(lb, ib, &bx, &by, &bz);
        out[(size_t)(ia * nb + ib) * nc * nd + cd] = Hb[cidx(ax, ay, az) * nbu + cidx(bx, by, bz)];
      }
    }
  }
  free(Hb);
  free(K);
  free(G);
  free(V);
}
