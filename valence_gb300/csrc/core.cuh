/* core.cuh -- the determinant-pair sum over a shared doubly occupied core
 * (core.cu): launch interface. */
#ifndef VSVB_CORE_CUH
#define VSVB_CORE_CUH
#include <cuda_runtime.h>

/* Orbital numbering of a core-mode handle: the 2P coupled orbitals of the
 * spin-coupled pairs are spatial orbitals 0..nC-1, the doubly occupied
 * (core) orbitals nC..nsp-1; there are no unpaired orbitals. */
struct CoreArgs {
  int nsp, nC, nD, P, nsc, ndet, nelec;
  long long nq;           /* determinant pairs: nsc^2 4^P */
  int np;                 /* orbital pairs nsp (nsp + 1) / 2 */
  int ncp;                /* coupled-orbital pairs nC (nC + 1) / 2 */
  int kx;                 /* columns of Wv and X: ncp + 2 */
  const double *So, *Ho;  /* nsp x nsp orbital overlap / core Hamiltonian */
  const double *csc;      /* [nsc] spin-coupling weights */
  const unsigned char *detorb; /* [ndet][2][P]: coupled orbital at block position r of spin s */
  const unsigned char *detpos; /* [ndet][nC]: spin << 5 | block position of coupled orbital a */
  const int *lst1, *off1; /* determinants by (a, spin of a): off1[2a+s] .. off1[2a+s+1] */
  const int *lst2, *off2; /* by (a, c, spin of a, spin of c): off2[4(a nC + c) + g] .. +1 */
  const int2 *pik;        /* [np]: orbital pair p -> (i, k), i >= k */
  double *fw;             /* core factorisation work: nD x (2 nD + nC) */
  double *G;              /* nD x nD: S_DD^-1 */
  double *Y;              /* nD x nC: S_DD^-1 S_DC */
  double *M;              /* nC x nC: S_CC - S_CD S_DD^-1 S_DC */
  double *P0;             /* nsp x nsp: S_DD^-1 on the core block, 0 elsewhere */
  double *U;              /* nsp x nC: e_c - S_DD^-1 S_Dc */
  double *s0;             /* det S_DD */
  double *dd;             /* [nq][2]: determinant of each spin block */
  double *L;              /* [nq][2][P*P]: first cofactors of the block, (bra position, ket position) */
  double *qf;             /* [nq][2]: w d_other / (2 d_s), the factor of the second cofactors of an
                           * unflagged block in the pair sums */
  int *pslot;             /* [nq]: 4 slot + flagged spins, or -1 */
  double *pool;           /* [cap][3][2][1 + P*P]: det and cofactors of block + k Pert, k = 1..3 */
  int *pcount;
  int cap;
  int *status;            /* |= 4: pool full; |= 8: singular core block */
  double *A0, *A1, *A2, *A2x, *R1;
  double *Wv, *X;         /* np x kx */
  const double *T, *sq;   /* orbital-pair ERI matrix and sqrt of its diagonal */
  double itol;
  double *part;           /* [ntile * ntile] per GEMM tile */
  int ntile;
  double enuc;
  int df;                 /* 1: the orbital-pair GEMMs in double-float (mixed path) */
  double *out;            /* [5] energy, e_num, e1, e2, wfnorm */
  int *nsing;             /* flagged determinant pairs */
};

/* buffers of the core-mode adjoint */
struct CoreGrad {
  double *Gam;        /* np x np: Gamma in orbital-pair layout (the sweep's dE_num/dT) */
  double *Yg;         /* np x kx: (T_masked / W) Wv */
  double *Axp;        /* [nchunk][kx][kx] partial Wv^T Yg */
  int nchunk;
  double *Ax;         /* kx x kx: dE/dA2x */
  double *Wvb;        /* np x kx: dE/dWv */
  double *KP, *KR;    /* nsp x nsp: exchange builds of T_masked / W with P0 and R1 */
  double *R1b, *P0b;  /* nsp x nsp */
  double *A1b;        /* nC x nC */
  double *Ub;         /* nsp x nC */
  double *Mbp;        /* [nq][2][P*P]: dE/dM_s per determinant pair */
  double *lam;        /* [nq]: each pair's share of sum <A-bar, A> */
  double *Mb;         /* nC x nC */
  double *sc;         /* [4]: A0-bar, Lambda */
  double *t1, *t2;    /* nsp x nsp work */
  double *Sbar, *Hbar; /* out: dE/dS_orb, dE/dh_orb */
};

/* before the ERI sweep (overlaps only); returns the kernels launched, or -1 */
int core_pre(const CoreArgs &a, cudaStream_t st);
/* Gamma stored in orbital-pair layout (gradient evaluations, before the sweep) */
int core_gamma(const CoreArgs &a, double *Gam, cudaStream_t st);
/* after the sweep: the pair-summed second-order density against the masked
 * orbital-pair ERIs (from Gam when stored, else recomputed tile by tile),
 * and the energy; returns the kernels launched, or -1 */
int core_post(const CoreArgs &a, const double *Gam, cudaStream_t st);
/* after core_post: dE/dS_orb and dE/dh_orb (and dE/dT = Gam / W for the
 * sweep's adjoint); returns the kernels launched, or -1 */
int core_adjoint(const CoreArgs &a, const CoreGrad &g, cudaStream_t st);
/* FMA count of the pair-summed density GEMM of one energy (the upper
 * triangle of Wv A2x Wv^T) */
double core_gemm_fma(const CoreArgs &a);
#endif
