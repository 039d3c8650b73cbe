/* density.cuh -- launch interface of the determinant-pair / assembly kernels. */
#ifndef VSVB_DENSITY_CUH
#define VSVB_DENSITY_CUH
#include <cuda_runtime.h>

#include "vsvb_internal.h"

struct DetCtx {
  DetSetup ds;
  const int *pair_slot;   /* [nsc][npair][2]: 0-based slots of pair_sc(k,1|2,isc) */
  const int *slot_pair;   /* [nsc][2*npair]: pair index of each coupled slot */
  const int *slot_which;  /* [nsc][2*npair]: 0 if the slot is pair_sc(k,1), 1 if (k,2) */
  const double *coeff_sc; /* [nsc] (1.0 when nspinc == 0) */
  const double *So, *Ho;  /* nsp x nsp orbital overlap / core Hamiltonian */
  double *det_a, *det_b;  /* [nq] determinants (exact LU on the exact-minor path) */
  double *detr_a, *detr_b; /* [nq] det(A + delta I) of a flagged block, det(A) elsewhere */
  double *Ta, *Tb;        /* [nq][n*n] inverses, of A + delta I on a flagged block */
  int *sing;              /* [nq] bit0 alpha, bit1 beta on the exact-minor path */
  int *nsing;             /* count of determinant pairs with a bit set (optional) */
  int *status;            /* value 2: a flagged block whose shift is singular too;
                           * value 4: more flagged determinant pairs than the pool holds */
  /* exact-minor pool: per flagged determinant pair one slot holding, per
   * spin block, inverse and determinant of A + k P (k = 1, 2, 3; P a fixed
   * rank-2 matrix), from which every struck determinant of A follows */
  double *xinv;           /* [xcap][3 (na*na + nb*nb)] */
  double *xdet;           /* [xcap][2][3] */
  int *xslot;             /* [nq] slot of pair q, -1 when none */
  int *xcount;            /* slots taken (reset per evaluation) */
  int xcap;
  int *abeq;              /* [nq] 1 when the beta block has the alpha block's orbitals and
                           * factorisation (doubly occupied orbitals, no unpaired ones) */
};

struct AsmArgs {
  const double *T;  /* np x np orbital-pair ERIs */
  const double *sq; /* [np] sqrt(max(T[p][p], 0)) */
  int np;
  double itol;
  long long ntasks;
  double *part_e1, *part_wf, *part_e2; /* [nq * nsplit] */
  int *status;
  /* adjoint pass */
  double inv_w, dw_coef;  /* 1/W and -E_num/(W^2 nelec) */
  const double *res;      /* when set: read e_num = res[1], W = res[4] on the device instead */
  double *Tbar, *Sbar, *Hbar;
  double *vtot;            /* [nq * nsplit] */
  double *Gglob;           /* [nq][na*na + nb*nb] */
  int g_in_smem;            /* copies of G per block in shared memory (0: G in global memory) */
  int skip_tbar; /* adjoint walk without dE/dT (single-sweep mode) */
  /* MODE 4 (unscaled adjoint walk): the dE/dS parts kept apart */
  double *Gs;     /* [nq][na*na + nb*nb] */
  double *vtot_s; /* [nq * nsplit] */
  double *D1;     /* [nsp*nsp] first-order cofactor densities */
};

__global__ void detpair_kernel(DetCtx d, double *scratch, int ld_scratch);
cudaError_t launch_assemble(int mode, dim3 grid, int threads, size_t smem, cudaStream_t st, const DetCtx &d,
                            const AsmArgs &a);
__global__ void energy_reduce_kernel(AsmArgs a, long long nslot, int nelec, double enuc, double *out);
__global__ void detpair_adjoint_kernel(DetCtx d, AsmArgs a, int nsplit);
__global__ void grad_scale_kernel(DetCtx d, AsmArgs a, int nsplit);
__global__ void hs_scale_kernel(DetCtx d, AsmArgs a, int nsplit, double alpha, double beta);
__global__ void spin_block_kernel(DetCtx d, AsmArgs a, int nsplit, double *BH, double *BS);
#endif
