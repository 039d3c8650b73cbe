/* onee.cuh -- launch interface of the one-electron / orbital-weight kernels. */
#ifndef VSVB_ONEE_CUH
#define VSVB_ONEE_CUH
#include <cuda_runtime.h>

#include "vsvb_internal.h"

struct Ao1eArgs {
  const GShell *shells;
  int nshell, nao, natom;
  const double *exps, *coefs;  /* normalised contraction coefficients */
  const double *angn;          /* per AO */
  const double *charge;        /* per atom */
  const double *atom_xyz;
  double *S, *H;               /* nao x nao */
};

/* orbital i's weight terms t in [term0[i], term0[i+1]): slot term_slot[t]
 * receives coeff[term_j[t]] (times coeff[term_m[t]] * ndf_scale[term_f[t]]
 * when the term goes through a derived basis function) */
struct OrbArgs {
  int norb_all;   /* orbitals + NDFs */
  int maxobs, nao;
  const int *obs_n, *obs_ao;  /* per orbital: OBS size, global AO ids [maxobs] */
  const int *term0, *term_slot, *term_j, *term_m, *term_f;
  const int *ndf_orb;         /* orbital index of each NDF */
  const double *coeff;        /* raw weights (device) */
  const double *S, *H;
  double *ndf_scale, *orb_scale;
  double *Craw, *C;           /* [norb_all * maxobs] */
  int *status;
  int fixed_orb;              /* orbital taken as given, not normalised (-1: none) */
};

struct XTerm {
  int oi, ok;            /* orbitals */
  int la, lb;            /* shell pair (A first) */
  int sAi, sBi, sAk, sBk;/* OBS slot of shell A/B in orbital i/k, -1 if absent */
  int aoA, aoB;          /* first global AO of shells A, B */
  int same_shell;
  int m0;                /* the pair's transfer matrix in hrr */
};

struct XtabArgs {
  const XTerm *terms;
  const long long *elem0;  /* first X element of each term */
  int nterm;
  long long nelem;
  const double *C;
  int maxobs;
  const double *angn;
  double dtol;
  double *xtab;
  double xbar_scale; /* adjoint: factor applied to dE/dX */
  const double *wres; /* when set: the factor is xbar_scale / wres[4] (W read on the device) */
  /* horizontal transfer folded into the weights: X'(op, e) = sum_ab X(op, ab) M(ab, e) */
  const long long *xh_elem0; /* first X' element of each term */
  long long nxh;
  const double *hrr;
  double *xtabh;
  float *xtabh32; /* the same in FP32 */
  int keep_orb;   /* an orbital exempt from the per-shell LCAO screen (-1: none) */
};

__global__ void ao_1e_kernel(Ao1eArgs a);
__global__ void ndf_norm_kernel(OrbArgs a);
__global__ void orb_norm_kernel(OrbArgs a);
__global__ void orb_1e_kernel(OrbArgs a, double *So, double *Ho);
__global__ void xtab_kernel(XtabArgs x);
__global__ void xtab_adjoint_kernel(XtabArgs x, const double *xbar, double *Cbar);
__global__ void xhrr_kernel(XtabArgs x);
__global__ void xhrr_adjoint_kernel(XtabArgs x, const double *xbarh, double *xbar);
__global__ void orb_1e_adjoint_kernel(OrbArgs a, const double *Sbar, const double *Hbar, int nsp, double *Cbar);
__global__ void orb_norm_adjoint_kernel(OrbArgs a, const double *Cbar, double *coeff_bar, double *ndf_bar);
__global__ void ndf_norm_adjoint_kernel(OrbArgs a, const double *ndf_bar, double *coeff_bar);
__global__ void entry_adjoint_kernel(OrbArgs a, int o, int j0, int nent, const double *Cbar, double *out, double scale,
                                     int *flag);
__global__ void hs_weights_kernel(double *coeff, const double *w, const int *src, int n, int j0, int nu);
#endif
