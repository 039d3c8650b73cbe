/* eri.cuh -- launch interface of the shell-quartet ERI kernels (eri.cu). */
#ifndef VSVB_ERI_CUH
#define VSVB_ERI_CUH
#include <cuda_runtime.h>

#include "vsvb_internal.h"

struct EriArgs {
  const ShellPair *pairs;
  const PrimPair *prims;
  const double *rys;       /* Chebyshev tables (device) */
  const int *pair_opid;    /* orbital-pair index of every pair term */
  const double *xtab;      /* X tables */
  double *T;               /* np x np orbital-pair ERIs (mode 0) */
  int np;
  double *qmax_out;        /* mode 1 */
  const double *Tbar;      /* mode 2: dE/dT */
  double *xbar;            /* mode 2: dE/dX */
};

/* cp >= cq are pair classes 0..5; mode 0 forward, 1 Schwarz, 2 adjoint. */
int eri_launch(int mode, int fp32, int cp, int cq, const EriArgs &a, const int2 *work, int nwork, int nsm,
               cudaStream_t st);
double eri_flops(int cp, int cq, int nprimP, int nprimQ, int nopP, int nopQ);
int eri_symmetrize(double *T, int np, cudaStream_t st);
int eri_set_tables(const int *off, const double *ax, const double *aw);
#endif
