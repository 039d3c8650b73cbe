/* eri.cuh -- launch interface of the shell-quartet ERI kernels (eri.cu). */
#ifndef VSVB_ERI_CUH
#define VSVB_ERI_CUH
#include <cuda_runtime.h>

#include "vsvb_internal.h"

struct RysConst {
  int off[5];            /* offset of each rule's Chebyshev block in the table */
  double ax[5][5];       /* large-T limit: x_i = ax / T */
  double aw[5][5];       /*                w_i = aw / sqrt(T) */
  float2 axf[5][5], awf[5][5]; /* the same as (hi, lo) FP32 pairs */
};

struct EriArgs {
  RysConst rc;
  const void *prim64, *prim32, *primdf; /* PrimT<double|float|df64> per primitive pair */
  const void *geom64, *geom32, *geomdf; /* GeomT<...> per shell pair */
  const ShellPair *pairs;
  const PrimPair *prims;
  const double *rys;       /* Chebyshev tables (device) */
  const float2 *rysdf;     /* the same coefficients as (hi, lo) FP32 pairs */
  const float *rys32;      /* and their FP32 roundings, for the FP32 kernels */
  const int *pair_opid;    /* orbital-pair index of every pair term */
  const double *xtab;      /* transferred weight tables X' = X M (nop x ne per pair) */
  const double *hrr;       /* per-pair transfer matrices M (n_a n_b x ne) */
  const float *xtab32;     /* X' in FP32 (the FP32 kernels' transform) */
  const float *Tbar32;     /* dE/dT in FP32 (the FP32 kernels' adjoint) */
  double *T;               /* np x np orbital-pair ERIs (mode 0) */
  int np;
  double *qmax_out;        /* mode 1: sqrt(max_ab |(ab|ab)|) per pair */
  double *q0max_out;       /* mode 1: sqrt(max_e |(e0|e0)|) per pair */
  const float *prim_q0;    /* per primitive pair (prims order): sqrt(max_e |(e0|e0)|) */
  float prim_lo, prim_hi;  /* evaluate the primitive quartets with prim_lo <= q0_p q0_q < prim_hi */
  const double *Tbar;      /* mode 2: dE/dT */
  double *xbar;            /* mode 2: dE/dX' */
  /* mode 4 (block mode): per shell pair its place in its atom pair's block
   * (off of shell A's functions in its atom, off of shell B's, flags: 1 shell
   * A on the pair's second atom, 2 both shells on one atom, 4 one shell;
   * functions of the pair's second atom), and the staging buffer of the
   * current chunk of atom quartets */
  const int4 *pair_blk;
  double *G;
};

/* arithmetic kinds of the ERI kernels */
enum { ERI_F64 = 0, ERI_F32 = 1, ERI_DF64 = 2 };

/* cp >= cq are pair classes 0..5; mode 0 forward, 1 Schwarz (F64 only),
 * 2 adjoint, 3 forward + adjoint.  Work items (P, Q, r0, r1): shell pairs P
 * (class cp) and Q, and the rows r0 <= ip < r1 of P's primitive pairs to
 * evaluate (a large quartet is split into row ranges).  max_blocks caps the
 * grid (the blocks then stride over the work list).
 * Mode 4 (block mode, classes 0..2): the transferred block (ab|cd) is added
 * into the staging buffer of its atom quartet; items (P, Q, g, w) with g the
 * block's offset in G, w = columns of the block | 1<<20 when P belongs to the
 * quartet's ket atom pair | 1<<21 when both atom pairs are the same (the
 * transposed block is added too). */
int eri_launch(int mode, int kind, int cp, int cq, const EriArgs &a, const int4 *work, int nwork, int max_blocks,
               cudaStream_t st);
int eri_dispatch_f64(int mode, int cp, int cq, const EriArgs &a, const int4 *w, int n, int max_blocks, cudaStream_t st);
int eri_dispatch_f32(int mode, int cp, int cq, const EriArgs &a, const int4 *w, int n, int max_blocks, cudaStream_t st);
int eri_dispatch_df64(int mode, int cp, int cq, const EriArgs &a, const int4 *w, int n, int max_blocks,
                      cudaStream_t st);
/* A forward + adjoint (mode 3) launch over the quartets of many molecules:
 * work item i belongs to molecule wmol[i] with arguments tab[wmol[i]]
 * (device arrays); a gives the primitive window of the launch. */
int eri_launch_tab(int kind, int cp, int cq, const EriArgs &a, const int4 *work, int nwork, int max_blocks,
                   cudaStream_t st, const EriArgs *tab, const int *wmol);
int eri_dispatch_tab_f64(int cp, int cq, const EriArgs &a, const int4 *w, int n, int max_blocks, cudaStream_t st,
                         const EriArgs *tab, const int *wmol);
int eri_dispatch_tab_f32(int cp, int cq, const EriArgs &a, const int4 *w, int n, int max_blocks, cudaStream_t st,
                         const EriArgs *tab, const int *wmol);
int eri_dispatch_tab_df64(int cp, int cq, const EriArgs &a, const int4 *w, int n, int max_blocks, cudaStream_t st,
                          const EriArgs *tab, const int *wmol);
double eri_flops(int mode, int cp, int cq, double nprimq, int nopP, int nopQ);
int eri_symmetrize(double *T, int np, double *sq, cudaStream_t st);
/* block mode: algorithmic FLOPs of the transfer (ab|cd) = M_P (e0|f0) M_Q^T
 * of one shell quartet (its non-zero terms) */
double eri_block_hrr_flops(int cp, int cq);
/* out[i] = (float)in[i] */
int eri_to_float(const double *in, float *out, size_t n, cudaStream_t st);
#endif
