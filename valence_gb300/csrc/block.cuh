/* block.cuh -- block mode of the orbital-pair ERI matrix for large s/p
 * systems (block.cu). */
#ifndef VSVB_BLOCK_CUH
#define VSVB_BLOCK_CUH
#include <cuda_runtime.h>

/* per-evaluation weights of the orbitals on each atom: for entry e (atom a,
 * its j-th orbital, function f of a) src[e] = (orbital, weight slot in that
 * orbital's basis set, first slot of the function's shell, components of
 * the shell) and ao[e] the function's global index (for angn) */
struct BlkCoefArgs {
  const int4 *src;
  const int *ao;
  int n;
  const double *C; /* normalised weights [norb][maxobs] */
  int maxobs;
  const double *angn;
  double dtol;
  double *catom; /* out: angn_f C_o(f), 0 where int2e's shell screen drops the shell */
};

struct BlkArgs {
  const int4 *aq;       /* per atom quartet: bra atom pair, ket atom pair, offset of its block in G, 1 = same pair */
  const int4 *ap;       /* per atom pair: first atom, second atom (<= first) */
  const int2 *atom_orb; /* per atom: first entry of its orbitals in orb / catom rows, their count */
  const int *atom_nf;   /* per atom: functions */
  const int *atom_c0;   /* per atom: offset of its weight block in catom ([orbital][function]) */
  const int *orb;       /* orbital (spatial, 0-based) of each (atom, j) */
  const double *catom;
  const double *G;      /* staging buffer of the chunk */
  double *G_clear;      /* the same, cleared after reading */
  double *U;            /* np x np, one orientation (T = U + U^T afterwards) */
  int np;
  int nfmax, nomax;     /* largest functions / orbitals on an atom (shared-memory layout) */
  int r1n;              /* blk_r1(nfmax, nomax) */
  int nomaxp;           /* nomax rounded up to a multiple of 8 */
};

int blk_coef(const BlkCoefArgs &a, cudaStream_t st);
/* one CTA per atom quartet aq0 .. aq0+n-1; tt 0 FP64, 1 FP32, 2 double-float */
int blk_transform(const BlkArgs &a, int aq0, int n, int tt, size_t smem_bytes, cudaStream_t st);
/* size of the first intermediate area, and the shared memory (bytes) of
 * blk_transform for the given maxima */
int blk_r1(int nfmax, int nomax);
size_t blk_transform_smem(int nfmax, int nomax, int tt);
/* algorithmic FLOPs of the four quarter transforms of one atom quartet */
double blk_transform_flops(int nfa, int nfb, int nfc, int nfd, int na, int nb, int nc, int nd);
#endif
