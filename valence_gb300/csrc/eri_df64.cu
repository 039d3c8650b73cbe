/*
 * eri_df64.cu -- instantiation of the shell-quartet ERI kernels
 * (eri_impl.cuh) with df64 arithmetic in the 2D tables and component sums.
 */
#include "eri_impl.cuh"

int eri_dispatch_df64(int mode, int cp, int cq, const EriArgs &a, const int4 *w, int n, int max_blocks, cudaStream_t st) {
  if (mode == 0) return dispatch<df64, 0>(cp, cq, a, w, n, max_blocks, st);
  if (mode == 3) return dispatch<df64, 3>(cp, cq, a, w, n, max_blocks, st);
  if (mode == 4) return dispatch_blk<df64>(cp, cq, a, w, n, max_blocks, st);
  return 3;
}

int eri_dispatch_tab_df64(int cp, int cq, const EriArgs &a, const int4 *w, int n, int max_blocks, cudaStream_t st,
                          const EriArgs *tab, const int *wmol) {
  return dispatch_tab<df64>(cp, cq, a, w, n, max_blocks, st, tab, wmol);
}
