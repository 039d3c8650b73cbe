/*
 * eri_f64.cu -- instantiation of the shell-quartet ERI kernels
 * (eri_impl.cuh) with double arithmetic in the 2D tables and component sums.
 */
#include "eri_impl.cuh"

int eri_dispatch_f64(int mode, int cp, int cq, const EriArgs &a, const int4 *w, int n, int max_blocks, cudaStream_t st) {
  if (mode == 0) return dispatch<double, 0>(cp, cq, a, w, n, max_blocks, st);
  if (mode == 1) return dispatch<double, 1>(cp, cq, a, w, n, max_blocks, st);
  if (mode == 2) return dispatch<double, 2>(cp, cq, a, w, n, max_blocks, st);
  if (mode == 3) return dispatch<double, 3>(cp, cq, a, w, n, max_blocks, st);
  if (mode == 4) return dispatch_blk<double>(cp, cq, a, w, n, max_blocks, st);
  return 3;
}

int eri_dispatch_tab_f64(int cp, int cq, const EriArgs &a, const int4 *w, int n, int max_blocks, cudaStream_t st,
                          const EriArgs *tab, const int *wmol) {
  return dispatch_tab<double>(cp, cq, a, w, n, max_blocks, st, tab, wmol);
}
