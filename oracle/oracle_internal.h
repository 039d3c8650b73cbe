/* oracle_internal.h -- ORACLE (test infrastructure) internals. */
#ifndef VSVB_ORACLE_INTERNAL_H
#define VSVB_ORACLE_INTERNAL_H
#include "vsvb_oracle.h"

typedef struct vo_shell {
  int l, nprim;
  const double *alpha, *coef;
  double xyz[3];
} vo_shell;

int vo_ncart(int l);
void vo_cart_comp(int l, int k, int *x, int *y, int *z);
void vo_shell_overlap_kinetic(const vo_shell *A, const vo_shell *B, double *ov, double *ke);
void vo_shell_nuclear(const vo_shell *A, const vo_shell *B, double zc, const double *C, double *out);
void vo_shell_eri(const vo_shell *A, const vo_shell *B, const vo_shell *C, const vo_shell *D, double *out);

#endif
