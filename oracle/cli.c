/* cli.c -- ORACLE (test infrastructure): command-line driver printing the
 * quantities VALENCE's test parser reads (testing/testing.py:174-191). */
#include <stdio.h>
#include <stdlib.h>
#include "vsvb_oracle.h"
int main(int argc, char **argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: %s input [nthreads]\n", argv[0]);
    return 2;
  }
  vo_input *in;
  char err[256];
  if (vo_read_input(argv[1], &in, err, sizeof err)) {
    fprintf(stderr, "%s\n", err);
    return 1;
  }
  vo_result r;
  vo_guess_energy(in, &r, argc > 2 ? atoi(argv[2]) : 0);
  printf(" nuclear repulsion %25.16f\n", r.enucrep);
  printf(" guess energy %25.16f\n", r.energy);
  printf(" e1 %25.16f e2 %25.16f wfnorm %25.16f tasks %lld dens2 %lld\n", r.e1, r.e2, r.wfnorm, r.ntasks, r.ndens2);
  vo_free_input(in);
  return 0;
}
