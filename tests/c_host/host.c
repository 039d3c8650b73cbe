/* A plain C99 host of the C ABI (include/vsvb_gpu.h): what a Fortran or C
 * caller links against.  Reads a VALENCE input, writes its 'orbitals' and
 * 'nelecwfn' text, and asks for a GPU handle; without a GPU the create call
 * must come back with a status code, never a crash.  Prints one line per step
 * for the test that runs it. */
#include <stdio.h>
#include <stdlib.h>

#include "vsvb_gpu.h"

int main(int argc, char **argv) {
  if (argc < 2) return 2;
  char err[256];
  vsvb_system_desc *d = NULL;
  int rc = vsvb_read_input(argv[1], &d, err, (int)sizeof err);
  printf("read %d natom %d totlen %d npair %d nspinc %d\n", rc, d ? d->natom : -1, d ? d->totlen : -1,
         d ? d->npair : -1, d ? d->nspinc : -1);
  if (rc) return 1;
  long n = 0;
  rc = vsvb_format_orbitals(d, NULL, -1.0, 0.0, 0, NULL, 0, &n);
  char *buf = (char *)malloc((size_t)n + 1);
  rc |= vsvb_format_orbitals(d, NULL, -1.0, 0.0, 0, buf, n + 1, &n);
  printf("orbitals %d %ld\n", rc, n);
  free(buf);
  rc = vsvb_format_nelecwfn(d, NULL, NULL, 0, &n);
  printf("nelecwfn %d %ld\n", rc, n);
  vsvb_options opt;
  vsvb_default_options(&opt);
  opt.precision = VSVB_MIXED_DF64;
  vsvb_gpu *h = NULL;
  rc = vsvb_gpu_create(d, &opt, &h);
  printf("create %d\n", rc);
  if (h) vsvb_gpu_destroy(h);
  vsvb_opt *o = NULL;
  rc = vsvb_opt_create(d, &opt, &o);
  printf("opt_create %d\n", rc);
  if (o) vsvb_opt_destroy(o);
  vsvb_free_desc(d);
  return 0;
}
