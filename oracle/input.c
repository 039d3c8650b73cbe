/*
 * input.c -- ORACLE (test infrastructure): reader for VALENCE input files.
 *
 * Restates xm_getdims / xm_input (xm_module.F90:25-335) and the tolerance
 * set-up of read_allocate_input (valence_initialize_module.F90:33-120).
 * Fortran list-directed input is record oriented: every READ statement
 * starts on a fresh line, takes values across as many lines as it needs and
 * drops whatever is left on its last line.  Blank lines carry no values.
 * The free text that ends most inputs is never reached.
 */
#include "vsvb_oracle.h"

#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  char *buf;
  size_t len, pos; /* pos = start of the next unread record */
  size_t cur;      /* cursor inside the current READ */
  int in_stmt;
  char tok[128];
  int bad;
} reader;

static void stmt_begin(reader *r) {
  r->cur = r->pos;
  r->in_stmt = 1;
}

static void stmt_end(reader *r) {
  /* drop the rest of the current record */
  size_t c = r->cur;
  while (c < r->len && r->buf[c] != '\n') c++;
  if (c < r->len) c++;
  r->pos = c;
  r->in_stmt = 0;
}

/* next value token of the current statement; separators are blanks, tabs,
 * commas and line ends */
static int next_tok(reader *r) {
  size_t c = r->cur;
  for (;;) {
    while (c < r->len && (r->buf[c] == ' ' || r->buf[c] == '\t' || r->buf[c] == ',' ||
                          r->buf[c] == '\r' || r->buf[c] == '\n'))
      c++;
    if (c >= r->len) {
      r->bad = 1;
      r->cur = c;
      return 0;
    }
    break;
  }
  size_t s = c;
  while (c < r->len && !(r->buf[c] == ' ' || r->buf[c] == '\t' || r->buf[c] == ',' ||
                         r->buf[c] == '\r' || r->buf[c] == '\n'))
    c++;
  size_t n = c - s;
  if (n >= sizeof(r->tok)) n = sizeof(r->tok) - 1;
  memcpy(r->tok, r->buf + s, n);
  r->tok[n] = 0;
  r->cur = c;
  return 1;
}

static int rd_int(reader *r) {
  if (!next_tok(r)) return 0;
  char *e;
  long v = strtol(r->tok, &e, 10);
  if (*e != 0) r->bad = 1;
  return (int)v;
}

static double rd_dbl(reader *r) {
  if (!next_tok(r)) return 0.0;
  for (char *p = r->tok; *p; ++p)
    if (*p == 'd' || *p == 'D') *p = 'e';
  char *e;
  double v = strtod(r->tok, &e);
  if (*e != 0) r->bad = 1;
  return v;
}

static void *xcalloc(size_t n, size_t s) { return calloc(n ? n : 1, s); }

void vo_free_input(vo_input *in) {
  if (!in) return;
  free(in->orbset);
  free(in->atom_t);
  free(in->coords);
  free(in->nuc_charge);
  free(in->map_atom2shell);
  free(in->num_shell_atom);
  free(in->map_shell2prim);
  free(in->ang_mom);
  free(in->exponent);
  free(in->uncoef);
  free(in->con_coeff);
  free(in->pair_sc);
  free(in->coeff_sc);
  free(in->xorb);
  free(in->root);
  free(in->orbas_atnum);
  free(in->orbas_atset);
  free(in->map_orbs);
  free(in->xpset);
  free(in->coeff);
  free(in->coeff_raw);
  free(in);
}

int vo_read_input(const char *path, vo_input **out, char *err, int errlen) {
  *out = NULL;
  FILE *f = fopen(path, "rb");
  if (!f) {
    snprintf(err, errlen, "problems opening input file: %s", path);
    return 1;
  }
  fseek(f, 0, SEEK_END);
  long sz = ftell(f);
  fseek(f, 0, SEEK_SET);
  reader r;
  memset(&r, 0, sizeof r);
  r.buf = (char *)malloc((size_t)sz + 1);
  r.len = fread(r.buf, 1, (size_t)sz, f);
  r.buf[r.len] = 0;
  fclose(f);

  vo_input *in = (vo_input *)calloc(1, sizeof(vo_input));
  /* A) dimensions */
  stmt_begin(&r);
  in->natom = rd_int(&r);
  in->natom_t = rd_int(&r);
  in->npair = rd_int(&r);
  in->nunpd = rd_int(&r);
  in->ndocc = rd_int(&r);
  in->totlen = rd_int(&r);
  in->xpmax = rd_int(&r);
  in->nspinc = rd_int(&r);
  in->num_sh = rd_int(&r);
  in->num_pr = rd_int(&r);
  in->nang = rd_int(&r);
  in->ndf = rd_int(&r);
  in->nset = rd_int(&r);
  in->nxorb = rd_int(&r);
  in->mxctr = rd_int(&r);
  stmt_end(&r);
  if (r.bad) {
    snprintf(err, errlen, "cannot read the dimension line");
    goto fail;
  }
  if (in->npair > 0 && in->nspinc < 1) {
    snprintf(err, errlen, "no spin couplings;");
    goto fail;
  }
  if (in->natom < 1 || in->natom_t < 1 || in->num_sh < 0 || in->num_pr < 0 || in->totlen < 1 ||
      in->mxctr < 1) {
    snprintf(err, errlen, "bad dimensions");
    goto fail;
  }
  in->norbs = 2 * in->npair + in->nunpd + in->ndocc + in->ndf;
  in->orbset = (int *)xcalloc(2 * (size_t)in->nset, sizeof(int));
  in->atom_t = (int *)xcalloc(in->natom, sizeof(int));
  in->coords = (double *)xcalloc(3 * (size_t)in->natom, sizeof(double));
  in->nuc_charge = (double *)xcalloc(in->natom_t, sizeof(double));
  in->map_atom2shell = (int *)xcalloc(in->natom_t, sizeof(int));
  in->num_shell_atom = (int *)xcalloc(in->natom_t, sizeof(int));
  in->map_shell2prim = (int *)xcalloc((size_t)in->num_sh + 1, sizeof(int));
  in->ang_mom = (int *)xcalloc(in->num_sh, sizeof(int));
  in->exponent = (double *)xcalloc(in->num_pr, sizeof(double));
  in->uncoef = (double *)xcalloc(in->num_pr, sizeof(double));
  in->con_coeff = (double *)xcalloc(in->num_pr, sizeof(double));
  in->pair_sc = (int *)xcalloc(2 * (size_t)in->npair * (in->nspinc > 0 ? in->nspinc : 1), sizeof(int));
  in->coeff_sc = (double *)xcalloc(in->nspinc > 0 ? in->nspinc : 1, sizeof(double));
  in->xorb = (int *)xcalloc(in->nxorb, sizeof(int));
  in->root = (int *)xcalloc(in->nxorb, sizeof(int));
  in->orbas_atnum = (int *)xcalloc(in->norbs, sizeof(int));
  in->orbas_atset = (int *)xcalloc((size_t)in->mxctr * in->norbs, sizeof(int));
  in->map_orbs = (int *)xcalloc((size_t)in->norbs + 1, sizeof(int));
  in->xpset = (int *)xcalloc(in->totlen, sizeof(int));
  in->coeff = (double *)xcalloc(in->totlen, sizeof(double));
  in->coeff_raw = (double *)xcalloc(in->totlen, sizeof(double));

  /* B) optimisation control */
  stmt_begin(&r);
  in->ntol_c = rd_int(&r);
  in->ntol_d = rd_int(&r);
  in->ntol_i = rd_int(&r);
  in->ntol_e_min = rd_int(&r);
  in->ntol_e_max = rd_int(&r);
  in->max_iter = rd_int(&r);
  in->ptbnmax = rd_dbl(&r);
  in->feather = rd_dbl(&r);
  for (int i = 0; i < in->nset; ++i) {
    in->orbset[2 * i] = rd_int(&r);
    in->orbset[2 * i + 1] = rd_int(&r);
  }
  stmt_end(&r);

  /* C) geometry */
  for (int i = 0; i < in->natom; ++i) {
    stmt_begin(&r);
    in->atom_t[i] = rd_int(&r);
    for (int j = 0; j < 3; ++j) in->coords[3 * i + j] = rd_dbl(&r);
    stmt_end(&r);
    if (in->atom_t[i] < 1 || in->atom_t[i] > in->natom_t) {
      snprintf(err, errlen, "atom %d has a bad type", i + 1);
      goto fail;
    }
  }

  /* D) basis sets */
  {
    int ns = 1, np = 1;
    for (int i = 0; i < in->natom_t; ++i) {
      in->map_atom2shell[i] = ns;
      stmt_begin(&r);
      in->nuc_charge[i] = rd_dbl(&r);
      int nshell = rd_int(&r);
      stmt_end(&r);
      in->num_shell_atom[i] = nshell;
      for (int j = 0; j < nshell; ++j) {
        if (ns > in->num_sh) {
          snprintf(err, errlen, "more shells than declared");
          goto fail;
        }
        in->map_shell2prim[ns - 1] = np;
        stmt_begin(&r);
        in->ang_mom[ns - 1] = rd_int(&r);
        int con_length = rd_int(&r);
        stmt_end(&r);
        if (np - 1 + con_length > in->num_pr || con_length < 1) {
          snprintf(err, errlen, "more primitives than declared");
          goto fail;
        }
        if (con_length == 1) {
          stmt_begin(&r);
          in->exponent[np - 1] = rd_dbl(&r);
          stmt_end(&r);
          in->uncoef[np - 1] = 1.0;
          np++;
        } else {
          for (int k = 0; k < con_length; ++k) {
            stmt_begin(&r);
            in->exponent[np - 1] = rd_dbl(&r);
            in->uncoef[np - 1] = rd_dbl(&r);
            stmt_end(&r);
            np++;
          }
        }
        ns++;
      }
    }
    if (ns - 1 <= in->num_sh) in->map_shell2prim[ns - 1] = np;
  }

  /* E) spin couplings */
  in->coeff_sc[0] = 1.0;
  if (in->npair > 0) {
    int np2 = in->npair;
    if (in->nspinc == 1) {
      stmt_begin(&r);
      for (int i = 0; i < np2; ++i) {
        in->pair_sc[i] = rd_int(&r);
        in->pair_sc[i + np2] = rd_int(&r);
      }
      stmt_end(&r);
    } else if (in->nspinc > 1) {
      stmt_begin(&r);
      for (int j = 0; j < in->nspinc; ++j) {
        in->coeff_sc[j] = rd_dbl(&r);
        for (int i = 0; i < np2; ++i) {
          in->pair_sc[i + np2 * (0 + 2 * j)] = rd_int(&r);
          in->pair_sc[i + np2 * (1 + 2 * j)] = rd_int(&r);
        }
      }
      stmt_end(&r);
    }
  }
  if (in->nxorb > 0) {
    stmt_begin(&r);
    for (int i = 0; i < in->nxorb; ++i) {
      in->xorb[i] = rd_int(&r);
      in->root[i] = rd_int(&r);
    }
    stmt_end(&r);
  }

  /* F, G) orbitals then NDFs, all in the same layout */
  {
    int j = 1;
    for (int i = 0; i < in->norbs; ++i) {
      stmt_begin(&r);
      in->orbas_atnum[i] = rd_int(&r);
      if (in->orbas_atnum[i] < 1 || in->orbas_atnum[i] > in->mxctr) {
        snprintf(err, errlen, "orbital %d: bad atom count", i + 1);
        goto fail;
      }
      for (int k = 0; k < in->orbas_atnum[i]; ++k) in->orbas_atset[k + in->mxctr * i] = rd_int(&r);
      int n = rd_int(&r);
      stmt_end(&r);
      in->map_orbs[i] = j;
      if (j - 1 + n > in->totlen || n < 0) {
        snprintf(err, errlen, "orbital %d: weight list longer than totlen", i + 1);
        goto fail;
      }
      stmt_begin(&r);
      for (int k = j; k < j + n; ++k) {
        in->xpset[k - 1] = rd_int(&r);
        in->coeff_raw[k - 1] = rd_dbl(&r);
      }
      stmt_end(&r);
      j += n;
    }
    in->map_orbs[in->norbs] = j;
  }
  if (r.bad) {
    snprintf(err, errlen, "premature end of input");
    goto fail;
  }
  /* tolerances (valence_initialize_module.F90:111-113) */
  in->dtol = pow(10.0, -(double)in->ntol_d);
  in->itol = pow(10.0, -(double)in->ntol_i);
  /* Angstrom -> bohr (tools_module.F90:6-17) */
  for (int i = 0; i < 3 * in->natom; ++i) in->coords[i] *= 1.889725987722;
  memcpy(in->coeff, in->coeff_raw, sizeof(double) * in->totlen);
  free(r.buf);
  *out = in;
  return 0;
fail:
  free(r.buf);
  vo_free_input(in);
  return 1;
}

void vo_set_coords_angstrom(vo_input *in, const double *xyz) {
  for (int i = 0; i < 3 * in->natom; ++i) in->coords[i] = xyz[i] * 1.889725987722;
}

void vo_set_coeff(vo_input *in, const double *coeff_raw) {
  memcpy(in->coeff_raw, coeff_raw, sizeof(double) * in->totlen);
  memcpy(in->coeff, coeff_raw, sizeof(double) * in->totlen);
}
