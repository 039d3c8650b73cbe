/*
 * vsvb_oracle.h -- CPU ORACLE for the VSVB energy hot path.
 *
 * THIS IS TEST INFRASTRUCTURE, NOT PRODUCT CODE.  Only the test suite, the
 * smoke check and the benchmark's CPU-baseline leg may load it, and only as
 * the checker / the timed CPU reference.  The GPU product never links it.
 *
 * It is a literal CPU restatement of VALENCE's guess-energy path
 * (src/valence.F90 of VALENCE-software/VALENCE):
 *   guess_energy            valence.F90:309-345
 *   vsvb_energy             valence.F90:1010-1434
 *   wfndet / schwarz_ints   valence.F90:1440-1523
 *   density .. det          valence.F90:1535-2056
 *   givdr / givens_single   valence.F90:2067-2144, givens.F90:230-262
 *   normal / ndf2obs        valence.F90:2157-2247
 *   norm_prim/cartesian/setangn   valence.F90:2264-2421
 *   set_up_unpaired_docc / build_abket / check_spin_and_locate
 *                           valence.F90:2444-2586, 2670-2714
 *   ovint / int1e / int2e   valence.F90:2891-3438
 *   input reader            xm_module.F90:25-335
 *   nuclear repulsion, Angstrom->bohr   tools_module.F90:6-40
 * The integrals that VALENCE takes from the third-party simint library
 * (simint-chem/simint-generator, unpinned HEAD, generated with -l 3 -p 3,
 * scalar, CCA component order) are restated here from the published
 * Obara-Saika / Head-Gordon-Pople recurrences with our own Boys function.
 * Parity is pinned against the reference's golden guess energies
 * (testing/testing.py:69-153, examples/test_examples.py:63-153).
 */
#ifndef VSVB_ORACLE_H
#define VSVB_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct vo_input {
  /* line A (xm_module.F90:38-39) */
  int natom, natom_t, npair, nunpd, ndocc, totlen, xpmax, nspinc;
  int num_sh, num_pr, nang, ndf, nset, nxorb, mxctr;
  /* line B (xm_module.F90:98-100) */
  int ntol_c, ntol_d, ntol_i, ntol_e_min, ntol_e_max, max_iter;
  double ptbnmax, feather;
  int *orbset;            /* 2*nset */
  /* geometry: atom_t 1-based types, coords in bohr after reading */
  int *atom_t;            /* natom */
  double *coords;         /* 3*natom, [3*i + x] */
  /* basis per atom type (1-based shell / primitive indices as in Fortran) */
  double *nuc_charge;     /* natom_t */
  int *map_atom2shell;    /* natom_t */
  int *num_shell_atom;    /* natom_t */
  int *map_shell2prim;    /* num_sh+1 */
  int *ang_mom;           /* num_sh */
  double *exponent;       /* num_pr */
  double *uncoef;         /* num_pr, unnormalized contraction coefficients */
  double *con_coeff;      /* num_pr, after norm_prim */
  /* spin couplings */
  int *pair_sc;           /* [k + npair*(s + 2*isc)], k<npair, s in {0,1} */
  double *coeff_sc;       /* max(nspinc,1) */
  int *xorb, *root;       /* nxorb */
  /* orbitals (1-based indices into coeff/xpset, as in Fortran) */
  int norbs;
  int *orbas_atnum;       /* norbs */
  int *orbas_atset;       /* [k + mxctr*i] (1-based atom numbers) */
  int *map_orbs;          /* norbs+1 */
  int *xpset;             /* totlen */
  double *coeff;          /* totlen (normalized in place by vo_prepare) */
  double *coeff_raw;      /* totlen (as read) */
  double dtol, itol;
} vo_input;

/* Parse a VALENCE input file with Fortran list-directed record semantics.
 * Returns 0 on success; on failure writes a message into err. */
int vo_read_input(const char *path, vo_input **out, char *err, int errlen);
void vo_free_input(vo_input *in);

/* Optional overrides before vo_guess_energy: coordinates in Angstrom
 * (3*natom) as valence_api_calculate_energy takes them, and raw
 * (unnormalized) orbital weights (totlen). */
void vo_set_coords_angstrom(vo_input *in, const double *xyz);
void vo_set_coeff(vo_input *in, const double *coeff_raw);

typedef struct vo_result {
  double enucrep;      /* nuclear repulsion */
  double energy;       /* guess energy = e_num/wfnorm + enucrep */
  double e1;           /* one-electron numerator */
  double e2;           /* two-electron numerator */
  double wfnorm;
  long long ntasks;    /* 2e tasks in the loop */
  long long ndens2;    /* density(2) calls */
} vo_result;

/* Literal guess energy (valence.F90:309-345). nthreads<=0: OpenMP default. */
int vo_guess_energy(vo_input *in, vo_result *res, int nthreads);
/* Same with only every stride-th two-electron task evaluated (CPU-baseline
 * timing on a bounded sample; the energy is then not the full energy). */
int vo_guess_energy_sampled(vo_input *in, vo_result *res, int nthreads, long long stride);
/* CPU-baseline timing on bounded samples of every phase: only every
 * schw_stride-th Schwarz-table entry (the others set so that they pass every
 * screen), every e1_stride-th one-electron term and every task_stride-th
 * two-electron task are evaluated.  phase_seconds[4]: set-up (normalisation,
 * orbital overlaps), Schwarz table, one-electron loop, task loop; each
 * extrapolates to the full run by its stride.  The energy is not the full
 * energy. */
int vo_guess_energy_timed(vo_input *in, vo_result *res, int nthreads, long long schw_stride, long long e1_stride,
                          long long task_stride, double *phase_seconds);

/* first_order_opt's Hamiltonian and overlap matrices (valence.F90:527-758)
 * for orbital iorb (1-based) of the wave function with the weights as set
 * (coeff_raw, normalised first as the reference's coeff is): nb x nb,
 * column-major, nb = map_orbs(iorb+1) - map_orbs(iorb), ham(ib,jb) the
 * energy numerator and ovl(ib,jb) the wave-function norm with the bra's
 * slot of iorb holding entry ib and the ket's entry jb, spin averaged for a
 * doubly occupied orbital when there are unpaired electrons; symmetrised. */
int vo_first_order_hs(vo_input *in, int iorb, double *ham, double *ovl, int nthreads);
/* spin_opt's (valence.F90:850-897): nspinc x nspinc over the couplings. */
int vo_spin_hs(vo_input *in, double *ham, double *ovl, int nthreads);
double vo_nuclear_repulsion(vo_input *in);
/* normal(iorb, iorb) (valence.F90:2157-2182) applied to coeff_raw */
int vo_normal(vo_input *in, int iorb);

/* Orbital-level integrals after vo_guess_energy's normalisation:
 * (io ko | jo lo) over the screened LCAO weights (1-based orbitals). */
double vo_int2e(vo_input *in, int io, int ko, int jo, int lo);
double vo_ovint(vo_input *in, int io, int jo);
double vo_int1e(vo_input *in, int io, int jo);

/* Contracted AO shell-quartet block (ab|cd) with CCA component order, raw
 * primitive normalisation (no angn factor), shells given as global shell
 * ids (see vo_num_global_shells).  out has n_a*n_b*n_c*n_d entries. */
int vo_num_global_shells(vo_input *in);
void vo_global_shell(vo_input *in, int g, int *atom, int *shell);
void vo_ao_eri_block(vo_input *in, int ga, int gb, int gc, int gd, double *out);

/* Boys function F_m(T) for m = 0..mmax into f. */
void vo_boys(int mmax, double t, double *f);

#ifdef __cplusplus
}
#endif
#endif
