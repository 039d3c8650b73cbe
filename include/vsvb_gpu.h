/*
 * vsvb_gpu.h -- C ABI of the GB300 (sm_103a) VSVB energy hot path.
 *
 * Drop-in boundary.  In VALENCE (VALENCE-software/VALENCE) the guess energy
 * is
 *     call wfndet                                           valence.F90:337
 *     call schwarz_ints( num_spatial_orbs, num_non_docc )   valence.F90:339
 *     call vsvb_energy( 0, num_non_docc, num_spatial_orbs,  valence.F90:341
 *                       energy, wfnorm, .false., .true. )
 *     call xm_equalize_scalar( energy/wfnorm )              valence.F90:342-343
 *     energy = energy/wfnorm + enucrep                      valence.F90:344
 * with the integrals from simint (int2e valence.F90:3184-3438, int1e
 * :3022-3176, ovint :2891-3012) and the cofactor densities from density ..
 * det .. givens_single (valence.F90:1535-2144, givens.F90:230-262).
 * vsvb_gpu_energy replaces that whole block: one call computes the orbital
 * normalisation (normal, valence.F90:2157-2182), the overlap/one-electron
 * orbital integrals, the Schwarz table, every screened orbital-quartet ERI and
 * its contraction with the spin-coupled cofactor densities, and returns the
 * same energy/wfnorm pair.  The Fortran side binds these entry points with
 * ISO_C_BINDING; nothing here takes a torch type.
 *
 * Conventions: all arrays are plain host pointers unless a name ends in
 * _dev.  Index arrays keep the reference's 1-based Fortran values exactly as
 * the module arrays hold them (integrals_module.F90:27-63,
 * density_module.F90:8-9).  Every entry point returns a vsvb_status; none
 * aborts, exits or traps.  A handle is not thread-safe; use one per host
 * thread.  The GPU path ignores MPI rank/size: run it on one rank only (the
 * reference's round-robin split, valence.F90:1158-1163, would otherwise be
 * summed twice by xm_equalize).
 */
#ifndef VSVB_GPU_H
#define VSVB_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum vsvb_status {
  VSVB_OK = 0,
  VSVB_ERR_INPUT = 1,       /* malformed input / inconsistent dimensions */
  VSVB_ERR_UNSUPPORTED = 2, /* e.g. angular momentum above d on the GPU */
  VSVB_ERR_CUDA = 3,        /* a CUDA runtime call failed */
  VSVB_ERR_SINGULAR = 4,    /* a determinant-pair block singular even when shifted (gradient), or rsg's overlap not positive definite */
  VSVB_ERR_NOMEM = 5,
  VSVB_ERR_TIMEOUT = 6,     /* a bounded device-side wait gave up */
  VSVB_ERR_NOT_NORMALISABLE = 7, /* an orbital has non-positive self-overlap */
  VSVB_ERR_TOO_LARGE = 8          /* request exceeds a fixed-size buffer (vsvb_det_factor_noalloc) */
} vsvb_status;

/* Precision modes of the ERI contraction. */
typedef enum vsvb_precision {
  VSVB_FP64 = 0,      /* every shell quartet in FP64 */
  VSVB_MIXED = 1,     /* quartets whose Schwarz bound is below mixed_threshold in FP32, the rest in FP64 */
  VSVB_MIXED_DF64 = 2 /* as VSVB_MIXED, but the rest in double-float (FP32 pairs, ~48-bit) on the FP32 pipes */
} vsvb_precision;

/*
 * System description: the reference's module arrays, borrowed for the
 * duration of vsvb_gpu_create.  Mirrors xm_getdims/xm_input
 * (xm_module.F90:25-335): the 15 dimension integers of input line A, the
 * density/integral tolerance exponents of line B, the geometry (bohr), the
 * basis per atom type, the spin couplings and the orbital expansions.
 */
typedef struct vsvb_system_desc {
  int natom, natom_t, npair, nunpd, ndocc, totlen, xpmax, nspinc;
  int num_sh, num_pr, nang, ndf, nxorb, mxctr;
  int ntol_d, ntol_i;             /* dtol = 10^-ntol_d, itol = 10^-ntol_i */
  const int *atom_t;              /* [natom], 1-based type */
  const double *coords;           /* [3*natom], bohr, coords(1:3, i) */
  const double *nuc_charge;       /* [natom_t] */
  const int *map_atom2shell;      /* [natom_t], 1-based */
  const int *num_shell_atom;      /* [natom_t] */
  const int *map_shell2prim;      /* [num_sh+1], 1-based */
  const int *ang_mom;             /* [num_sh] */
  const double *exponent;         /* [num_pr] */
  const double *con_coeff;        /* [num_pr], as read (before norm_prim) */
  const int *pair_sc;             /* [npair*2*max(nspinc,1)], pair_sc(k,s,isc) column-major */
  const double *coeff_sc;         /* [max(nspinc,1)] */
  const int *orbas_atnum;         /* [norbs] */
  const int *orbas_atset;         /* [mxctr*norbs], orbas_atset(k,i) column-major */
  const int *map_orbs;            /* [norbs+1], 1-based */
  const int *xpset;               /* [totlen] */
  const double *coeff;            /* [totlen] raw orbital weights */
  /* optimisation control (line B and the excited-state record; read by
   * vsvb_read_input, used by vsvb_opt_minimize only) */
  int ntol_e_min, ntol_e_max, max_iter, nset;
  double ptbnmax, feather;        /* direct minimisation: first perturbation, its reduction factor */
  const int *orbset;              /* [2*nset], orbset(1:2, iset): first and last orbital of each set */
  const int *xorb, *root;         /* [nxorb]: orbital xorb(i) takes eigenvector root(i) (0 = lowest) */
} vsvb_system_desc;

typedef struct vsvb_options {
  int precision;          /* vsvb_precision */
  double mixed_threshold; /* Schwarz bound below which a quartet runs in FP32 (default 1e-6) */
  double ao_screen;       /* AO shell-quartet Schwarz screen (default 1e-15) */
  int device;             /* CUDA device ordinal (default 0) */
  int grad_mode;          /* 0 (default): one ERI sweep yields T and dE/dX, the adjoint
                           * weights taken from the unscreened cofactor densities;
                           * 1: a second sweep recomputes the ERIs against the
                           * exactly screened dE/dT (valence.F90:1189-1190,1286-1287) */
  double prim_screen;     /* primitive-quartet Schwarz screen: a primitive quartet whose bound
                           * sqrt(max (e0|e0)_p) sqrt(max (f0|f0)_q) falls below this is skipped
                           * (default 1e-17; 0 evaluates every primitive quartet) */
  int prim_split;         /* mixed paths: the primitive quartets of the FP64-class shell
                           * quartets whose bound falls below mixed_threshold also run in
                           * FP32 (default 1; 0 keeps whole shell quartets in one arithmetic) */
  int cuda_graph;         /* energy + gradient calls replay one captured CUDA graph of the
                           * whole evaluation from the second call on (default 1) */
  int autotune;           /* pick the ERI grid caps and assembly task splits by timing them on
                           * this device at create (default 0: fixed heuristics) */
  int block_mode;         /* orbital-pair ERIs per atom quartet (s and p shells only): each
                           * shell quartet's (ab|cd) block is staged per atom quartet and
                           * transformed once per atom quartet.  0 (default): on for large
                           * s/p systems (more than 5e7 candidate shell quartets), 1: on,
                           * -1: off.  Energies only; a gradient call returns
                           * VSVB_ERR_UNSUPPORTED on a block-mode handle */
  int core_mode;          /* the determinant-pair sum over the doubly occupied core shared by
                           * every determinant, in closed form: one P x P factorisation per
                           * pair and spin (P coupled pairs) and one pass over the orbital-pair
                           * ERIs, in place of the per-pair task loop (valence.F90:1153-1433).
                           * Needs 1-10 spin-coupled pairs and no unpaired orbitals.
                           * 0 (default): on from 4096 determinant pairs with grad_mode 0, 1: on (else
                           * VSVB_ERR_UNSUPPORTED at create), -1: off.  Gradients with
                           * grad_mode 0 only (VSVB_ERR_UNSUPPORTED otherwise) */
} vsvb_options;

typedef struct vsvb_energy_result {
  double energy;   /* e_num/wfnorm + enucrep (valence.F90:344) */
  double e_num;    /* one- plus two-electron numerator */
  double e1, e2;   /* its parts */
  double wfnorm;   /* valence.F90:1106 */
  double enucrep;  /* tools_module.F90:19-40 */
  double err_est;  /* mixed paths: estimate of |E_mixed - E_fp64| from the FP32 quartets
                      (FP32 rounding of the untransferred integral sizes behind them, in units
                      of the two-electron energy per Schwarz-bound mass); 0 on FP64 */
  long long n_quartets_fp64, n_quartets_fp32; /* AO shell quartets evaluated */
  long long n_tasks;                           /* orbital-quartet tasks (valence.F90:1153-1157) */
  int n_singular_pairs;                        /* determinant pairs on the exact-minor path */
  int n_kernel_launches;                       /* kernels this call enqueued */
  double n_prim_quartets;                      /* primitive quartets evaluated (after the screen) */
  double n_prim_quartets_fp32;                 /* of which in FP32 */
} vsvb_energy_result;

typedef struct vsvb_gpu vsvb_gpu;

void vsvb_default_options(vsvb_options *opt);

/* Parse a VALENCE input file (xm_module.F90:25-335 record semantics) into a
 * description that owns its arrays; free it with vsvb_free_desc.  Coordinates
 * are converted to bohr (tools_module.F90:6-17). */
int vsvb_read_input(const char *path, vsvb_system_desc **desc, char *err, int errlen);
void vsvb_free_desc(vsvb_system_desc *desc);

/* The reference's 'orbitals' output (xm_output, xm_module.F90:464-577): per
 * orbital -- spin-coupled, unpaired, doubly occupied, then after a blank
 * line the derived basis functions -- format(5x,i2,5x,10i4) with the atom
 * list and length and format(4(i4,1x,f13.8)) with the (basis index, weight)
 * pairs, then the total energy (and, with done, the convergence line).
 * coeff: weights to write (NULL: desc->coeff).  vsvb_format_orbitals writes
 * the text to buf (cap bytes including the terminating zero; NULL buf: only
 * *len); vsvb_write_orbitals writes it to a file. */
int vsvb_format_orbitals(const vsvb_system_desc *desc, const double *coeff, double energy, double etol, int done,
                         char *buf, long cap, long *len);
int vsvb_write_orbitals(const char *path, const vsvb_system_desc *desc, const double *coeff, double energy,
                        double etol, int done);

/* The 'nelecwfn' file written beside 'orbitals' when nspinc > 1
 * (xm_module.F90:480-505): each coupling's weight (coeff_sc, NULL: the
 * description's) with its pairs, then the excited-state roots. */
int vsvb_format_nelecwfn(const vsvb_system_desc *desc, const double *coeff_sc, char *buf, long cap, long *len);
int vsvb_write_nelecwfn(const char *path, const vsvb_system_desc *desc, const double *coeff_sc);

/* Build a handle: normalises primitives (norm_prim, valence.F90:2264-2305),
 * builds the shell-pair tables, AO one-electron matrices, Schwarz bounds and
 * quartet schedules on the GPU.  Replaces the set-up half of
 * calculate_vsvb_energy (valence.F90:70-182). */
int vsvb_gpu_create(const vsvb_system_desc *desc, const vsvb_options *opt, vsvb_gpu **out);
void vsvb_gpu_destroy(vsvb_gpu *h);
const char *vsvb_gpu_last_error(const vsvb_gpu *h);

/* Guess energy for the given raw orbital weights (coeff, totlen host doubles;
 * NULL = the weights given at create).  Replaces valence.F90:337-344. */
int vsvb_gpu_energy(vsvb_gpu *h, const double *coeff, vsvb_energy_result *out);

/* Energy and its gradient with respect to the raw weights
 * (grad[totlen], host).  No counterpart exists in the reference, whose
 * optimiser (first_order_opt, valence.F90:527-844) diagonalises per-orbital
 * H/S matrices instead; this is the adjoint that a gradient optimiser
 * consumes.  The backward pass recomputes the ERIs. */
int vsvb_gpu_energy_grad(vsvb_gpu *h, const double *coeff, vsvb_energy_result *out, double *grad);

/* Same two calls with the weights/gradient already in device memory
 * (coeff_dev, grad_dev: totlen doubles on this handle's device); they enqueue
 * on the handle's stream and synchronise before returning. */
int vsvb_gpu_energy_device(vsvb_gpu *h, const double *coeff_dev, vsvb_energy_result *out);
int vsvb_gpu_energy_grad_device(vsvb_gpu *h, const double *coeff_dev, vsvb_energy_result *out, double *grad_dev);

/* Batched energies+gradients of independent molecules (one handle each) in
 * one call: all handles must live on the same device.  weights[i] / grads[i]
 * are host arrays of handle i's totlen (grads may be NULL for energy only). */
int vsvb_gpu_batch_energy_grad(vsvb_gpu *const *handles, int n, const double *const *weights,
                               vsvb_energy_result *results, double *const *grads);

/* Batched energy + gradient of many molecules as ONE CUDA graph launch.
 * vsvb_batch_create takes handles on one device, runs one warm-up
 * evaluation on each, and keeps
 * them borrowed for the batch's life.  vsvb_batch_energy_grad copies
 * weights_dev[i] (device, handle i's totlen) in, evaluates every molecule
 * -- each on its own stream branch of the graph, so their kernels run
 * concurrently -- and writes dE/dweights to grads_dev[i] (device) and the
 * energies to results[i] (host, may be NULL).  The graph is captured on the
 * first call and replayed while the pointer arrays stay the same; changed
 * pointers trigger a new capture.  stream: a cudaStream_t to launch on, or
 * NULL for the batch's own.  Returns after the results are on the host. */
typedef struct vsvb_batch vsvb_batch;
int vsvb_batch_create(vsvb_gpu *const *handles, int n, vsvb_batch **batch);
int vsvb_batch_energy_grad(vsvb_batch *batch, const double *const *weights_dev, double *const *grads_dev,
                           vsvb_energy_result *results, void *stream);
int vsvb_batch_launches(const vsvb_batch *batch); /* kernels per graph launch */
const char *vsvb_batch_last_error(const vsvb_batch *batch);
void vsvb_batch_destroy(vsvb_batch *batch);

/* Run the handle's work on a caller-owned stream (a cudaStream_t passed as
 * void*; NULL restores the handle's own stream).  Lets a host time calls with
 * CUDA events on the stream the kernels are launched on. */
int vsvb_gpu_set_stream(vsvb_gpu *h, void *stream);

/* Spin-coupling weights coeff_sc (nspinc doubles, host) for the following
 * evaluations, in place of the description's: the reference's spin_opt
 * (valence.F90:927-930) changes them between energy calls.  A captured CUDA
 * graph stays valid (the weights live in device memory). */
int vsvb_gpu_set_spin_coeffs(vsvb_gpu *h, const double *coeff_sc);

/* Diagnostics for roofline reporting: run the forward ERI pass once with a
 * CUDA event pair around every class launch.  Per launch i (up to cap):
 * ms[i] its duration, flops[i] its algorithmic FLOP count (Rys roots, 2D
 * tables, component sums and the orbital-pair transform, counted per
 * primitive quartet / shell quartet), cls[i] = 100*prec + 10*bra + ket.
 * Returns the number of launches or a negative status. */
int vsvb_gpu_eri_profile(vsvb_gpu *h, double *ms, double *flops, int *cls, int cap);
/* The same with the launches one after another in mode 0 (forward) or 3
 * (forward + adjoint; needs a previous vsvb_gpu_energy_grad on the handle,
 * whose dE/dT it reuses).  cls[i] = 100*k + 10*bra + ket, k = 0 FP64,
 * 1 FP32, 2 double-float, 3 the FP32 tail of an FP64-class schedule. */
int vsvb_gpu_eri_profile_mode(vsvb_gpu *h, int mode, double *ms, double *flops, int *cls, int cap);

/* In-situ timing of the ERI class launches inside ordinary calls: with
 * vsvb_gpu_set_sweep_timing(h, 1) every ERI sweep records a CUDA event pair
 * around each class launch on the side stream it runs on (the launches of
 * one sweep run concurrently).  vsvb_gpu_sweep_times then returns, for the
 * last sweep, per class launch i (up to cap): ms[i] its duration, flops[i]
 * its algorithmic FLOP count for the sweep's mode (forward, or forward plus
 * adjoint on the fused gradient path), cls[i] = 100*kind + 10*bra + ket with
 * kind 0 FP64, 1 FP32, 2 double-float.  Returns the number of launches (0
 * when timing is off) or a negative status. */
int vsvb_gpu_set_sweep_timing(vsvb_gpu *h, int on);
int vsvb_gpu_sweep_times(vsvb_gpu *h, double *ms, double *flops, int *cls, int cap);
/* The launch geometry in use (after the autotuner, if enabled): the
 * assembly task splits per determinant pair, and per ERI launch of the
 * sweep (up to cap) its class code and grid cap in blocks per SM.  Returns
 * the number of ERI launches written. */
int vsvb_gpu_launch_config(const vsvb_gpu *h, int *nsplit, int *codes, int *blocks_per_sm, int cap);

/* Wall time of the last ERI sweep (fork to join on the handle's stream) in
 * *ms; 0 when timing is off. */
int vsvb_gpu_sweep_wall_ms(vsvb_gpu *h, double *ms);

/* Measured FP64 and FP32 FMA throughput of this device in FLOP/s (a dependent
 * FMA chain kernel sized to fill every SM), for roofline denominators. */
int vsvb_gpu_fma_peak(int device, double *fp64_flops, double *fp32_flops);

/* Batched determinant and inverse of nmat dense n x n matrices (row-major,
 * device memory, a_dev[nmat*n*n]) by Gauss-Jordan elimination with partial
 * pivoting: the factorisation applied to every spin block of every
 * determinant pair, replacing givdr/givens_single (valence.F90:2067-2144,
 * givens.F90:230-262).  Outputs (device): det_dev[nmat], inv_dev[nmat*n*n]
 * (row-major inverse), sing_dev[nmat] = 1 when a pivot falls below 1e-7 of
 * the matrix's largest entry (the determinant then comes from LU and the
 * inverse is zero).  Enqueues on stream (a cudaStream_t, NULL = default)
 * and synchronises it.  Allocates n x 2n doubles of scratch per matrix. */
int vsvb_det_factor(const double *a_dev, int n, int nmat, double *det_dev, double *inv_dev, int *sing_dev,
                    void *stream);

/* Same factorisation without any device allocation, for callers that may
 * not call cudaMalloc (their device memory is owned by another framework's
 * allocator, or allocation is forbidden in the phase they run in).  Has no
 * counterpart in the reference.  Scratch is a fixed 4 MiB device array per
 * device (2*n*n*nmat doubles at most, else VSVB_ERR_TOO_LARGE) held for the
 * life of the process; the first call on a device resolves that array's
 * address once and keeps it, so the library must not be used across a
 * cudaDeviceReset.  Every call synchronises its stream before returning, so
 * no call may be made while that stream is capturing.  Concurrent calls share
 * the array and must not overlap on the GPU.  Arguments and results as
 * vsvb_det_factor. */
int vsvb_det_factor_noalloc(const double *a_dev, int n, int nmat, double *det_dev, double *inv_dev, int *sing_dev,
                            void *stream);

/*
 * Wave-function optimisation (the reference's minimize_energy with
 * first_order_opt, spin_opt and demgs_opt, valence.F90:350-936, 2744-2885).
 * An optimiser owns a copy of the description, a handle for energies and,
 * created on first use, one handle per orbital (two for a DOCC orbital when
 * there are unpaired electrons) for first_order_opt's matrices.
 */
typedef struct vsvb_opt vsvb_opt;

typedef struct vsvb_opt_result {
  double energy;         /* final energy (the last eigenvalue + enucrep, as the reference reports it) */
  double guess_energy;   /* energy of the normalised input weights */
  double etol;           /* the last tolerance of the feathering loop, kcal/mol */
  double seconds;        /* wall time of the call */
  int iterations;        /* num_iter of minimize_energy */
  int converged;         /* the reference's 'calculation converged' test */
  long long n_energy_evals, n_hs_builds;
} vsvb_opt_result;

int vsvb_opt_create(const vsvb_system_desc *desc, const vsvb_options *opt, vsvb_opt **out);
void vsvb_opt_destroy(vsvb_opt *o);
const char *vsvb_opt_last_error(const vsvb_opt *o);

/* first_order_opt's Hamiltonian and overlap (valence.F90:609-758) of orbital
 * iorb (1-based) for raw weights coeff (totlen) and, when nspinc > 0, the
 * spin-coupling weights coeff_sc (NULL: keep the current ones): nb x nb
 * column-major, nb = map_orbs(iorb+1) - map_orbs(iorb), element (ib, jb) the
 * energy numerator / wave-function norm with the bra's slot of iorb holding
 * entry ib and the ket's entry jb; symmetric. */
int vsvb_opt_first_order_hs(vsvb_opt *o, const double *coeff, const double *coeff_sc, int iorb, double *ham,
                            double *ovl);
/* spin_opt's matrices (valence.F90:866-897), nspinc x nspinc. */
int vsvb_opt_spin_hs(vsvb_opt *o, const double *coeff, double *ham, double *ovl);

/* minimize_energy (valence.F90:2744-2885) from raw weights coeff (totlen,
 * updated in place to the optimised, normalised weights) and coeff_sc
 * (nspinc, updated; may be NULL without spin couplings), with the
 * description's max_iter, ntol_e_min..ntol_e_max, orbital sets, excited-state
 * roots and ptbnmax/feather (direct minimisation when ptbnmax > 0 and there
 * are no excited-state roots). */
int vsvb_opt_minimize(vsvb_opt *o, double *coeff, double *coeff_sc, vsvb_opt_result *res);

/* Files vsvb_opt_minimize writes as the reference does (xm_output 'save'
 * after the guess energy and after every orbital or coupling update, 'done'
 * on convergence, valence.F90:192,453,489,2823,2859,2882): the orbitals file
 * at orbitals_path and, with more than one coupling, the coupling file at
 * nelecwfn_path.  NULL switches a file off (the default). */
int vsvb_opt_set_output(vsvb_opt *o, const char *orbitals_path, const char *nelecwfn_path);

/* EISPACK rsg (rsg.F) on the GPU: ham w = e ovl w for symmetric ham and
 * positive-definite ovl (n x n, column-major, leading dimension ld);
 * eigenvalues ascending into eig, eigenvectors (w^T ovl w = 1) into the
 * columns of w (leading dimension ldw).  VSVB_ERR_SINGULAR when ovl is not
 * positive definite (rsg's ierr = 7n+1).  n <= 1024. */
int vsvb_rsg(int n, const double *ham, const double *ovl, int ld, double *eig, double *w, int ldw);

/* Sizes of a handle (for bindings). */
int vsvb_gpu_totlen(const vsvb_gpu *h);
int vsvb_gpu_num_orbitals(const vsvb_gpu *h);

/* Diagnostics used by the parity tests: copy the orbital-pair ERI matrix
 * T[p*np+q] = (i k | j l) for pairs p=(i,k), q=(j,l) (0-based, i>=k,
 * index i*(i+1)/2+k) of the last evaluation, np = n(n+1)/2, n = spatial
 * orbitals.  Returns np, or a negative vsvb_status. */
int vsvb_gpu_debug_orbital_eri(vsvb_gpu *h, double *out, size_t cap);
/* Sampled entries of the same matrix: out[i] = T[idx[i]] (idx[i] < np*np),
 * for systems whose T is too large to copy whole.  Returns np, or a
 * negative vsvb_status. */
int vsvb_gpu_debug_orbital_eri_at(vsvb_gpu *h, const long long *idx, int n, double *out);
/* Block mode (vsvb_options.block_mode) figures of one energy evaluation:
 * algorithmic FLOPs of the ERI launches per kind (FP64, FP32, double-float;
 * primitive-quartet work as in vsvb_gpu_eri_profile plus the transfer to
 * (ab|cd)), of the per-atom-quartet transforms (FP64, FP32, double-float),
 * and counts: atom quartets, chunks, kernel launches of the sweep.  Returns
 * 1 when the handle runs in block mode, 0 when not. */
int vsvb_gpu_block_stats(const vsvb_gpu *h, double *eri_flops3, double *transform_flops3, long long *counts3);
/* Core mode (vsvb_options.core_mode): FMAs of the pair-summed density GEMM
 * of one energy evaluation, and counts2 = {determinant pairs, coupled
 * orbitals}.  Returns 1 on a core-mode handle, 0 otherwise, negative on error. */
int vsvb_gpu_core_stats(const vsvb_gpu *h, double *gemm_fma, long long *counts2);
/* Orbital overlap and core-Hamiltonian matrices of the last evaluation
 * (n x n, row-major). */
int vsvb_gpu_debug_orbital_1e(vsvb_gpu *h, double *s, double *hcore, size_t cap);

#ifdef __cplusplus
}
#endif
#endif
