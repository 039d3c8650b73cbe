/* handle_internal.h -- what the optimiser (optimize.cu) uses of a handle
 * beyond the public C ABI. */
#ifndef VSVB_HANDLE_INTERNAL_H
#define VSVB_HANDLE_INTERNAL_H
#include <cuda_runtime.h>

#include "../../include/vsvb_gpu.h"

/* A handle for first_order_opt's matrices of one orbital.  d is the
 * description of the wave function as first_order_opt sets it up
 * (valence.F90:555-603): split 0 -- the orbitals as given, the substituted
 * orbital is spatial orbital sub itself; split 1 / 2 -- d carries one orbital
 * more than its counts say (the substituted one), and the first DOCC pair's
 * alpha / beta slot holds it (spatial orbital sub = 2*npair+nunpd, or +1). */
int vsvb_gpu_create_sub(const vsvb_system_desc *d, const vsvb_options *opt, int split, int sub, vsvb_gpu **out);

/* Columns nu = 0..nb-1 of first_order_opt's H and S (nb x nb, column-major,
 * device): the evaluation's weights are w_dev[src[t]] (src[t] >= 0) and, on
 * the substituted orbital's entries j0..j0+nb, the unit vector e_nu.  Each
 * column is half the derivative of the energy numerator / the norm with
 * respect to those entries (both are quadratic forms in them). */
int gpu_hs_columns(vsvb_gpu *h, const double *w_dev, const int *src_dev, int j0, int nb, double *H_dev, double *S_dev);

/* spin_opt's coupling blocks (nsc x nsc, row isc, column jsc; device) for
 * weights w_dev: the energy numerator and the norm of the determinant pairs
 * of bra coupling isc and ket coupling jsc. */
int gpu_spin_blocks(vsvb_gpu *h, const double *w_dev, double *BH_dev, double *BS_dev);

/* the spin-coupling weights of the following evaluations (host array, nsc) */
int gpu_set_spin_coeffs(vsvb_gpu *h, const double *csc);
/* normal() (valence.F90:2157-2182) factors for host weights w: per derived
 * basis function (ndf) and per orbital (nsp) */
int gpu_orbital_scales(vsvb_gpu *h, const double *w, double *ndf_scale, double *orb_scale);
cudaStream_t gpu_stream(vsvb_gpu *h);
int gpu_nsc(const vsvb_gpu *h);
#endif
