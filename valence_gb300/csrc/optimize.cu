/*
 * optimize.cu -- the reference's wave-function optimisation on the GPU path.
 *
 *   first_order_opt (valence.F90:527-844)  vsvb_opt_first_order_hs
 *     The reference builds the orbital's H and S element by element: for every
 *     pair (ib, jb) of its expansion entries a full non-symmetric energy
 *     evaluation with the bra's slot of the orbital holding entry ib and the
 *     ket's entry jb, nb(nb+1)/2 evaluations.  Both matrices are the
 *     quadratic forms of the energy numerator and of the norm in that slot's
 *     weights, so column jb is half the derivative of either at weights
 *     e_jb: nb forward passes with the adjoint of each (gpu_hs_columns).
 *     A DOCC orbital is split as the reference splits it (:578-603), its
 *     alpha slot holding the substituted weights; with unpaired electrons
 *     the beta-slot matrices are added (spin averaging, :708-749).
 *   spin_opt (:850-936)                     vsvb_opt_spin_hs
 *     one walk with every coupling weight 1, summed per coupling pair.
 *   rsg (EISPACK rsg.F: reduc, tred2, tql2, rebak)  vsvb_rsg
 *     H w = e S w on one CTA: Cholesky S = L L^T, A = L^-1 H L^-T, cyclic
 *     Jacobi rotations in parallel (round-robin) order, w = L^-T v; ascending
 *     eigenvalues, w^T S w = 1.
 *   demgs_opt (:350-524), minimize_energy (:2744-2885)  vsvb_opt_minimize
 *     the host control loop over GPU evaluations, in the reference's order
 *     and with its convergence tests.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "../../include/vsvb_gpu.h"
#include "handle_internal.h"

namespace {

constexpr double kTokcal = 627.509469; /* valence.F90:2756 */
constexpr int kRsgMax = 1024;

/* ---------------- rsg on one CTA ---------------- */

struct RsgArgs {
  int n, m;              /* order; m = n rounded up to even (round-robin) */
  const double *H, *S;   /* n x n column-major, leading dimension ld */
  int ld;
  double *L, *A, *V, *Y; /* n x n work (column-major, ld n) */
  double *eig, *W;       /* out: n, n x n (leading dimension ldw) */
  int ldw;
  int *info;             /* 0, or 7n+1 when S is not positive definite (rsg's ierr) */
};

__device__ __forceinline__ double &at(double *a, int n, int i, int j) { return a[(size_t)j * n + i]; }

__global__ void __launch_bounds__(256) rsg_kernel(RsgArgs r) {
  const int n = r.n, m = r.m, tid = threadIdx.x, nt = blockDim.x;
  __shared__ double cs[kRsgMax / 2], sn[kRsgMax / 2];
  __shared__ int top[kRsgMax / 2], bot[kRsgMax / 2];
  __shared__ int fail;
  __shared__ double red[256];
  __shared__ int order[kRsgMax];
  if (tid == 0) fail = 0;
  /* Cholesky (right-looking) of S into L (lower) */
  for (int t = tid; t < n * n; t += nt) {
    const int i = t % n, j = t / n;
    r.L[t] = i >= j ? r.S[(size_t)j * r.ld + i] : 0.0;
  }
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    if (tid == 0) {
      const double d = at(r.L, n, k, k);
      if (!(d > 0.0)) fail = 1;
      at(r.L, n, k, k) = d > 0.0 ? sqrt(d) : 1.0;
    }
    __syncthreads();
    if (fail) break;
    const double lkk = at(r.L, n, k, k);
    for (int i = k + 1 + tid; i < n; i += nt) at(r.L, n, i, k) /= lkk;
    __syncthreads();
    const int rem = n - k - 1;
    for (int t = tid; t < rem * rem; t += nt) {
      const int i = k + 1 + t % rem, j = k + 1 + t / rem;
      if (j <= i) at(r.L, n, i, j) -= at(r.L, n, i, k) * at(r.L, n, j, k);
    }
    __syncthreads();
  }
  if (fail) {
    if (tid == 0) *r.info = 7 * n + 1;
    return;
  }
  /* Y = L^-1 H (a column per thread), then row i of A = (L^-1 Y(i,:)^T)^T */
  for (int c = tid; c < n; c += nt)
    for (int i = 0; i < n; ++i) {
      double v = r.H[(size_t)c * r.ld + i];
      for (int j = 0; j < i; ++j) v -= at(r.L, n, i, j) * at(r.Y, n, j, c);
      at(r.Y, n, i, c) = v / at(r.L, n, i, i);
    }
  __syncthreads();
  for (int row = tid; row < n; row += nt)
    for (int c = 0; c < n; ++c) {
      double v = at(r.Y, n, row, c);
      for (int j = 0; j < c; ++j) v -= at(r.L, n, c, j) * at(r.A, n, row, j);
      at(r.A, n, row, c) = v / at(r.L, n, c, c);
    }
  __syncthreads();
  for (int t = tid; t < n * n; t += nt) {
    const int i = t % n, j = t / n;
    if (i < j) {
      const double v = 0.5 * (at(r.A, n, i, j) + at(r.A, n, j, i));
      at(r.A, n, i, j) = v;
      at(r.A, n, j, i) = v;
    }
    r.V[t] = i == j ? 1.0 : 0.0;
  }
  /* round-robin pairing of m indices (index n is a dummy when n is odd) */
  for (int i = tid; i < m / 2; i += nt) {
    top[i] = 2 * i;
    bot[i] = 2 * i + 1;
  }
  __syncthreads();
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0, all = 0.0;
    for (int t = tid; t < n * n; t += nt) {
      const double v = r.A[t] * r.A[t];
      all += v;
      if (t % n != t / n) off += v;
    }
    red[tid] = off;
    __syncthreads();
    for (int s = nt / 2; s > 0; s >>= 1) {
      if (tid < s) red[tid] += red[tid + s];
      __syncthreads();
    }
    off = red[0];
    __syncthreads();
    red[tid] = all;
    __syncthreads();
    for (int s = nt / 2; s > 0; s >>= 1) {
      if (tid < s) red[tid] += red[tid + s];
      __syncthreads();
    }
    all = red[0];
    __syncthreads();
    if (!(off > 1e-30 * all)) break;
    for (int round = 0; round < m - 1; ++round) {
      for (int i = tid; i < m / 2; i += nt) {
        const int p = min(top[i], bot[i]), q = max(top[i], bot[i]);
        double c = 1.0, s = 0.0;
        if (q < n) {
          const double apq = at(r.A, n, p, q);
          if (apq != 0.0) {
            const double theta = (at(r.A, n, q, q) - at(r.A, n, p, p)) / (2.0 * apq);
            const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
            c = 1.0 / sqrt(t * t + 1.0);
            s = t * c;
          }
        }
        cs[i] = c;
        sn[i] = s;
      }
      __syncthreads();
      /* A <- J^T A (rows p, q), then A <- A J and V <- V J (columns p, q) */
      for (int t = tid; t < (m / 2) * n; t += nt) {
        const int i = t / n, k = t % n;
        const int p = min(top[i], bot[i]), q = max(top[i], bot[i]);
        if (q >= n || sn[i] == 0.0) continue;
        const double a = at(r.A, n, p, k), b = at(r.A, n, q, k);
        at(r.A, n, p, k) = cs[i] * a - sn[i] * b;
        at(r.A, n, q, k) = sn[i] * a + cs[i] * b;
      }
      __syncthreads();
      for (int t = tid; t < (m / 2) * n; t += nt) {
        const int i = t / n, k = t % n;
        const int p = min(top[i], bot[i]), q = max(top[i], bot[i]);
        if (q >= n || sn[i] == 0.0) continue;
        const double a = at(r.A, n, k, p), b = at(r.A, n, k, q);
        at(r.A, n, k, p) = cs[i] * a - sn[i] * b;
        at(r.A, n, k, q) = sn[i] * a + cs[i] * b;
        const double va = at(r.V, n, k, p), vb = at(r.V, n, k, q);
        at(r.V, n, k, p) = cs[i] * va - sn[i] * vb;
        at(r.V, n, k, q) = sn[i] * va + cs[i] * vb;
      }
      __syncthreads();
      if (tid == 0 && m > 2) {
        /* index top[0] stays; the others rotate one place */
        const int last_top = top[m / 2 - 1], first_bot = bot[0];
        for (int i = m / 2 - 1; i > 1; --i) top[i] = top[i - 1];
        if (m / 2 > 1) top[1] = first_bot;
        for (int i = 0; i < m / 2 - 1; ++i) bot[i] = bot[i + 1];
        bot[m / 2 - 1] = last_top;
      }
      __syncthreads();
    }
  }
  /* ascending order, then w = L^-T v */
  if (tid == 0) {
    for (int i = 0; i < n; ++i) order[i] = i;
    for (int i = 0; i < n; ++i) {
      int b = i;
      for (int j = i + 1; j < n; ++j)
        if (at(r.A, n, order[j], order[j]) < at(r.A, n, order[b], order[b])) b = j;
      const int t = order[i];
      order[i] = order[b];
      order[b] = t;
    }
    for (int i = 0; i < n; ++i) r.eig[i] = at(r.A, n, order[i], order[i]);
    *r.info = 0;
  }
  __syncthreads();
  for (int c = tid; c < n; c += nt) {
    const int src = order[c];
    for (int i = n - 1; i >= 0; --i) {
      double v = at(r.V, n, i, src);
      for (int j = i + 1; j < n; ++j) v -= at(r.L, n, j, i) * r.W[(size_t)c * r.ldw + j];
      r.W[(size_t)c * r.ldw + i] = v / at(r.L, n, i, i);
    }
  }
}

/* ---------------- descriptions ---------------- */

/* an owned copy of a system description */
struct DescCopy {
  vsvb_system_desc d{};
  std::vector<int> atom_t, map_atom2shell, num_shell_atom, map_shell2prim, ang_mom, pair_sc, orbas_atnum,
      orbas_atset, map_orbs, xpset, orbset, xorb, root;
  std::vector<double> coords, nuc_charge, exponent, con_coeff, coeff_sc, coeff;
  void wire() {
    d.atom_t = atom_t.data();
    d.coords = coords.data();
    d.nuc_charge = nuc_charge.data();
    d.map_atom2shell = map_atom2shell.data();
    d.num_shell_atom = num_shell_atom.data();
    d.map_shell2prim = map_shell2prim.data();
    d.ang_mom = ang_mom.data();
    d.exponent = exponent.data();
    d.con_coeff = con_coeff.data();
    d.pair_sc = pair_sc.data();
    d.coeff_sc = coeff_sc.data();
    d.orbas_atnum = orbas_atnum.data();
    d.orbas_atset = orbas_atset.data();
    d.map_orbs = map_orbs.data();
    d.xpset = xpset.data();
    d.coeff = coeff.data();
    d.orbset = orbset.data();
    d.xorb = xorb.data();
    d.root = root.data();
  }
};

template <typename T>
std::vector<T> copy_of(const T *p, size_t n) {
  std::vector<T> v(n + 1, T{});
  if (p && n) std::copy(p, p + n, v.begin());
  return v;
}

void copy_desc(const vsvb_system_desc *s, DescCopy &c) {
  c.d = *s;
  const int norbs = 2 * s->npair + s->nunpd + s->ndocc + s->ndf, nsc = s->nspinc > 0 ? s->nspinc : 1;
  c.atom_t = copy_of(s->atom_t, s->natom);
  c.coords = copy_of(s->coords, 3 * (size_t)s->natom);
  c.nuc_charge = copy_of(s->nuc_charge, s->natom_t);
  c.map_atom2shell = copy_of(s->map_atom2shell, s->natom_t);
  c.num_shell_atom = copy_of(s->num_shell_atom, s->natom_t);
  c.map_shell2prim = copy_of(s->map_shell2prim, (size_t)s->num_sh + 1);
  c.ang_mom = copy_of(s->ang_mom, s->num_sh);
  c.exponent = copy_of(s->exponent, s->num_pr);
  c.con_coeff = copy_of(s->con_coeff, s->num_pr);
  c.pair_sc = copy_of(s->pair_sc, 2 * (size_t)s->npair * nsc);
  c.coeff_sc = copy_of(s->coeff_sc, nsc);
  c.orbas_atnum = copy_of(s->orbas_atnum, norbs);
  c.orbas_atset = copy_of(s->orbas_atset, (size_t)s->mxctr * norbs);
  c.map_orbs = copy_of(s->map_orbs, (size_t)norbs + 1);
  c.xpset = copy_of(s->xpset, s->totlen);
  c.coeff = copy_of(s->coeff, s->totlen);
  c.orbset = copy_of(s->orbset, 2 * (size_t)std::max(s->nset, 0));
  c.xorb = copy_of(s->xorb, std::max(s->nxorb, 0));
  c.root = copy_of(s->root, std::max(s->nxorb, 0));
  c.wire();
}

/* first_order_opt's wave function for DOCC orbital o (0-based): the orbital
 * list with the substituted orbital and o as the first DOCC pair's alpha /
 * beta slots (split 1) or beta / alpha (split 2), the other DOCC orbitals
 * after them, derived basis functions last.  src maps each weight of the new
 * list to the caller's weights (-1 on the substituted orbital). */
void split_desc(const DescCopy &in, int o, int split, DescCopy &out, std::vector<int> &src, int &j0) {
  const vsvb_system_desc &d = in.d;
  const int nnd = 2 * d.npair + d.nunpd, norbs = nnd + d.ndocc + d.ndf, mx = d.mxctr;
  std::vector<int> list; /* original orbital per new position; -2 = the substituted one */
  for (int i = 0; i < nnd; ++i) list.push_back(i);
  if (split == 1) {
    list.push_back(-2);
    list.push_back(o);
  } else {
    list.push_back(o);
    list.push_back(-2);
  }
  for (int i = nnd; i < nnd + d.ndocc; ++i)
    if (i != o) list.push_back(i);
  for (int i = nnd + d.ndocc; i < norbs; ++i) list.push_back(i);
  out = in;
  out.orbas_atnum.assign(list.size() + 1, 0);
  out.orbas_atset.assign((size_t)mx * (list.size() + 1), 0);
  out.map_orbs.assign(list.size() + 2, 0);
  out.xpset.clear();
  out.coeff.clear();
  src.clear();
  out.map_orbs[0] = 1;
  for (size_t k = 0; k < list.size(); ++k) {
    const int from = list[k] == -2 ? o : list[k];
    out.orbas_atnum[k] = in.orbas_atnum[from];
    for (int a = 0; a < mx; ++a) out.orbas_atset[a + (size_t)mx * k] = in.orbas_atset[a + (size_t)mx * from];
    if (list[k] == -2) j0 = (int)out.xpset.size();
    for (int j = in.map_orbs[from] - 1; j < in.map_orbs[from + 1] - 1; ++j) {
      out.xpset.push_back(in.xpset[j]);
      out.coeff.push_back(in.coeff[j]);
      src.push_back(list[k] == -2 ? -1 : j);
    }
    out.map_orbs[k + 1] = (int)out.xpset.size() + 1;
  }
  out.d.totlen = (int)out.xpset.size();
  out.xpset.push_back(0);
  out.coeff.push_back(0.0);
  out.wire();
}

template <typename T>
struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  cudaError_t alloc(size_t count) {
    if (count <= n && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    n = count;
    return cudaMalloc(&p, sizeof(T) * std::max<size_t>(count, 1));
  }
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

/* one first_order_opt handle: orbital o with split 0/1/2 */
struct SubHandle {
  vsvb_gpu *h = nullptr;
  DescCopy desc;
  DevBuf<int> src;
  int j0 = 0, nb = 0;
  int csc_version = -1;
  ~SubHandle() {
    if (h) vsvb_gpu_destroy(h);
  }
};

}  // namespace

struct vsvb_opt {
  vsvb_options opt{};
  DescCopy desc;
  std::string err;
  vsvb_gpu *main = nullptr;
  std::map<std::pair<int, int>, SubHandle *> subs;
  std::vector<double> csc; /* spin-coupling weights in use */
  int csc_version = 0, main_csc_version = -1;
  DevBuf<double> w, H, S, H2, S2, BH, BS;
  int nnd = 0, nsp = 0, nsc = 1;
  double enuc = 0.0;
  std::string out_orbitals, out_nelecwfn; /* xm_output files (empty: off) */
  double etol_kcal = 0.0;                 /* the loop's current tolerance, for 'done' */
  long long n_energy = 0, n_hs = 0;
  ~vsvb_opt() {
    for (auto &kv : subs) delete kv.second;
    if (main) vsvb_gpu_destroy(main);
  }
};

namespace {

int opt_fail(vsvb_opt *o, int rc, const std::string &what) {
  o->err = what;
  return rc;
}

int cuda_check(vsvb_opt *o, cudaError_t e, const char *what) {
  if (e == cudaSuccess) return VSVB_OK;
  return opt_fail(o, VSVB_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define OK_OR_RETURN(expr)   \
  do {                       \
    int rc_ = (expr);        \
    if (rc_) return rc_;     \
  } while (0)

int sync_main_spin(vsvb_opt *o) {
  if (o->main_csc_version == o->csc_version) return VSVB_OK;
  int rc = gpu_set_spin_coeffs(o->main, o->csc.data());
  if (rc) return opt_fail(o, rc, vsvb_gpu_last_error(o->main));
  o->main_csc_version = o->csc_version;
  return VSVB_OK;
}

int get_sub(vsvb_opt *o, int orb, int split, SubHandle **out) {
  auto key = std::make_pair(orb, split);
  auto it = o->subs.find(key);
  if (it == o->subs.end()) {
    auto *s = new SubHandle();
    const vsvb_system_desc &d = o->desc.d;
    std::vector<int> src;
    int sub;
    if (split == 0) {
      s->desc = o->desc;
      s->desc.wire();
      s->j0 = d.map_orbs[orb] - 1;
      src.resize(d.totlen);
      for (int t = 0; t < d.totlen; ++t) src[t] = t;
      sub = orb;
    } else {
      split_desc(o->desc, orb, split, s->desc, src, s->j0);
      sub = o->nnd + (split == 1 ? 0 : 1);
    }
    s->nb = d.map_orbs[orb + 1] - d.map_orbs[orb];
    for (int k = 0; k < s->nb; ++k) src[s->j0 + k] = -1;
    int rc = vsvb_gpu_create_sub(&s->desc.d, &o->opt, split, sub, &s->h);
    if (rc) {
      std::string e = s->h ? vsvb_gpu_last_error(s->h) : "create failed";
      delete s;
      return opt_fail(o, rc, e);
    }
    if (s->src.alloc(src.size()) != cudaSuccess ||
        cudaMemcpy(s->src.p, src.data(), sizeof(int) * src.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
      delete s;
      return opt_fail(o, VSVB_ERR_CUDA, "upload of the weight map failed");
    }
    it = o->subs.emplace(key, s).first;
  }
  SubHandle *s = it->second;
  if (s->csc_version != o->csc_version) {
    int rc = gpu_set_spin_coeffs(s->h, o->csc.data());
    if (rc) return opt_fail(o, rc, vsvb_gpu_last_error(s->h));
    s->csc_version = o->csc_version;
  }
  *out = s;
  return VSVB_OK;
}

/* H, S (nb x nb, column-major, symmetrised) of orbital orb (0-based) */
int first_order_hs(vsvb_opt *o, const double *coeff, int orb, double *ham, double *ovl) {
  const vsvb_system_desc &d = o->desc.d;
  const int nb = d.map_orbs[orb + 1] - d.map_orbs[orb];
  OK_OR_RETURN(cuda_check(o, o->w.alloc(d.totlen), "alloc"));
  OK_OR_RETURN(cuda_check(o, cudaMemcpy(o->w.p, coeff, sizeof(double) * d.totlen, cudaMemcpyHostToDevice), "copy"));
  const size_t nn = (size_t)nb * nb;
  OK_OR_RETURN(cuda_check(o, o->H.alloc(nn), "alloc"));
  OK_OR_RETURN(cuda_check(o, o->S.alloc(nn), "alloc"));
  std::vector<double> h(nn), s(nn);
  const bool docc = orb >= o->nnd;
  SubHandle *sh = nullptr;
  OK_OR_RETURN(get_sub(o, orb, docc ? 1 : 0, &sh));
  int rc = gpu_hs_columns(sh->h, o->w.p, sh->src.p, sh->j0, nb, o->H.p, o->S.p);
  if (rc) return opt_fail(o, rc, vsvb_gpu_last_error(sh->h));
  OK_OR_RETURN(cuda_check(o, cudaMemcpy(h.data(), o->H.p, sizeof(double) * nn, cudaMemcpyDeviceToHost), "copy"));
  OK_OR_RETURN(cuda_check(o, cudaMemcpy(s.data(), o->S.p, sizeof(double) * nn, cudaMemcpyDeviceToHost), "copy"));
  o->n_hs++;
  if (docc && d.nunpd > 0) {
    /* spin average: the beta slot substituted (valence.F90:708-749) */
    OK_OR_RETURN(get_sub(o, orb, 2, &sh));
    rc = gpu_hs_columns(sh->h, o->w.p, sh->src.p, sh->j0, nb, o->H.p, o->S.p);
    if (rc) return opt_fail(o, rc, vsvb_gpu_last_error(sh->h));
    std::vector<double> h2(nn), s2(nn);
    OK_OR_RETURN(cuda_check(o, cudaMemcpy(h2.data(), o->H.p, sizeof(double) * nn, cudaMemcpyDeviceToHost), "copy"));
    OK_OR_RETURN(cuda_check(o, cudaMemcpy(s2.data(), o->S.p, sizeof(double) * nn, cudaMemcpyDeviceToHost), "copy"));
    for (size_t k = 0; k < nn; ++k) {
      h[k] += h2[k];
      s[k] += s2[k];
    }
    o->n_hs++;
  }
  for (int i = 0; i < nb; ++i)
    for (int j = 0; j < nb; ++j) {
      ham[(size_t)j * nb + i] = 0.5 * (h[(size_t)j * nb + i] + h[(size_t)i * nb + j]);
      ovl[(size_t)j * nb + i] = 0.5 * (s[(size_t)j * nb + i] + s[(size_t)i * nb + j]);
    }
  return VSVB_OK;
}

int spin_hs(vsvb_opt *o, const double *coeff, double *ham, double *ovl) {
  const int nsc = o->nsc;
  const vsvb_system_desc &d = o->desc.d;
  OK_OR_RETURN(sync_main_spin(o));
  OK_OR_RETURN(cuda_check(o, o->w.alloc(d.totlen), "alloc"));
  OK_OR_RETURN(cuda_check(o, cudaMemcpy(o->w.p, coeff, sizeof(double) * d.totlen, cudaMemcpyHostToDevice), "copy"));
  OK_OR_RETURN(cuda_check(o, o->BH.alloc((size_t)nsc * nsc), "alloc"));
  OK_OR_RETURN(cuda_check(o, o->BS.alloc((size_t)nsc * nsc), "alloc"));
  int rc = gpu_spin_blocks(o->main, o->w.p, o->BH.p, o->BS.p);
  if (rc) return opt_fail(o, rc, vsvb_gpu_last_error(o->main));
  std::vector<double> bh((size_t)nsc * nsc), bs((size_t)nsc * nsc);
  OK_OR_RETURN(cuda_check(o, cudaMemcpy(bh.data(), o->BH.p, sizeof(double) * bh.size(), cudaMemcpyDeviceToHost), "copy"));
  OK_OR_RETURN(cuda_check(o, cudaMemcpy(bs.data(), o->BS.p, sizeof(double) * bs.size(), cudaMemcpyDeviceToHost), "copy"));
  /* block (isc, jsc) is row isc * nsc + jsc; the symmetric task walk splits
   * a coupling pair's terms between (isc, jsc) and (jsc, isc) */
  for (int i = 0; i < nsc; ++i)
    for (int j = 0; j < nsc; ++j) {
      ham[(size_t)j * nsc + i] = 0.5 * (bh[(size_t)i * nsc + j] + bh[(size_t)j * nsc + i]);
      ovl[(size_t)j * nsc + i] = 0.5 * (bs[(size_t)i * nsc + j] + bs[(size_t)j * nsc + i]);
    }
  return VSVB_OK;
}

int energy_of(vsvb_opt *o, const double *coeff, double *e) {
  OK_OR_RETURN(sync_main_spin(o));
  vsvb_energy_result r;
  int rc = vsvb_gpu_energy(o->main, coeff, &r);
  if (rc) return opt_fail(o, rc, vsvb_gpu_last_error(o->main));
  o->n_energy++;
  *e = r.energy;
  return VSVB_OK;
}

/* normal(iorb, iorb) (valence.F90:2157-2182) on the host weights */
int normalise(vsvb_opt *o, double *coeff, int orb) {
  std::vector<double> sc(o->nsp);
  int rc = gpu_orbital_scales(o->main, coeff, nullptr, sc.data());
  if (rc) return opt_fail(o, rc, vsvb_gpu_last_error(o->main));
  const vsvb_system_desc &d = o->desc.d;
  for (int j = d.map_orbs[orb] - 1; j < d.map_orbs[orb + 1] - 1; ++j) coeff[j] *= sc[orb];
  return VSVB_OK;
}

int rsg_device(vsvb_opt *o, int n, const double *ham, const double *ovl, double *eig, double *w) {
  int rc = vsvb_rsg(n, ham, ovl, n, eig, w, n);
  if (rc == VSVB_ERR_SINGULAR) return opt_fail(o, rc, "rsg: the overlap matrix is not positive definite");
  if (rc) return opt_fail(o, rc, "rsg failed");
  return VSVB_OK;
}

int root_of(const vsvb_system_desc &d, int iorb1) {
  int r = 0;
  for (int i = 0; i < d.nxorb; ++i)
    if (d.xorb[i] == iorb1) r = d.root[i];
  return r;
}

/* xm_output (xm_module.F90:464-577): the orbitals file, and with more than
 * one coupling the coupling file, for the current weights */
int save_output(vsvb_opt *o, const double *coeff, double energy, bool done) {
  if (!o->out_orbitals.empty()) {
    int rc = vsvb_write_orbitals(o->out_orbitals.c_str(), &o->desc.d, coeff, energy, o->etol_kcal, done ? 1 : 0);
    if (rc) return opt_fail(o, rc, "cannot write " + o->out_orbitals);
  }
  if (!o->out_nelecwfn.empty() && o->desc.d.nspinc > 1) {
    int rc = vsvb_write_nelecwfn(o->out_nelecwfn.c_str(), &o->desc.d, o->csc.data());
    if (rc) return opt_fail(o, rc, "cannot write " + o->out_nelecwfn);
  }
  return VSVB_OK;
}

/* first_order_opt (valence.F90:527-844) on orbital orb: the new energy */
int first_order_opt(vsvb_opt *o, double *coeff, int orb, double *energy) {
  const vsvb_system_desc &d = o->desc.d;
  const int nb = d.map_orbs[orb + 1] - d.map_orbs[orb];
  std::vector<double> ham((size_t)nb * nb), ovl((size_t)nb * nb), eig(nb), w((size_t)nb * nb);
  OK_OR_RETURN(first_order_hs(o, coeff, orb, ham.data(), ovl.data()));
  OK_OR_RETURN(rsg_device(o, nb, ham.data(), ovl.data(), eig.data(), w.data()));
  const int r = root_of(d, orb + 1);
  if (r < 0 || r >= nb) return opt_fail(o, VSVB_ERR_INPUT, "excited-state root outside the orbital's expansion");
  *energy = eig[r] + o->enuc;
  const int j0 = d.map_orbs[orb] - 1;
  for (int i = 0; i < nb; ++i) coeff[j0 + i] = w[(size_t)r * nb + i];
  return normalise(o, coeff, orb);
}

/* spin_opt (valence.F90:850-936) */
int spin_opt(vsvb_opt *o, const double *coeff, double *energy) {
  const int nsc = o->nsc;
  std::vector<double> ham((size_t)nsc * nsc), ovl((size_t)nsc * nsc), eig(nsc), w((size_t)nsc * nsc);
  OK_OR_RETURN(spin_hs(o, coeff, ham.data(), ovl.data()));
  OK_OR_RETURN(rsg_device(o, nsc, ham.data(), ovl.data(), eig.data(), w.data()));
  *energy = eig[0] + o->enuc;
  for (int i = 0; i < nsc; ++i) o->csc[i] = w[i];
  o->csc_version++;
  return VSVB_OK;
}

/* demgs_opt (valence.F90:350-524) on orbital orb */
int demgs_opt(vsvb_opt *o, double *coeff, int orb, double etol, double *energy) {
  const vsvb_system_desc &d = o->desc.d;
  const int j0 = d.map_orbs[orb] - 1, nb = d.map_orbs[orb + 1] - d.map_orbs[orb];
  std::vector<char> lock(nb);
  double perturb = d.ptbnmax;
  while (kTokcal * perturb * perturb >= etol) {
    std::fill(lock.begin(), lock.end(), 0);
    bool updated = true;
    while (updated) {
      updated = false;
      for (int i = 0; i < nb; ++i) {
        if (lock[i]) continue;
        const int ic = j0 + i;
        const double eprev = *energy, origc = coeff[ic];
        double e;
        coeff[ic] = origc + perturb;
        OK_OR_RETURN(normalise(o, coeff, orb));
        OK_OR_RETURN(energy_of(o, coeff, &e));
        if (e < eprev) {
          updated = true;
          *energy = e;
          OK_OR_RETURN(save_output(o, coeff, e, false));
          continue;
        }
        coeff[ic] = origc - perturb;
        OK_OR_RETURN(normalise(o, coeff, orb));
        OK_OR_RETURN(energy_of(o, coeff, &e));
        if (e < eprev) {
          updated = true;
          *energy = e;
          OK_OR_RETURN(save_output(o, coeff, e, false));
          continue;
        }
        coeff[ic] = origc;
        lock[i] = 1;
        OK_OR_RETURN(normalise(o, coeff, orb));
        *energy = eprev;
      }
    }
    perturb *= d.feather;
  }
  return VSVB_OK;
}

}  // namespace

extern "C" {

int vsvb_rsg(int n, const double *ham, const double *ovl, int ld, double *eig, double *w, int ldw) {
  if (n < 1 || n > kRsgMax || !ham || !ovl || !eig || !w || ld < n || ldw < n) return VSVB_ERR_INPUT;
  const size_t nn = (size_t)n * n;
  double *buf = nullptr;
  int *info = nullptr;
  const size_t ntot = 2 * (size_t)ld * n + 4 * nn + n + (size_t)ldw * n;
  if (cudaMalloc(&buf, sizeof(double) * ntot) != cudaSuccess) return VSVB_ERR_NOMEM;
  if (cudaMalloc(&info, sizeof(int)) != cudaSuccess) {
    cudaFree(buf);
    return VSVB_ERR_NOMEM;
  }
  RsgArgs r{};
  r.n = n;
  r.m = n + (n & 1);
  double *Hd = buf, *Sd = Hd + (size_t)ld * n;
  r.H = Hd;
  r.S = Sd;
  r.ld = ld;
  r.L = Sd + (size_t)ld * n;
  r.A = r.L + nn;
  r.V = r.A + nn;
  r.Y = r.V + nn;
  r.eig = r.Y + nn;
  r.W = r.eig + n;
  r.ldw = ldw;
  r.info = info;
  int rc = VSVB_OK, hinfo = 0;
  if (cudaMemcpy(Hd, ham, sizeof(double) * ld * n, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(Sd, ovl, sizeof(double) * ld * n, cudaMemcpyHostToDevice) != cudaSuccess)
    rc = VSVB_ERR_CUDA;
  if (!rc) {
    rsg_kernel<<<1, 256>>>(r);
    if (cudaGetLastError() != cudaSuccess || cudaMemcpy(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = VSVB_ERR_CUDA;
  }
  if (!rc && hinfo) rc = VSVB_ERR_SINGULAR;
  if (!rc && (cudaMemcpy(eig, r.eig, sizeof(double) * n, cudaMemcpyDeviceToHost) != cudaSuccess ||
              cudaMemcpy(w, r.W, sizeof(double) * ldw * n, cudaMemcpyDeviceToHost) != cudaSuccess))
    rc = VSVB_ERR_CUDA;
  cudaFree(buf);
  cudaFree(info);
  return rc;
}

int vsvb_opt_create(const vsvb_system_desc *d, const vsvb_options *opt, vsvb_opt **out) {
  if (!d || !out) return VSVB_ERR_INPUT;
  auto *o = new vsvb_opt();
  *out = o;
  vsvb_default_options(&o->opt);
  if (opt) o->opt = *opt;
  o->opt.autotune = 0;
  o->opt.core_mode = -1; /* the H/S builds read the per-pair walk's quantities */
  copy_desc(d, o->desc);
  o->nnd = 2 * d->npair + d->nunpd;
  o->nsp = o->nnd + d->ndocc;
  o->nsc = d->nspinc > 0 ? d->nspinc : 1;
  o->csc.assign(o->nsc, 1.0);
  if (d->nspinc > 0) o->csc.assign(d->coeff_sc, d->coeff_sc + d->nspinc);
  int rc = vsvb_gpu_create(&o->desc.d, &o->opt, &o->main);
  if (rc) return opt_fail(o, rc, o->main ? vsvb_gpu_last_error(o->main) : "create failed");
  vsvb_energy_result r;
  rc = vsvb_gpu_energy(o->main, nullptr, &r);
  if (rc) return opt_fail(o, rc, vsvb_gpu_last_error(o->main));
  o->enuc = r.enucrep;
  o->main_csc_version = o->csc_version;
  return VSVB_OK;
}

void vsvb_opt_destroy(vsvb_opt *o) { delete o; }

int vsvb_opt_set_output(vsvb_opt *o, const char *orbitals_path, const char *nelecwfn_path) {
  if (!o) return VSVB_ERR_INPUT;
  o->out_orbitals = orbitals_path ? orbitals_path : "";
  o->out_nelecwfn = nelecwfn_path ? nelecwfn_path : "";
  return VSVB_OK;
}

const char *vsvb_opt_last_error(const vsvb_opt *o) { return o ? o->err.c_str() : "null optimiser"; }

int vsvb_opt_first_order_hs(vsvb_opt *o, const double *coeff, const double *coeff_sc, int iorb, double *ham,
                            double *ovl) {
  if (!o || !coeff || !ham || !ovl || iorb < 1 || iorb > o->nsp) return VSVB_ERR_INPUT;
  if (coeff_sc && o->desc.d.nspinc > 0) {
    o->csc.assign(coeff_sc, coeff_sc + o->nsc);
    o->csc_version++;
  }
  return first_order_hs(o, coeff, iorb - 1, ham, ovl);
}

int vsvb_opt_spin_hs(vsvb_opt *o, const double *coeff, double *ham, double *ovl) {
  if (!o || !coeff || !ham || !ovl) return VSVB_ERR_INPUT;
  if (o->desc.d.nspinc < 1) return opt_fail(o, VSVB_ERR_INPUT, "no spin couplings");
  return spin_hs(o, coeff, ham, ovl);
}

int vsvb_opt_minimize(vsvb_opt *o, double *coeff, double *coeff_sc, vsvb_opt_result *res) {
  if (!o || !coeff || !res) return VSVB_ERR_INPUT;
  auto t0 = std::chrono::steady_clock::now();
  std::memset(res, 0, sizeof(*res));
  const vsvb_system_desc &d = o->desc.d;
  if (coeff_sc && d.nspinc > 0) {
    o->csc.assign(coeff_sc, coeff_sc + o->nsc);
    o->csc_version++;
  }
  o->n_energy = o->n_hs = 0;
  /* calculate_vsvb_energy normalises the NDFs, then the orbitals */
  {
    std::vector<double> ndf(std::max(d.ndf, 1)), sc(o->nsp);
    int rc = gpu_orbital_scales(o->main, coeff, ndf.data(), sc.data());
    if (rc) return opt_fail(o, rc, vsvb_gpu_last_error(o->main));
    for (int f = 0; f < d.ndf; ++f)
      for (int j = d.map_orbs[o->nsp + f] - 1; j < d.map_orbs[o->nsp + f + 1] - 1; ++j) coeff[j] *= ndf[f];
    for (int i = 0; i < o->nsp; ++i)
      for (int j = d.map_orbs[i] - 1; j < d.map_orbs[i + 1] - 1; ++j) coeff[j] *= sc[i];
  }
  double energy = 0.0;
  OK_OR_RETURN(energy_of(o, coeff, &energy));
  res->guess_energy = energy;
  o->etol_kcal = 0.0;
  OK_OR_RETURN(save_output(o, coeff, energy, false));
  const bool dem_gs = d.ptbnmax > 0.0 && d.nxorb == 0;
  int num_iter = 0;
  double eprv_sc = 0.0, eprv_orb = 0.0, etol = 1.0;
  for (int ntol = d.ntol_e_min; ntol <= d.ntol_e_max; ++ntol) {
    etol = std::pow(10.0, -ntol);
    o->etol_kcal = etol;
    bool finished = false;
    while (!finished) {
      eprv_sc = energy;
      bool orbconv = false;
      while (!orbconv && num_iter < d.max_iter) {
        eprv_orb = energy;
        for (int iset = 0; iset < d.nset; ++iset) {
          const int lo = d.orbset[2 * iset], hi = d.orbset[2 * iset + 1];
          if (lo < 1 || hi > o->nsp) return opt_fail(o, VSVB_ERR_INPUT, "orbital set outside the wave function");
          bool setcnv = false;
          while (!setcnv && num_iter < d.max_iter) {
            const double eprv_set = energy;
            ++num_iter;
            for (int iorb = lo; iorb <= hi; ++iorb) {
              if (dem_gs) {
                OK_OR_RETURN(demgs_opt(o, coeff, iorb - 1, etol, &energy));
              } else {
                OK_OR_RETURN(first_order_opt(o, coeff, iorb - 1, &energy));
                OK_OR_RETURN(save_output(o, coeff, energy, false));
              }
            }
            setcnv = std::fabs(energy - eprv_set) * kTokcal < etol;
            if (lo == hi && dem_gs) setcnv = true;
          }
        }
        orbconv = std::fabs(energy - eprv_orb) * kTokcal < etol;
        if (d.nset == 1) {
          orbconv = true;
          eprv_orb = energy;
        }
      }
      if (d.nspinc > 1) {
        ++num_iter;
        OK_OR_RETURN(spin_opt(o, coeff, &energy));
        OK_OR_RETURN(save_output(o, coeff, energy, false));
        finished = std::fabs(energy - eprv_sc) * kTokcal < etol;
      } else {
        finished = true;
      }
      if (num_iter >= d.max_iter) finished = true;
    }
  }
  const double eprev = d.nspinc > 1 ? eprv_sc : eprv_orb;
  res->energy = energy;
  res->iterations = num_iter;
  res->converged = num_iter < d.max_iter && std::fabs(energy - eprev) * kTokcal < etol;
  if (res->converged) OK_OR_RETURN(save_output(o, coeff, energy, true));
  res->etol = etol;
  res->n_energy_evals = o->n_energy;
  res->n_hs_builds = o->n_hs;
  if (coeff_sc && d.nspinc > 0) std::copy(o->csc.begin(), o->csc.end(), coeff_sc);
  res->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return VSVB_OK;
}

}  /* extern "C" */
