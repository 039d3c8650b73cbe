/*
 * handle.cu -- the C ABI (include/vsvb_gpu.h): handle set-up and the energy /
 * gradient pipelines on one CUDA stream.
 *
 * Set-up mirrors calculate_vsvb_energy (valence.F90:70-182): norm_prim per
 * shell (:2264-2305), CCA component factors angn (:2337-2421), nuclear
 * repulsion (tools_module.F90:19-40), then builds what the GPU kernels need:
 * global shells, the orbital basis sets (OBS) with their weight scatter
 * terms (ovint/int1e/int2e scatter, :2919-2947; ndf2obs, :2191-2247),
 * unique shell pairs with primitive-pair data and the orbital pairs that
 * touch them, AO one-electron matrices, AO Schwarz bounds and a quartet
 * schedule sorted by angular-momentum class (and by precision on the mixed
 * path), and the spin-coupling maps of dbra/dket (:1648-1870).
 *
 * Evaluation (guess_energy, :309-345, with vsvb_energy, :1010-1434):
 *   ndf_norm, orb_norm -> orb_1e -> xtab -> eri (per class) -> detpair ->
 *   assemble -> energy_reduce,
 * and for the gradient a second walk of the same tasks (assemble<GRAD>),
 * the determinant-pair adjoint, the ERI adjoint (ERIs recomputed) and the
 * chain back through the X tables, the orbital integrals and normal().
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <functional>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <set>
#include <string>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "../../include/vsvb_gpu.h"
#include "block.cuh"
#include "core.cuh"
#include "density.cuh"
#include "eri.cuh"
#include "handle_internal.h"
#include "onee.cuh"
#include "vsvb_internal.h"

#include "rys_tables.inc"

namespace {

template <typename T>
struct DBuf {
  T *p = nullptr;
  size_t n = 0;
  cudaError_t alloc(size_t count) {
    free();
    n = count;
    if (count == 0) return cudaSuccess;
    return cudaMalloc(&p, sizeof(T) * count);
  }
  cudaError_t upload(const std::vector<T> &v) {
    cudaError_t e = alloc(v.size());
    if (e != cudaSuccess || v.empty()) return e;
    return cudaMemcpy(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice);
  }
  void free() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  ~DBuf() { free(); }
};

int ncart(int l) { return (l + 1) * (l + 2) / 2; }

/* Cartesian exponents of component k of angular momentum l in CCA order
 * (x-power descending, then y-power descending) */
void cart_exp(int l, int k, int e[3]) {
  for (int lx = l; lx >= 0; --lx) {
    const int n = l - lx + 1;
    if (k < n) {
      e[0] = lx;
      e[1] = l - lx - k;
      e[2] = k;
      return;
    }
    k -= n;
  }
  e[0] = e[1] = e[2] = 0;
}
int cca_index(const int e[3]) {
  const int l = e[0] + e[1] + e[2], u = l - e[0];
  return u * (u + 1) / 2 + e[2];
}

/* horizontal transfer of a shell pair (la, lb) with AB = A - B as a matrix:
 * (a b| = sum_e M(ab, e) (e 0|, e over the Cartesian functions of angular
 * momentum la .. la+lb on centre A.  Per direction
 * (a, b)_1D = sum_k binom(b, k) AB^(b-k) (a+k, 0)_1D. */
int pair_ne(int la, int lb) {
  int n = 0;
  for (int l = la; l <= la + lb; ++l) n += ncart(l);
  return n;
}
void hrr_matrix(int la, int lb, const double AB[3], std::vector<double> &out) {
  const int na = ncart(la), nb = ncart(lb), ne = pair_ne(la, lb);
  int off[8] = {0};
  for (int l = la + 1; l <= la + lb + 1; ++l) off[l - la] = off[l - la - 1] + ncart(l - 1);
  static const double binom[3][3] = {{1, 0, 0}, {1, 1, 0}, {1, 2, 1}};
  const size_t base = out.size();
  out.resize(base + (size_t)na * nb * ne, 0.0);
  for (int ia = 0; ia < na; ++ia)
    for (int ib = 0; ib < nb; ++ib) {
      int a[3], b[3];
      cart_exp(la, ia, a);
      cart_exp(lb, ib, b);
      for (int kx = 0; kx <= b[0]; ++kx)
        for (int ky = 0; ky <= b[1]; ++ky)
          for (int kz = 0; kz <= b[2]; ++kz) {
            const int k[3] = {kx, ky, kz};
            double c = 1.0;
            for (int d = 0; d < 3; ++d) c *= binom[b[d]][k[d]] * std::pow(AB[d], b[d] - k[d]);
            const int e[3] = {a[0] + kx, a[1] + ky, a[2] + kz};
            const int col = off[kx + ky + kz] + cca_index(e);
            out[base + (size_t)(ia * nb + ib) * ne + col] += c;
          }
    }
}
int pair_class(int la, int lb) { return la * (la + 1) / 2 + lb; } /* la >= lb */

double dblfac(int n) {
  double d = 1.0;
  for (int i = 3; i <= n; i += 2) d *= (double)i;
  return d;
}

}  // namespace

struct vsvb_gpu {
  vsvb_options opt;
  std::string err;
  int dev = 0, nsm = 152;
  cudaStream_t st = nullptr;     /* stream in use */
  cudaStream_t own_st = nullptr; /* the handle's own stream */
  static constexpr int NAUX = 6;  /* side streams for concurrent ERI class launches */
  cudaStream_t aux[NAUX] = {};
  cudaEvent_t ev_fork = nullptr, ev_join[NAUX] = {};
  /* CUDA graph of one energy + gradient evaluation (forward + adjoint),
   * captured on the second call and replayed after that */
  bool warm = false;
  cudaGraphExec_t gexec = nullptr;
  int graph_launches = 0;
  /* in-situ timing of the class launches of the last sweep (optional) */
  bool sweep_timing = false;
  int sweep_mode = -1;
  std::vector<cudaEvent_t> sweep_ev; /* 2 per class launch */
  cudaEvent_t sweep_t0 = nullptr, sweep_t1 = nullptr; /* fork and join of the last sweep */
  /* one ERI launch of a sweep: a class schedule (list 0: FP64-class shell
   * quartets, 1: FP32-class), the arithmetic it runs in and the window
   * [lo, hi) of primitive-quartet bounds it evaluates */
  struct SweepItem {
    int list, kind, a, c;
    float lo, hi;
    double nprimq;           /* primitive quartets inside the window */
    double flops_fwd, flops_grad;
    int code;                /* 100*k + 10*a + c; k = kind, or 3 for the FP32 tail of an FP64-class list */
    int bps = 16;            /* grid cap: blocks per SM (autotuned) */
    int wl = -1;             /* its own quartet list: item_wh / item_wd */
  };
  /* per launch: the quartets with work in its window, most primitive
   * quartets first */
  std::vector<std::vector<int4>> item_wh; /* (P, Q, first row, end row of P's primitives) */
  std::vector<DBuf<int4>> item_wd;
  std::vector<SweepItem> sweep; /* by decreasing work */
  int launches = 0;              /* kernels enqueued by the current call */
  /* dims */
  int natom = 0, nsh = 0, nao = 0, norb_all = 0, nsp = 0, ndf = 0, totlen = 0, maxobs = 0, np = 0;
  DetSetup ds{};
  double enuc = 0.0, dtol = 0.0, itol = 0.0;
  long long ntasks = 0;
  int nsplit = 1, nsplit_max = 1; /* task splits per determinant pair (assembly grids) */
  std::vector<double> coeff0;
  /* schedules: [prec][cp][cq] */
  /* [0] FP64-class quartets (their FP32 tail split off on the mixed paths),
   * [1] FP32-class, [2] FP64-class kept whole on the mixed paths */
  std::vector<int2> work_h[3][6][6];
  long long nq_fp64 = 0, nq_fp32 = 0;
  double nprimq_fp32 = 0.0, nprimq_all = 0.0; /* primitive quartets evaluated in FP32 / in total */
  double err_bound = 0.0; /* sum over FP32 quartets of the Schwarz bound */
  double bound_all = 0.0; /* the same over every evaluated quartet */
  /* device data */
  DBuf<GShell> shells;
  DBuf<double> exps, coefs, angn, charge, axyz, rys;
  DBuf<float2> rysdf;
  DBuf<float> rys32;
  DBuf<double> S_ao, H_ao;
  DBuf<ShellPair> pairs;
  DBuf<PrimPair> prims;
  DBuf<PrimT<double>> prim64;
  DBuf<PrimT<float>> prim32;
  DBuf<PrimT<df64>> primdf;
  DBuf<float> prim_q0; /* per primitive pair: sqrt(max_e |(e0|e0)|), pairs sorted descending */
  DBuf<GeomT<double>> geom64;
  DBuf<GeomT<float>> geom32;
  DBuf<GeomT<df64>> geomdf;
  RysConst rc{};
  DBuf<int> pair_opid;
  DBuf<XTerm> xterms;
  DBuf<long long> xelem0, xh_elem0;
  DBuf<double> hrr, xtabh;
  DBuf<float> xtabh32, Tbar32;
  long long nxelem = 0, nxh = 0;
  int nxterm = 0;
  DBuf<int> obs_n, obs_ao, term0, term_slot, term_j, term_m, term_f, ndf_orb;
  DBuf<double> coeff_d, ndf_scale, orb_scale, Craw, C, So, Ho, xtab, T, sqT, qmax, q0max;
  DBuf<int> pair_slot, slot_pair, slot_which, sing, status, nsing, xslot, xcount, abeq;
  DBuf<double> xinv, xdet; /* exact-minor pool of flagged determinant pairs */
  int xcap = 0;
  DBuf<double> coeff_sc, det_a, det_b, detr_a, detr_b, Ta, Tb, scratch;
  int ld_scratch = 0;
  DBuf<double> part_e1, part_wf, part_e2, result;
  /* adjoint */
  DBuf<double> Tbar, Sbar, Hbar, xbar, xbarh, Cbar, vtot, Gglob, coeff_bar;
  DBuf<double> Gs, vtot_s, D1; /* dE/dS parts of the fused (unscaled) adjoint walk */
  DBuf<double> ndf_bar;        /* dE/d(scale) of each derived basis function */
  bool grad_ready = false;
  int last_singular = 0;
  /* first_order_opt configuration (vsvb_opt): hs_split 1 / 2 when the
   * description carries one orbital more than its counts, the alpha / beta
   * slot of the first DOCC pair holding it; hs_sub its spatial index, taken
   * as given (not normalised); -1 on ordinary handles */
  int hs_split = 0, hs_sub = -1;
  DBuf<int> hs_flag;
  std::vector<double> csc_h; /* the spin-coupling weights in use */
  /* block mode (block.cu): atom quartets in chunks whose staging blocks fit
   * one of two alternating buffers of blk_gsize doubles */
  bool blk_on = false;
  struct BlkLaunch {
    long long off; /* into blk_work */
    int n, kind, cp, cq;
    float lo, hi;
  };
  struct BlkChunk {
    int aq0, naq, tt; /* atom quartets, transform arithmetic (0 FP64, 1 FP32) */
    int l0, nl;       /* its ERI launches in blk_launch */
  };
  std::vector<BlkLaunch> blk_launch;
  std::vector<BlkChunk> blk_chunk;
  size_t blk_gsize = 0;
  int blk_nfmax = 1, blk_nomax = 1, blk_ncoef = 0;
  size_t blk_smem[3] = {0, 0, 0};
  double blk_eri_flops[3] = {0, 0, 0};  /* per ERI kind, one sweep */
  double blk_tr_flops[3] = {0, 0, 0};   /* transform, FP64 / FP32 / double-float */
  long long blk_naq = 0;
  DBuf<int4> blk_pair, blk_aq, blk_ap, blk_work, blk_csrc;
  DBuf<int2> blk_atom_orb;
  DBuf<int> blk_atom_nf, blk_atom_c0, blk_orb, blk_cao;
  DBuf<double> blk_catom, blk_G;
  cudaEvent_t blk_done[2] = {nullptr, nullptr};
  /* core mode (core.cu): the determinant-pair sum over the shared doubly
   * occupied core in closed form */
  bool core_on = false;
  int core_nt = 0;
  DBuf<unsigned char> core_detorb, core_detpos;
  DBuf<int> core_lst1, core_off1, core_lst2, core_off2, core_pslot, core_pcount;
  DBuf<int2> core_pik;
  DBuf<double> core_fw, core_G, core_Y, core_M, core_P0, core_U, core_s0, core_dd, core_L, core_qf, core_pool;
  DBuf<double> core_A0, core_A1, core_A2, core_A2x, core_R1, core_Wv, core_X, core_part;
  int core_cap = 0;
  /* core-mode adjoint (core.cu CoreGrad) */
  static constexpr int CORE_NCHUNK = 64;
  DBuf<double> cg_Yg, cg_Axp, cg_Ax, cg_Wvb, cg_KP, cg_KR, cg_R1b, cg_P0b, cg_A1b, cg_Ub, cg_Mbp, cg_lam, cg_Mb, cg_sc,
      cg_t1, cg_t2;
};

namespace {

int cuda_fail(vsvb_gpu *h, cudaError_t e, const char *what) {
  h->err = std::string(what) + ": " + cudaGetErrorString(e);
  return VSVB_ERR_CUDA;
}

#define CK(call, what)                              \
  do {                                              \
    cudaError_t e_ = (call);                        \
    if (e_ != cudaSuccess) return cuda_fail(h, e_, what); \
  } while (0)

OrbArgs orb_args(vsvb_gpu *h) {
  OrbArgs a{};
  a.norb_all = h->norb_all;
  a.maxobs = h->maxobs;
  a.nao = h->nao;
  a.obs_n = h->obs_n.p;
  a.obs_ao = h->obs_ao.p;
  a.term0 = h->term0.p;
  a.term_slot = h->term_slot.p;
  a.term_j = h->term_j.p;
  a.term_m = h->term_m.p;
  a.term_f = h->term_f.p;
  a.ndf_orb = h->ndf_orb.p;
  a.coeff = h->coeff_d.p;
  a.S = h->S_ao.p;
  a.H = h->H_ao.p;
  a.ndf_scale = h->ndf_scale.p;
  a.orb_scale = h->orb_scale.p;
  a.Craw = h->Craw.p;
  a.C = h->C.p;
  a.status = h->status.p;
  a.fixed_orb = h->hs_sub;
  return a;
}

XtabArgs xtab_args(vsvb_gpu *h) {
  XtabArgs x{};
  x.terms = h->xterms.p;
  x.elem0 = h->xelem0.p;
  x.nterm = h->nxterm;
  x.nelem = h->nxelem;
  x.C = h->C.p;
  x.maxobs = h->maxobs;
  x.angn = h->angn.p;
  x.dtol = h->dtol;
  x.xtab = h->xtab.p;
  x.xbar_scale = 1.0;
  x.xh_elem0 = h->xh_elem0.p;
  x.nxh = h->nxh;
  x.hrr = h->hrr.p;
  x.xtabh = h->xtabh.p;
  x.xtabh32 = h->xtabh32.p;
  /* first_order_opt's substituted orbital: its matrices are the bilinear
   * forms over every shell of the orbital, as the reference's one-shell dummy
   * orbitals give them, so no shell of it is screened out */
  x.keep_orb = h->hs_sub;
  return x;
}

EriArgs eri_args(vsvb_gpu *h) {
  EriArgs a{};
  a.rc = h->rc;
  a.prim64 = h->prim64.p;
  a.prim32 = h->prim32.p;
  a.primdf = h->primdf.p;
  a.geom64 = h->geom64.p;
  a.geom32 = h->geom32.p;
  a.geomdf = h->geomdf.p;
  a.pairs = h->pairs.p;
  a.prims = h->prims.p;
  a.rys = h->rys.p;
  a.rysdf = h->rysdf.p;
  a.rys32 = h->rys32.p;
  a.pair_opid = h->pair_opid.p;
  a.xtab = h->xtabh.p;
  a.hrr = h->hrr.p;
  a.xtab32 = h->xtabh32.p;
  a.Tbar32 = h->Tbar32.p;
  a.T = h->T.p;
  a.np = h->np;
  a.qmax_out = h->qmax.p;
  a.q0max_out = h->q0max.p;
  a.prim_q0 = h->prim_q0.p;
  a.prim_lo = (float)h->opt.prim_screen;
  a.prim_hi = INFINITY;
  a.Tbar = h->Tbar.p;
  a.xbar = h->xbarh.p;
  return a;
}

DetCtx det_ctx(vsvb_gpu *h) {
  DetCtx d{};
  d.ds = h->ds;
  d.pair_slot = h->pair_slot.p;
  d.slot_pair = h->slot_pair.p;
  d.slot_which = h->slot_which.p;
  d.coeff_sc = h->coeff_sc.p;
  d.So = h->So.p;
  d.Ho = h->Ho.p;
  d.det_a = h->det_a.p;
  d.det_b = h->det_b.p;
  d.detr_a = h->detr_a.p;
  d.detr_b = h->detr_b.p;
  d.Ta = h->Ta.p;
  d.Tb = h->Tb.p;
  d.sing = h->sing.p;
  d.nsing = h->nsing.p;
  d.xinv = h->xinv.p;
  d.xdet = h->xdet.p;
  d.xslot = h->xslot.p;
  d.xcount = h->xcount.p;
  d.xcap = h->xcap;
  d.abeq = h->abeq.p;
  d.status = h->status.p;
  return d;
}

AsmArgs asm_args(vsvb_gpu *h) {
  AsmArgs a{};
  a.T = h->T.p;
  a.sq = h->sqT.p;
  a.np = h->np;
  a.itol = h->itol;
  a.ntasks = h->ntasks;
  a.part_e1 = h->part_e1.p;
  a.part_wf = h->part_wf.p;
  a.part_e2 = h->part_e2.p;
  a.status = nullptr;
  a.Tbar = h->Tbar.p;
  a.Sbar = h->Sbar.p;
  a.Hbar = h->Hbar.p;
  a.vtot = h->vtot.p;
  a.Gglob = h->Gglob.p;
  a.Gs = h->Gs.p;
  a.vtot_s = h->vtot_s.p;
  a.D1 = h->D1.p;
  int na = h->ds.nalpha, nb = h->ds.nbeta;
  {
    /* dJ/dT accumulators: one copy per warp of the 128-thread block when
     * they fit, else one per block, else global memory */
    const size_t gbytes = (size_t)(na * na + nb * nb) * sizeof(double);
    a.g_in_smem = 4 * gbytes <= 40 * 1024 ? 4 : (gbytes <= 40 * 1024 ? 1 : 0);
  }
  return a;
}

int setup_core(vsvb_gpu *h, const std::vector<int> &pslot);

CoreGrad core_grad(vsvb_gpu *h) {
  CoreGrad g{};
  g.Gam = h->Tbar.p;
  g.Yg = h->cg_Yg.p;
  g.Axp = h->cg_Axp.p;
  g.nchunk = vsvb_gpu::CORE_NCHUNK;
  g.Ax = h->cg_Ax.p;
  g.Wvb = h->cg_Wvb.p;
  g.KP = h->cg_KP.p;
  g.KR = h->cg_KR.p;
  g.R1b = h->cg_R1b.p;
  g.P0b = h->cg_P0b.p;
  g.A1b = h->cg_A1b.p;
  g.Ub = h->cg_Ub.p;
  g.Mbp = h->cg_Mbp.p;
  g.lam = h->cg_lam.p;
  g.Mb = h->cg_Mb.p;
  g.sc = h->cg_sc.p;
  g.t1 = h->cg_t1.p;
  g.t2 = h->cg_t2.p;
  g.Sbar = h->Sbar.p;
  g.Hbar = h->Hbar.p;
  return g;
}

CoreArgs core_args(vsvb_gpu *h) {
  CoreArgs c{};
  const DetSetup &ds = h->ds;
  c.nsp = ds.nsp;
  c.P = ds.npair;
  c.nC = 2 * ds.npair;
  c.nD = ds.nsp - c.nC;
  c.nsc = ds.nsc;
  c.ndet = ds.nsc << ds.npair;
  c.nelec = ds.nelec;
  c.nq = ds.nq;
  c.np = h->np;
  c.ncp = c.nC * (c.nC + 1) / 2;
  c.kx = c.ncp + 2;
  c.So = h->So.p;
  c.Ho = h->Ho.p;
  c.csc = h->coeff_sc.p;
  c.detorb = h->core_detorb.p;
  c.detpos = h->core_detpos.p;
  c.lst1 = h->core_lst1.p;
  c.off1 = h->core_off1.p;
  c.lst2 = h->core_lst2.p;
  c.off2 = h->core_off2.p;
  c.pik = h->core_pik.p;
  c.fw = h->core_fw.p;
  c.G = h->core_G.p;
  c.Y = h->core_Y.p;
  c.M = h->core_M.p;
  c.P0 = h->core_P0.p;
  c.U = h->core_U.p;
  c.s0 = h->core_s0.p;
  c.dd = h->core_dd.p;
  c.L = h->core_L.p;
  c.qf = h->core_qf.p;
  c.pslot = h->core_pslot.p;
  c.pool = h->core_pool.p;
  c.pcount = h->core_pcount.p;
  c.cap = h->core_cap;
  c.status = h->status.p;
  c.A0 = h->core_A0.p;
  c.A1 = h->core_A1.p;
  c.A2 = h->core_A2.p;
  c.A2x = h->core_A2x.p;
  c.R1 = h->core_R1.p;
  c.Wv = h->core_Wv.p;
  c.X = h->core_X.p;
  c.T = h->T.p;
  c.sq = h->sqT.p;
  c.itol = h->itol;
  c.part = h->core_part.p;
  c.ntile = h->core_nt;
  c.enuc = h->enuc;
  c.df = h->opt.precision == VSVB_MIXED_DF64;
  c.out = h->result.p;
  c.nsing = h->nsing.p;
  return c;
}

/* arithmetic of a schedule: list 1 holds the quartets below the mixed
 * threshold (FP32); list 0 the rest, in FP64 or, on VSVB_MIXED_DF64, in
 * double-float */
int eri_kind(const vsvb_gpu *h, int list) {
  if (list == 1) return ERI_F32;
  return h->opt.precision == VSVB_MIXED_DF64 ? ERI_DF64 : ERI_F64;
}

/* ---------------- set-up ---------------- */

/* the primitive-pair table in every kernel arithmetic */
int upload_prims(vsvb_gpu *h, const std::vector<PrimPair> &prims) {
  std::vector<PrimT<double>> p64(prims.size());
  std::vector<PrimT<float>> p32(prims.size());
  std::vector<PrimT<df64>> pdf(prims.size());
  for (size_t i = 0; i < prims.size(); ++i) {
    for (int k = 0; k < 3; ++k) {
      p64[i].P[k] = prims[i].P[k];
      p32[i].P[k] = (float)prims[i].P[k];
      pdf[i].P[k] = df64(prims[i].P[k]);
    }
    p64[i].p = prims[i].p;
    p64[i].inv_p = prims[i].inv_p;
    p64[i].Kp = prims[i].Kp;
    p32[i].p = (float)prims[i].p;
    p32[i].inv_p = (float)prims[i].inv_p;
    p32[i].Kp = (float)prims[i].Kp;
    pdf[i].p = df64(prims[i].p);
    pdf[i].inv_p = df64(prims[i].inv_p);
    pdf[i].Kp = df64(prims[i].Kp);
  }
  CK(h->prims.upload(prims), "upload prims");
  CK(h->prim64.upload(p64), "upload prim64");
  CK(h->prim32.upload(p32), "upload prim32");
  CK(h->primdf.upload(pdf), "upload primdf");
  return VSVB_OK;
}

/* Block-mode set-up (block.cu): atom pairs and their shell pairs, the
 * per-atom orbital weight tables, the atom quartets above the AO screen
 * sorted by bound (largest first) and cut into chunks whose staging blocks
 * fit one buffer, and per chunk the shell-quartet lists of every (bra class,
 * ket class, precision), built by worker threads straight into device
 * memory. */
int build_block(vsvb_gpu *h, const vsvb_system_desc *d, const std::vector<GShell> &sh, const std::vector<int> &first_sh,
                const std::vector<std::vector<int>> &orbs_on_atom, const std::vector<std::vector<int>> &slot_of_shell,
                const std::vector<ShellPair> &pairs, const std::vector<float> &q0f, const std::vector<double> &q0,
                const std::vector<double> &amp) {
  const int nat = d->natom;
  std::vector<int> atom_nf(nat), atom_c0(nat), borb, cao;
  std::vector<int2> atom_orb(nat);
  std::vector<int4> csrc;
  int nfmax = 1, nomax = 1;
  for (int a = 0; a < nat; ++a) {
    int nf = 0;
    for (int g = first_sh[a]; g < first_sh[a + 1]; ++g) nf += ncart(sh[g].l);
    atom_nf[a] = nf;
    nfmax = std::max(nfmax, nf);
    atom_orb[a] = make_int2((int)borb.size(), 0);
    atom_c0[a] = (int)csrc.size();
    for (int o : orbs_on_atom[a]) {
      borb.push_back(o);
      atom_orb[a].y++;
      for (int g = first_sh[a]; g < first_sh[a + 1]; ++g) {
        const int slot = slot_of_shell[o][g], nc = ncart(sh[g].l);
        for (int c = 0; c < nc; ++c) {
          csrc.push_back(make_int4(o, slot < 0 ? -1 : slot + c, slot, nc));
          cao.push_back(sh[g].ao0 + c);
        }
      }
    }
    nomax = std::max(nomax, atom_orb[a].y);
  }
  h->blk_nfmax = nfmax;
  h->blk_nomax = nomax;
  h->blk_smem[0] = blk_transform_smem(nfmax, nomax, 0);
  h->blk_smem[1] = blk_transform_smem(nfmax, nomax, 1);
  h->blk_smem[2] = blk_transform_smem(nfmax, nomax, 2);
  if (h->blk_smem[0] > 227 * 1024) {
    h->err = "block mode: an atom's functions and orbitals exceed the transform's shared memory";
    return VSVB_ERR_UNSUPPORTED;
  }
  h->blk_ncoef = (int)csrc.size();
  CK(h->blk_atom_nf.upload(atom_nf), "upload blk");
  CK(h->blk_atom_c0.upload(atom_c0), "upload blk");
  CK(h->blk_atom_orb.upload(atom_orb), "upload blk");
  CK(h->blk_orb.upload(borb.empty() ? std::vector<int>(1, 0) : borb), "upload blk");
  CK(h->blk_csrc.upload(csrc.empty() ? std::vector<int4>(1, make_int4(0, -1, 0, 0)) : csrc), "upload blk");
  CK(h->blk_cao.upload(cao.empty() ? std::vector<int>(1, 0) : cao), "upload blk");
  CK(h->blk_catom.alloc(std::max<size_t>(csrc.size(), 1)), "alloc blk");
  /* atom pairs (first atom >= second) and each shell pair's place */
  std::vector<int> ap_of(nat * nat, -1);
  std::vector<int4> aps;
  std::vector<std::vector<int>> ap_pairs;
  std::vector<double> ap_q;
  std::vector<int4> pblk(pairs.size());
  for (size_t p = 0; p < pairs.size(); ++p) {
    const int sA = pairs[p].shA, sB = pairs[p].shB, aA = sh[sA].atom, aB = sh[sB].atom;
    const int X = std::max(aA, aB), Y = std::min(aA, aB);
    int &ap = ap_of[X * nat + Y];
    if (ap < 0) {
      ap = (int)aps.size();
      aps.push_back(make_int4(X, Y, atom_nf[X] * atom_nf[Y], 0));
      ap_pairs.emplace_back();
      ap_q.push_back(0.0);
    }
    ap_pairs[ap].push_back((int)p);
    ap_q[ap] = std::max(ap_q[ap], pairs[p].qmax);
    const int offA = sh[sA].ao0 - sh[first_sh[aA]].ao0, offB = sh[sB].ao0 - sh[first_sh[aB]].ao0;
    const int flags = (X != Y && aA == Y ? 1 : 0) | (X == Y ? 2 : 0) | (sA == sB ? 4 : 0);
    pblk[p] = make_int4(offA, offB, flags, atom_nf[Y]);
  }
  CK(h->blk_pair.upload(pblk.empty() ? std::vector<int4>(1, make_int4(0, 0, 0, 0)) : pblk), "upload blk");
  CK(h->blk_ap.upload(aps.empty() ? std::vector<int4>(1, make_int4(0, 0, 0, 0)) : aps), "upload blk");
  /* atom quartets above the screen, largest bound first */
  struct AQ {
    int i, j;
    double b;
  };
  std::vector<AQ> aqs;
  for (int i = 0; i < (int)aps.size(); ++i)
    for (int j = 0; j <= i; ++j) {
      const double b = ap_q[i] * ap_q[j];
      if (b >= h->opt.ao_screen) aqs.push_back({i, j, b});
    }
  std::stable_sort(aqs.begin(), aqs.end(), [](const AQ &x, const AQ &y) { return x.b > y.b; });
  h->blk_naq = (long long)aqs.size();
  /* chunks: staging blocks of one chunk fit blk_gsize doubles */
  /* 512 MiB of FP64 per buffer: enough shell quartets per class launch to
   * fill the GPU with the one-lane-per-quartet kernels */
  const size_t gbudget = (size_t)1 << 26;
  size_t gmax = 0;
  std::vector<int4> aqd(aqs.size());
  {
    size_t off = 0;
    int c0 = 0;
    for (size_t k = 0; k < aqs.size(); ++k) {
      const size_t sz = (size_t)aps[aqs[k].i].z * aps[aqs[k].j].z;
      if (off > 0 && off + sz > gbudget) {
        h->blk_chunk.push_back({c0, (int)k - c0, 0, 0, 0});
        c0 = (int)k;
        off = 0;
      }
      aqd[k] = make_int4(aqs[k].i, aqs[k].j, (int)off, aqs[k].i == aqs[k].j ? 1 : 0);
      off += sz;
      gmax = std::max(gmax, off);
    }
    if (!aqs.empty()) h->blk_chunk.push_back({c0, (int)aqs.size() - c0, 0, 0, 0});
  }
  h->blk_gsize = std::max<size_t>(gmax, 1);
  CK(h->blk_aq.upload(aqd.empty() ? std::vector<int4>(1, make_int4(0, 0, 0, 0)) : aqd), "upload blk");
  CK(h->blk_G.alloc(2 * h->blk_gsize), "alloc blk G");
  CK(cudaMemset(h->blk_G.p, 0, sizeof(double) * h->blk_G.n), "memset blk G");
  const bool mixed = h->opt.precision == VSVB_MIXED || h->opt.precision == VSVB_MIXED_DF64;
  const float eps = (float)h->opt.prim_screen, tau = (float)h->opt.mixed_threshold;
  const bool split = mixed && h->opt.prim_split;
  const int kind64 = eri_kind(h, 0);
  auto window = [&](int P, int Q, float lo, float hi, double &sum) -> double {
    const float *a = q0f.data() + pairs[P].prim0, *b = q0f.data() + pairs[Q].prim0;
    const int na = pairs[P].nprim, nb = pairs[Q].nprim;
    double n = 0.0;
    sum = 0.0;
    int jlo = nb, jhi = nb;
    for (int i = 0; i < na; ++i) {
      if (!(a[i] * b[0] >= lo)) break;
      while (jlo > 0 && !(a[i] * b[jlo - 1] >= lo)) --jlo;
      while (jhi > 0 && !(a[i] * b[jhi - 1] >= hi)) --jhi;
      n += jlo - jhi;
      for (int j = jhi; j < jlo; ++j) sum += (double)a[i] * b[j];
    }
    return n;
  };
  /* per chunk: the quartet lists of each (cp, cq, precision), counted in a
   * first pass and written in a second, both over worker threads */
  const int nch = (int)h->blk_chunk.size();
  struct ChunkStat {
    long long cnt[3][3][2];
    long long nq64, nq32;
    double nprim_all, nprim32, errb, ball;
    double prim[3][3][2][2]; /* primitive quartets per (cp, cq, precision, main / FP32 tail) */
  };
  std::vector<ChunkStat> cs(nch);
  for (auto &c : cs) std::memset(&c, 0, sizeof(c));
  auto for_quartets = [&](int c, auto &&f) {
    const auto &ch = h->blk_chunk[c];
    for (int k = ch.aq0; k < ch.aq0 + ch.naq; ++k) {
      const AQ &q = aqs[k];
      const int ncol = aps[q.j].z;
      for (int P : ap_pairs[q.i])
        for (int Q : ap_pairs[q.j]) {
          if (q.i == q.j && Q > P) continue;
          const double b = pairs[P].qmax * pairs[Q].qmax;
          if (b < h->opt.ao_screen) continue;
          int a = P, cc = Q, swp = 0;
          if (pairs[a].cls < pairs[cc].cls) {
            std::swap(a, cc);
            swp = 1;
          }
          const int prec = (mixed && b < h->opt.mixed_threshold) ? 1 : 0;
          f(pairs[a].cls, pairs[cc].cls, prec, make_int4(a, cc, aqd[k].z, ncol | (swp << 20) | ((q.i == q.j) << 21)), b,
            P, Q);
        }
    }
  };
  const int nthr = std::max(1, std::min<int>(16, (int)std::thread::hardware_concurrency()));
  auto run_threads = [&](auto &&job) {
    std::vector<std::thread> th;
    for (int t = 0; t < nthr; ++t) th.emplace_back([&, t]() {
      for (int c = t; c < nch; c += nthr) job(c);
    });
    for (auto &x : th) x.join();
  };
  run_threads([&](int c) {
    ChunkStat &st = cs[c];
    for_quartets(c, [&](int cp, int cq, int prec, int4, double b, int P, int Q) {
      st.cnt[cp][cq][prec]++;
      int a = P, cc = Q;
      if (pairs[a].cls < pairs[cc].cls) std::swap(a, cc);
      double sb = 0.0;
      const double nall = window(a, cc, eps, INFINITY, sb);
      st.ball += b;
      st.nprim_all += nall;
      if (prec) {
        st.nq32++;
        st.nprim32 += nall;
        st.errb += amp[P] * amp[Q];
        st.prim[cp][cq][1][0] += nall;
      } else {
        st.nq64++;
        if (split) {
          const double nt = window(a, cc, eps, tau, sb);
          st.nprim32 += nt;
          st.errb += sb * (amp[P] / std::max(q0[P], 1e-300)) * (amp[Q] / std::max(q0[Q], 1e-300));
          st.prim[cp][cq][0][1] += nt;
          st.prim[cp][cq][0][0] += nall - nt;
        } else {
          st.prim[cp][cq][0][0] += nall;
        }
      }
    });
  });
  /* offsets, launches and totals */
  long long total = 0;
  std::vector<long long> off((size_t)nch * 18, 0);
  for (int c = 0; c < nch; ++c) {
    auto &ch = h->blk_chunk[c];
    const ChunkStat &st = cs[c];
    h->nq_fp64 += st.nq64;
    h->nq_fp32 += st.nq32;
    h->nprimq_all += st.nprim_all;
    h->nprimq_fp32 += st.nprim32;
    h->err_bound += st.errb;
    h->bound_all += st.ball;
    ch.l0 = (int)h->blk_launch.size();
    /* transform in FP32 when every quartet of the chunk is FP32-class; the
     * others in the FP64-class arithmetic of the handle (double-float on
     * VSVB_MIXED_DF64) */
    ch.tt = (mixed && aqs[ch.aq0].b < h->opt.mixed_threshold) ? 1 : (kind64 == ERI_DF64 ? 2 : 0);
    for (int a = 0; a < 3; ++a)
      for (int cq = 0; cq <= a; ++cq)
        for (int prec = 0; prec < 2; ++prec) {
          const long long n = st.cnt[a][cq][prec];
          off[(size_t)c * 18 + (a * 3 + cq) * 2 + prec] = total;
          if (n == 0) continue;
          const double hf = (double)n * eri_block_hrr_flops(a, cq);
          if (prec == 1) {
            h->blk_launch.push_back({total, (int)n, ERI_F32, a, cq, eps, INFINITY});
            h->blk_eri_flops[ERI_F32] += eri_flops(1, a, cq, st.prim[a][cq][1][0], 0, 0) + hf;
          } else {
            h->blk_launch.push_back({total, (int)n, kind64, a, cq, split ? std::max(eps, tau) : eps, INFINITY});
            h->blk_eri_flops[kind64] += eri_flops(1, a, cq, st.prim[a][cq][0][0], 0, 0) + hf;
            if (split) {
              h->blk_launch.push_back({total, (int)n, ERI_F32, a, cq, eps, tau});
              h->blk_eri_flops[ERI_F32] += eri_flops(1, a, cq, st.prim[a][cq][0][1], 0, 0);
            }
          }
          total += n;
        }
    ch.nl = (int)h->blk_launch.size() - ch.l0;
    for (int k = ch.aq0; k < ch.aq0 + ch.naq; ++k) {
      const int4 p1 = aps[aqs[k].i], p2 = aps[aqs[k].j];
      h->blk_tr_flops[ch.tt] += blk_transform_flops(atom_nf[p1.x], atom_nf[p1.y], atom_nf[p2.x], atom_nf[p2.y],
                                                    atom_orb[p1.x].y, atom_orb[p1.y].y, atom_orb[p2.x].y,
                                                    atom_orb[p2.y].y);
    }
  }
  CK(h->blk_work.alloc(std::max<long long>(total, 1)), "alloc blk work");
  int fill_err = 0;
  run_threads([&](int c) {
    if (cudaSetDevice(h->dev) != cudaSuccess) {
      fill_err = 1;
      return;
    }
    std::vector<int4> lst[3][3][2];
    for_quartets(c, [&](int cp, int cq, int prec, int4 item, double, int, int) { lst[cp][cq][prec].push_back(item); });
    for (int a = 0; a < 3; ++a)
      for (int cq = 0; cq <= a; ++cq)
        for (int prec = 0; prec < 2; ++prec) {
          auto &v = lst[a][cq][prec];
          if (v.empty()) continue;
          /* most primitive quartets first: neighbouring lanes of the
           * one-lane-per-quartet kernels get similar work */
          std::stable_sort(v.begin(), v.end(), [&](const int4 &x, const int4 &y) {
            return pairs[x.x].nprim * pairs[x.y].nprim > pairs[y.x].nprim * pairs[y.y].nprim;
          });
          const long long o = off[(size_t)c * 18 + (a * 3 + cq) * 2 + prec];
          if (cudaMemcpy(h->blk_work.p + o, v.data(), sizeof(int4) * v.size(), cudaMemcpyHostToDevice) != cudaSuccess)
            fill_err = 1;
        }
  });
  if (fill_err) {
    h->err = "block mode: upload of the quartet lists failed";
    return VSVB_ERR_CUDA;
  }
  for (int k = 0; k < 2; ++k) CK(cudaEventCreateWithFlags(&h->blk_done[k], cudaEventDisableTiming), "cudaEventCreate");
  return VSVB_OK;
}

int build(vsvb_gpu *h, const vsvb_system_desc *d) {
  if (d->npair > 0 && d->nspinc < 1) {
    h->err = "no spin couplings;";
    return VSVB_ERR_INPUT;
  }
  for (int s = 0; s < d->num_sh; ++s)
    if (d->ang_mom[s] < 0 || d->ang_mom[s] > VSVB_LMAX) {
      h->err = "angular momentum above d is not supported on the GPU path";
      return VSVB_ERR_UNSUPPORTED;
    }
  if (d->npair > 15) {
    h->err = "more than 15 spin-coupled pairs";
    return VSVB_ERR_UNSUPPORTED;
  }
  CK(cudaSetDevice(h->dev), "cudaSetDevice");
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, h->dev), "cudaGetDeviceProperties");
  h->nsm = prop.multiProcessorCount;
  CK(cudaStreamCreateWithFlags(&h->own_st, cudaStreamNonBlocking), "cudaStreamCreate");
  h->st = h->own_st;
  for (int k = 0; k < vsvb_gpu::NAUX; ++k) {
    CK(cudaStreamCreateWithFlags(&h->aux[k], cudaStreamNonBlocking), "cudaStreamCreate");
    CK(cudaEventCreateWithFlags(&h->ev_join[k], cudaEventDisableTiming), "cudaEventCreate");
  }
  CK(cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming), "cudaEventCreate");

  const int norbs = 2 * d->npair + d->nunpd + d->ndocc + d->ndf + (h->hs_split ? 1 : 0);
  h->natom = d->natom;
  h->ndf = d->ndf;
  h->norb_all = norbs;
  h->nsp = 2 * d->npair + d->nunpd + d->ndocc + (h->hs_split ? 1 : 0);
  h->totlen = d->totlen;
  h->dtol = std::pow(10.0, -(double)d->ntol_d);
  h->itol = std::pow(10.0, -(double)d->ntol_i);
  h->coeff0.assign(d->coeff, d->coeff + d->totlen);

  /* norm_prim (valence.F90:2264-2305) */
  std::vector<double> cc(d->num_pr);
  const double pi32 = std::pow(std::acos(-1.0), 1.5);
  for (int s = 0; s < d->num_sh; ++s) {
    int l = d->ang_mom[s], k0 = d->map_shell2prim[s] - 1, n = d->map_shell2prim[s + 1] - d->map_shell2prim[s];
    double fac = pi32 * dblfac(2 * l - 1) * std::pow(2.0, -l), fax = -1.5 - l;
    for (int i = 0; i < n; ++i) cc[k0 + i] = d->con_coeff[k0 + i] * std::pow(fac * std::pow(2.0 * d->exponent[k0 + i], fax), -0.5);
    double sovl = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) sovl += fac * cc[k0 + i] * cc[k0 + j] * std::pow(d->exponent[k0 + i] + d->exponent[k0 + j], fax);
    sovl = std::pow(sovl, -0.5);
    for (int i = 0; i < n; ++i) cc[k0 + i] *= sovl;
  }
  /* angn per component in CCA order (setangn, valence.F90:2395-2421) */
  auto angn_of = [](int l, int k) {
    int n = 0;
    for (int i = 0; i <= l; ++i)
      for (int j = 0; j <= i; ++j) {
        if (n == k) {
          int x = l - i, y = i - j, z = j;
          return std::sqrt(dblfac(2 * l - 1) / (dblfac(2 * x - 1) * dblfac(2 * y - 1) * dblfac(2 * z - 1)));
        }
        ++n;
      }
    return 1.0;
  };
  /* global shells */
  std::vector<GShell> sh;
  std::vector<int> first_sh(d->natom + 1);
  std::vector<double> angn;
  int ao = 0;
  for (int a = 0; a < d->natom; ++a) {
    first_sh[a] = (int)sh.size();
    int t = d->atom_t[a] - 1;
    for (int s = 0; s < d->num_shell_atom[t]; ++s) {
      int gs = d->map_atom2shell[t] - 1 + s;
      GShell g{};
      g.l = d->ang_mom[gs];
      g.nprim = d->map_shell2prim[gs + 1] - d->map_shell2prim[gs];
      g.prim0 = d->map_shell2prim[gs] - 1;
      g.atom = a;
      g.ao0 = ao;
      for (int k = 0; k < 3; ++k) g.xyz[k] = d->coords[3 * a + k];
      for (int k = 0; k < ncart(g.l); ++k) angn.push_back(angn_of(g.l, k));
      ao += ncart(g.l);
      sh.push_back(g);
    }
  }
  first_sh[d->natom] = (int)sh.size();
  h->nsh = (int)sh.size();
  h->nao = ao;
  /* nuclear repulsion */
  h->enuc = 0.0;
  for (int i = 1; i < d->natom; ++i)
    for (int j = 0; j < i; ++j) {
      double zij = d->nuc_charge[d->atom_t[i] - 1] * d->nuc_charge[d->atom_t[j] - 1];
      if (std::fabs(zij) > 1e-12) {
        double r2 = 0.0;
        for (int k = 0; k < 3; ++k) r2 += std::pow(d->coords[3 * i + k] - d->coords[3 * j + k], 2);
        if (r2 > 1e-5) h->enuc += zij * std::pow(r2, -0.5);
      }
    }
  /* orbital basis sets */
  std::vector<std::vector<int>> obs(norbs);
  std::vector<std::vector<int>> slot_of_shell(norbs, std::vector<int>(h->nsh, -1));
  std::vector<std::vector<int>> orb_atoms(norbs);
  for (int o = 0; o < norbs; ++o) {
    for (int k = 0; k < d->orbas_atnum[o]; ++k) {
      int a = d->orbas_atset[k + (size_t)d->mxctr * o] - 1;
      if (a < 0 || a >= d->natom) {
        h->err = "orbital on a non-existent atom";
        return VSVB_ERR_INPUT;
      }
      orb_atoms[o].push_back(a);
      for (int g = first_sh[a]; g < first_sh[a + 1]; ++g) {
        if (slot_of_shell[o][g] < 0) slot_of_shell[o][g] = (int)obs[o].size();
        for (int c = 0; c < ncart(sh[g].l); ++c) obs[o].push_back(sh[g].ao0 + c);
      }
    }
    h->maxobs = std::max(h->maxobs, (int)obs[o].size());
  }
  /* weight scatter terms */
  std::vector<int> term0(norbs + 1, 0), tslot, tj, tm, tf, ndf_orb;
  const int nfirst_ndf = norbs - d->ndf;
  for (int f = 0; f < d->ndf; ++f) ndf_orb.push_back(nfirst_ndf + f);
  for (int o = 0; o < norbs; ++o) {
    term0[o] = (int)tslot.size();
    for (int j = d->map_orbs[o] - 1; j < d->map_orbs[o + 1] - 1; ++j) {
      int xp = d->xpset[j];
      if (xp >= 1) {
        if (xp > (int)obs[o].size()) {
          h->err = "weight address outside its orbital basis set";
          return VSVB_ERR_INPUT;
        }
        tslot.push_back(xp - 1);
        tj.push_back(j);
        tm.push_back(-1);
        tf.push_back(-1);
      } else {
        if (o >= nfirst_ndf) {
          h->err = "a derived basis function refers to another one";
          return VSVB_ERR_INPUT;
        }
        int indf = xp + norbs - 1; /* 0-based orbital index of the NDF */
        if (indf < nfirst_ndf || indf >= norbs) {
          h->err = "bad derived-basis-function reference";
          return VSVB_ERR_INPUT;
        }
        /* ndf2obs: NDF atom AO ranges, then the matching orbital atom offsets */
        std::vector<int> beg, end, target;
        int ib = 0;
        for (int a : orb_atoms[indf]) {
          beg.push_back(ib + 1);
          for (int g = first_sh[a]; g < first_sh[a + 1]; ++g) ib += ncart(sh[g].l);
          end.push_back(ib);
        }
        target.assign(orb_atoms[indf].size(), 0);
        int ob = 1;
        for (int a : orb_atoms[o]) {
          for (size_t jat = 0; jat < orb_atoms[indf].size(); ++jat)
            if (orb_atoms[indf][jat] == a) target[jat] = ob;
          for (int g = first_sh[a]; g < first_sh[a + 1]; ++g) ob += ncart(sh[g].l);
        }
        int shift = 0;
        for (int m = d->map_orbs[indf] - 1; m < d->map_orbs[indf + 1] - 1; ++m) {
          int xm = d->xpset[m];
          for (size_t ia = 0; ia < orb_atoms[indf].size(); ++ia)
            if (xm >= beg[ia] && xm <= end[ia]) shift = target[ia] - beg[ia];
          int slot = xm + shift - 1;
          if (slot < 0 || slot >= (int)obs[o].size()) {
            h->err = "derived basis function outside the orbital basis set";
            return VSVB_ERR_INPUT;
          }
          tslot.push_back(slot);
          tj.push_back(j);
          tm.push_back(m);
          tf.push_back(indf - nfirst_ndf);
        }
      }
    }
  }
  term0[norbs] = (int)tslot.size();
  std::vector<int> obs_n(norbs), obs_ao((size_t)norbs * std::max(h->maxobs, 1), 0);
  for (int o = 0; o < norbs; ++o) {
    obs_n[o] = (int)obs[o].size();
    for (size_t k = 0; k < obs[o].size(); ++k) obs_ao[(size_t)o * h->maxobs + k] = obs[o][k];
  }
  /* device uploads for the one-electron stage */
  std::vector<double> charge(d->natom), axyz(3 * d->natom);
  for (int a = 0; a < d->natom; ++a) {
    charge[a] = d->nuc_charge[d->atom_t[a] - 1];
    for (int k = 0; k < 3; ++k) axyz[3 * a + k] = d->coords[3 * a + k];
  }
  CK(h->shells.upload(sh), "upload shells");
  CK(h->exps.upload(std::vector<double>(d->exponent, d->exponent + d->num_pr)), "upload exps");
  CK(h->coefs.upload(cc), "upload coefs");
  CK(h->angn.upload(angn), "upload angn");
  CK(h->charge.upload(charge), "upload charge");
  CK(h->axyz.upload(axyz), "upload xyz");
  CK(h->S_ao.alloc((size_t)h->nao * h->nao), "alloc S");
  CK(h->H_ao.alloc((size_t)h->nao * h->nao), "alloc H");
  {
    Ao1eArgs a{};
    a.shells = h->shells.p;
    a.nshell = h->nsh;
    a.nao = h->nao;
    a.natom = d->natom;
    a.exps = h->exps.p;
    a.coefs = h->coefs.p;
    a.angn = h->angn.p;
    a.charge = h->charge.p;
    a.atom_xyz = h->axyz.p;
    a.S = h->S_ao.p;
    a.H = h->H_ao.p;
    int npairs = h->nsh * (h->nsh + 1) / 2;
    ao_1e_kernel<<<(unsigned)(((long long)npairs * 32 + 127) / 128), 128, 0, h->st>>>(a);
    CK(cudaGetLastError(), "ao_1e_kernel");
  }
  CK(h->obs_n.upload(obs_n), "upload obs");
  CK(h->obs_ao.upload(obs_ao), "upload obs");
  CK(h->term0.upload(term0), "upload terms");
  CK(h->term_slot.upload(tslot), "upload terms");
  CK(h->term_j.upload(tj), "upload terms");
  CK(h->term_m.upload(tm), "upload terms");
  CK(h->term_f.upload(tf), "upload terms");
  CK(h->ndf_orb.upload(ndf_orb), "upload ndf");

  /* shell pairs, orbital pairs, X terms */
  const int nsp = h->nsp;
  h->np = nsp * (nsp + 1) / 2;
  std::vector<std::vector<int>> orbs_on_atom(d->natom);
  for (int o = 0; o < nsp; ++o)
    for (int a : orb_atoms[o])
      if (orbs_on_atom[a].empty() || orbs_on_atom[a].back() != o) orbs_on_atom[a].push_back(o);
  std::vector<ShellPair> pairs;
  std::vector<PrimPair> prims;
  std::vector<int> opid;
  std::vector<XTerm> xterms;
  std::vector<long long> xelem0, xh_elem0;
  std::vector<double> hrr;
  long long nx = 0, nxh = 0;
  for (int A0 = 0; A0 < h->nsh; ++A0)
    for (int B0 = 0; B0 <= A0; ++B0) {
      int A = A0, B = B0;
      if (sh[A].l < sh[B].l) std::swap(A, B);
      /* orbital pairs touching (A,B) */
      std::set<std::pair<int, int>> ops;
      for (int i : orbs_on_atom[sh[A].atom])
        for (int k : orbs_on_atom[sh[B].atom]) ops.insert({std::max(i, k), std::min(i, k)});
      if (ops.empty()) continue;
      ShellPair P{};
      P.shA = A;
      P.shB = B;
      P.cls = pair_class(sh[A].l, sh[B].l);
      P.prim0 = (int)prims.size();
      for (int k = 0; k < 3; ++k) {
        P.A[k] = sh[A].xyz[k];
        P.B[k] = sh[B].xyz[k];
      }
      double ab2 = 0.0;
      for (int k = 0; k < 3; ++k) ab2 += (P.A[k] - P.B[k]) * (P.A[k] - P.B[k]);
      for (int ia = 0; ia < sh[A].nprim; ++ia)
        for (int ib = 0; ib < sh[B].nprim; ++ib) {
          double al = d->exponent[sh[A].prim0 + ia], be = d->exponent[sh[B].prim0 + ib];
          double p = al + be;
          double K = cc[sh[A].prim0 + ia] * cc[sh[B].prim0 + ib] * std::exp(-al * be / p * ab2);
          if (std::fabs(K) < 1e-24) continue;
          PrimPair pp{};
          for (int k = 0; k < 3; ++k) pp.P[k] = (al * P.A[k] + be * P.B[k]) / p;
          pp.p = p;
          pp.inv_p = 1.0 / p;
          pp.Kp = K / p;
          prims.push_back(pp);
        }
      P.nprim = (int)prims.size() - P.prim0;
      if (P.nprim == 0) continue;
      P.op0 = (int)opid.size();
      P.nop = (int)ops.size();
      P.x0 = (int)nx;
      P.xh0 = (int)nxh;
      P.m0 = (int)hrr.size();
      {
        const double AB[3] = {P.A[0] - P.B[0], P.A[1] - P.B[1], P.A[2] - P.B[2]};
        hrr_matrix(sh[A].l, sh[B].l, AB, hrr);
      }
      for (auto &ik : ops) {
        int i = ik.first, k = ik.second;
        opid.push_back(i * (i + 1) / 2 + k);
        XTerm t{};
        t.oi = i;
        t.ok = k;
        t.la = sh[A].l;
        t.lb = sh[B].l;
        t.sAi = slot_of_shell[i][A];
        t.sBi = slot_of_shell[i][B];
        t.sAk = slot_of_shell[k][A];
        t.sBk = slot_of_shell[k][B];
        t.aoA = sh[A].ao0;
        t.aoB = sh[B].ao0;
        t.same_shell = A == B;
        t.m0 = P.m0;
        xterms.push_back(t);
        xelem0.push_back(nx);
        xh_elem0.push_back(nxh);
        nx += ncart(sh[A].l) * ncart(sh[B].l);
        nxh += pair_ne(sh[A].l, sh[B].l);
      }
      pairs.push_back(P);
    }
  if (nx > (long long)0x7fffffff || nxh > (long long)0x7fffffff || hrr.size() > (size_t)0x7fffffff) {
    h->err = "weight tables exceed 2^31 elements";
    return VSVB_ERR_UNSUPPORTED;
  }
  h->nxelem = nx;
  h->nxh = nxh;
  h->nxterm = (int)xterms.size();
  CK(h->pairs.upload(pairs), "upload pairs");
  {
    int rc = upload_prims(h, prims);
    if (rc) return rc;
  }
  {
    std::vector<GeomT<double>> g64(pairs.size());
    std::vector<GeomT<float>> g32(pairs.size());
    std::vector<GeomT<df64>> gdf(pairs.size());
    for (size_t i = 0; i < pairs.size(); ++i)
      for (int k = 0; k < 3; ++k) {
        const double A = pairs[i].A[k], AB = pairs[i].A[k] - pairs[i].B[k];
        g64[i].A[k] = A;
        g64[i].AB[k] = AB;
        g32[i].A[k] = (float)A;
        g32[i].AB[k] = (float)AB;
        gdf[i].A[k] = df64(A);
        gdf[i].AB[k] = df64(AB);
      }
    CK(h->geom64.upload(g64), "upload geom64");
    CK(h->geom32.upload(g32), "upload geom32");
    CK(h->geomdf.upload(gdf), "upload geomdf");
  }
  CK(h->pair_opid.upload(opid), "upload opid");
  CK(h->xterms.upload(xterms), "upload xterms");
  CK(h->xelem0.upload(xelem0), "upload xelem0");
  CK(h->xh_elem0.upload(xh_elem0.empty() ? std::vector<long long>(1, 0) : xh_elem0), "upload xh_elem0");
  CK(h->hrr.upload(hrr.empty() ? std::vector<double>(1, 0.0) : hrr), "upload hrr");
  CK(h->xtab.alloc(std::max<long long>(nx, 1)), "alloc xtab");
  CK(h->xtabh.alloc(std::max<long long>(nxh, 1)), "alloc xtabh");
  CK(h->xtabh32.alloc(std::max<long long>(nxh, 1)), "alloc xtabh32");
  CK(h->qmax.alloc(std::max<size_t>(pairs.size(), 1)), "alloc qmax");
  CK(h->q0max.alloc(std::max<size_t>(pairs.size(), 1)), "alloc q0max");
  CK(h->T.alloc(std::max<size_t>((size_t)h->np * h->np, 1)), "alloc T");
  CK(h->sqT.alloc(std::max<size_t>((size_t)h->np, 1)), "alloc sqT");
  /* Rys tables */
  CK(h->rys.upload(std::vector<double>(rys_table_data, rys_table_data + sizeof(rys_table_data) / sizeof(double))),
     "upload rys");
  {
    const size_t nt = sizeof(rys_table_data) / sizeof(double);
    std::vector<float2> df(nt);
    for (size_t i = 0; i < nt; ++i) {
      const float hi = (float)rys_table_data[i];
      df[i] = make_float2(hi, (float)(rys_table_data[i] - (double)hi));
    }
    CK(h->rysdf.upload(df), "upload rysdf");
    std::vector<float> f32(nt);
    for (size_t i = 0; i < nt; ++i) f32[i] = df[i].x;
    CK(h->rys32.upload(f32), "upload rys32");
  }
  for (int k = 0; k < 5; ++k) {
    h->rc.off[k] = rys_table_offset[k];
    for (int r = 0; r < 5; ++r) {
      h->rc.ax[k][r] = rys_asym_x[k][r];
      h->rc.aw[k][r] = rys_asym_w[k][r];
      const float axh = (float)rys_asym_x[k][r], awh = (float)rys_asym_w[k][r];
      h->rc.axf[k][r] = make_float2(axh, (float)(rys_asym_x[k][r] - (double)axh));
      h->rc.awf[k][r] = make_float2(awh, (float)(rys_asym_w[k][r] - (double)awh));
    }
  }
  /* Schwarz bounds (diagonal quartets) */
  std::vector<double> q0;
  std::vector<float> q0f; /* per primitive pair, sorted descending within each shell pair */
  {
    std::vector<int4> diag[6];
    for (size_t p = 0; p < pairs.size(); ++p) diag[pairs[p].cls].push_back(make_int4((int)p, (int)p, 0, 1 << 30));
    EriArgs ea = eri_args(h);
    ea.prim_lo = 0.f;
    ea.prim_hi = INFINITY;
    DBuf<int4> wd[6];
    for (int c = 0; c < 6; ++c) {
      if (diag[c].empty()) continue;
      CK(wd[c].upload(diag[c]), "upload diag");
      if (eri_launch(1, 0, c, c, ea, wd[c].p, (int)diag[c].size(), h->nsm * 16, h->st)) {
        h->err = "Schwarz kernel launch failed";
        return VSVB_ERR_CUDA;
      }
    }
    std::vector<double> q(pairs.size());
    q0.assign(pairs.size(), 0.0);
    CK(cudaStreamSynchronize(h->st), "schwarz sync");
    if (!pairs.empty()) {
      CK(cudaMemcpy(q.data(), h->qmax.p, sizeof(double) * q.size(), cudaMemcpyDeviceToHost), "qmax");
      CK(cudaMemcpy(q0.data(), h->q0max.p, sizeof(double) * q0.size(), cudaMemcpyDeviceToHost), "q0max");
    }
    for (size_t p = 0; p < pairs.size(); ++p) pairs[p].qmax = q[p];
    CK(h->pairs.upload(pairs), "upload pairs");
  }
  /* primitive Schwarz bounds: the same diagonal pass over one-primitive
   * copies of every shell pair gives sqrt(max_e |(e0|e0)|) per primitive
   * pair; each pair's primitives are then sorted by it, descending, so that
   * the kernels' primitive screen q0_p q0_q < prim_screen cuts a tail */
  {
    std::vector<ShellPair> vp;
    std::vector<GeomT<double>> vg;
    std::vector<int4> vdiag[6];
    for (size_t pi = 0; pi < pairs.size(); ++pi) {
      GeomT<double> g;
      for (int k = 0; k < 3; ++k) {
        g.A[k] = pairs[pi].A[k];
        g.AB[k] = pairs[pi].A[k] - pairs[pi].B[k];
      }
      for (int ip = 0; ip < pairs[pi].nprim; ++ip) {
        ShellPair v = pairs[pi];
        v.prim0 = pairs[pi].prim0 + ip;
        v.nprim = 1;
        vdiag[v.cls].push_back(make_int4((int)vp.size(), (int)vp.size(), 0, 1 << 30));
        vp.push_back(v);
        vg.push_back(g);
      }
    }
    DBuf<ShellPair> vp_d;
    DBuf<GeomT<double>> vg_d;
    DBuf<double> vq, vq0;
    DBuf<int4> wd[6];
    CK(vp_d.upload(vp), "upload prim pairs");
    CK(vg_d.upload(vg), "upload prim geometry");
    CK(vq.alloc(std::max<size_t>(vp.size(), 1)), "alloc prim bounds");
    CK(vq0.alloc(std::max<size_t>(vp.size(), 1)), "alloc prim bounds");
    EriArgs ea = eri_args(h);
    ea.pairs = vp_d.p;
    ea.geom64 = vg_d.p;
    ea.qmax_out = vq.p;
    ea.q0max_out = vq0.p;
    ea.prim_lo = 0.f;
    ea.prim_hi = INFINITY;
    for (int c = 0; c < 6; ++c) {
      if (vdiag[c].empty()) continue;
      CK(wd[c].upload(vdiag[c]), "upload prim diag");
      if (eri_launch(1, 0, c, c, ea, wd[c].p, (int)vdiag[c].size(), h->nsm * 16, h->st)) {
        h->err = "primitive Schwarz kernel launch failed";
        return VSVB_ERR_CUDA;
      }
    }
    std::vector<double> pq0(vp.size());
    CK(cudaStreamSynchronize(h->st), "prim schwarz sync");
    if (!vp.empty()) CK(cudaMemcpy(pq0.data(), vq0.p, sizeof(double) * pq0.size(), cudaMemcpyDeviceToHost), "prim q0");
    /* vp is in prims order, so pq0[i] belongs to prims[i] */
    q0f.assign(prims.size(), 0.f);
    for (size_t pi = 0; pi < pairs.size(); ++pi) {
      const int p0 = pairs[pi].prim0, n = pairs[pi].nprim;
      std::vector<int> ord(n);
      for (int k = 0; k < n; ++k) ord[k] = k;
      std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return pq0[p0 + x] > pq0[p0 + y]; });
      std::vector<PrimPair> seg(n);
      for (int k = 0; k < n; ++k) {
        seg[k] = prims[p0 + ord[k]];
        q0f[p0 + k] = (float)pq0[p0 + ord[k]];
      }
      for (int k = 0; k < n; ++k) prims[p0 + k] = seg[k];
    }
    int rc = upload_prims(h, prims);
    if (rc) return rc;
    CK(h->prim_q0.upload(q0f.empty() ? std::vector<float>(1, 0.f) : q0f), "upload prim q0");
  }
  /* size of the arithmetic behind a pair's transferred integrals: the
   * (e0|e0) bound times the largest row 1-norm of its transfer matrix */
  std::vector<double> amp(pairs.size(), 0.0);
  for (size_t p = 0; p < pairs.size(); ++p) {
    const int la = sh[pairs[p].shA].l, lb = sh[pairs[p].shB].l;
    const int nab = ncart(la) * ncart(lb), ne = pair_ne(la, lb);
    double mx = 0.0;
    for (int ab = 0; ab < nab; ++ab) {
      double r = 0.0;
      for (int e = 0; e < ne; ++e) r += std::fabs(hrr[pairs[p].m0 + (size_t)ab * ne + e]);
      mx = std::max(mx, r);
    }
    amp[p] = q0[p] * mx;
  }
  /* quartet schedule */
  const bool mixed = h->opt.precision == VSVB_MIXED || h->opt.precision == VSVB_MIXED_DF64;
  const float eps = (float)h->opt.prim_screen, tau = (float)h->opt.mixed_threshold;
  const bool split = mixed && h->opt.prim_split;
  /* primitive quartets of (P, Q) with lo <= q0_p q0_q < hi (FP32 products,
   * as the kernels form them; rows cut where q0_p q0_q(first) < lo), and
   * the sum of their bounds */
  auto window = [&](int P, int Q, float lo, float hi, double &sum) -> double {
    const float *a = q0f.data() + pairs[P].prim0, *b = q0f.data() + pairs[Q].prim0;
    const int na = pairs[P].nprim, nb = pairs[Q].nprim;
    double n = 0.0;
    sum = 0.0;
    int jlo = nb, jhi = nb;
    for (int i = 0; i < na; ++i) {
      if (!(a[i] * b[0] >= lo)) break;
      while (jlo > 0 && !(a[i] * b[jlo - 1] >= lo)) --jlo;
      while (jhi > 0 && !(a[i] * b[jhi - 1] >= hi)) --jhi;
      n += jlo - jhi;
      for (int j = jhi; j < jlo; ++j) sum += (double)a[i] * b[j];
    }
    return n;
  };
  /* the primitive split of an FP64-class quartet on the mixed paths (its
   * small primitive quartets in a second, FP32 launch) pays when the
   * quartet's double-float integrals outweigh its transform.  In the
   * double-float launch the transform runs on the FP64 pipe and the
   * integrals on the FP32 pipe side by side; while the FP64 transform is the
   * longer of the two, the small primitives cost nothing there, and the FP32
   * launch would only repeat the transform.  Rates as in the roofline:
   * double-float integrals at 3/16 of the FP32 FMA rate against the
   * transform at the FP64 rate, a factor 5.5 on this part.  Measured with
   * the split everywhere / nowhere / this rule at factors 5.5, 1.5: the C/H
   * chain 14.8 / 18.1 / 16.1, 15.1 ms; the 128-atom chain (transforms of
   * ~36 x 36 orbital pairs) 491 / 465 / 459, 470 ms.  The rule takes 3, and
   * splits every quartet whose transform block has at most 256 orbital-pair
   * products (C/H chain 15.5 ms, 128-atom chain 451 ms; at most 1024: 14.8
   * and 475 ms) */
  auto split_pays = [&](int a, int c) -> bool {
    if (!split) return false;
    double sb = 0.0;
    const double nall = window(a, c, eps, INFINITY, sb);
    const double pf = eri_flops(0, pairs[a].cls, pairs[c].cls, 1.0, 0, 0);
    const double tr = eri_flops(3, pairs[a].cls, pairs[c].cls, 0.0, pairs[a].nop, pairs[c].nop);
    return nall * pf > 3.0 * tr || (long long)pairs[a].nop * pairs[c].nop <= 256;
  };
  /* the same per row of P's primitive pairs (rows[i] for i < na) */
  auto window_rows = [&](int P, int Q, float lo, float hi, std::vector<int> &rows) {
    const float *a = q0f.data() + pairs[P].prim0, *b = q0f.data() + pairs[Q].prim0;
    const int na = pairs[P].nprim, nb = pairs[Q].nprim;
    rows.assign(na, 0);
    int jlo = nb, jhi = nb;
    for (int i = 0; i < na; ++i) {
      if (!(a[i] * b[0] >= lo)) break;
      while (jlo > 0 && !(a[i] * b[jlo - 1] >= lo)) --jlo;
      while (jhi > 0 && !(a[i] * b[jhi - 1] >= hi)) --jhi;
      rows[i] = jlo - jhi;
    }
  };
  h->err_bound = 0.0;
  h->bound_all = 0.0;
  {
    /* block mode: s and p shells only, not for first_order_opt's handles */
    bool sp_only = true;
    for (const GShell &g : sh) sp_only = sp_only && g.l <= 1;
    const double ncand = 0.5 * (double)pairs.size() * ((double)pairs.size() + 1.0);
    const bool want = h->opt.block_mode > 0 || (h->opt.block_mode == 0 && ncand > 5e7);
    if (want && (!sp_only || h->hs_split)) {
      if (h->opt.block_mode > 0) {
        h->err = "block mode needs s and p shells only";
        return VSVB_ERR_UNSUPPORTED;
      }
    } else if (want) {
      h->blk_on = true;
    }
  }
  if (h->blk_on) {
    int rc = build_block(h, d, sh, first_sh, orbs_on_atom, slot_of_shell, pairs, q0f, q0, amp);
    if (rc) return rc;
  } else {
    h->err_bound = 0.0;
    h->bound_all = 0.0;
    /* host threads over contiguous ranges of P (equal numbers of (P, Q)
     * candidates), merged in P order: the same lists as one thread */
    const size_t npr = pairs.size();
    const int nthr = npr > 2000 ? std::max(1, std::min(16, (int)std::thread::hardware_concurrency())) : 1;
    auto run_threads = [&](int n, const std::function<void(int)> &f) {
      std::vector<std::thread> th;
      for (int k = 1; k < n; ++k) th.emplace_back(f, k);
      f(0);
      for (auto &t : th) t.join();
    };
    {
      struct Part {
        double bound_all = 0.0, nprimq_all = 0.0, nprimq_fp32 = 0.0, err_bound = 0.0;
        long long nq32 = 0, nq64 = 0;
        std::vector<int2> w[3][6][6];
      };
      std::vector<size_t> cut(nthr + 1);
      for (int k = 0; k <= nthr; ++k) cut[k] = (size_t)std::llround((double)npr * std::sqrt((double)k / nthr));
      cut[nthr] = npr;
      std::vector<Part> parts(nthr);
      run_threads(nthr, [&](int k) {
        Part &pt = parts[k];
        for (size_t P = cut[k]; P < cut[k + 1]; ++P)
          for (size_t Q = 0; Q <= P; ++Q) {
            double b = pairs[P].qmax * pairs[Q].qmax;
            if (b < h->opt.ao_screen) continue;
            int a = (int)P, c = (int)Q;
            if (pairs[a].cls < pairs[c].cls) std::swap(a, c);
            int prec = (mixed && b < h->opt.mixed_threshold) ? 1 : 0;
            pt.bound_all += b;
            double sb = 0.0;
            const double nall = window(a, c, eps, INFINITY, sb);
            pt.nprimq_all += nall;
            if (prec) {
              pt.nq32++;
              pt.nprimq_fp32 += nall;
              pt.err_bound += amp[P] * amp[Q];
            } else {
              pt.nq64++;
              if (!split_pays(a, c)) {
                if (split) prec = 2;
              } else {
                /* the FP32 tail: its bound mass in units of the pair bounds,
                 * with the transfer norms of both pairs */
                const double nt = window(a, c, eps, tau, sb);
                pt.nprimq_fp32 += nt;
                pt.err_bound += sb * (amp[P] / std::max(q0[P], 1e-300)) * (amp[Q] / std::max(q0[Q], 1e-300));
              }
            }
            pt.w[prec][pairs[a].cls][pairs[c].cls].push_back(make_int2(a, c));
          }
      });
      for (const Part &pt : parts) {
        h->bound_all += pt.bound_all;
        h->nprimq_all += pt.nprimq_all;
        h->nprimq_fp32 += pt.nprimq_fp32;
        h->err_bound += pt.err_bound;
        h->nq_fp32 += pt.nq32;
        h->nq_fp64 += pt.nq64;
        for (int p = 0; p < 3; ++p)
          for (int a = 0; a < 6; ++a)
            for (int c = 0; c < 6; ++c) {
              auto &dst = h->work_h[p][a][c];
              dst.insert(dst.end(), pt.w[p][a][c].begin(), pt.w[p][a][c].end());
            }
      }
    }
    {
      /* a quartet with more than this many primitive quartets in a launch's
       * window is split into row ranges of P's primitives, so that the largest
       * quartets do not leave a tail of lone CTAs at the end of the launch */
      constexpr int SPLIT_PRIMQ = 512;
      /* one task per (list, bra class, ket class), on host threads; results
       * appended in task order */
      struct Task {
        int p, a, c;
        std::vector<vsvb_gpu::SweepItem> items;
        std::vector<std::vector<int4>> lists;
      };
      std::vector<Task> tasks;
      for (int p = 0; p < 3; ++p)
        for (int a = 0; a < 6; ++a)
          for (int c = 0; c < 6; ++c)
            if (!h->work_h[p][a][c].empty()) tasks.push_back({p, a, c, {}, {}});
      std::atomic<int> next(0);
      run_threads(std::min<int>(nthr, (int)tasks.size()), [&](int) {
        std::vector<int> rows;
        for (int ti = next++; ti < (int)tasks.size(); ti = next++) {
          Task &tk = tasks[ti];
          const int p = tk.p, a = tk.a, c = tk.c;
          const auto &w = h->work_h[p][a][c];
          /* launches over this list: FP32-class lists in FP32; FP64-class
           * lists in the handle's FP64-class arithmetic, and with the split
           * their primitive quartets below tau in FP32 */
          std::vector<vsvb_gpu::SweepItem> items;
          if (p == 1) {
            items.push_back({p, ERI_F32, a, c, eps, INFINITY, 0, 0, 0, 100 * ERI_F32 + 10 * a + c});
          } else if (p == 2) {
            items.push_back({p, eri_kind(h, 0), a, c, eps, INFINITY, 0, 0, 0, 100 * eri_kind(h, 0) + 10 * a + c});
          } else if (split) {
            items.push_back({p, eri_kind(h, 0), a, c, std::max(eps, tau), INFINITY, 0, 0, 0, 100 * eri_kind(h, 0) + 10 * a + c});
            items.push_back({p, ERI_F32, a, c, eps, tau, 0, 0, 0, 300 + 10 * a + c});
          } else {
            items.push_back({p, eri_kind(h, 0), a, c, eps, INFINITY, 0, 0, 0, 100 * eri_kind(h, 0) + 10 * a + c});
          }
          for (auto &it : items) {
            std::vector<std::pair<double, int4>> kept;
            for (const int2 &q : w) {
              window_rows(q.x, q.y, it.lo, it.hi, rows);
              double n = 0.0;
              for (int r : rows) n += r;
              if (n <= 0.0) continue;
              const int parts = (int)std::ceil(n / SPLIT_PRIMQ);
              const double target = n / parts;
              int r0 = 0;
              double acc = 0.0;
              for (int r = 0; r < (int)rows.size(); ++r) {
                acc += rows[r];
                const bool last = r + 1 == (int)rows.size();
                if (acc > 0.0 && (acc >= target || last)) {
                  kept.push_back({acc, make_int4(q.x, q.y, r0, last ? 1 << 30 : r + 1)});
                  it.flops_fwd += eri_flops(0, a, c, acc, pairs[q.x].nop, pairs[q.y].nop);
                  it.flops_grad += eri_flops(3, a, c, acc, pairs[q.x].nop, pairs[q.y].nop);
                  r0 = r + 1;
                  acc = 0.0;
                } else if (acc == 0.0) {
                  r0 = r + 1;
                }
              }
              it.nprimq += n;
            }
            if (kept.empty()) continue;
            /* the quartets of one atom quartet update and read the same
             * blocks of T and dE/dT (every shell pair of an atom pair has
             * the same orbital pairs), so they run next to each other,
             * where those blocks stay in L2: items grouped by atom
             * quartet, groups by their total work, largest first, items
             * within a group by work */
            const long long na = d->natom;
            auto aq = [&](const int4 &q) -> long long {
              const ShellPair &P = pairs[q.x], &Q = pairs[q.y];
              return ((sh[P.shA].atom * na + sh[P.shB].atom) * na + sh[Q.shA].atom) * na + sh[Q.shB].atom;
            };
            std::unordered_map<long long, double> gwork;
            gwork.reserve(kept.size());
            for (const auto &k : kept) gwork[aq(k.second)] += k.first;
            std::vector<std::tuple<double, long long, double, int4>> ord;
            ord.reserve(kept.size());
            for (const auto &k : kept) {
              const long long g = aq(k.second);
              ord.emplace_back(gwork[g], g, k.first, k.second);
            }
            std::stable_sort(ord.begin(), ord.end(), [](const auto &x, const auto &y) {
              if (std::get<0>(x) != std::get<0>(y)) return std::get<0>(x) > std::get<0>(y);
              if (std::get<1>(x) != std::get<1>(y)) return std::get<1>(x) < std::get<1>(y);
              return std::get<2>(x) > std::get<2>(y);
            });
            std::vector<int4> lst(ord.size());
            for (size_t k = 0; k < ord.size(); ++k) lst[k] = std::get<3>(ord[k]);
            tk.lists.push_back(std::move(lst));
            tk.items.push_back(it);
          }
        }
      });
      std::vector<std::vector<int4>> iwl;
      for (auto &tk : tasks)
        for (size_t k = 0; k < tk.items.size(); ++k) {
          tk.items[k].wl = (int)iwl.size();
          iwl.push_back(std::move(tk.lists[k]));
          h->sweep.push_back(tk.items[k]);
        }
      std::sort(h->sweep.begin(), h->sweep.end(), [](const vsvb_gpu::SweepItem &x, const vsvb_gpu::SweepItem &y) {
        return x.flops_fwd > y.flops_fwd;
      });
      h->item_wh = std::move(iwl);
      h->item_wd = std::vector<DBuf<int4>>(h->item_wh.size());
      for (size_t k = 0; k < h->item_wh.size(); ++k) CK(h->item_wd[k].upload(h->item_wh[k]), "upload item work");
    }
  }

  /* determinant pairs */
  DetSetup &ds = h->ds;
  ds.npair = d->npair;
  ds.nunpd = d->nunpd;
  ds.ndocc = d->ndocc;
  ds.nelec = 2 * d->npair + 2 * d->ndocc + d->nunpd;
  ds.nalpha = d->npair + d->nunpd + d->ndocc;
  ds.nbeta = d->npair + d->ndocc;
  ds.nnd = 2 * d->npair + d->nunpd;
  ds.nsd = ds.nnd + (h->hs_split ? 2 : 0);
  ds.nsp = nsp;
  ds.nsc = d->nspinc > 0 ? d->nspinc : 1;
  ds.nq = (long long)ds.nsc * ds.nsc << (2 * d->npair);
  std::vector<int> pslot((size_t)ds.nsc * d->npair * 2), spair((size_t)ds.nsc * 2 * d->npair, -1),
      swhich((size_t)ds.nsc * 2 * d->npair, -1);
  std::vector<double> csc(ds.nsc, 1.0);
  for (int isc = 0; isc < ds.nsc; ++isc) {
    if (d->nspinc > 0) csc[isc] = d->coeff_sc[isc];
    for (int k = 0; k < d->npair; ++k)
      for (int s = 0; s < 2; ++s) {
        int slot = d->pair_sc[k + d->npair * (s + 2 * isc)] - 1;
        if (slot < 0 || slot >= 2 * d->npair) {
          h->err = "spin-coupling pair outside the coupled orbitals";
          return VSVB_ERR_INPUT;
        }
        pslot[(isc * d->npair + k) * 2 + s] = slot;
        spair[isc * 2 * d->npair + slot] = k;
        swhich[isc * 2 * d->npair + slot] = s;
      }
    for (int s = 0; s < 2 * d->npair; ++s)
      if (spair[isc * 2 * d->npair + s] < 0) {
        h->err = "spin coupling does not cover every coupled orbital";
        return VSVB_ERR_INPUT;
      }
  }
  CK(h->pair_slot.upload(pslot.empty() ? std::vector<int>(1, 0) : pslot), "upload sc");
  CK(h->slot_pair.upload(spair.empty() ? std::vector<int>(1, 0) : spair), "upload sc");
  CK(h->slot_which.upload(swhich.empty() ? std::vector<int>(1, 0) : swhich), "upload sc");
  CK(h->coeff_sc.upload(csc), "upload coeff_sc");
  h->csc_h = csc;
  const long long nq_all = ds.nq;
  {
    /* core mode: every determinant pair shares the doubly occupied core
     * (no unpaired orbitals, the usual slot layout); automatic from 4096
     * determinant pairs */
    const bool fits = d->nunpd == 0 && !h->hs_split && d->npair >= 1 && d->npair <= 10;
    if (h->opt.core_mode > 0 && !fits) {
      h->err = "core mode needs spin-coupled pairs (at most 10) and no unpaired orbitals";
      return VSVB_ERR_UNSUPPORTED;
    }
    h->core_on = fits && (h->opt.core_mode > 0 || (h->opt.core_mode == 0 && nq_all >= 4096 && h->opt.grad_mode == 0));
  }
  if (h->core_on) {
    int rc = setup_core(h, pslot);
    if (rc) return rc;
  }
  /* per-pair buffers of the factorised path (one element in core mode) */
  const long long nq = h->core_on ? 1 : nq_all;
  const int na = ds.nalpha, nb = ds.nbeta;
  CK(h->det_a.alloc(nq), "alloc det");
  CK(h->det_b.alloc(nq), "alloc det");
  CK(h->detr_a.alloc(nq), "alloc det");
  CK(h->detr_b.alloc(nq), "alloc det");
  CK(h->Ta.alloc(std::max<long long>(nq * na * na, 1)), "alloc Ta");
  CK(h->Tb.alloc(std::max<long long>(nq * nb * nb, 1)), "alloc Tb");
  CK(h->sing.alloc(nq), "alloc sing");
  {
    /* exact-minor pool: one slot per flagged determinant pair, up to 1 GiB */
    const size_t per = (size_t)3 * ((size_t)na * na + (size_t)nb * nb);
    const size_t cap = std::max<size_t>(1, ((size_t)1 << 27) / std::max<size_t>(per, 1));
    h->xcap = (int)std::min<size_t>(std::min<size_t>((size_t)nq, cap), (size_t)1 << 30);
    CK(h->xinv.alloc(std::max<size_t>((size_t)h->xcap * per, 1)), "alloc exact-minor pool");
    CK(h->xdet.alloc((size_t)h->xcap * 6), "alloc exact-minor pool");
    CK(h->xslot.alloc(nq), "alloc exact-minor pool");
    CK(h->xcount.alloc(1), "alloc exact-minor pool");
    CK(h->abeq.alloc(nq), "alloc block flags");
  }
  CK(h->nsing.alloc(1), "alloc nsing");
  h->ld_scratch = 2 * std::max(na, nb) * std::max(std::max(na, nb), 1);
  CK(h->scratch.alloc(std::max<long long>(nq * h->ld_scratch, 1)), "alloc scratch");
  long long ntij = (long long)nsp * (nsp + 1) / 2;
  h->ntasks = ntij * (ntij + 1) / 2;
  long long work = std::max<long long>(h->ntasks, (long long)ds.nelec * ds.nelec);
  long long want = (16LL * h->nsm + nq_all - 1) / nq_all;
  long long maxs = (work + 127) / 128;
  h->nsplit = (int)std::max<long long>(1, std::min(want, maxs));
  h->nsplit_max = (int)std::max<long long>(1, std::min(4 * want, maxs)); /* autotuner range */
  size_t nslot = (size_t)nq_all * h->nsplit_max;
  CK(h->part_e1.alloc(nslot), "alloc parts");
  CK(h->part_wf.alloc(nslot), "alloc parts");
  CK(h->part_e2.alloc(nslot), "alloc parts");
  CK(h->result.alloc(8), "alloc result");
  CK(h->status.alloc(1), "alloc status");
  /* per-evaluation orbital buffers */
  CK(h->coeff_d.alloc(h->totlen), "alloc coeff");
  CK(h->ndf_scale.alloc(std::max(h->ndf, 1)), "alloc ndf");
  CK(h->orb_scale.alloc(norbs), "alloc scale");
  CK(h->Craw.alloc((size_t)norbs * h->maxobs), "alloc C");
  CK(h->C.alloc((size_t)norbs * h->maxobs), "alloc C");
  CK(h->So.alloc((size_t)nsp * nsp), "alloc So");
  CK(h->Ho.alloc((size_t)nsp * nsp), "alloc Ho");
  CK(cudaStreamSynchronize(h->st), "set-up sync");
  return VSVB_OK;
}

/* core-mode tables: per determinant (coupling, spin-flip bits) the coupled
 * orbital at each block position of each spin and the reverse map, the
 * determinants grouped by the spins of one or two coupled orbitals, the
 * orbital-pair index map; and the buffers of core.cu */
int setup_core(vsvb_gpu *h, const std::vector<int> &pslot) {
  const DetSetup &ds = h->ds;
  const int P = ds.npair, nC = 2 * P, nsc = ds.nsc, nsp = ds.nsp, nD = nsp - nC;
  const int ndet = nsc << P;
  std::vector<unsigned char> orb((size_t)ndet * 2 * P), pos((size_t)ndet * nC);
  for (int dt = 0; dt < ndet; ++dt) {
    const int sc = dt >> P, bits = dt & ((1 << P) - 1);
    for (int sp = 0; sp < 2; ++sp)
      for (int r = 0; r < P; ++r) {
        const int o = pslot[((size_t)sc * P + r) * 2 + (sp ^ ((bits >> r) & 1))];
        orb[((size_t)dt * 2 + sp) * P + r] = (unsigned char)o;
        pos[(size_t)dt * nC + o] = (unsigned char)((sp << 5) | r);
      }
  }
  auto spin = [&](int dt, int o) { return pos[(size_t)dt * nC + o] >> 5; };
  std::vector<int> l1, o1(2 * nC + 1), l2, o2(4 * nC * nC + 1);
  for (int x = 0; x < nC; ++x)
    for (int sp = 0; sp < 2; ++sp) {
      o1[2 * x + sp] = (int)l1.size();
      for (int dt = 0; dt < ndet; ++dt)
        if (spin(dt, x) == sp) l1.push_back(dt);
    }
  o1[2 * nC] = (int)l1.size();
  for (int x = 0; x < nC; ++x)
    for (int y = 0; y < nC; ++y)
      for (int g = 0; g < 4; ++g) {
        o2[4 * (x * nC + y) + g] = (int)l2.size();
        for (int dt = 0; dt < ndet; ++dt)
          if (2 * spin(dt, x) + spin(dt, y) == g) l2.push_back(dt);
      }
  o2[4 * nC * nC] = (int)l2.size();
  std::vector<int2> pik((size_t)h->np);
  for (int i = 0; i < nsp; ++i)
    for (int k = 0; k <= i; ++k) pik[(size_t)i * (i + 1) / 2 + k] = make_int2(i, k);
  CK(h->core_detorb.upload(orb), "upload core tables");
  CK(h->core_detpos.upload(pos), "upload core tables");
  CK(h->core_lst1.upload(l1), "upload core tables");
  CK(h->core_off1.upload(o1), "upload core tables");
  CK(h->core_lst2.upload(l2), "upload core tables");
  CK(h->core_off2.upload(o2), "upload core tables");
  CK(h->core_pik.upload(pik), "upload core tables");
  const long long nq = ds.nq;
  const int P2 = P * P, ncp = nC * (nC + 1) / 2, kx = ncp + 2;
  CK(h->core_fw.alloc(std::max<size_t>((size_t)nD * (2 * nD + nC), 1)), "alloc core");
  CK(h->core_G.alloc(std::max<size_t>((size_t)nD * nD, 1)), "alloc core");
  CK(h->core_Y.alloc(std::max<size_t>((size_t)nD * nC, 1)), "alloc core");
  CK(h->core_M.alloc((size_t)nC * nC), "alloc core");
  CK(h->core_P0.alloc((size_t)nsp * nsp), "alloc core");
  CK(h->core_U.alloc((size_t)nsp * nC), "alloc core");
  CK(h->core_s0.alloc(1), "alloc core");
  CK(h->core_dd.alloc((size_t)nq * 2), "alloc core");
  CK(h->core_L.alloc((size_t)nq * 2 * P2), "alloc core");
  CK(h->core_qf.alloc((size_t)nq * 2), "alloc core");
  CK(h->core_pslot.alloc((size_t)nq), "alloc core");
  CK(h->core_pcount.alloc(1), "alloc core");
  /* flagged-pair pool: three perturbed factorisations per spin, up to 512 MiB */
  const size_t per = (size_t)6 * (1 + P2);
  h->core_cap = (int)std::min<size_t>((size_t)nq, ((size_t)1 << 26) / per);
  CK(h->core_pool.alloc(std::max<size_t>((size_t)h->core_cap * per, 1)), "alloc core");
  CK(h->core_A0.alloc(1), "alloc core");
  CK(h->core_A1.alloc((size_t)nC * nC), "alloc core");
  CK(h->core_A2.alloc((size_t)nC * nC * nC * nC), "alloc core");
  CK(h->core_A2x.alloc((size_t)kx * kx), "alloc core");
  CK(h->core_R1.alloc((size_t)nsp * nsp), "alloc core");
  CK(h->core_Wv.alloc((size_t)h->np * kx), "alloc core");
  CK(h->core_X.alloc((size_t)h->np * kx), "alloc core");
  h->core_nt = (h->np + 63) / 64;
  CK(h->core_part.alloc((size_t)h->core_nt * h->core_nt), "alloc core");
  return VSVB_OK;
}

int alloc_grad(vsvb_gpu *h) {
  if (h->grad_ready) return VSVB_OK;
  const long long nq = h->ds.nq;
  const int na = h->ds.nalpha, nb = h->ds.nbeta;
  CK(h->Tbar.alloc(std::max<size_t>((size_t)h->np * h->np, 1)), "alloc Tbar");
  CK(h->Tbar32.alloc(std::max<size_t>((size_t)h->np * h->np, 1)), "alloc Tbar32");
  CK(h->Sbar.alloc((size_t)h->nsp * h->nsp), "alloc Sbar");
  CK(h->Hbar.alloc((size_t)h->nsp * h->nsp), "alloc Hbar");
  CK(h->xbar.alloc(std::max<long long>(h->nxelem, 1)), "alloc xbar");
  CK(h->xbarh.alloc(std::max<long long>(h->nxh, 1)), "alloc xbarh");
  CK(h->Cbar.alloc((size_t)h->norb_all * h->maxobs), "alloc Cbar");
  if (h->core_on) {
    /* the pair sums' adjoint instead of the per-pair walk buffers */
    const int P = h->ds.npair, nC = 2 * P, kx = nC * (nC + 1) / 2 + 2, n = h->nsp;
    const size_t nn = (size_t)n * n;
    CK(h->cg_Yg.alloc((size_t)h->np * kx), "alloc core adjoint");
    CK(h->cg_Axp.alloc((size_t)vsvb_gpu::CORE_NCHUNK * kx * kx), "alloc core adjoint");
    CK(h->cg_Ax.alloc((size_t)kx * kx), "alloc core adjoint");
    CK(h->cg_Wvb.alloc((size_t)h->np * kx), "alloc core adjoint");
    CK(h->cg_KP.alloc(nn), "alloc core adjoint");
    CK(h->cg_KR.alloc(nn), "alloc core adjoint");
    CK(h->cg_R1b.alloc(nn), "alloc core adjoint");
    CK(h->cg_P0b.alloc(nn), "alloc core adjoint");
    CK(h->cg_A1b.alloc((size_t)nC * nC), "alloc core adjoint");
    CK(h->cg_Ub.alloc((size_t)n * nC), "alloc core adjoint");
    CK(h->cg_Mbp.alloc((size_t)h->ds.nq * 2 * P * P), "alloc core adjoint");
    CK(h->cg_lam.alloc((size_t)h->ds.nq), "alloc core adjoint");
    CK(h->cg_Mb.alloc((size_t)nC * nC), "alloc core adjoint");
    CK(h->cg_sc.alloc(4), "alloc core adjoint");
    CK(h->cg_t1.alloc(nn), "alloc core adjoint");
    CK(h->cg_t2.alloc(nn), "alloc core adjoint");
  }
  const long long nqw = h->core_on ? 1 : nq;
  CK(h->vtot.alloc((size_t)nqw * h->nsplit_max), "alloc vtot");
  CK(h->Gglob.alloc(std::max<long long>(nqw * (na * na + nb * nb), 1)), "alloc G");
  CK(h->Gs.alloc(std::max<long long>(nqw * (na * na + nb * nb), 1)), "alloc Gs");
  CK(h->vtot_s.alloc((size_t)nqw * h->nsplit_max), "alloc vtot_s");
  CK(h->D1.alloc((size_t)h->nsp * h->nsp), "alloc D1");
  CK(h->coeff_bar.alloc(h->totlen), "alloc coeff_bar");
  CK(h->ndf_bar.alloc(std::max(h->ndf, 1)), "alloc ndf_bar");
  h->grad_ready = true;
  return VSVB_OK;
}

int alloc_grad(vsvb_gpu *h);

/* one sweep over every class schedule, spread over the side streams (largest
 * classes first), joined back into the handle's stream */
int eri_sweep(vsvb_gpu *h, int mode) {
  cudaStream_t st = h->st;
  EriArgs ea = eri_args(h);
  if (h->sweep_timing && !h->sweep_t0) {
    CK(cudaEventCreate(&h->sweep_t0), "cudaEventCreate");
    CK(cudaEventCreate(&h->sweep_t1), "cudaEventCreate");
  }
  if (h->sweep_timing) CK(cudaEventRecord(h->sweep_t0, st), "event record");
  CK(cudaEventRecord(h->ev_fork, st), "event record");
  for (int k = 0; k < vsvb_gpu::NAUX; ++k) CK(cudaStreamWaitEvent(h->aux[k], h->ev_fork, 0), "stream wait");
  int i = 0;
  if (h->sweep_timing && h->sweep_ev.size() < 2 * h->sweep.size()) {
    for (size_t k = h->sweep_ev.size(); k < 2 * h->sweep.size(); ++k) {
      cudaEvent_t e;
      CK(cudaEventCreate(&e), "cudaEventCreate");
      h->sweep_ev.push_back(e);
    }
  }
  for (const auto &it : h->sweep) {
    const int n = (int)h->item_wh[it.wl].size();
    cudaStream_t sa = h->aux[i % vsvb_gpu::NAUX];
    ea.prim_lo = it.lo;
    ea.prim_hi = it.hi;
    if (h->sweep_timing) CK(cudaEventRecord(h->sweep_ev[2 * i], sa), "event record");
    if (eri_launch(mode, it.kind, it.a, it.c, ea, h->item_wd[it.wl].p, n, h->nsm * it.bps, sa)) {
      h->err = "ERI kernel launch failed";
      return VSVB_ERR_CUDA;
    }
    if (h->sweep_timing) CK(cudaEventRecord(h->sweep_ev[2 * i + 1], sa), "event record");
    h->launches++;
    ++i;
  }
  h->sweep_mode = mode;
  for (int k = 0; k < vsvb_gpu::NAUX; ++k) {
    CK(cudaEventRecord(h->ev_join[k], h->aux[k]), "event record");
    CK(cudaStreamWaitEvent(st, h->ev_join[k], 0), "stream wait");
  }
  if (h->sweep_timing) CK(cudaEventRecord(h->sweep_t1, st), "event record");
  return VSVB_OK;
}

/* block mode: the orbital-pair matrix U (into T) chunk by chunk.  The ERI
 * launches of chunk c run on the side streams into staging buffer c % 2
 * (after the transform of chunk c - 2 has freed it); the handle's stream
 * joins them and transforms the chunk, so the integrals of chunk c + 1 run
 * while chunk c is transformed. */
int block_sweep(vsvb_gpu *h) {
  cudaStream_t st = h->st;
  {
    BlkCoefArgs ca{};
    ca.src = h->blk_csrc.p;
    ca.ao = h->blk_cao.p;
    ca.n = h->blk_ncoef;
    ca.C = h->C.p;
    ca.maxobs = h->maxobs;
    ca.angn = h->angn.p;
    ca.dtol = h->dtol;
    ca.catom = h->blk_catom.p;
    if (blk_coef(ca, st)) {
      h->err = "block weight launch failed";
      return VSVB_ERR_CUDA;
    }
    h->launches++;
  }
  if (h->sweep_timing && !h->sweep_t0) {
    CK(cudaEventCreate(&h->sweep_t0), "cudaEventCreate");
    CK(cudaEventCreate(&h->sweep_t1), "cudaEventCreate");
  }
  if (h->sweep_timing) CK(cudaEventRecord(h->sweep_t0, st), "event record");
  /* the transforms leave the staging buffers cleared; clearing them here as
   * well keeps an evaluation correct after one that stopped part-way */
  CK(cudaMemsetAsync(h->blk_G.p, 0, sizeof(double) * h->blk_G.n, st), "memset staging");
  CK(cudaEventRecord(h->ev_fork, st), "event record");
  for (int k = 0; k < vsvb_gpu::NAUX; ++k) CK(cudaStreamWaitEvent(h->aux[k], h->ev_fork, 0), "stream wait");
  EriArgs ea = eri_args(h);
  ea.pair_blk = h->blk_pair.p;
  BlkArgs ba{};
  ba.aq = h->blk_aq.p;
  ba.ap = h->blk_ap.p;
  ba.atom_orb = h->blk_atom_orb.p;
  ba.atom_nf = h->blk_atom_nf.p;
  ba.atom_c0 = h->blk_atom_c0.p;
  ba.orb = h->blk_orb.p;
  ba.catom = h->blk_catom.p;
  ba.U = h->T.p;
  ba.np = h->np;
  ba.nfmax = h->blk_nfmax;
  ba.nomax = h->blk_nomax;
  ba.r1n = blk_r1(h->blk_nfmax, h->blk_nomax);
  ba.nomaxp = (h->blk_nomax + 7) / 8 * 8;
  int rr = 0;
  for (size_t c = 0; c < h->blk_chunk.size(); ++c) {
    const auto &ch = h->blk_chunk[c];
    const int buf = (int)(c & 1);
    double *G = h->blk_G.p + (size_t)buf * h->blk_gsize;
    if (c >= 2)
      for (int k = 0; k < vsvb_gpu::NAUX; ++k) CK(cudaStreamWaitEvent(h->aux[k], h->blk_done[buf], 0), "stream wait");
    ea.G = G;
    for (int l = ch.l0; l < ch.l0 + ch.nl; ++l) {
      const auto &L = h->blk_launch[l];
      ea.prim_lo = L.lo;
      ea.prim_hi = L.hi;
      cudaStream_t sa = h->aux[rr++ % vsvb_gpu::NAUX];
      if (eri_launch(4, L.kind, L.cp, L.cq, ea, h->blk_work.p + L.off, L.n, h->nsm * 16, sa)) {
        h->err = "block ERI launch failed";
        return VSVB_ERR_CUDA;
      }
      h->launches++;
    }
    for (int k = 0; k < vsvb_gpu::NAUX; ++k) {
      CK(cudaEventRecord(h->ev_join[k], h->aux[k]), "event record");
      CK(cudaStreamWaitEvent(st, h->ev_join[k], 0), "stream wait");
    }
    ba.G = G;
    ba.G_clear = G;
    if (blk_transform(ba, ch.aq0, ch.naq, ch.tt, h->blk_smem[ch.tt], st)) {
      h->err = "block transform launch failed";
      return VSVB_ERR_CUDA;
    }
    h->launches++;
    CK(cudaEventRecord(h->blk_done[buf], st), "event record");
  }
  h->sweep_mode = 4;
  if (h->sweep_timing) CK(cudaEventRecord(h->sweep_t1, st), "event record");
  return VSVB_OK;
}

/* forward pass on coeff_d; leaves E in result[0..4] (device).  With fused,
 * the ERI sweep also accumulates the (unscaled) adjoint dE/dX from the
 * unscreened cofactor densities. */
/* the forward pass in two halves around the ERI sweep, so that a batch can
 * run one sweep for all its molecules between them */
int forward_pre(vsvb_gpu *h, bool fused);
int forward_post(vsvb_gpu *h, bool fused);

int forward(vsvb_gpu *h, bool fused = false) {
  int rc = forward_pre(h, fused);
  if (rc) return rc;
  rc = h->blk_on ? block_sweep(h) : eri_sweep(h, fused ? 3 : 0);
  if (rc) return rc;
  return forward_post(h, fused); /* launches keep counting across the three */
}

int forward_pre(vsvb_gpu *h, bool fused) {
  cudaStream_t st = h->st;
  h->launches = 0;
  CK(cudaMemsetAsync(h->status.p, 0, sizeof(int), st), "memset status");
  OrbArgs oa = orb_args(h);
  size_t osh = sizeof(double) * std::max(h->maxobs, 1);
  if (h->ndf > 0) {
    ndf_norm_kernel<<<h->ndf, 128, osh, st>>>(oa);
    CK(cudaGetLastError(), "ndf_norm");
    h->launches++;
  }
  orb_norm_kernel<<<h->nsp, 128, osh, st>>>(oa);
  CK(cudaGetLastError(), "orb_norm");
  orb_1e_kernel<<<dim3(h->nsp, h->nsp), 128, 0, st>>>(oa, h->So.p, h->Ho.p);
  CK(cudaGetLastError(), "orb_1e");
  h->launches += 2;
  if (h->nxelem > 0 && !h->blk_on) {
    XtabArgs xa = xtab_args(h);
    xtab_kernel<<<(unsigned)((h->nxelem + 255) / 256), 256, 0, st>>>(xa);
    CK(cudaGetLastError(), "xtab");
    xhrr_kernel<<<(unsigned)((h->nxh + 255) / 256), 256, 0, st>>>(xa);
    CK(cudaGetLastError(), "xhrr");
    h->launches += 2;
  }
  CK(cudaMemsetAsync(h->sing.p, 0, sizeof(int) * h->sing.n, st), "memset sing");
  CK(cudaMemsetAsync(h->xcount.p, 0, sizeof(int), st), "memset pool count");
  CK(cudaMemsetAsync(h->nsing.p, 0, sizeof(int), st), "memset nsing");
  if (h->core_on) {
    /* the pair sums over the shared core need the overlaps only */
    const int nl = core_pre(core_args(h), st);
    if (nl < 0) {
      h->err = "core-mode launch failed";
      return VSVB_ERR_CUDA;
    }
    h->launches += nl;
    if (fused) {
      /* Gamma is the sweep's dE_num/dT */
      int rc = alloc_grad(h);
      if (rc) return rc;
      CK(cudaMemsetAsync(h->xbarh.p, 0, sizeof(double) * h->xbarh.n, st), "memset xbarh");
      if (core_gamma(core_args(h), h->Tbar.p, st) < 0 || eri_to_float(h->Tbar.p, h->Tbar32.p, h->Tbar.n, st)) {
        h->err = "core-mode launch failed";
        return VSVB_ERR_CUDA;
      }
      h->launches += 2;
    }
    CK(cudaMemsetAsync(h->T.p, 0, sizeof(double) * h->T.n, st), "memset T");
    return VSVB_OK;
  }
  DetCtx dc = det_ctx(h);
  detpair_kernel<<<(unsigned)h->ds.nq, std::max(h->ds.nalpha, h->ds.nbeta) > 64 ? 512 : 128, 0, st>>>(
      dc, h->scratch.p, h->ld_scratch);
  CK(cudaGetLastError(), "detpair");
  h->launches++;
  if (fused) {
    int rc = alloc_grad(h);
    if (rc) return rc;
    CK(cudaMemsetAsync(h->Tbar.p, 0, sizeof(double) * h->Tbar.n, st), "memset Tbar");
    CK(cudaMemsetAsync(h->xbarh.p, 0, sizeof(double) * h->xbarh.n, st), "memset xbarh");
    AsmArgs ad = asm_args(h);
    CK(launch_assemble(2, dim3((unsigned)h->ds.nq, h->nsplit), 128, 0, st, dc, ad), "density walk");
    if (eri_to_float(h->Tbar.p, h->Tbar32.p, h->Tbar.n, st)) {
      h->err = "Tbar conversion launch failed";
      return VSVB_ERR_CUDA;
    }
    h->launches += 2;
  }
  CK(cudaMemsetAsync(h->T.p, 0, sizeof(double) * h->T.n, st), "memset T");
  return VSVB_OK;
}

int forward_post(vsvb_gpu *h, bool fused) {
  cudaStream_t st = h->st;
  DetCtx dc = det_ctx(h);
  if (eri_symmetrize(h->T.p, h->np, h->sqT.p, st)) {
    h->err = "symmetrize launch failed";
    return VSVB_ERR_CUDA;
  }
  h->launches++;
  if (h->core_on) {
    const int nl = core_post(core_args(h), fused ? h->Tbar.p : nullptr, st);
    if (nl < 0) {
      h->err = "core-mode launch failed";
      return VSVB_ERR_CUDA;
    }
    h->launches += nl;
    return VSVB_OK;
  }
  AsmArgs aa = asm_args(h);
  if (fused) {
    /* one walk for the energy sums and the (unscaled) adjoint quantities */
    const int na = h->ds.nalpha, nb = h->ds.nbeta;
    CK(cudaMemsetAsync(h->Gglob.p, 0, sizeof(double) * h->Gglob.n, st), "memset G");
    CK(cudaMemsetAsync(h->Gs.p, 0, sizeof(double) * h->Gs.n, st), "memset Gs");
    CK(cudaMemsetAsync(h->D1.p, 0, sizeof(double) * h->D1.n, st), "memset D1");
    aa.status = h->status.p;
    aa.skip_tbar = 1;
    const size_t gsh = sizeof(double) * (size_t)(na * na + nb * nb) * aa.g_in_smem;
    CK(launch_assemble(4, dim3((unsigned)h->ds.nq, h->nsplit), 128, gsh, st, dc, aa), "energy + adjoint walk");
  } else {
    CK(launch_assemble(0, dim3((unsigned)h->ds.nq, h->nsplit), 128, 0, st, dc, aa), "assemble");
  }
  energy_reduce_kernel<<<1, 256, 0, st>>>(aa, h->ds.nq * h->nsplit, h->ds.nelec, h->enuc, h->result.p);
  CK(cudaGetLastError(), "reduce");
  h->launches += 2;
  return VSVB_OK;
}

/* the result record of handle h from the device result r[0..4] */
void fill_result(const vsvb_gpu *h, const double *r, vsvb_energy_result *out) {
  {
    std::memset(out, 0, sizeof(*out));
    out->energy = r[0];
    out->e_num = r[1];
    out->e1 = r[2];
    out->e2 = r[3];
    out->wfnorm = r[4];
    out->enucrep = h->enuc;
    out->n_quartets_fp64 = h->nq_fp64;
    out->n_quartets_fp32 = h->nq_fp32;
    out->n_tasks = h->ntasks;
    out->n_kernel_launches = h->launches;
    out->n_prim_quartets = h->nprimq_all;
    out->n_prim_quartets_fp32 = h->nprimq_fp32;
    /* error estimate of the FP32 quartets: FP32 rounding (2^-24) of the
     * arithmetic behind their integrals -- per quartet the (e0|e0) bounds
     * times the transfer-matrix norms of both pairs -- converted to energy by
     * the two-electron energy per unit of Schwarz-bound mass,
     * |e2/W| / sum_PQ b_PQ, with a factor 2^-5 for the looseness of these
     * product bounds (on the C/H chain at thresholds 1e-6 .. all-FP32 the
     * measured error stays 5-90x below the estimate) */
    if (h->nq_fp32 > 0 && h->bound_all > 0.0 && r[4] != 0.0)
      out->err_est = std::ldexp(std::fabs(r[3] / r[4]) * (h->err_bound / h->bound_all), -29);
  }
}

int finish_result(vsvb_gpu *h, vsvb_energy_result *out) {
  double r[5];
  int status = 0, nsing = 0;
  CK(cudaMemcpyAsync(r, h->result.p, sizeof(double) * 5, cudaMemcpyDeviceToHost, h->st), "copy result");
  CK(cudaMemcpyAsync(&status, h->status.p, sizeof(int), cudaMemcpyDeviceToHost, h->st), "copy status");
  CK(cudaMemcpyAsync(&nsing, h->nsing.p, sizeof(int), cudaMemcpyDeviceToHost, h->st), "copy nsing");
  CK(cudaStreamSynchronize(h->st), "sync");
  if (status & 1) {
    h->err = "an orbital has non-positive self-overlap";
    return VSVB_ERR_NOT_NORMALISABLE;
  }
  if (status & 4) {
    h->err = "more singular determinant pairs than the exact-minor pool holds";
    return VSVB_ERR_UNSUPPORTED;
  }
  if (status & 8) {
    h->err = "the doubly occupied orbitals' overlap block is singular";
    return VSVB_ERR_SINGULAR;
  }
  if (out) {
    fill_result(h, r, out);
    out->n_singular_pairs = nsing;
  }
  return VSVB_OK;
}

/* Autotuner: launch geometry picked by timing on this device, once per
 * handle (vsvb_options.autotune).
 *  - per ERI launch of the sweep: the grid cap, 2/4/8/16 blocks per SM
 *    (beyond it the blocks stride over the quartet list);
 *  - the task splits per determinant pair of the assembly grids, from half
 *    to four times the default.
 * Each candidate runs 3 times on the handle's own data (min taken); the
 * choice changes launch shapes only, never the arithmetic. */
int autotune(vsvb_gpu *h) {
  if ((h->sweep.empty() && h->ntasks == 0) || h->blk_on || h->core_on) return VSVB_OK;
  int rc = forward(h); /* weight tables, T and determinant pairs for the timed launches */
  if (rc) return rc;
  CK(cudaStreamSynchronize(h->st), "autotune sync");
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0), "cudaEventCreate");
  CK(cudaEventCreate(&e1), "cudaEventCreate");
  auto time_it = [&](auto &&launch) -> float {
    float best = 1e30f;
    for (int r = 0; r < 3; ++r) {
      cudaEventRecord(e0, h->st);
      if (launch()) return -1.f;
      cudaEventRecord(e1, h->st);
      if (cudaEventSynchronize(e1) != cudaSuccess) return -1.f;
      float t = 0.f;
      cudaEventElapsedTime(&t, e0, e1);
      best = std::min(best, t);
    }
    return best;
  };
  /* ERI grid caps (forward launches into a scratch copy of U) */
  EriArgs ea = eri_args(h);
  int fail = 0;
  for (auto &it : h->sweep) {
    const int n = (int)h->item_wh[it.wl].size();
    ea.prim_lo = it.lo;
    ea.prim_hi = it.hi;
    float best = 1e30f;
    int pick = it.bps;
    for (int bps : {2, 4, 8, 16}) {
      const float t = time_it([&]() {
        return eri_launch(0, it.kind, it.a, it.c, ea, h->item_wd[it.wl].p, n, h->nsm * bps, h->st);
      });
      if (t < 0.f) {
        fail = 1;
        break;
      }
      if (t < best * 0.97f) {
        best = t;
        pick = bps;
      }
    }
    if (fail) break;
    it.bps = pick;
  }
  /* assembly task splits */
  if (!fail) {
    DetCtx dc = det_ctx(h);
    AsmArgs aa = asm_args(h);
    const int base = h->nsplit;
    float best = 1e30f;
    int pick = base;
    for (int ns : {base / 2, base, 2 * base, 4 * base}) {
      if (ns < 1 || ns > h->nsplit_max) continue;
      const float t = time_it([&]() {
        return (int)(launch_assemble(0, dim3((unsigned)h->ds.nq, ns), 128, 0, h->st, dc, aa) != cudaSuccess);
      });
      if (t < 0.f) {
        fail = 1;
        break;
      }
      if (t < best * 0.97f) {
        best = t;
        pick = ns;
      }
    }
    h->nsplit = pick;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (fail) {
    h->err = "autotune launch failed";
    return VSVB_ERR_CUDA;
  }
  CK(cudaMemsetAsync(h->T.p, 0, sizeof(double) * h->T.n, h->st), "memset T");
  CK(cudaStreamSynchronize(h->st), "autotune sync");
  return VSVB_OK;
}

/* adjoint pass; reads e_num and W from the forward pass's device result, so
 * forward + backward enqueue without a host round trip (and can be captured
 * into a CUDA graph) */
int backward(vsvb_gpu *h, bool fused) {
  int rc = alloc_grad(h);
  if (rc) return rc;
  cudaStream_t st = h->st;
  const int na = h->ds.nalpha, nb = h->ds.nbeta;
  if (!fused) {
    CK(cudaMemsetAsync(h->Tbar.p, 0, sizeof(double) * h->Tbar.n, st), "memset");
    CK(cudaMemsetAsync(h->xbarh.p, 0, sizeof(double) * h->xbarh.n, st), "memset");
  }
  CK(cudaMemsetAsync(h->Cbar.p, 0, sizeof(double) * h->Cbar.n, st), "memset");
  CK(cudaMemsetAsync(h->coeff_bar.p, 0, sizeof(double) * h->coeff_bar.n, st), "memset");
  DetCtx dc = det_ctx(h);
  AsmArgs aa = asm_args(h);
  aa.status = h->status.p;
  aa.res = h->result.p;
  if (h->core_on) {
    /* dE/dS_orb and dE/dh_orb of the pair sums; dE/dT went into the sweep */
    const int nl = core_adjoint(core_args(h), core_grad(h), st);
    if (nl < 0) {
      h->err = "core-mode adjoint launch failed";
      return VSVB_ERR_CUDA;
    }
    h->launches += nl;
  } else if (fused) {
    /* the forward walk accumulated the adjoint quantities unscaled */
    grad_scale_kernel<<<(unsigned)h->ds.nq, 128, 0, st>>>(dc, aa, h->nsplit);
    CK(cudaGetLastError(), "grad scale");
  } else {
    CK(cudaMemsetAsync(h->Sbar.p, 0, sizeof(double) * h->Sbar.n, st), "memset");
    CK(cudaMemsetAsync(h->Hbar.p, 0, sizeof(double) * h->Hbar.n, st), "memset");
    CK(cudaMemsetAsync(h->Gglob.p, 0, sizeof(double) * h->Gglob.n, st), "memset");
    aa.skip_tbar = 0;
    size_t gsh = sizeof(double) * (size_t)(na * na + nb * nb) * aa.g_in_smem;
    CK(launch_assemble(1, dim3((unsigned)h->ds.nq, h->nsplit), 128, gsh, st, dc, aa), "assemble grad");
  }
  if (!h->core_on) {
    detpair_adjoint_kernel<<<(unsigned)h->ds.nq, 128, 0, st>>>(dc, aa, h->nsplit);
    CK(cudaGetLastError(), "detpair adjoint");
  }
  if (!fused) {
    int rc2 = eri_sweep(h, 2);
    if (rc2) return rc2;
  }
  if (h->nxelem > 0) {
    XtabArgs xa = xtab_args(h);
    if (fused) xa.wres = h->result.p; /* the sweep used the unscaled densities: scale by 1/W */
    xhrr_adjoint_kernel<<<(unsigned)((h->nxelem + 255) / 256), 256, 0, st>>>(xa, h->xbarh.p, h->xbar.p);
    CK(cudaGetLastError(), "xhrr adjoint");
    xtab_adjoint_kernel<<<(unsigned)((h->nxelem + 255) / 256), 256, 0, st>>>(xa, h->xbar.p, h->Cbar.p);
    CK(cudaGetLastError(), "xtab adjoint");
    h->launches++;
  }
  OrbArgs oa = orb_args(h);
  orb_1e_adjoint_kernel<<<h->nsp, 128, 0, st>>>(oa, h->Sbar.p, h->Hbar.p, h->nsp, h->Cbar.p);
  CK(cudaGetLastError(), "orb_1e adjoint");
  if (h->ndf > 0) CK(cudaMemsetAsync(h->ndf_bar.p, 0, sizeof(double) * h->ndf, st), "memset ndf_bar");
  orb_norm_adjoint_kernel<<<h->nsp, 128, sizeof(double) * std::max(h->maxobs, 1), st>>>(oa, h->Cbar.p,
                                                                                     h->coeff_bar.p, h->ndf_bar.p);
  CK(cudaGetLastError(), "orb_norm adjoint");
  if (h->ndf > 0) {
    ndf_norm_adjoint_kernel<<<h->ndf, 128, 2 * sizeof(double) * std::max(h->maxobs, 1), st>>>(oa, h->ndf_bar.p,
                                                                                            h->coeff_bar.p);
    CK(cudaGetLastError(), "ndf_norm adjoint");
    h->launches++;
  }
  h->launches += 5;
  return VSVB_OK;
}

}  // namespace

extern "C" {

void vsvb_default_options(vsvb_options *o) {
  if (!o) return;
  o->precision = VSVB_FP64;
  o->mixed_threshold = 1e-6;
  o->ao_screen = 1e-15;
  o->device = 0;
  o->grad_mode = 0;
  o->prim_screen = 1e-17;
  o->prim_split = 1;
  o->cuda_graph = 1;
  o->autotune = 0;
  o->block_mode = 0;
  o->core_mode = 0;
}

int vsvb_gpu_create(const vsvb_system_desc *d, const vsvb_options *opt, vsvb_gpu **out) {
  if (!d || !out) return VSVB_ERR_INPUT;
  *out = nullptr;
  auto *h = new vsvb_gpu();
  vsvb_default_options(&h->opt);
  if (opt) h->opt = *opt;
  h->dev = h->opt.device;
  int rc = build(h, d);
  if (!rc && h->opt.autotune) rc = autotune(h);
  *out = h;
  return rc;
}

void vsvb_gpu_destroy(vsvb_gpu *h) {
  if (!h) return;
  cudaSetDevice(h->dev);
  if (h->st) cudaStreamSynchronize(h->st);
  cudaStream_t st = h->own_st;
  for (int k = 0; k < vsvb_gpu::NAUX; ++k) {
    if (h->aux[k]) cudaStreamDestroy(h->aux[k]);
    if (h->ev_join[k]) cudaEventDestroy(h->ev_join[k]);
  }
  if (h->ev_fork) cudaEventDestroy(h->ev_fork);
  if (h->gexec) cudaGraphExecDestroy(h->gexec);
  for (cudaEvent_t e : h->sweep_ev) cudaEventDestroy(e);
  if (h->sweep_t0) cudaEventDestroy(h->sweep_t0);
  if (h->sweep_t1) cudaEventDestroy(h->sweep_t1);
  for (int k = 0; k < 2; ++k)
    if (h->blk_done[k]) cudaEventDestroy(h->blk_done[k]);
  delete h;
  if (st) cudaStreamDestroy(st);
}

const char *vsvb_gpu_last_error(const vsvb_gpu *h) { return h ? h->err.c_str() : "null handle"; }

int vsvb_gpu_totlen(const vsvb_gpu *h) { return h ? h->totlen : -1; }
int vsvb_gpu_num_orbitals(const vsvb_gpu *h) { return h ? h->nsp : -1; }

int vsvb_gpu_energy_device(vsvb_gpu *h, const double *coeff_dev, vsvb_energy_result *out) {
  if (!h) return VSVB_ERR_INPUT;
  CK(cudaSetDevice(h->dev), "cudaSetDevice");
  CK(cudaMemcpyAsync(h->coeff_d.p, coeff_dev, sizeof(double) * h->totlen, cudaMemcpyDeviceToDevice, h->st), "copy coeff");
  int rc = forward(h);
  if (rc) return rc;
  return finish_result(h, out);
}

int vsvb_gpu_energy(vsvb_gpu *h, const double *coeff, vsvb_energy_result *out) {
  if (!h) return VSVB_ERR_INPUT;
  CK(cudaSetDevice(h->dev), "cudaSetDevice");
  const double *src = coeff ? coeff : h->coeff0.data();
  CK(cudaMemcpyAsync(h->coeff_d.p, src, sizeof(double) * h->totlen, cudaMemcpyHostToDevice, h->st), "copy coeff");
  int rc = forward(h);
  if (rc) return rc;
  return finish_result(h, out);
}

/* forward + adjoint on h->st: eagerly, or as a replay of the captured CUDA
 * graph of the same sequence.  The first call runs eagerly (it allocates the
 * adjoint buffers and sets kernel attributes); the second captures and
 * replays.  A failed capture falls back to eager launches for good. */
static int enqueue_eval(vsvb_gpu *h, bool fused) {
  const bool graph = h->opt.cuda_graph && !h->sweep_timing && h->warm;
  if (graph && !h->gexec) {
    if (cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      int rc = forward(h, fused);
      const int nl = h->launches;
      if (!rc) rc = backward(h, fused);
      h->graph_launches = nl + h->launches;
      cudaGraph_t g = nullptr;
      const cudaError_t e = cudaStreamEndCapture(h->st, &g);
      if (rc == 0 && e == cudaSuccess && g && cudaGraphInstantiate(&h->gexec, g, 0) == cudaSuccess) {
        cudaGraphDestroy(g);
      } else {
        if (g) cudaGraphDestroy(g);
        h->gexec = nullptr;
        h->opt.cuda_graph = 0;
        (void)cudaGetLastError();
        if (rc) return rc;
      }
    } else {
      (void)cudaGetLastError();
      h->opt.cuda_graph = 0;
    }
  }
  if (graph && h->gexec) {
    CK(cudaGraphLaunch(h->gexec, h->st), "graph launch");
    h->launches = h->graph_launches;
    return VSVB_OK;
  }
  int rc = forward(h, fused);
  if (rc) return rc;
  const int nl = h->launches;
  rc = backward(h, fused);
  h->launches += nl;
  if (rc) return rc;
  h->warm = true;
  return VSVB_OK;
}

static int energy_grad_common(vsvb_gpu *h, vsvb_energy_result *out, double *grad, bool grad_on_device) {
  if (h->blk_on) {
    h->err = "the gradient is not available on a block-mode handle";
    return VSVB_ERR_UNSUPPORTED;
  }
  if (h->core_on && h->opt.grad_mode != 0) {
    h->err = "a core-mode handle takes the fused gradient (grad_mode 0) only";
    return VSVB_ERR_UNSUPPORTED;
  }
  const bool fused = h->opt.grad_mode == 0;
  int rc = enqueue_eval(h, fused);
  if (rc) return rc;
  CK(cudaMemcpyAsync(grad, h->coeff_bar.p, sizeof(double) * h->totlen,
                     grad_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h->st),
     "copy grad");
  vsvb_energy_result r;
  rc = finish_result(h, &r); /* copies the result and status, one stream sync */
  if (rc) return rc;
  int status = 0;
  CK(cudaMemcpy(&status, h->status.p, sizeof(int), cudaMemcpyDeviceToHost), "status");
  if (status & 2) {
    h->err = "gradient through a determinant pair whose overlap block stays singular when shifted";
    return VSVB_ERR_SINGULAR;
  }
  if (out) *out = r;
  return VSVB_OK;
}

int vsvb_gpu_energy_grad(vsvb_gpu *h, const double *coeff, vsvb_energy_result *out, double *grad) {
  if (!h || !grad) return VSVB_ERR_INPUT;
  CK(cudaSetDevice(h->dev), "cudaSetDevice");
  const double *src = coeff ? coeff : h->coeff0.data();
  CK(cudaMemcpyAsync(h->coeff_d.p, src, sizeof(double) * h->totlen, cudaMemcpyHostToDevice, h->st), "copy coeff");
  return energy_grad_common(h, out, grad, false);
}

int vsvb_gpu_energy_grad_device(vsvb_gpu *h, const double *coeff_dev, vsvb_energy_result *out, double *grad_dev) {
  if (!h || !grad_dev) return VSVB_ERR_INPUT;
  CK(cudaSetDevice(h->dev), "cudaSetDevice");
  CK(cudaMemcpyAsync(h->coeff_d.p, coeff_dev, sizeof(double) * h->totlen, cudaMemcpyDeviceToDevice, h->st), "copy coeff");
  return energy_grad_common(h, out, grad_dev, true);
}

int vsvb_gpu_batch_energy_grad(vsvb_gpu *const *hs, int n, const double *const *weights, vsvb_energy_result *res,
                               double *const *grads) {
  for (int i = 0; i < n; ++i) {
    int rc = grads ? vsvb_gpu_energy_grad(hs[i], weights ? weights[i] : nullptr, res ? &res[i] : nullptr, grads[i])
                   : vsvb_gpu_energy(hs[i], weights ? weights[i] : nullptr, res ? &res[i] : nullptr);
    if (rc) return rc;
  }
  return VSVB_OK;
}

}  // extern "C"

/* ---------------- batched evaluation as one CUDA graph ---------------- */

struct vsvb_batch {
  std::vector<vsvb_gpu *> hs;
  int dev = 0;
  std::string err;
  cudaStream_t st = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> join;
  cudaGraphExec_t exec = nullptr;
  std::vector<const double *> w; /* pointers the graph was captured with */
  std::vector<double *> g;
  DBuf<double> res; /* [n][5] */
  DBuf<int> stat;   /* [n] */
  int launches = 0;
  /* one ERI sweep for every molecule (all handles per quartet, fused
   * gradient): the molecules' class launches merged per (arithmetic, bra
   * class, ket class, primitive window), each item tagged with its molecule */
  bool merged = false;
  struct Group {
    int kind, a, c, n;
    float lo, hi;
    long long off;
  };
  std::vector<Group> groups;
  DBuf<int4> gwork;
  DBuf<int> gmol;
  DBuf<EriArgs> etab;
  static constexpr int NAUX = 6;
  cudaStream_t aux[NAUX] = {};
  cudaEvent_t sfork = nullptr, sjoin[NAUX] = {};
  std::vector<cudaEvent_t> pre; /* per molecule: its half before the sweep is done */
};

namespace {

int batch_fail(vsvb_batch *b, cudaError_t e, const char *what) {
  b->err = std::string(what) + ": " + cudaGetErrorString(e);
  return VSVB_ERR_CUDA;
}
#define BCK(call, what)                                \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) return batch_fail(b, e_, what); \
  } while (0)

/* the merged evaluation on the batch's streams: per molecule (on its own
 * stream) weights in and the forward half before the sweep; one sweep of
 * merged class launches over every molecule's quartets on the side streams;
 * per molecule the rest of the forward pass, the adjoint and the results */
int batch_enqueue_merged(vsvb_batch *b, const double *const *w, double *const *g, int &launches) {
  const int n = (int)b->hs.size();
  launches = 0;
  BCK(cudaEventRecord(b->fork, b->st), "event record");
  int rc = VSVB_OK;
  for (int i = 0; i < n && !rc; ++i) {
    vsvb_gpu *h = b->hs[i];
    cudaStream_t saved = h->st;
    h->st = h->own_st;
    if (cudaStreamWaitEvent(h->st, b->fork, 0) != cudaSuccess ||
        cudaMemcpyAsync(h->coeff_d.p, w[i], sizeof(double) * h->totlen, cudaMemcpyDeviceToDevice, h->st) != cudaSuccess)
      rc = VSVB_ERR_CUDA;
    if (!rc) rc = forward_pre(h, true);
    launches += h->launches;
    if (!rc && (cudaEventRecord(b->pre[i], h->st) != cudaSuccess ||
                cudaStreamWaitEvent(b->st, b->pre[i], 0) != cudaSuccess))
      rc = VSVB_ERR_CUDA;
    if (rc && h->err.size()) b->err = "molecule " + std::to_string(i) + ": " + h->err;
    h->st = saved;
  }
  if (rc) return rc;
  BCK(cudaEventRecord(b->sfork, b->st), "event record");
  for (int k = 0; k < vsvb_batch::NAUX; ++k) BCK(cudaStreamWaitEvent(b->aux[k], b->sfork, 0), "stream wait");
  EriArgs a0 = eri_args(b->hs[0]);
  for (size_t k = 0; k < b->groups.size(); ++k) {
    const auto &G = b->groups[k];
    a0.prim_lo = G.lo;
    a0.prim_hi = G.hi;
    if (eri_launch_tab(G.kind, G.a, G.c, a0, b->gwork.p + G.off, G.n, b->hs[0]->nsm * 16,
                       b->aux[k % vsvb_batch::NAUX], b->etab.p, b->gmol.p + G.off)) {
      b->err = "merged ERI launch failed";
      return VSVB_ERR_CUDA;
    }
    ++launches;
  }
  for (int k = 0; k < vsvb_batch::NAUX; ++k) {
    BCK(cudaEventRecord(b->sjoin[k], b->aux[k]), "event record");
    BCK(cudaStreamWaitEvent(b->st, b->sjoin[k], 0), "stream wait");
  }
  BCK(cudaEventRecord(b->sfork, b->st), "event record");
  for (int i = 0; i < n && !rc; ++i) {
    vsvb_gpu *h = b->hs[i];
    cudaStream_t saved = h->st;
    h->st = h->own_st;
    if (cudaStreamWaitEvent(h->st, b->sfork, 0) != cudaSuccess) rc = VSVB_ERR_CUDA;
    h->launches = 0;
    if (!rc) rc = forward_post(h, true);
    const int nl = h->launches;
    if (!rc) rc = backward(h, true);
    launches += nl + h->launches;
    if (!rc && (cudaMemcpyAsync(g[i], h->coeff_bar.p, sizeof(double) * h->totlen, cudaMemcpyDeviceToDevice,
                                h->st) != cudaSuccess ||
                cudaMemcpyAsync(b->res.p + 5 * i, h->result.p, sizeof(double) * 5, cudaMemcpyDeviceToDevice,
                                h->st) != cudaSuccess ||
                cudaMemcpyAsync(b->stat.p + i, h->status.p, sizeof(int), cudaMemcpyDeviceToDevice, h->st) != cudaSuccess ||
                cudaEventRecord(b->join[i], h->st) != cudaSuccess ||
                cudaStreamWaitEvent(b->st, b->join[i], 0) != cudaSuccess))
      rc = VSVB_ERR_CUDA;
    if (rc && h->err.size()) b->err = "molecule " + std::to_string(i) + ": " + h->err;
    h->st = saved;
  }
  return rc;
}

/* capture every handle's evaluation (copy weights in, forward + adjoint,
 * copy gradient and result out) as one graph: merged (one sweep for all
 * molecules) when the batch allows it, otherwise each handle on its own
 * stream branch forked from and joined into the batch stream */
int batch_capture(vsvb_batch *b, const double *const *w, double *const *g) {
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  const int n = (int)b->hs.size();
  BCK(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal), "begin capture");
  int rc = VSVB_OK, launches = 0;
  if (b->merged) {
    rc = batch_enqueue_merged(b, w, g, launches);
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(b->st, &graph);
    if (rc || e != cudaSuccess || !graph) {
      if (graph) cudaGraphDestroy(graph);
      (void)cudaGetLastError();
      if (b->err.empty()) b->err = "batch capture failed";
      return rc ? rc : VSVB_ERR_CUDA;
    }
    const cudaError_t ei = cudaGraphInstantiate(&b->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) {
      b->exec = nullptr;
      return batch_fail(b, ei, "graph instantiate");
    }
    b->w.assign(w, w + n);
    b->g.assign(g, g + n);
    b->launches = launches;
    return VSVB_OK;
  }
  BCK(cudaEventRecord(b->fork, b->st), "event record");
  for (int i = 0; i < n && !rc; ++i) {
    vsvb_gpu *h = b->hs[i];
    cudaStream_t saved = h->st;
    h->st = h->own_st;
    const bool fused = h->opt.grad_mode == 0;
    if (cudaStreamWaitEvent(h->st, b->fork, 0) != cudaSuccess ||
        cudaMemcpyAsync(h->coeff_d.p, w[i], sizeof(double) * h->totlen, cudaMemcpyDeviceToDevice, h->st) != cudaSuccess)
      rc = VSVB_ERR_CUDA;
    if (!rc) rc = forward(h, fused);
    const int nl = h->launches;
    if (!rc) rc = backward(h, fused);
    launches += nl + h->launches;
    if (!rc && (cudaMemcpyAsync(g[i], h->coeff_bar.p, sizeof(double) * h->totlen, cudaMemcpyDeviceToDevice,
                                h->st) != cudaSuccess ||
                cudaMemcpyAsync(b->res.p + 5 * i, h->result.p, sizeof(double) * 5, cudaMemcpyDeviceToDevice,
                                h->st) != cudaSuccess ||
                cudaMemcpyAsync(b->stat.p + i, h->status.p, sizeof(int), cudaMemcpyDeviceToDevice, h->st) != cudaSuccess ||
                cudaEventRecord(b->join[i], h->st) != cudaSuccess ||
                cudaStreamWaitEvent(b->st, b->join[i], 0) != cudaSuccess))
      rc = VSVB_ERR_CUDA;
    if (rc && h->err.size()) b->err = "molecule " + std::to_string(i) + ": " + h->err;
    h->st = saved;
  }
  cudaGraph_t graph = nullptr;
  const cudaError_t e = cudaStreamEndCapture(b->st, &graph);
  if (rc || e != cudaSuccess || !graph) {
    if (graph) cudaGraphDestroy(graph);
    (void)cudaGetLastError();
    if (b->err.empty()) b->err = "batch capture failed";
    return rc ? rc : VSVB_ERR_CUDA;
  }
  const cudaError_t ei = cudaGraphInstantiate(&b->exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ei != cudaSuccess) {
    b->exec = nullptr;
    return batch_fail(b, ei, "graph instantiate");
  }
  b->w.assign(w, w + n);
  b->g.assign(g, g + n);
  b->launches = launches;
  return VSVB_OK;
}

}  // namespace

extern "C" {

int vsvb_batch_create(vsvb_gpu *const *handles, int n, vsvb_batch **out) {
  if (!handles || n < 1 || !out) return VSVB_ERR_INPUT;
  *out = nullptr;
  auto *b = new vsvb_batch();
  b->dev = handles[0]->dev;
  for (int i = 0; i < n; ++i) {
    vsvb_gpu *h = handles[i];
    if (!h || h->dev != b->dev) {
      delete b;
      return VSVB_ERR_INPUT;
    }
    b->hs.push_back(h);
  }
  *out = b;
  BCK(cudaSetDevice(b->dev), "cudaSetDevice");
  BCK(cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking), "cudaStreamCreate");
  BCK(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming), "cudaEventCreate");
  b->join.assign(n, nullptr);
  for (int i = 0; i < n; ++i) BCK(cudaEventCreateWithFlags(&b->join[i], cudaEventDisableTiming), "cudaEventCreate");
  BCK(b->res.alloc((size_t)5 * n), "alloc results");
  BCK(b->stat.alloc((size_t)n), "alloc status");
  /* one eager evaluation per handle: allocates its adjoint buffers and sets
   * kernel attributes, neither of which may happen inside a capture */
  std::vector<double> grad;
  for (vsvb_gpu *h : b->hs) {
    if (h->warm) continue;
    grad.assign(h->totlen, 0.0);
    int rc = vsvb_gpu_energy_grad(h, nullptr, nullptr, grad.data());
    if (rc) {
      b->err = "warm-up: " + h->err;
      return rc;
    }
  }
  /* merged sweep: every handle on the per-quartet path with the fused
   * gradient (one ERI sweep per evaluation) */
  b->merged = true;
  for (vsvb_gpu *h : b->hs) b->merged = b->merged && !h->blk_on && h->opt.grad_mode == 0;
  if (b->merged) {
    std::map<std::tuple<int, int, int, float, float>, std::vector<std::pair<int, int>>> key;
    for (int i = 0; i < n; ++i)
      for (const auto &it : b->hs[i]->sweep) key[std::make_tuple(it.kind, it.a, it.c, it.lo, it.hi)].push_back({i, it.wl});
    std::vector<int4> work;
    std::vector<int> mol;
    for (const auto &kv : key) {
      vsvb_batch::Group G{};
      G.kind = std::get<0>(kv.first);
      G.a = std::get<1>(kv.first);
      G.c = std::get<2>(kv.first);
      G.lo = std::get<3>(kv.first);
      G.hi = std::get<4>(kv.first);
      G.off = (long long)work.size();
      for (const auto &m : kv.second) {
        const auto &lst = b->hs[m.first]->item_wh[m.second];
        work.insert(work.end(), lst.begin(), lst.end());
        mol.insert(mol.end(), lst.size(), m.first);
      }
      G.n = (int)(work.size() - G.off);
      if (G.n > 0) b->groups.push_back(G);
    }
    /* most work first over the side streams */
    std::stable_sort(b->groups.begin(), b->groups.end(),
                     [](const vsvb_batch::Group &x, const vsvb_batch::Group &y) { return x.n > y.n; });
    std::vector<EriArgs> tab;
    for (vsvb_gpu *h : b->hs) tab.push_back(eri_args(h));
    BCK(b->gwork.upload(work.empty() ? std::vector<int4>(1, make_int4(0, 0, 0, 0)) : work), "upload merged work");
    BCK(b->gmol.upload(mol.empty() ? std::vector<int>(1, 0) : mol), "upload merged work");
    BCK(b->etab.upload(tab), "upload argument table");
    for (int k = 0; k < vsvb_batch::NAUX; ++k) {
      BCK(cudaStreamCreateWithFlags(&b->aux[k], cudaStreamNonBlocking), "cudaStreamCreate");
      BCK(cudaEventCreateWithFlags(&b->sjoin[k], cudaEventDisableTiming), "cudaEventCreate");
    }
    BCK(cudaEventCreateWithFlags(&b->sfork, cudaEventDisableTiming), "cudaEventCreate");
    b->pre.assign(n, nullptr);
    for (int i = 0; i < n; ++i) BCK(cudaEventCreateWithFlags(&b->pre[i], cudaEventDisableTiming), "cudaEventCreate");
    /* one eager merged evaluation: sets the merged kernels' attributes
     * outside any capture */
    std::vector<DBuf<double>> wd(n), gd(n);
    std::vector<const double *> wp(n);
    std::vector<double *> gp(n);
    for (int i = 0; i < n; ++i) {
      BCK(wd[i].upload(b->hs[i]->coeff0), "upload weights");
      BCK(gd[i].alloc(b->hs[i]->totlen), "alloc gradient");
      wp[i] = wd[i].p;
      gp[i] = gd[i].p;
    }
    int launches = 0;
    int rc = batch_enqueue_merged(b, wp.data(), gp.data(), launches);
    if (rc) return rc;
    BCK(cudaStreamSynchronize(b->st), "merged warm-up");
  }
  return VSVB_OK;
}

int vsvb_batch_energy_grad(vsvb_batch *b, const double *const *weights_dev, double *const *grads_dev,
                           vsvb_energy_result *results, void *stream) {
  if (!b || !weights_dev || !grads_dev) return VSVB_ERR_INPUT;
  const int n = (int)b->hs.size();
  BCK(cudaSetDevice(b->dev), "cudaSetDevice");
  bool same = b->exec && (int)b->w.size() == n;
  for (int i = 0; same && i < n; ++i) same = b->w[i] == weights_dev[i] && b->g[i] == grads_dev[i];
  if (!same) {
    int rc = batch_capture(b, weights_dev, grads_dev);
    if (rc) return rc;
  }
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : b->st;
  BCK(cudaGraphLaunch(b->exec, st), "graph launch");
  std::vector<double> r((size_t)5 * n);
  std::vector<int> stat(n);
  BCK(cudaMemcpyAsync(r.data(), b->res.p, sizeof(double) * r.size(), cudaMemcpyDeviceToHost, st), "copy results");
  BCK(cudaMemcpyAsync(stat.data(), b->stat.p, sizeof(int) * n, cudaMemcpyDeviceToHost, st), "copy status");
  BCK(cudaStreamSynchronize(st), "sync");
  for (int i = 0; i < n; ++i) {
    if (stat[i] & 1) {
      b->err = "molecule " + std::to_string(i) + ": an orbital has non-positive self-overlap";
      return VSVB_ERR_NOT_NORMALISABLE;
    }
    if (stat[i] & 4) {
      b->err = "molecule " + std::to_string(i) + ": more singular determinant pairs than the exact-minor pool holds";
      return VSVB_ERR_UNSUPPORTED;
    }
    if (stat[i] & 2) {
      b->err = "molecule " + std::to_string(i) + ": gradient through a determinant pair whose overlap block stays singular when shifted";
      return VSVB_ERR_SINGULAR;
    }
    if (results) {
      fill_result(b->hs[i], r.data() + 5 * i, &results[i]);
      results[i].n_kernel_launches = b->launches;
    }
  }
  return VSVB_OK;
}

int vsvb_batch_launches(const vsvb_batch *b) { return b ? b->launches : -1; }

const char *vsvb_batch_last_error(const vsvb_batch *b) { return b ? b->err.c_str() : "null batch"; }

void vsvb_batch_destroy(vsvb_batch *b) {
  if (!b) return;
  cudaSetDevice(b->dev);
  if (b->st) cudaStreamSynchronize(b->st);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  for (cudaEvent_t e : b->join)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : b->pre)
    if (e) cudaEventDestroy(e);
  for (int k = 0; k < vsvb_batch::NAUX; ++k) {
    if (b->aux[k]) cudaStreamDestroy(b->aux[k]);
    if (b->sjoin[k]) cudaEventDestroy(b->sjoin[k]);
  }
  if (b->sfork) cudaEventDestroy(b->sfork);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->st) cudaStreamDestroy(b->st);
  delete b;
}

int vsvb_gpu_set_stream(vsvb_gpu *h, void *stream) {
  if (!h) return VSVB_ERR_INPUT;
  h->st = stream ? static_cast<cudaStream_t>(stream) : h->own_st;
  return VSVB_OK;
}

int vsvb_gpu_set_spin_coeffs(vsvb_gpu *h, const double *coeff_sc) { return gpu_set_spin_coeffs(h, coeff_sc); }

int vsvb_gpu_eri_profile_mode(vsvb_gpu *h, int mode, double *ms, double *flops, int *cls, int cap) {
  if (!h || (mode != 0 && mode != 3)) return -VSVB_ERR_INPUT;
  if (mode == 3 && !h->grad_ready) return -VSVB_ERR_INPUT;
  if (cudaSetDevice(h->dev) != cudaSuccess) return -VSVB_ERR_CUDA;
  EriArgs ea = eri_args(h);
  if (cudaMemsetAsync(h->T.p, 0, sizeof(double) * h->T.n, h->st) != cudaSuccess) return -VSVB_ERR_CUDA;
  if (mode == 3 && cudaMemsetAsync(h->xbarh.p, 0, sizeof(double) * h->xbarh.n, h->st) != cudaSuccess)
    return -VSVB_ERR_CUDA;
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return -VSVB_ERR_CUDA;
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return -VSVB_ERR_CUDA;
  }
  int k = 0, rc = 0;
  for (const auto &it : h->sweep) {
    if (k >= cap) break;
    ea.prim_lo = it.lo;
    ea.prim_hi = it.hi;
    cudaEventRecord(e0, h->st);
    if (eri_launch(mode, it.kind, it.a, it.c, ea, h->item_wd[it.wl].p, (int)h->item_wh[it.wl].size(),
                   h->nsm * it.bps, h->st)) {
      rc = -VSVB_ERR_CUDA;
      break;
    }
    cudaEventRecord(e1, h->st);
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      rc = -VSVB_ERR_CUDA;
      break;
    }
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    ms[k] = t;
    flops[k] = mode == 0 ? it.flops_fwd : it.flops_grad;
    cls[k] = it.code;
    ++k;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc ? rc : k;
}

int vsvb_gpu_eri_profile(vsvb_gpu *h, double *ms, double *flops, int *cls, int cap) {
  return vsvb_gpu_eri_profile_mode(h, 0, ms, flops, cls, cap);
}

int vsvb_gpu_set_sweep_timing(vsvb_gpu *h, int on) {
  if (!h) return VSVB_ERR_INPUT;
  h->sweep_timing = on != 0;
  return VSVB_OK;
}

int vsvb_gpu_sweep_times(vsvb_gpu *h, double *ms, double *flops, int *cls, int cap) {
  if (!h) return -VSVB_ERR_INPUT;
  if (!h->sweep_timing || h->sweep_mode < 0) return 0;
  if (cudaSetDevice(h->dev) != cudaSuccess) return -VSVB_ERR_CUDA;
  std::vector<ShellPair> pairs(h->pairs.n);
  if (!pairs.empty() &&
      cudaMemcpy(pairs.data(), h->pairs.p, sizeof(ShellPair) * pairs.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
    return -VSVB_ERR_CUDA;
  int k = 0;
  for (size_t i = 0; i < h->sweep.size() && k < cap; ++i, ++k) {
    const auto &it = h->sweep[i];
    if (cudaEventSynchronize(h->sweep_ev[2 * i + 1]) != cudaSuccess) return -VSVB_ERR_CUDA;
    float t = 0.f;
    if (cudaEventElapsedTime(&t, h->sweep_ev[2 * i], h->sweep_ev[2 * i + 1]) != cudaSuccess) return -VSVB_ERR_CUDA;
    ms[k] = t;
    flops[k] = h->sweep_mode == 0 ? it.flops_fwd : it.flops_grad;
    cls[k] = it.code;
  }
  return k;
}

int vsvb_gpu_launch_config(const vsvb_gpu *h, int *nsplit, int *codes, int *blocks_per_sm, int cap) {
  if (!h) return -VSVB_ERR_INPUT;
  if (nsplit) *nsplit = h->nsplit;
  int k = 0;
  for (const auto &it : h->sweep) {
    if (k >= cap) break;
    if (codes) codes[k] = it.code;
    if (blocks_per_sm) blocks_per_sm[k] = it.bps;
    ++k;
  }
  return k;
}

int vsvb_gpu_sweep_wall_ms(vsvb_gpu *h, double *ms) {
  if (!h || !ms) return VSVB_ERR_INPUT;
  *ms = 0.0;
  if (!h->sweep_timing || h->sweep_mode < 0 || !h->sweep_t1) return VSVB_OK;
  CK(cudaSetDevice(h->dev), "cudaSetDevice");
  CK(cudaEventSynchronize(h->sweep_t1), "event sync");
  float t = 0.f;
  CK(cudaEventElapsedTime(&t, h->sweep_t0, h->sweep_t1), "event time");
  *ms = t;
  return VSVB_OK;
}

int vsvb_gpu_debug_orbital_eri(vsvb_gpu *h, double *out, size_t cap) {
  if (!h) return -VSVB_ERR_INPUT;
  size_t n = (size_t)h->np * h->np;
  if (cap < n) return -VSVB_ERR_INPUT;
  if (cudaMemcpy(out, h->T.p, sizeof(double) * n, cudaMemcpyDeviceToHost) != cudaSuccess) return -VSVB_ERR_CUDA;
  return h->np;
}

int vsvb_gpu_debug_orbital_eri_at(vsvb_gpu *h, const long long *idx, int n, double *out) {
  if (!h || (n > 0 && (!idx || !out))) return VSVB_ERR_INPUT;
  CK(cudaSetDevice(h->dev), "cudaSetDevice");
  CK(cudaStreamSynchronize(h->st), "sync");
  const long long nt = (long long)h->np * h->np;
  for (int i = 0; i < n; ++i) {
    if (idx[i] < 0 || idx[i] >= nt) {
      h->err = "orbital-pair ERI index out of range";
      return VSVB_ERR_INPUT;
    }
    CK(cudaMemcpy(out + i, h->T.p + idx[i], sizeof(double), cudaMemcpyDeviceToHost), "copy T entry");
  }
  return h->np;
}

int vsvb_gpu_block_stats(const vsvb_gpu *h, double *eri_flops3, double *transform_flops2, long long *counts3) {
  if (!h) return -VSVB_ERR_INPUT;
  if (eri_flops3)
    for (int k = 0; k < 3; ++k) eri_flops3[k] = h->blk_eri_flops[k];
  if (transform_flops2)
    for (int k = 0; k < 3; ++k) transform_flops2[k] = h->blk_tr_flops[k];
  if (counts3) {
    counts3[0] = h->blk_naq;
    counts3[1] = (long long)h->blk_chunk.size();
    counts3[2] = (long long)h->blk_launch.size() + (long long)h->blk_chunk.size();
  }
  return h->blk_on ? 1 : 0;
}

int vsvb_gpu_core_stats(const vsvb_gpu *h, double *gemm_fma, long long *counts2) {
  if (!h) return -VSVB_ERR_INPUT;
  if (!h->core_on) return 0;
  vsvb_gpu *hh = const_cast<vsvb_gpu *>(h);
  const CoreArgs c = core_args(hh);
  if (gemm_fma) *gemm_fma = core_gemm_fma(c);
  if (counts2) {
    counts2[0] = c.nq;
    counts2[1] = (long long)c.nC;
  }
  return 1;
}

int vsvb_gpu_debug_orbital_1e(vsvb_gpu *h, double *s, double *hc, size_t cap) {
  if (!h) return -VSVB_ERR_INPUT;
  size_t n = (size_t)h->nsp * h->nsp;
  if (cap < n) return -VSVB_ERR_INPUT;
  if (cudaMemcpy(s, h->So.p, sizeof(double) * n, cudaMemcpyDeviceToHost) != cudaSuccess) return -VSVB_ERR_CUDA;
  if (cudaMemcpy(hc, h->Ho.p, sizeof(double) * n, cudaMemcpyDeviceToHost) != cudaSuccess) return -VSVB_ERR_CUDA;
  return h->nsp;
}

}  /* extern "C" */

/* ---- first_order_opt / spin_opt support (handle_internal.h) ---- */

int vsvb_gpu_create_sub(const vsvb_system_desc *d, const vsvb_options *opt, int split, int sub, vsvb_gpu **out) {
  if (!d || !out) return VSVB_ERR_INPUT;
  *out = nullptr;
  auto *h = new vsvb_gpu();
  vsvb_default_options(&h->opt);
  if (opt) h->opt = *opt;
  h->opt.autotune = 0;
  h->opt.cuda_graph = 0;
  h->dev = h->opt.device;
  h->hs_split = split;
  h->hs_sub = sub;
  int rc = build(h, d);
  *out = h;
  return rc;
}

int gpu_hs_columns(vsvb_gpu *h, const double *w_dev, const int *src_dev, int j0, int nb, double *H_dev, double *S_dev) {
  if (!h || h->hs_sub < 0) return VSVB_ERR_INPUT;
  CK(cudaSetDevice(h->dev), "cudaSetDevice");
  cudaStream_t st = h->st;
  if (!h->hs_flag.p) CK(h->hs_flag.alloc(1), "alloc flag");
  CK(cudaMemsetAsync(h->hs_flag.p, 0, sizeof(int), st), "memset flag");
  const unsigned nq = (unsigned)h->ds.nq;
  for (int nu = 0; nu < nb; ++nu) {
    hs_weights_kernel<<<(h->totlen + 255) / 256, 256, 0, st>>>(h->coeff_d.p, w_dev, src_dev, h->totlen, j0, nu);
    CK(cudaGetLastError(), "hs weights");
    int rc = forward(h, true);
    if (rc) return rc;
    DetCtx dc = det_ctx(h);
    AsmArgs aa = asm_args(h);
    OrbArgs oa = orb_args(h);
    /* pass 0: d(E_num)/dw, pass 1: d(W)/dw, from the same forward walk */
    for (int pass = 0; pass < 2; ++pass) {
      CK(cudaMemsetAsync(h->Cbar.p, 0, sizeof(double) * h->Cbar.n, st), "memset Cbar");
      const double alpha = pass == 0 ? 1.0 : 0.0, beta = pass == 0 ? 0.0 : 1.0 / (double)h->ds.nelec;
      hs_scale_kernel<<<nq, 128, 0, st>>>(dc, aa, h->nsplit, alpha, beta);
      CK(cudaGetLastError(), "hs scale");
      detpair_adjoint_kernel<<<nq, 128, 0, st>>>(dc, aa, h->nsplit);
      CK(cudaGetLastError(), "detpair adjoint");
      if (pass == 0 && h->nxelem > 0) {
        XtabArgs xa = xtab_args(h); /* unscaled densities in the sweep: factor 1 */
        xhrr_adjoint_kernel<<<(unsigned)((h->nxelem + 255) / 256), 256, 0, st>>>(xa, h->xbarh.p, h->xbar.p);
        CK(cudaGetLastError(), "xhrr adjoint");
        xtab_adjoint_kernel<<<(unsigned)((h->nxelem + 255) / 256), 256, 0, st>>>(xa, h->xbar.p, h->Cbar.p);
        CK(cudaGetLastError(), "xtab adjoint");
      }
      orb_1e_adjoint_kernel<<<h->nsp, 128, 0, st>>>(oa, h->Sbar.p, h->Hbar.p, h->nsp, h->Cbar.p);
      CK(cudaGetLastError(), "orb_1e adjoint");
      entry_adjoint_kernel<<<1, 32, 0, st>>>(oa, h->hs_sub, j0, nb, h->Cbar.p,
                                             (pass == 0 ? H_dev : S_dev) + (size_t)nu * nb, 0.5, h->hs_flag.p);
      CK(cudaGetLastError(), "entry adjoint");
    }
  }
  int flag = 0;
  CK(cudaMemcpyAsync(&flag, h->hs_flag.p, sizeof(int), cudaMemcpyDeviceToHost, st), "copy flag");
  CK(cudaStreamSynchronize(st), "sync");
  if (flag & 1) {
    h->err = "an orbital has non-positive self-overlap";
    return VSVB_ERR_NOT_NORMALISABLE;
  }
  if (flag & 4) {
    h->err = "more singular determinant pairs than the exact-minor pool holds";
    return VSVB_ERR_UNSUPPORTED;
  }
  if (flag & 2) {
    h->err = "first_order_opt matrices through a determinant pair whose overlap block stays singular when shifted";
    return VSVB_ERR_SINGULAR;
  }
  return VSVB_OK;
}

int gpu_set_spin_coeffs(vsvb_gpu *h, const double *csc) {
  if (!h || !csc) return VSVB_ERR_INPUT;
  CK(cudaSetDevice(h->dev), "cudaSetDevice");
  h->csc_h.assign(csc, csc + h->ds.nsc);
  CK(cudaMemcpyAsync(h->coeff_sc.p, h->csc_h.data(), sizeof(double) * h->ds.nsc, cudaMemcpyHostToDevice, h->st),
     "copy coeff_sc");
  CK(cudaStreamSynchronize(h->st), "sync");
  return VSVB_OK;
}

int gpu_spin_blocks(vsvb_gpu *h, const double *w_dev, double *BH_dev, double *BS_dev) {
  if (!h) return VSVB_ERR_INPUT;
  CK(cudaSetDevice(h->dev), "cudaSetDevice");
  cudaStream_t st = h->st;
  const std::vector<double> keep = h->csc_h, ones(h->ds.nsc, 1.0);
  CK(cudaMemcpyAsync(h->coeff_sc.p, ones.data(), sizeof(double) * h->ds.nsc, cudaMemcpyHostToDevice, st), "copy");
  CK(cudaMemcpyAsync(h->coeff_d.p, w_dev, sizeof(double) * h->totlen, cudaMemcpyDeviceToDevice, st), "copy coeff");
  int rc = forward(h, false);
  if (rc) return rc;
  AsmArgs aa = asm_args(h);
  spin_block_kernel<<<h->ds.nsc * h->ds.nsc, 256, 0, st>>>(det_ctx(h), aa, h->nsplit, BH_dev, BS_dev);
  CK(cudaGetLastError(), "spin blocks");
  CK(cudaMemcpyAsync(h->coeff_sc.p, keep.data(), sizeof(double) * h->ds.nsc, cudaMemcpyHostToDevice, st), "copy");
  return finish_result(h, nullptr);
}

cudaStream_t gpu_stream(vsvb_gpu *h) { return h ? h->st : nullptr; }
int gpu_nsc(const vsvb_gpu *h) { return h ? h->ds.nsc : 0; }

int gpu_orbital_scales(vsvb_gpu *h, const double *w, double *ndf_scale, double *orb_scale) {
  if (!h || !w) return VSVB_ERR_INPUT;
  CK(cudaSetDevice(h->dev), "cudaSetDevice");
  cudaStream_t st = h->st;
  CK(cudaMemcpyAsync(h->coeff_d.p, w, sizeof(double) * h->totlen, cudaMemcpyHostToDevice, st), "copy coeff");
  CK(cudaMemsetAsync(h->status.p, 0, sizeof(int), st), "memset status");
  OrbArgs oa = orb_args(h);
  const size_t osh = sizeof(double) * std::max(h->maxobs, 1);
  if (h->ndf > 0) ndf_norm_kernel<<<h->ndf, 128, osh, st>>>(oa);
  orb_norm_kernel<<<h->nsp, 128, osh, st>>>(oa);
  CK(cudaGetLastError(), "orb_norm");
  if (ndf_scale && h->ndf > 0)
    CK(cudaMemcpyAsync(ndf_scale, h->ndf_scale.p, sizeof(double) * h->ndf, cudaMemcpyDeviceToHost, st), "copy");
  if (orb_scale) CK(cudaMemcpyAsync(orb_scale, h->orb_scale.p, sizeof(double) * h->nsp, cudaMemcpyDeviceToHost, st), "copy");
  return finish_result(h, nullptr);
}
