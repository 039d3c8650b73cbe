/*
 * input.cpp -- reader for VALENCE input files into a vsvb_system_desc.
 *
 * Follows xm_getdims / xm_input (xm_module.F90:25-335) and the checks of
 * read_allocate_input (valence_initialize_module.F90:33-120): Fortran
 * list-directed reads, where each READ starts on a new line, may continue
 * over following lines and discards the rest of its last line.  Errors are
 * returned as VSVB_ERR_INPUT with a message (the reference stops through
 * xm_abort instead).
 */
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/vsvb_gpu.h"

namespace {

struct Owned {
  vsvb_system_desc d;
  std::vector<int> atom_t, map_atom2shell, num_shell_atom, map_shell2prim, ang_mom, pair_sc, orbas_atnum,
      orbas_atset, map_orbs, xpset, orbset, xorb, root;
  std::vector<double> coords, nuc_charge, exponent, con_coeff, coeff_sc, coeff;
};

class Records {
 public:
  explicit Records(std::string text) : s_(std::move(text)) {}
  void begin() { cur_ = pos_; }
  void end() {
    size_t c = cur_;
    while (c < s_.size() && s_[c] != '\n') ++c;
    if (c < s_.size()) ++c;
    pos_ = c;
  }
  bool tok(std::string &t) {
    auto sep = [](char ch) { return ch == ' ' || ch == '\t' || ch == ',' || ch == '\r' || ch == '\n'; };
    size_t c = cur_;
    while (c < s_.size() && sep(s_[c])) ++c;
    if (c >= s_.size()) {
      bad_ = true;
      cur_ = c;
      return false;
    }
    size_t b = c;
    while (c < s_.size() && !sep(s_[c])) ++c;
    t.assign(s_, b, c - b);
    cur_ = c;
    return true;
  }
  int i() {
    std::string t;
    if (!tok(t)) return 0;
    char *e = nullptr;
    long v = std::strtol(t.c_str(), &e, 10);
    if (*e) bad_ = true;
    return static_cast<int>(v);
  }
  double f() {
    std::string t;
    if (!tok(t)) return 0.0;
    for (auto &ch : t)
      if (ch == 'd' || ch == 'D') ch = 'e';
    char *e = nullptr;
    double v = std::strtod(t.c_str(), &e);
    if (*e) bad_ = true;
    return v;
  }
  bool bad() const { return bad_; }

 private:
  std::string s_;
  size_t pos_ = 0, cur_ = 0;
  bool bad_ = false;
};

int fail(char *err, int errlen, const char *msg) {
  if (err && errlen > 0) std::snprintf(err, errlen, "%s", msg);
  return VSVB_ERR_INPUT;
}

}  // namespace

extern "C" int vsvb_read_input(const char *path, vsvb_system_desc **out, char *err, int errlen) {
  if (!out) return VSVB_ERR_INPUT;
  *out = nullptr;
  FILE *fp = std::fopen(path, "rb");
  if (!fp) return fail(err, errlen, "problems opening input file");
  std::string text;
  char buf[65536];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof buf, fp)) > 0) text.append(buf, n);
  std::fclose(fp);
  Records r(text);
  auto *o = new Owned();
  vsvb_system_desc &d = o->d;
  std::memset(&d, 0, sizeof d);
  r.begin();
  d.natom = r.i();
  d.natom_t = r.i();
  d.npair = r.i();
  d.nunpd = r.i();
  d.ndocc = r.i();
  d.totlen = r.i();
  d.xpmax = r.i();
  d.nspinc = r.i();
  d.num_sh = r.i();
  d.num_pr = r.i();
  d.nang = r.i();
  d.ndf = r.i();
  int nset = r.i();
  d.nxorb = r.i();
  d.mxctr = r.i();
  r.end();
  if (r.bad() || d.natom < 1 || d.natom_t < 1 || d.num_sh < 0 || d.num_pr < 0 || d.totlen < 1 || d.mxctr < 1 ||
      nset < 0 || d.npair < 0 || d.nunpd < 0 || d.ndocc < 0 || d.ndf < 0) {
    delete o;
    return fail(err, errlen, "bad dimension line");
  }
  if (d.npair > 0 && d.nspinc < 1) {
    delete o;
    return fail(err, errlen, "no spin couplings;");
  }
  int norbs = 2 * d.npair + d.nunpd + d.ndocc + d.ndf;
  r.begin();
  int ntol_c = r.i();
  (void)ntol_c;
  d.ntol_d = r.i();
  d.ntol_i = r.i();
  d.ntol_e_min = r.i();
  d.ntol_e_max = r.i();
  d.max_iter = r.i();
  d.ptbnmax = r.f();
  d.feather = r.f();
  d.nset = nset;
  o->orbset.assign(2 * (size_t)nset + 1, 0);
  for (int k = 0; k < 2 * nset; ++k) o->orbset[k] = r.i();
  r.end();
  o->atom_t.resize(d.natom);
  o->coords.resize(3 * (size_t)d.natom);
  for (int a = 0; a < d.natom; ++a) {
    r.begin();
    o->atom_t[a] = r.i();
    for (int k = 0; k < 3; ++k) o->coords[3 * a + k] = r.f() * 1.889725987722;
    r.end();
    if (o->atom_t[a] < 1 || o->atom_t[a] > d.natom_t) {
      delete o;
      return fail(err, errlen, "atom with a bad type");
    }
  }
  o->nuc_charge.resize(d.natom_t);
  o->map_atom2shell.resize(d.natom_t);
  o->num_shell_atom.resize(d.natom_t);
  o->map_shell2prim.assign((size_t)d.num_sh + 1, 0);
  o->ang_mom.assign(d.num_sh, 0);
  o->exponent.assign(d.num_pr, 0.0);
  o->con_coeff.assign(d.num_pr, 0.0);
  int ns = 1, np = 1;
  for (int t = 0; t < d.natom_t; ++t) {
    o->map_atom2shell[t] = ns;
    r.begin();
    o->nuc_charge[t] = r.f();
    int nshell = r.i();
    r.end();
    o->num_shell_atom[t] = nshell;
    for (int s = 0; s < nshell; ++s) {
      if (ns > d.num_sh) {
        delete o;
        return fail(err, errlen, "more shells than declared");
      }
      o->map_shell2prim[ns - 1] = np;
      r.begin();
      o->ang_mom[ns - 1] = r.i();
      int nc = r.i();
      r.end();
      if (nc < 1 || np - 1 + nc > d.num_pr) {
        delete o;
        return fail(err, errlen, "more primitives than declared");
      }
      if (nc == 1) {
        r.begin();
        o->exponent[np - 1] = r.f();
        r.end();
        o->con_coeff[np - 1] = 1.0;
        ++np;
      } else {
        for (int k = 0; k < nc; ++k) {
          r.begin();
          o->exponent[np - 1] = r.f();
          o->con_coeff[np - 1] = r.f();
          r.end();
          ++np;
        }
      }
      ++ns;
    }
  }
  /* the reference reads only what the shells need; declared counts may be
   * larger (its arrays are allocated from them) */
  o->map_shell2prim[ns - 1] = np;
  d.num_sh = ns - 1;
  d.num_pr = np - 1;
  int nsc = d.nspinc > 0 ? d.nspinc : 1;
  o->pair_sc.assign((size_t)2 * d.npair * nsc, 0);
  o->coeff_sc.assign(nsc, 1.0);
  if (d.npair > 0) {
    r.begin();
    if (d.nspinc == 1) {
      for (int k = 0; k < d.npair; ++k) {
        o->pair_sc[k] = r.i();
        o->pair_sc[k + d.npair] = r.i();
      }
    } else {
      for (int j = 0; j < d.nspinc; ++j) {
        o->coeff_sc[j] = r.f();
        for (int k = 0; k < d.npair; ++k) {
          o->pair_sc[k + d.npair * (0 + 2 * j)] = r.i();
          o->pair_sc[k + d.npair * (1 + 2 * j)] = r.i();
        }
      }
    }
    r.end();
  }
  o->xorb.assign((size_t)d.nxorb + 1, 0);
  o->root.assign((size_t)d.nxorb + 1, 0);
  if (d.nxorb > 0) {
    r.begin();
    for (int k = 0; k < d.nxorb; ++k) {
      o->xorb[k] = r.i();
      o->root[k] = r.i();
    }
    r.end();
  }
  o->orbas_atnum.assign(norbs, 0);
  o->orbas_atset.assign((size_t)d.mxctr * norbs, 0);
  o->map_orbs.assign((size_t)norbs + 1, 0);
  o->xpset.assign(d.totlen, 0);
  o->coeff.assign(d.totlen, 0.0);
  int j = 1;
  for (int i = 0; i < norbs; ++i) {
    r.begin();
    o->orbas_atnum[i] = r.i();
    if (o->orbas_atnum[i] < 1 || o->orbas_atnum[i] > d.mxctr) {
      delete o;
      return fail(err, errlen, "orbital with a bad atom count");
    }
    for (int k = 0; k < o->orbas_atnum[i]; ++k) {
      int a = r.i();
      if (a < 1 || a > d.natom) {
        delete o;
        return fail(err, errlen, "orbital on a non-existent atom");
      }
      o->orbas_atset[k + (size_t)d.mxctr * i] = a;
    }
    int nexp = r.i();
    r.end();
    if (nexp < 0 || j - 1 + nexp > d.totlen) {
      delete o;
      return fail(err, errlen, "orbital weight list longer than totlen");
    }
    o->map_orbs[i] = j;
    r.begin();
    for (int k = j; k < j + nexp; ++k) {
      o->xpset[k - 1] = r.i();
      o->coeff[k - 1] = r.f();
    }
    r.end();
    j += nexp;
  }
  o->map_orbs[norbs] = j;
  if (r.bad()) {
    delete o;
    return fail(err, errlen, "premature end of input");
  }
  d.atom_t = o->atom_t.data();
  d.coords = o->coords.data();
  d.nuc_charge = o->nuc_charge.data();
  d.map_atom2shell = o->map_atom2shell.data();
  d.num_shell_atom = o->num_shell_atom.data();
  d.map_shell2prim = o->map_shell2prim.data();
  d.ang_mom = o->ang_mom.data();
  d.exponent = o->exponent.data();
  d.con_coeff = o->con_coeff.data();
  d.pair_sc = o->pair_sc.data();
  d.coeff_sc = o->coeff_sc.data();
  d.orbas_atnum = o->orbas_atnum.data();
  d.orbas_atset = o->orbas_atset.data();
  d.map_orbs = o->map_orbs.data();
  d.xpset = o->xpset.data();
  d.coeff = o->coeff.data();
  d.orbset = o->orbset.data();
  d.xorb = o->xorb.data();
  d.root = o->root.data();
  *out = &o->d;
  return VSVB_OK;
}

extern "C" void vsvb_free_desc(vsvb_system_desc *d) {
  if (!d) return;
  /* d is the first member of Owned */
  delete reinterpret_cast<Owned *>(d);
}

/* ---- the orbitals file (xm_output, xm_module.F90:464-577) ---------------- */

namespace {

/* Fortran Iw: right-justified, '*' fill when it does not fit */
void fort_i(std::string &o, long v, int w) {
  char b[64];
  const int n = std::snprintf(b, sizeof b, "%ld", v);
  if (n > w) o.append(w, '*');
  else o.append(w - n, ' ').append(b);
}

/* Fortran Fw.d */
void fort_f(std::string &o, double v, int w, int d) {
  char b[128];
  const int n = std::snprintf(b, sizeof b, "%*.*f", w, d, v);
  if (n > w) o.append(w, '*');
  else o.append(b);
}

/* Fortran Ew.d: [-]0.ddE+ee right-justified */
void fort_e(std::string &o, double v, int w, int d) {
  char b[128];
  if (v == 0.0) {
    std::snprintf(b, sizeof b, "0.%0*dE+00", d, 0);
  } else {
    int e = (int)std::floor(std::log10(std::fabs(v))) + 1;
    double m = std::fabs(v) / std::pow(10.0, e);
    /* rounding may carry the mantissa to 1.0 */
    const double scale = std::pow(10.0, d);
    double mr = std::round(m * scale) / scale;
    if (mr >= 1.0) {
      mr /= 10.0;
      ++e;
    }
    std::snprintf(b, sizeof b, "%s0.%0*ldE%c%02d", v < 0 ? "-" : "", d, (long)std::llround(mr * scale),
                  e < 0 ? '-' : '+', e < 0 ? -e : e);
  }
  const int n = (int)std::strlen(b);
  if (n > w) o.append(w, '*');
  else o.append(w - n, ' ').append(b);
}

/* one orbital: format(5x,1i2,5x,10i4) for the atom list and length, then
 * format(4(1i4,1x,1f13.8)) for its (xpset, coeff) pairs; both with Fortran
 * format reversion (a new record per exhausted format) */
void orbital_block(std::string &o, const vsvb_system_desc *d, const double *coeff, int i) {
  const int natl = d->orbas_atnum[i];
  std::vector<long> items;
  items.push_back(natl);
  for (int j = 0; j < natl; ++j) items.push_back(d->orbas_atset[(size_t)i * d->mxctr + j]);
  const int b = d->map_orbs[i] - 1, e = d->map_orbs[i + 1] - 1;
  items.push_back(e - b);
  size_t k = 0;
  while (k < items.size()) {
    o.append(5, ' ');
    fort_i(o, items[k++], 2);
    o.append(5, ' ');
    for (int f = 0; f < 10 && k < items.size(); ++f) fort_i(o, items[k++], 4);
    o.push_back('\n');
  }
  for (int j = b; j < e;) {
    for (int f = 0; f < 4 && j < e; ++f, ++j) {
      fort_i(o, d->xpset[j], 4);
      o.push_back(' ');
      fort_f(o, coeff[j], 13, 8);
    }
    o.push_back('\n');
  }
}

}  // namespace

extern "C" int vsvb_format_orbitals(const vsvb_system_desc *d, const double *coeff, double energy, double etol,
                                    int done, char *buf, long cap, long *len) {
  if (!d || (!buf && cap > 0)) return VSVB_ERR_INPUT;
  const double *c = coeff ? coeff : d->coeff;
  const int norbs = 2 * d->npair + d->nunpd + d->ndocc;
  std::string o;
  /* spin-coupled, unpaired and doubly occupied orbitals, then the NDF */
  for (int i = 0; i < norbs; ++i) orbital_block(o, d, c, i);
  o.push_back('\n');
  for (int i = norbs; i < norbs + d->ndf; ++i) orbital_block(o, d, c, i);
  o.append("\n total energy in atomic units ");
  fort_f(o, energy, 32, 16);
  o.push_back('\n');
  if (done) {
    o.append(" converged to ");
    fort_e(o, etol, 10, 2);
    o.append(" kCal/mol\n");
  }
  o.push_back('\n');
  if (len) *len = (long)o.size();
  if (!buf) return VSVB_OK;
  if ((long)o.size() + 1 > cap) return VSVB_ERR_TOO_LARGE;
  std::memcpy(buf, o.c_str(), o.size() + 1);
  return VSVB_OK;
}

extern "C" int vsvb_write_orbitals(const char *path, const vsvb_system_desc *d, const double *coeff, double energy,
                                   double etol, int done) {
  if (!path) return VSVB_ERR_INPUT;
  long n = 0;
  int rc = vsvb_format_orbitals(d, coeff, energy, etol, done, nullptr, 0, &n);
  if (rc) return rc;
  std::vector<char> b((size_t)n + 1);
  rc = vsvb_format_orbitals(d, coeff, energy, etol, done, b.data(), n + 1, &n);
  if (rc) return rc;
  FILE *f = std::fopen(path, "w");
  if (!f) return VSVB_ERR_INPUT;
  const bool ok = std::fwrite(b.data(), 1, (size_t)n, f) == (size_t)n;
  return std::fclose(f) == 0 && ok ? VSVB_OK : VSVB_ERR_INPUT;
}

/* The 'nelecwfn' file xm_output writes beside 'orbitals' when there is more
 * than one spin coupling (xm_module.F90:480-505): per coupling
 * format(1x,1f13.8,7(2i3,2x)) with the weight and its pairs (format reversion
 * continues past seven pairs on a record of 7(2i3,2x)), then the excited-state
 * roots in format(1x,7(2i3,2x)) and a blank record. */
extern "C" int vsvb_format_nelecwfn(const vsvb_system_desc *d, const double *coeff_sc, char *buf, long cap,
                                    long *len) {
  if (!d || !len) return VSVB_ERR_INPUT;
  std::string o, rec;
  const int nsc = d->nspinc > 0 ? d->nspinc : 1;
  /* X editing at the end of a record writes nothing: records end at their
   * last value */
  auto flush = [&]() {
    while (!rec.empty() && rec.back() == ' ') rec.pop_back();
    o += rec;
    o += '\n';
    rec.clear();
  };
  for (int j = 0; j < nsc; ++j) {
    rec = " ";
    fort_f(rec, coeff_sc ? coeff_sc[j] : d->coeff_sc[j], 13, 8);
    for (int k = 0; k < d->npair; ++k) {
      if (k > 0 && k % 7 == 0) flush();
      fort_i(rec, d->pair_sc[k + d->npair * (0 + 2 * j)], 3);
      fort_i(rec, d->pair_sc[k + d->npair * (1 + 2 * j)], 3);
      rec += "  ";
    }
    flush();
  }
  rec = " ";
  for (int i = 0; i < d->nxorb; ++i) {
    if (i > 0 && i % 7 == 0) flush();
    fort_i(rec, d->xorb[i], 3);
    fort_i(rec, d->root[i], 3);
    rec += "  ";
  }
  flush();
  o += '\n'; /* write(11,*) */
  *len = (long)o.size();
  if (buf) {
    if (cap < (long)o.size() + 1) return VSVB_ERR_TOO_LARGE;
    std::memcpy(buf, o.data(), o.size());
    buf[o.size()] = 0;
  }
  return VSVB_OK;
}

extern "C" int vsvb_write_nelecwfn(const char *path, const vsvb_system_desc *d, const double *coeff_sc) {
  if (!path) return VSVB_ERR_INPUT;
  long n = 0;
  int rc = vsvb_format_nelecwfn(d, coeff_sc, nullptr, 0, &n);
  if (rc) return rc;
  std::vector<char> b((size_t)n + 1);
  rc = vsvb_format_nelecwfn(d, coeff_sc, b.data(), n + 1, &n);
  if (rc) return rc;
  FILE *f = std::fopen(path, "w");
  if (!f) return VSVB_ERR_INPUT;
  const bool ok = std::fwrite(b.data(), 1, (size_t)n, f) == (size_t)n;
  return std::fclose(f) == 0 && ok ? VSVB_OK : VSVB_ERR_INPUT;
}

