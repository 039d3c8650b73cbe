"""ctypes binding of the CPU oracle (test infrastructure only).

The oracle is a literal C restatement of VALENCE's guess-energy path
(src/valence.F90:309-345, 1010-2144, 2157-3438); see oracle/vsvb_oracle.h.
"""
import ctypes
import json
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
_lib = None


class VoResult(ctypes.Structure):
    _fields_ = [("enucrep", ctypes.c_double), ("energy", ctypes.c_double), ("e1", ctypes.c_double),
                ("e2", ctypes.c_double), ("wfnorm", ctypes.c_double), ("ntasks", ctypes.c_longlong),
                ("ndens2", ctypes.c_longlong)]


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_build", "libvsvb_oracle.so"))
        _lib.vo_read_input.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p, ctypes.c_int]
        _lib.vo_guess_energy.argtypes = [ctypes.c_void_p, ctypes.POINTER(VoResult), ctypes.c_int]
        _lib.vo_free_input.argtypes = [ctypes.c_void_p]
        _lib.vo_set_coeff.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
        _lib.vo_set_coords_angstrom.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
        _lib.vo_int2e.argtypes = [ctypes.c_void_p] + [ctypes.c_int] * 4
        _lib.vo_int2e.restype = ctypes.c_double
        _lib.vo_ovint.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        _lib.vo_ovint.restype = ctypes.c_double
        _lib.vo_int1e.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        _lib.vo_int1e.restype = ctypes.c_double
        _lib.vo_boys.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.POINTER(ctypes.c_double)]
        _lib.vo_guess_energy_sampled.argtypes = [ctypes.c_void_p, ctypes.POINTER(VoResult), ctypes.c_int,
                                                 ctypes.c_longlong]
        _lib.vo_guess_energy_timed.argtypes = [ctypes.c_void_p, ctypes.POINTER(VoResult), ctypes.c_int,
                                               ctypes.c_longlong, ctypes.c_longlong, ctypes.c_longlong,
                                               ctypes.POINTER(ctypes.c_double)]
    return _lib


class Oracle:
    """One parsed input held by the oracle."""

    def __init__(self, path):
        self.h = ctypes.c_void_p()
        err = ctypes.create_string_buffer(256)
        if lib().vo_read_input(path.encode(), ctypes.byref(self.h), err, 256):
            raise ValueError(err.value.decode())

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.vo_free_input(self.h)
            self.h = None

    def set_coeff(self, c):
        c = np.ascontiguousarray(c, dtype=np.float64)
        lib().vo_set_coeff(self.h, c.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))

    def set_coords_angstrom(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        lib().vo_set_coords_angstrom(self.h, x.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))

    def guess_energy(self, nthreads=0):
        r = VoResult()
        lib().vo_guess_energy(self.h, ctypes.byref(r), nthreads)
        return r

    def guess_energy_sampled(self, nthreads=0, stride=1):
        r = VoResult()
        lib().vo_guess_energy_sampled(self.h, ctypes.byref(r), nthreads, stride)
        return r

    def guess_energy_timed(self, nthreads=0, schw_stride=1, e1_stride=1, task_stride=1):
        """Phase times (set-up, Schwarz table, one-electron loop, task loop)
        of a run that evaluates only every stride-th item of each phase."""
        r = VoResult()
        t = (ctypes.c_double * 4)()
        lib().vo_guess_energy_timed(self.h, ctypes.byref(r), nthreads, schw_stride, e1_stride, task_stride, t)
        return r, list(t)

    def int2e(self, io, ko, jo, lo):
        return lib().vo_int2e(self.h, io, ko, jo, lo)

    def ovint(self, io, jo):
        return lib().vo_ovint(self.h, io, jo)

    def int1e(self, io, jo):
        return lib().vo_int1e(self.h, io, jo)


def boys(mmax, t):
    f = (ctypes.c_double * (mmax + 1))()
    lib().vo_boys(mmax, t, f)
    return np.array(f[:])


def goldens():
    with open(os.path.join(GOLDEN, "reference_goldens.json")) as f:
        return json.load(f)


class VoInput(ctypes.Structure):
    """Layout of struct vo_input (oracle/vsvb_oracle.h)."""
    _fields_ = [(n, ctypes.c_int) for n in ("natom", "natom_t", "npair", "nunpd", "ndocc", "totlen", "xpmax",
                                            "nspinc", "num_sh", "num_pr", "nang", "ndf", "nset", "nxorb", "mxctr",
                                            "ntol_c", "ntol_d", "ntol_i", "ntol_e_min", "ntol_e_max", "max_iter")] + [
        ("ptbnmax", ctypes.c_double), ("feather", ctypes.c_double), ("orbset", ctypes.POINTER(ctypes.c_int)),
        ("atom_t", ctypes.POINTER(ctypes.c_int)), ("coords", ctypes.POINTER(ctypes.c_double)),
        ("nuc_charge", ctypes.POINTER(ctypes.c_double)), ("map_atom2shell", ctypes.POINTER(ctypes.c_int)),
        ("num_shell_atom", ctypes.POINTER(ctypes.c_int)), ("map_shell2prim", ctypes.POINTER(ctypes.c_int)),
        ("ang_mom", ctypes.POINTER(ctypes.c_int)), ("exponent", ctypes.POINTER(ctypes.c_double)),
        ("uncoef", ctypes.POINTER(ctypes.c_double)), ("con_coeff", ctypes.POINTER(ctypes.c_double)),
        ("pair_sc", ctypes.POINTER(ctypes.c_int)), ("coeff_sc", ctypes.POINTER(ctypes.c_double)),
        ("xorb", ctypes.POINTER(ctypes.c_int)), ("root", ctypes.POINTER(ctypes.c_int)), ("norbs", ctypes.c_int),
        ("orbas_atnum", ctypes.POINTER(ctypes.c_int)), ("orbas_atset", ctypes.POINTER(ctypes.c_int)),
        ("map_orbs", ctypes.POINTER(ctypes.c_int)), ("xpset", ctypes.POINTER(ctypes.c_int)),
        ("coeff", ctypes.POINTER(ctypes.c_double)), ("coeff_raw", ctypes.POINTER(ctypes.c_double)),
        ("dtol", ctypes.c_double), ("itol", ctypes.c_double)]


TOKCAL = 627.509469  # valence.F90:2756


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class OptOracle(Oracle):
    """The reference's orbital / spin-coupling optimisation (minimize_energy,
    valence.F90:2744-2885; first_order_opt :527-844; spin_opt :850-936) on
    the oracle's literal H/S builds.  EISPACK rsg (a generalised symmetric
    eigensolver, rsg.F) is scipy.linalg.eigh here: ascending eigenvalues,
    eigenvectors normalised to w^T S w = 1."""

    def __init__(self, path):
        super().__init__(path)
        L = lib()
        L.vo_first_order_hs.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                        ctypes.POINTER(ctypes.c_double), ctypes.c_int]
        L.vo_spin_hs.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                 ctypes.c_int]
        L.vo_nuclear_repulsion.argtypes = [ctypes.c_void_p]
        L.vo_nuclear_repulsion.restype = ctypes.c_double
        L.vo_normal.argtypes = [ctypes.c_void_p, ctypes.c_int]
        self.inp = ctypes.cast(self.h, ctypes.POINTER(VoInput)).contents

    def coeff_raw(self):
        return np.ctypeslib.as_array(self.inp.coeff_raw, shape=(self.inp.totlen,)).copy()

    def coeff_sc(self):
        return np.ctypeslib.as_array(self.inp.coeff_sc, shape=(max(self.inp.nspinc, 1),)).copy()

    def set_coeff_sc(self, c):
        for k, v in enumerate(c):
            self.inp.coeff_sc[k] = float(v)

    def norbas(self, iorb):
        return self.inp.map_orbs[iorb] - self.inp.map_orbs[iorb - 1]

    def first_order_hs(self, iorb, nthreads=0):
        n = self.norbas(iorb)
        ham, ovl = np.zeros((n, n)), np.zeros((n, n))
        hf, of = np.asfortranarray(ham), np.asfortranarray(ovl)
        if lib().vo_first_order_hs(self.h, iorb, _dp(hf), _dp(of), nthreads):
            raise ValueError("bad orbital")
        return hf, of

    def spin_hs(self, nthreads=0):
        n = self.inp.nspinc
        hf, of = np.zeros((n, n), order="F"), np.zeros((n, n), order="F")
        if lib().vo_spin_hs(self.h, _dp(hf), _dp(of), nthreads):
            raise ValueError("no spin couplings")
        return hf, of

    def enucrep(self):
        return lib().vo_nuclear_repulsion(self.h)

    def _root_of(self, iorb):
        r = 0
        for k in range(self.inp.nxorb):
            if self.inp.xorb[k] == iorb:
                r = self.inp.root[k]
        return r

    def first_order_opt(self, iorb, nthreads=0):
        """valence.F90:527-844: H/S, rsg, the selected root into iorb."""
        import scipy.linalg
        ham, ovl = self.first_order_hs(iorb, nthreads)
        eig, w = scipy.linalg.eigh(ham, ovl)
        r = self._root_of(iorb)
        c = self.coeff_raw()
        b0 = self.inp.map_orbs[iorb - 1] - 1
        c[b0:b0 + len(eig)] = w[:, r]
        self.set_coeff(c)
        return eig[r] + self.enucrep()

    def demgs_opt(self, iorb, etol, energy, nthreads=0):
        """demgs_opt (valence.F90:350-524): coordinate-wise perturbation of
        the orbital's normalised weights, largest step first, feathered down
        until tokcal * perturb^2 < etol.  normal() follows every change, and
        a rejected +step leaves the other weights at their +step scale, as in
        the reference."""
        inp = self.inp
        j0 = inp.map_orbs[iorb - 1] - 1
        nb = self.norbas(iorb)
        perturb = inp.ptbnmax

        def trial(i, value):
            c = self.coeff_raw()
            c[j0 + i] = value
            self.set_coeff(c)
            lib().vo_normal(self.h, iorb)
            return self.guess_energy(nthreads).energy

        while TOKCAL * perturb * perturb >= etol:
            lock = [False] * nb
            updated = True
            while updated:
                updated = False
                for i in range(nb):
                    if lock[i]:
                        continue
                    origc, eprev = self.coeff_raw()[j0 + i], energy
                    e = trial(i, origc + perturb)
                    if e < eprev:
                        updated, energy = True, e
                        continue
                    e = trial(i, origc - perturb)
                    if e < eprev:
                        updated, energy = True, e
                        continue
                    c = self.coeff_raw()
                    c[j0 + i] = origc
                    self.set_coeff(c)
                    lib().vo_normal(self.h, iorb)
                    lock[i] = True
                    energy = eprev
            perturb *= inp.feather
        return energy

    def spin_opt(self, nthreads=0):
        """valence.F90:850-936: lowest root into coeff_sc (not normalised)."""
        import scipy.linalg
        ham, ovl = self.spin_hs(nthreads)
        eig, w = scipy.linalg.eigh(ham, ovl)
        self.set_coeff_sc(w[:, 0])
        return eig[0] + self.enucrep()

    def minimize_energy(self, nthreads=0):
        """minimize_energy (valence.F90:2744-2885) after guess_energy, with
        first_order_opt, or demgs_opt when ptbnmax > 0 and there are no
        excited-state roots.  Returns the final energy and the number of
        iterations."""
        inp = self.inp
        dem_gs = inp.ptbnmax > 0.0 and inp.nxorb == 0
        # calculate_vsvb_energy normalises the weights before anything else
        for iorb in range(1, inp.norbs - inp.ndf + 1):
            lib().vo_normal(self.h, iorb)
        energy = self.guess_energy(nthreads).energy
        num_iter = 0
        eprv_sc = eprv_orb = 0.0
        sets = [(inp.orbset[2 * s], inp.orbset[2 * s + 1]) for s in range(inp.nset)]
        for ntol in range(inp.ntol_e_min, inp.ntol_e_max + 1):
            etol = 10.0 ** (-ntol)
            finished = False
            while not finished:
                eprv_sc = energy
                orbconv = False
                while not orbconv and num_iter < inp.max_iter:
                    eprv_orb = energy
                    for lo, hi in sets:
                        setcnv = False
                        while not setcnv and num_iter < inp.max_iter:
                            eprv_set = energy
                            num_iter += 1
                            for iorb in range(lo, hi + 1):
                                if dem_gs:
                                    energy = self.demgs_opt(iorb, etol, energy, nthreads)
                                else:
                                    energy = self.first_order_opt(iorb, nthreads)
                            setcnv = abs(energy - eprv_set) * TOKCAL < etol
                            if lo == hi and dem_gs:
                                setcnv = True
                    orbconv = abs(energy - eprv_orb) * TOKCAL < etol
                    if len(sets) == 1:
                        orbconv = True
                        eprv_orb = energy
                if inp.nspinc > 1:
                    num_iter += 1
                    energy = self.spin_opt(nthreads)
                    finished = abs(energy - eprv_sc) * TOKCAL < etol
                else:
                    finished = True
                if num_iter >= inp.max_iter:
                    finished = True
        return energy, num_iter
