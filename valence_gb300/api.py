"""Python host for libvsvb_gb300.so.

Mirrors VALENCE's library API (src/valence_api.F90):
    valence_api_initialize(info, call_mpi_init, comm)   valence_api.F90:9-35
    valence_api_calculate_energy(x, v)                  valence_api.F90:37-108
    valence_api_finalize(call_mpi_finalize)             valence_api.F90:114-134
with the same meaning: initialise from an input file, then energies for
Cartesian coordinates x (Angstrom, 3*natom) in hartree.  The reference reads
the input file named by argv(1) (valence_initialize_module.F90:49-53); here the
path is an argument.  Errors raise VSVBError (the reference stops through
xm_abort).  There is no CPU path: without the built library every entry point
raises.
"""
import ctypes
import os

import numpy as np

FP64 = 0
MIXED = 1
MIXED_DF64 = 2

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def library_path():
    return os.path.join(_HERE, "_build", "libvsvb_gb300.so")


class VSVBError(RuntimeError):
    pass


class Desc(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("natom", "natom_t", "npair", "nunpd", "ndocc", "totlen", "xpmax",
                                             "nspinc", "num_sh", "num_pr", "nang", "ndf", "nxorb", "mxctr",
                                             "ntol_d", "ntol_i")] + [
        ("atom_t", ctypes.POINTER(ctypes.c_int)), ("coords", ctypes.POINTER(ctypes.c_double)),
        ("nuc_charge", ctypes.POINTER(ctypes.c_double)), ("map_atom2shell", ctypes.POINTER(ctypes.c_int)),
        ("num_shell_atom", ctypes.POINTER(ctypes.c_int)), ("map_shell2prim", ctypes.POINTER(ctypes.c_int)),
        ("ang_mom", ctypes.POINTER(ctypes.c_int)), ("exponent", ctypes.POINTER(ctypes.c_double)),
        ("con_coeff", ctypes.POINTER(ctypes.c_double)), ("pair_sc", ctypes.POINTER(ctypes.c_int)),
        ("coeff_sc", ctypes.POINTER(ctypes.c_double)), ("orbas_atnum", ctypes.POINTER(ctypes.c_int)),
        ("orbas_atset", ctypes.POINTER(ctypes.c_int)), ("map_orbs", ctypes.POINTER(ctypes.c_int)),
        ("xpset", ctypes.POINTER(ctypes.c_int)), ("coeff", ctypes.POINTER(ctypes.c_double)),
        ("ntol_e_min", ctypes.c_int), ("ntol_e_max", ctypes.c_int), ("max_iter", ctypes.c_int), ("nset", ctypes.c_int),
        ("ptbnmax", ctypes.c_double), ("feather", ctypes.c_double), ("orbset", ctypes.POINTER(ctypes.c_int)),
        ("xorb", ctypes.POINTER(ctypes.c_int)), ("root", ctypes.POINTER(ctypes.c_int))]


class Options(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("mixed_threshold", ctypes.c_double), ("ao_screen", ctypes.c_double),
                ("device", ctypes.c_int), ("grad_mode", ctypes.c_int), ("prim_screen", ctypes.c_double),
                ("prim_split", ctypes.c_int), ("cuda_graph", ctypes.c_int), ("autotune", ctypes.c_int),
                ("block_mode", ctypes.c_int), ("core_mode", ctypes.c_int)]


class Result(ctypes.Structure):
    _fields_ = [("energy", ctypes.c_double), ("e_num", ctypes.c_double), ("e1", ctypes.c_double),
                ("e2", ctypes.c_double), ("wfnorm", ctypes.c_double), ("enucrep", ctypes.c_double),
                ("err_est", ctypes.c_double), ("n_quartets_fp64", ctypes.c_longlong),
                ("n_quartets_fp32", ctypes.c_longlong), ("n_tasks", ctypes.c_longlong),
                ("n_singular_pairs", ctypes.c_int), ("n_kernel_launches", ctypes.c_int),
                ("n_prim_quartets", ctypes.c_double), ("n_prim_quartets_fp32", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class OptResult(ctypes.Structure):
    _fields_ = [("energy", ctypes.c_double), ("guess_energy", ctypes.c_double), ("etol", ctypes.c_double),
                ("seconds", ctypes.c_double), ("iterations", ctypes.c_int), ("converged", ctypes.c_int),
                ("n_energy_evals", ctypes.c_longlong), ("n_hs_builds", ctypes.c_longlong)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def lib():
    global _LIB
    if _LIB is None:
        p = library_path()
        if not os.path.exists(p):
            raise VSVBError("libvsvb_gb300.so is not built (run __graft_entry__.build())")
        L = ctypes.CDLL(p)
        P, D, I = ctypes.POINTER, ctypes.c_double, ctypes.c_int
        L.vsvb_read_input.argtypes = [ctypes.c_char_p, P(P(Desc)), ctypes.c_char_p, I]
        L.vsvb_free_desc.argtypes = [P(Desc)]
        L.vsvb_default_options.argtypes = [P(Options)]
        L.vsvb_gpu_create.argtypes = [P(Desc), P(Options), P(ctypes.c_void_p)]
        L.vsvb_gpu_destroy.argtypes = [ctypes.c_void_p]
        L.vsvb_gpu_last_error.argtypes = [ctypes.c_void_p]
        L.vsvb_gpu_last_error.restype = ctypes.c_char_p
        L.vsvb_gpu_energy.argtypes = [ctypes.c_void_p, P(D), P(Result)]
        L.vsvb_gpu_energy_grad.argtypes = [ctypes.c_void_p, P(D), P(Result), P(D)]
        L.vsvb_gpu_energy_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p, P(Result)]
        L.vsvb_gpu_energy_grad_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p, P(Result), ctypes.c_void_p]
        L.vsvb_gpu_totlen.argtypes = [ctypes.c_void_p]
        L.vsvb_gpu_num_orbitals.argtypes = [ctypes.c_void_p]
        L.vsvb_gpu_debug_orbital_eri.argtypes = [ctypes.c_void_p, P(D), ctypes.c_size_t]
        L.vsvb_gpu_debug_orbital_1e.argtypes = [ctypes.c_void_p, P(D), P(D), ctypes.c_size_t]
        L.vsvb_gpu_debug_orbital_eri_at.argtypes = [ctypes.c_void_p, P(ctypes.c_longlong), I, P(D)]
        L.vsvb_gpu_block_stats.argtypes = [ctypes.c_void_p, P(D), P(D), P(ctypes.c_longlong)]
        L.vsvb_gpu_core_stats.argtypes = [ctypes.c_void_p, P(D), P(ctypes.c_longlong)]
        L.vsvb_gpu_batch_energy_grad.argtypes = [P(ctypes.c_void_p), I, P(P(D)), P(Result), P(P(D))]
        L.vsvb_gpu_set_stream.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.vsvb_gpu_set_spin_coeffs.argtypes = [ctypes.c_void_p, P(D)]
        L.vsvb_gpu_eri_profile.argtypes = [ctypes.c_void_p, P(D), P(D), P(I), I]
        L.vsvb_gpu_eri_profile_mode.argtypes = [ctypes.c_void_p, I, P(D), P(D), P(I), I]
        L.vsvb_gpu_set_sweep_timing.argtypes = [ctypes.c_void_p, I]
        L.vsvb_gpu_sweep_times.argtypes = [ctypes.c_void_p, P(D), P(D), P(I), I]
        L.vsvb_gpu_sweep_wall_ms.argtypes = [ctypes.c_void_p, P(D)]
        L.vsvb_gpu_launch_config.argtypes = [ctypes.c_void_p, P(I), P(I), P(I), I]
        L.vsvb_gpu_fma_peak.argtypes = [I, P(D), P(D)]
        L.vsvb_det_factor.argtypes = [ctypes.c_void_p, I, I, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_void_p]
        L.vsvb_det_factor_noalloc.argtypes = L.vsvb_det_factor.argtypes
        L.vsvb_format_orbitals.argtypes = [P(Desc), P(D), D, D, I, ctypes.c_char_p, ctypes.c_long,
                                           P(ctypes.c_long)]
        L.vsvb_write_orbitals.argtypes = [ctypes.c_char_p, P(Desc), P(D), D, D, I]
        L.vsvb_batch_create.argtypes = [P(ctypes.c_void_p), I, P(ctypes.c_void_p)]
        L.vsvb_batch_energy_grad.argtypes = [ctypes.c_void_p, P(ctypes.c_void_p), P(ctypes.c_void_p), P(Result),
                                             ctypes.c_void_p]
        L.vsvb_batch_launches.argtypes = [ctypes.c_void_p]
        L.vsvb_batch_last_error.argtypes = [ctypes.c_void_p]
        L.vsvb_batch_last_error.restype = ctypes.c_char_p
        L.vsvb_batch_destroy.argtypes = [ctypes.c_void_p]
        L.vsvb_opt_create.argtypes = [P(Desc), P(Options), P(ctypes.c_void_p)]
        L.vsvb_opt_destroy.argtypes = [ctypes.c_void_p]
        L.vsvb_opt_last_error.argtypes = [ctypes.c_void_p]
        L.vsvb_opt_last_error.restype = ctypes.c_char_p
        L.vsvb_opt_first_order_hs.argtypes = [ctypes.c_void_p, P(D), P(D), I, P(D), P(D)]
        L.vsvb_opt_spin_hs.argtypes = [ctypes.c_void_p, P(D), P(D), P(D)]
        L.vsvb_opt_minimize.argtypes = [ctypes.c_void_p, P(D), P(D), P(OptResult)]
        L.vsvb_rsg.argtypes = [I, P(D), P(D), I, P(D), P(D), I]
        L.vsvb_opt_set_output.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p]
        L.vsvb_format_nelecwfn.argtypes = [P(Desc), P(D), ctypes.c_char_p, ctypes.c_long, P(ctypes.c_long)]
        L.vsvb_write_nelecwfn.argtypes = [ctypes.c_char_p, P(Desc), P(D)]
        _LIB = L
    return _LIB


def format_orbitals(desc, coeff=None, energy=0.0, etol=0.0, done=False):
    """The reference's 'orbitals' file text (xm_output) for a parsed input
    description (read_input) and optional new weights."""
    c = None if coeff is None else np.ascontiguousarray(coeff, dtype=np.float64)
    n = ctypes.c_long()
    rc = lib().vsvb_format_orbitals(desc, None if c is None else _dptr(c), energy, etol, int(done), None, 0,
                                    ctypes.byref(n))
    if rc:
        raise VSVBError(f"format_orbitals failed ({rc})")
    buf = ctypes.create_string_buffer(n.value + 1)
    rc = lib().vsvb_format_orbitals(desc, None if c is None else _dptr(c), energy, etol, int(done), buf,
                                    n.value + 1, ctypes.byref(n))
    if rc:
        raise VSVBError(f"format_orbitals failed ({rc})")
    return buf.value.decode()


def format_nelecwfn(desc, coeff_sc=None):
    """The reference's 'nelecwfn' file text (xm_output with nspinc > 1)."""
    c = None if coeff_sc is None else np.ascontiguousarray(coeff_sc, dtype=np.float64)
    n = ctypes.c_long()
    if lib().vsvb_format_nelecwfn(desc, None if c is None else _dptr(c), None, 0, ctypes.byref(n)):
        raise VSVBError("format_nelecwfn failed")
    buf = ctypes.create_string_buffer(n.value + 1)
    if lib().vsvb_format_nelecwfn(desc, None if c is None else _dptr(c), buf, n.value + 1, ctypes.byref(n)):
        raise VSVBError("format_nelecwfn failed")
    return buf.value.decode()


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def read_input(path):
    """Parse a VALENCE input file into a description owned by the library."""
    d = ctypes.POINTER(Desc)()
    err = ctypes.create_string_buffer(256)
    rc = lib().vsvb_read_input(os.fsencode(path), ctypes.byref(d), err, 256)
    if rc:
        raise VSVBError(f"input error ({rc}): {err.value.decode()}")
    return d


def make_options(precision=FP64, mixed_threshold=1e-6, ao_screen=1e-15, device=0, grad_mode=0, prim_screen=None,
                 prim_split=None, cuda_graph=None, autotune=None, block_mode=None, core_mode=None):
    o = Options()
    lib().vsvb_default_options(ctypes.byref(o))
    o.precision = precision
    o.mixed_threshold = mixed_threshold
    o.ao_screen = ao_screen
    o.device = device
    o.grad_mode = grad_mode
    if prim_screen is not None:
        o.prim_screen = prim_screen
    if prim_split is not None:
        o.prim_split = int(prim_split)
    if cuda_graph is not None:
        o.cuda_graph = int(cuda_graph)
    if autotune is not None:
        o.autotune = int(autotune)
    if block_mode is not None:
        o.block_mode = int(block_mode)
    if core_mode is not None:
        o.core_mode = int(core_mode)
    return o


class System:
    """One molecule on the GPU: a parsed input plus a device handle."""

    def __init__(self, path, precision=FP64, mixed_threshold=1e-6, ao_screen=1e-15, device=0, coords_angstrom=None,
                 grad_mode=0, prim_screen=None, prim_split=None, cuda_graph=None, autotune=None, block_mode=None,
                 core_mode=None):
        self.path = path
        self._desc = read_input(path)
        d = self._desc.contents
        self.natom = d.natom
        self.totlen = d.totlen
        self.coeff0 = np.ctypeslib.as_array(d.coeff, shape=(d.totlen,)).copy()
        self._coords_bohr = np.ctypeslib.as_array(d.coords, shape=(3 * d.natom,))
        if coords_angstrom is not None:
            self._coords_bohr[:] = np.asarray(coords_angstrom, dtype=np.float64).ravel() * 1.889725987722
        self.opt = make_options(precision, mixed_threshold, ao_screen, device, grad_mode, prim_screen, prim_split,
                                cuda_graph, autotune, block_mode, core_mode)
        self._h = ctypes.c_void_p()
        rc = lib().vsvb_gpu_create(self._desc, ctypes.byref(self.opt), ctypes.byref(self._h))
        if rc:
            msg = lib().vsvb_gpu_last_error(self._h).decode() if self._h else ""
            self.close()
            raise VSVBError(f"vsvb_gpu_create failed ({rc}): {msg}")

    def close(self):
        if getattr(self, "_h", None):
            lib().vsvb_gpu_destroy(self._h)
            self._h = None
        if getattr(self, "_desc", None):
            lib().vsvb_free_desc(self._desc)
            self._desc = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc:
            raise VSVBError(f"{what} failed ({rc}): {lib().vsvb_gpu_last_error(self._h).decode()}")

    def energy(self, coeff=None):
        r = Result()
        c = None if coeff is None else np.ascontiguousarray(coeff, dtype=np.float64)
        self._check(lib().vsvb_gpu_energy(self._h, None if c is None else _dptr(c), ctypes.byref(r)), "energy")
        return r.as_dict()

    def energy_grad(self, coeff=None):
        r = Result()
        c = None if coeff is None else np.ascontiguousarray(coeff, dtype=np.float64)
        g = np.zeros(self.totlen)
        self._check(lib().vsvb_gpu_energy_grad(self._h, None if c is None else _dptr(c), ctypes.byref(r), _dptr(g)),
                    "energy_grad")
        return r.as_dict(), g

    def set_spin_coeffs(self, coeff_sc):
        """Spin-coupling weights (nspinc) for the following evaluations."""
        c = np.ascontiguousarray(coeff_sc, dtype=np.float64)
        self._check(lib().vsvb_gpu_set_spin_coeffs(self._h, _dptr(c)), "set_spin_coeffs")

    def energy_device(self, coeff_ptr):
        """Energy with the weights already in device memory (a raw pointer)."""
        r = Result()
        self._check(lib().vsvb_gpu_energy_device(self._h, ctypes.c_void_p(coeff_ptr), ctypes.byref(r)), "energy")
        return r.as_dict()

    def energy_grad_device(self, coeff_ptr, grad_ptr):
        r = Result()
        self._check(lib().vsvb_gpu_energy_grad_device(self._h, ctypes.c_void_p(coeff_ptr), ctypes.byref(r),
                                                      ctypes.c_void_p(grad_ptr)), "energy_grad")
        return r.as_dict()

    def set_stream(self, stream_ptr):
        """Enqueue this system's work on a caller-owned CUDA stream (an int
        cudaStream_t, e.g. torch.cuda.current_stream().cuda_stream; 0 restores
        the handle's own stream)."""
        self._check(lib().vsvb_gpu_set_stream(self._h, ctypes.c_void_p(stream_ptr or None)), "set_stream")

    def eri_profile(self, cap=128, mode=0):
        """Per ERI launch of one sweep run one after another (mode 0 forward,
        3 forward + adjoint): ms, algorithmic FLOPs and class code."""
        ms = np.zeros(cap)
        fl = np.zeros(cap)
        cl = np.zeros(cap, dtype=np.int32)
        n = lib().vsvb_gpu_eri_profile_mode(self._h, mode, _dptr(ms), _dptr(fl),
                                            cl.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), cap)
        if n < 0:
            raise VSVBError("eri_profile failed")
        return [dict(cls=int(cl[i]), ms=float(ms[i]), flops=float(fl[i])) for i in range(n)]

    def set_sweep_timing(self, on=True):
        """Record CUDA events around every ERI class launch of later calls."""
        self._check(lib().vsvb_gpu_set_sweep_timing(self._h, 1 if on else 0), "set_sweep_timing")

    def sweep_times(self, cap=128):
        """Per class launch of the last ERI sweep: duration (ms, in situ,
        concurrent with the other classes) and algorithmic FLOPs."""
        ms = np.zeros(cap)
        fl = np.zeros(cap)
        cl = np.zeros(cap, dtype=np.int32)
        n = lib().vsvb_gpu_sweep_times(self._h, _dptr(ms), _dptr(fl), cl.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), cap)
        if n < 0:
            raise VSVBError("sweep_times failed")
        return [dict(cls=int(cl[i]), ms=float(ms[i]), flops=float(fl[i])) for i in range(n)]

    def launch_config(self, cap=256):
        """Launch geometry in use: {"nsplit": task splits, "eri": [(class code, blocks per SM)]}."""
        ns = ctypes.c_int()
        codes = (ctypes.c_int * cap)()
        bps = (ctypes.c_int * cap)()
        k = lib().vsvb_gpu_launch_config(self._h, ctypes.byref(ns), codes, bps, cap)
        if k < 0:
            raise VSVBError("launch_config failed")
        return {"nsplit": ns.value, "eri": [(codes[i], bps[i]) for i in range(k)]}

    def sweep_wall_ms(self):
        """Wall time (ms) of the last ERI sweep, fork to join."""
        v = ctypes.c_double()
        self._check(lib().vsvb_gpu_sweep_wall_ms(self._h, ctypes.byref(v)), "sweep_wall_ms")
        return v.value

    def orbital_eri(self):
        n = lib().vsvb_gpu_num_orbitals(self._h)
        np_ = n * (n + 1) // 2
        out = np.zeros(np_ * np_)
        rc = lib().vsvb_gpu_debug_orbital_eri(self._h, _dptr(out), out.size)
        if rc < 0:
            raise VSVBError("debug_orbital_eri failed")
        return out.reshape(np_, np_)

    def orbital_eri_at(self, p, q):
        """Entries T[p[i], q[i]] of the orbital-pair ERI matrix of the last
        evaluation (orbital-pair indices i*(i+1)/2+k, i >= k)."""
        n = lib().vsvb_gpu_num_orbitals(self._h)
        np_ = n * (n + 1) // 2
        idx = np.ascontiguousarray(np.asarray(p, dtype=np.int64) * np_ + np.asarray(q, dtype=np.int64))
        out = np.zeros(idx.size)
        rc = lib().vsvb_gpu_debug_orbital_eri_at(self._h, idx.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)),
                                                 int(idx.size), _dptr(out))
        if rc < 0 or rc > 0 and rc != np_:
            raise VSVBError(f"debug_orbital_eri_at failed ({rc}): {lib().vsvb_gpu_last_error(self._h).decode()}")
        return out

    def block_stats(self):
        """Block-mode figures: whether the handle runs in block mode, the
        algorithmic FLOPs of one sweep per ERI kind and of the transforms, and
        the atom quartets, chunks and launches of the sweep."""
        ef = (ctypes.c_double * 3)()
        tf = (ctypes.c_double * 3)()
        cn = (ctypes.c_longlong * 3)()
        on = lib().vsvb_gpu_block_stats(self._h, ef, tf, cn)
        return {"on": bool(on), "eri_flops": {"fp64": ef[0], "fp32": ef[1], "df64": ef[2]},
                "transform_flops": {"fp64": tf[0], "fp32": tf[1], "df64": tf[2]},
                "atom_quartets": cn[0], "chunks": cn[1], "launches": cn[2]}

    def core_stats(self):
        """Core-mode figures: whether the handle sums the determinant pairs
        over the shared core, the FMAs of its pair-summed density GEMM per
        evaluation, the determinant pairs and the coupled orbitals."""
        f = ctypes.c_double()
        cn = (ctypes.c_longlong * 2)()
        on = lib().vsvb_gpu_core_stats(self._h, ctypes.byref(f), cn)
        if on < 0:
            raise VSVBError("core_stats failed")
        return {"on": bool(on), "gemm_fma": f.value, "determinant_pairs": cn[0], "coupled_orbitals": cn[1]}

    def orbital_1e(self):
        n = lib().vsvb_gpu_num_orbitals(self._h)
        s = np.zeros(n * n)
        h = np.zeros(n * n)
        rc = lib().vsvb_gpu_debug_orbital_1e(self._h, _dptr(s), _dptr(h), n * n)
        if rc < 0:
            raise VSVBError("debug_orbital_1e failed")
        return s.reshape(n, n), h.reshape(n, n)


def batch_energy_grad(systems, weights=None, with_grad=True):
    """Energies (and gradients) of independent molecules in one library call."""
    n = len(systems)
    hs = (ctypes.c_void_p * n)(*[s._h for s in systems])
    ws = [np.ascontiguousarray(w if w is not None else s.coeff0, dtype=np.float64)
          for s, w in zip(systems, weights or [None] * n)]
    wp = (ctypes.POINTER(ctypes.c_double) * n)(*[_dptr(w) for w in ws])
    res = (Result * n)()
    grads = [np.zeros(s.totlen) for s in systems] if with_grad else None
    gp = (ctypes.POINTER(ctypes.c_double) * n)(*[_dptr(g) for g in grads]) if with_grad else None
    rc = lib().vsvb_gpu_batch_energy_grad(hs, n, wp, res, gp)
    if rc:
        raise VSVBError(f"batch failed ({rc}): {lib().vsvb_gpu_last_error(systems[0]._h).decode()}")
    return [r.as_dict() for r in res], grads


def det_factor(a, stream=0):
    """Determinants and inverses of a batch of square matrices held in a
    CUDA torch tensor of shape (nmat, n, n), float64.  Returns (det, inv,
    singular) as CUDA tensors."""
    import torch
    a = a.contiguous()
    nmat, n, _ = a.shape
    det = torch.empty(nmat, dtype=torch.float64, device=a.device)
    inv = torch.empty_like(a)
    sing = torch.empty(nmat, dtype=torch.int32, device=a.device)
    rc = lib().vsvb_det_factor(ctypes.c_void_p(a.data_ptr()), n, nmat, ctypes.c_void_p(det.data_ptr()),
                               ctypes.c_void_p(inv.data_ptr()), ctypes.c_void_p(sing.data_ptr()),
                               ctypes.c_void_p(stream or None))
    if rc:
        raise VSVBError(f"vsvb_det_factor failed ({rc})")
    return det, inv, sing


def fma_peak(device=0):
    """Measured FP64 and FP32 FMA throughput (FLOP/s) of the device."""
    a, b = ctypes.c_double(), ctypes.c_double()
    if lib().vsvb_gpu_fma_peak(device, ctypes.byref(a), ctypes.byref(b)):
        raise VSVBError("fma_peak failed")
    return a.value, b.value


# --- reference-shaped API ---------------------------------------------------

_STATE = {}


def valence_api_initialize(input_path, precision=FP64, mixed_threshold=1e-6, device=0):
    """Counterpart of valence_api_initialize (valence_api.F90:9-35): read the
    input once; returns info = 0 on success (the reference always returns 0)."""
    _STATE.clear()
    _STATE.update(path=input_path, precision=precision, mixed_threshold=mixed_threshold, device=device, sys=None,
                  coords=None)
    return 0


def valence_api_calculate_energy(x):
    """Counterpart of valence_api_calculate_energy (valence_api.F90:37-108):
    x = 3*natom Cartesian coordinates in Angstrom; returns the guess energy in
    hartree (energy/wfnorm + enucrep, valence.F90:344)."""
    if "path" not in _STATE:
        raise VSVBError("valence_api_initialize has not been called")
    x = np.asarray(x, dtype=np.float64).ravel()
    s = _STATE.get("sys")
    if s is None or _STATE.get("coords") is None or not np.array_equal(_STATE["coords"], x):
        if s is not None:
            s.close()
        s = System(_STATE["path"], precision=_STATE["precision"], mixed_threshold=_STATE["mixed_threshold"],
                   device=_STATE["device"], coords_angstrom=x)
        _STATE["sys"], _STATE["coords"] = s, x.copy()
    return s.energy()["energy"]


def valence_api_finalize():
    """Counterpart of valence_api_finalize (valence_api.F90:114-134)."""
    s = _STATE.get("sys")
    if s is not None:
        s.close()
    _STATE.clear()


# --- torch binding ----------------------------------------------------------

try:
    import torch

    class VSVBEnergy(torch.autograd.Function):
        """E(weights) with dE/dweights from the GPU adjoint (ERIs recomputed in
        the backward pass).  weights: 1-D float64 tensor of length totlen."""

        @staticmethod
        def forward(ctx, weights, system):
            w = weights.detach().to("cpu", torch.float64).contiguous().numpy()
            r, g = system.energy_grad(w)
            ctx.save_for_backward(torch.from_numpy(g).to(weights.device))
            return torch.tensor(r["energy"], dtype=torch.float64, device=weights.device)

        @staticmethod
        def backward(ctx, gout):
            (g,) = ctx.saved_tensors
            return gout * g, None
except ImportError:  # pragma: no cover
    VSVBEnergy = None


class Batch:
    """Energy + gradient of many molecules as one CUDA graph launch
    (vsvb_batch_*).  systems: System objects on one device; they must stay
    alive while the batch is used."""

    def __init__(self, systems):
        self.systems = list(systems)
        arr = (ctypes.c_void_p * len(self.systems))(*[s._h for s in self.systems])
        self._b = ctypes.c_void_p()
        rc = lib().vsvb_batch_create(arr, len(self.systems), ctypes.byref(self._b))
        if rc:
            msg = lib().vsvb_batch_last_error(self._b).decode() if self._b else ""
            self.close()
            raise VSVBError(f"vsvb_batch_create failed ({rc}): {msg}")

    def energy_grad_device(self, weight_ptrs, grad_ptrs, stream=None):
        """weight_ptrs / grad_ptrs: device addresses (one per molecule).
        Returns the list of result dicts."""
        n = len(self.systems)
        w = (ctypes.c_void_p * n)(*weight_ptrs)
        g = (ctypes.c_void_p * n)(*grad_ptrs)
        res = (Result * n)()
        rc = lib().vsvb_batch_energy_grad(self._b, w, g, res, ctypes.c_void_p(stream) if stream else None)
        if rc:
            raise VSVBError(f"vsvb_batch_energy_grad failed ({rc}): {lib().vsvb_batch_last_error(self._b).decode()}")
        return [r.as_dict() for r in res]

    @property
    def launches(self):
        return lib().vsvb_batch_launches(self._b)

    def close(self):
        if getattr(self, "_b", None):
            lib().vsvb_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def rsg(ham, ovl):
    """EISPACK rsg on the GPU (vsvb_rsg): eigenvalues ascending and
    eigenvectors (columns, w^T ovl w = 1) of ham w = e ovl w."""
    h = np.asfortranarray(ham, dtype=np.float64)
    s = np.asfortranarray(ovl, dtype=np.float64)
    n = h.shape[0]
    eig, w = np.zeros(n), np.zeros((n, n), order="F")
    rc = lib().vsvb_rsg(n, _dptr(h), _dptr(s), n, _dptr(eig), _dptr(w), n)
    if rc:
        raise VSVBError(f"vsvb_rsg failed ({rc})")
    return eig, w


class Optimizer:
    """The reference's wave-function optimisation (minimize_energy with
    first_order_opt / spin_opt / demgs_opt, valence.F90:350-936, 2744-2885)
    on the GPU path (vsvb_opt_*)."""

    def __init__(self, path, precision=FP64, device=0, **kw):
        self.path = path
        self._desc = read_input(path)
        d = self._desc.contents
        self.totlen, self.nspinc = d.totlen, d.nspinc
        self.npair, self.nunpd, self.ndocc, self.ndf = d.npair, d.nunpd, d.ndocc, d.ndf
        self.map_orbs = np.ctypeslib.as_array(d.map_orbs, shape=(2 * d.npair + d.nunpd + d.ndocc + d.ndf + 1,)).copy()
        self.coeff0 = np.ctypeslib.as_array(d.coeff, shape=(d.totlen,)).copy()
        self.coeff_sc0 = np.ctypeslib.as_array(d.coeff_sc, shape=(max(d.nspinc, 1),)).copy()
        self.opt = make_options(precision, kw.get("mixed_threshold", 1e-6), kw.get("ao_screen", 1e-15), device,
                                0, kw.get("prim_screen"), kw.get("prim_split"), None, None)
        self._o = ctypes.c_void_p()
        rc = lib().vsvb_opt_create(self._desc, ctypes.byref(self.opt), ctypes.byref(self._o))
        if rc:
            msg = lib().vsvb_opt_last_error(self._o).decode() if self._o else ""
            self.close()
            raise VSVBError(f"vsvb_opt_create failed ({rc}): {msg}")

    def close(self):
        if getattr(self, "_o", None):
            lib().vsvb_opt_destroy(self._o)
            self._o = None
        if getattr(self, "_desc", None):
            lib().vsvb_free_desc(self._desc)
            self._desc = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc:
            raise VSVBError(f"{what} failed ({rc}): {lib().vsvb_opt_last_error(self._o).decode()}")

    def desc_counts(self):
        return {"npair": self.npair, "nunpd": self.nunpd, "ndocc": self.ndocc, "ndf": self.ndf,
                "nnd": 2 * self.npair + self.nunpd}

    def first_order_hs(self, iorb, coeff=None, coeff_sc=None):
        c = np.ascontiguousarray(self.coeff0 if coeff is None else coeff, dtype=np.float64)
        csc = None if coeff_sc is None else np.ascontiguousarray(coeff_sc, dtype=np.float64)
        n = int(self.map_orbs[iorb] - self.map_orbs[iorb - 1])
        h, s = np.zeros((n, n), order="F"), np.zeros((n, n), order="F")
        self._check(lib().vsvb_opt_first_order_hs(self._o, _dptr(c), None if csc is None else _dptr(csc), iorb,
                                                  _dptr(h), _dptr(s)), "first_order_hs")
        return h, s

    def spin_hs(self, coeff=None):
        c = np.ascontiguousarray(self.coeff0 if coeff is None else coeff, dtype=np.float64)
        n = self.nspinc
        h, s = np.zeros((n, n), order="F"), np.zeros((n, n), order="F")
        self._check(lib().vsvb_opt_spin_hs(self._o, _dptr(c), _dptr(h), _dptr(s)), "spin_hs")
        return h, s

    def set_output(self, orbitals_path=None, nelecwfn_path=None):
        """Write the 'orbitals' (and 'nelecwfn') files during minimize, as the
        reference does after every update and on convergence."""
        enc = lambda p: None if p is None else os.fsencode(p)
        self._check(lib().vsvb_opt_set_output(self._o, enc(orbitals_path), enc(nelecwfn_path)), "set_output")

    def minimize(self, coeff=None, coeff_sc=None):
        """Returns (result dict, optimised weights, spin-coupling weights)."""
        c = np.array(self.coeff0 if coeff is None else coeff, dtype=np.float64)
        csc = np.array(self.coeff_sc0 if coeff_sc is None else coeff_sc, dtype=np.float64)
        r = OptResult()
        self._check(lib().vsvb_opt_minimize(self._o, _dptr(c), _dptr(csc), ctypes.byref(r)), "minimize")
        return r.as_dict(), c, csc
