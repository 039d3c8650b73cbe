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
