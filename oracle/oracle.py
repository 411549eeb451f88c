"""ctypes wrapper of the CPU oracle (oracle.c) - TEST INFRASTRUCTURE ONLY.

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
checker of the CUDA library; never by the library itself.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "taxila-lbm_gb300"))
from taxila import params as P  # noqa: E402

_lib = None


def build(force=False):
    """Compile oracle.c with oracle/Makefile (gcc, -ffp-contract=off)."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(
            os.path.getmtime(os.path.join(HERE, f)) for f in ("oracle.c", "oracle.h", "ff_stencil_oracle.h")):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.POINTER(P.TxParams)]
        L.orc_destroy.argtypes = [C.c_void_p]
        for fn in ("orc_set_walls", "orc_set_fi"):
            getattr(L, fn).argtypes = [C.c_void_p, C.c_void_p]
        L.orc_set_state.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_set_species.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_set_bc_values.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.orc_init.argtypes = [C.c_void_p]
        L.orc_step.argtypes = [C.c_void_p, C.c_int]
        L.orc_delta_norm.argtypes = [C.c_void_p, C.c_int]
        L.orc_delta_norm.restype = C.c_double
        L.orc_get.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.orc_field_size.argtypes = [C.c_void_p, C.c_int]
        L.orc_field_size.restype = C.c_long
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_set_threads.restype = C.c_int
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


class Oracle:
    """The reference's flow step on the CPU, natural-order arrays in and out."""

    def __init__(self, params, threads=0):
        self.p = P.copy_params(params)
        self.L = lib()
        if threads:
            self.L.orc_set_threads(int(threads))
        self.h = self.L.orc_create(C.byref(self.p))
        if not self.h:
            raise MemoryError("orc_create failed")

    def close(self):
        if self.h:
            self.L.orc_destroy(self.h)
            self.h = None

    __del__ = close

    def set_walls(self, walls):
        self._walls = np.ascontiguousarray(walls, dtype=np.float64).ravel()
        assert self._walls.size == self.p.nsites
        self.L.orc_set_walls(self.h, _ptr(self._walls))

    def set_state(self, rho, u=None):
        rho = np.ascontiguousarray(rho, dtype=np.float64).ravel()
        u = None if u is None else np.ascontiguousarray(u, dtype=np.float64).ravel()
        self.L.orc_set_state(self.h, _ptr(rho), _ptr(u))

    def set_fi(self, fi):
        fi = np.ascontiguousarray(fi, dtype=np.float64).ravel()
        self.L.orc_set_fi(self.h, _ptr(fi))

    def set_species(self, conc, flux=None):
        conc = np.ascontiguousarray(conc, dtype=np.float64).ravel()
        flux = None if flux is None else np.ascontiguousarray(flux, dtype=np.float64).ravel()
        if self.L.orc_set_species(self.h, _ptr(conc), _ptr(flux)):
            raise ValueError("the parameters declare no species")

    def set_bc_values(self, face, vals):
        vals = np.ascontiguousarray(vals, dtype=np.float64).ravel()
        rc = self.L.orc_set_bc_values(self.h, int(face), _ptr(vals))
        if rc:
            raise ValueError("face %d is not a density face" % face)

    def init(self):
        self.L.orc_init(self.h)

    def step(self, n=1):
        rc = self.L.orc_step(self.h, int(n))
        if rc:
            raise RuntimeError("orc_step before orc_init")

    def get(self, field):
        n = self.L.orc_field_size(self.h, int(field))
        out = np.empty(n, dtype=np.float64)
        self.L.orc_get(self.h, int(field), _ptr(out))
        return out

    def delta_norm(self, field=P.FIELD_RHO):
        return self.L.orc_delta_norm(self.h, int(field))
