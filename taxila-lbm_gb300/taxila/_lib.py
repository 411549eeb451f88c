"""ctypes binding of libtaxila_gb300.so (include/taxila_gb300.h).

The library is the compute path; there is no fallback.  Loading fails with
an error that names the missing file when it has not been built.
"""
import ctypes as C
import os

import numpy as np

from . import params as P

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_ROOT, "libtaxila_gb300.so")

_lib = None


class TxProbe(C.Structure):
    """tx_probe of include/taxila_gb300.h."""
    _fields_ = [("id", C.c_int32), ("pad_", C.c_int32), ("du_max", C.c_double), ("u_max", C.c_double),
                ("u_sum", C.c_double * 3), ("pore_sites", C.c_int64), ("steps", C.c_int64),
                ("mass", C.c_double * P.MAXC)]


class TxError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (P.ERR_NAMES.get(code, "TX_ERR_%d" % code), msg))
        self.code = code


def load():
    """Load the CUDA library (build it with taxila-lbm_gb300/build.py)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libtaxila_gb300.so not found at %s: run __graft_entry__.build() "
                          "(or python taxila-lbm_gb300/build.py) first" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    vp, i32, i64, dp = C.c_void_p, C.c_int32, C.c_int64, C.POINTER(C.c_double)
    sig = {
        "tx_params_default": ([C.POINTER(P.TxParams)], C.c_int),
        "tx_create": ([C.POINTER(P.TxParams), C.POINTER(vp)], C.c_int),
        "tx_destroy": ([vp], C.c_int),
        "tx_last_error": ([vp], C.c_char_p),
        "tx_upload_walls": ([vp, dp], C.c_int),
        "tx_upload_state": ([vp, dp, dp], C.c_int),
        "tx_upload_fi": ([vp, dp], C.c_int),
        "tx_upload_species": ([vp, dp, dp], C.c_int),
        "tx_upload_bc_values": ([vp, i32, dp], C.c_int),
        "tx_init": ([vp], C.c_int),
        "tx_step": ([vp, i32], C.c_int),
        "tx_step_species": ([vp, i32], C.c_int),
        "tx_delta_norm": ([vp, i32, dp], C.c_int),
        "tx_download": ([vp, i32, dp], C.c_int),
        "tx_conservation": ([vp, dp], C.c_int),
        "tx_field_size": ([vp, i32], i64),
        "tx_sync": ([vp], C.c_int),
        "tx_set_timing": ([vp, i32], C.c_int),
        "tx_get_timing": ([vp, dp, dp, C.POINTER(i64)], C.c_int),
        "tx_get_stream": ([vp], vp),
        "tx_kernel_name": ([vp], C.c_char_p),
        "tx_step_static": ([C.POINTER(P.TxParams), vp, vp, vp, i32, vp], C.c_int),
        "tx_batch_create": ([C.POINTER(P.TxParams), i64, C.POINTER(vp)], C.c_int),
        "tx_batch_destroy": ([vp], C.c_int),
        "tx_batch_last_error": ([vp], C.c_char_p),
        "tx_batch_lattice_bytes": ([C.POINTER(P.TxParams)], i64),
        "tx_batch_bytes_in_use": ([vp], i64),
        "tx_batch_count": ([vp], i32),
        "tx_batch_add": ([vp, C.POINTER(P.TxParams), dp, dp, dp, dp, C.POINTER(i32)], C.c_int),
        "tx_batch_remove": ([vp, i32], C.c_int),
        "tx_batch_step": ([vp, i32], C.c_int),
        "tx_batch_launch": ([vp, i32], C.c_int),
        "tx_batch_sync": ([vp], C.c_int),
        "tx_batch_probe": ([vp, i32, C.POINTER(TxProbe), C.POINTER(i32)], C.c_int),
        "tx_batch_download": ([vp, i32, i32, dp], C.c_int),
        "tx_batch_set_tiles": ([vp, i32, i32, i32, i32], C.c_int),
        "tx_batch_tune": ([vp, i32, C.POINTER(i32)], C.c_int),
        "tx_batch_set_graph": ([vp, i32], C.c_int),
        "tx_batch_stream": ([vp], vp),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64).ravel()


def step_static(params, walls_dev, fi_in_dev, fi_out_dev, nsteps, stream=None):
    """tx_step_static on caller-owned device arrays (addresses as ints)."""
    L = load()
    p = P.copy_params(params)
    rc = L.tx_step_static(C.byref(p), C.c_void_p(walls_dev), C.c_void_p(fi_in_dev), C.c_void_p(fi_out_dev),
                          int(nsteps), C.c_void_p(stream) if stream else None)
    if rc:
        raise TxError(rc, L.tx_last_error(None).decode())


class Handle:
    """One tx_handle: a lattice resident on the GPU."""

    def __init__(self, params):
        self.L = load()
        self.p = P.copy_params(params)
        h = C.c_void_p()
        rc = self.L.tx_create(C.byref(self.p), C.byref(h))
        if rc:
            raise TxError(rc, self.L.tx_last_error(None).decode())
        self.h = h

    def _check(self, rc):
        if rc:
            raise TxError(rc, self.L.tx_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.L.tx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload_walls(self, walls):
        w = f64(walls)
        assert w.size == self.p.nsites
        self._check(self.L.tx_upload_walls(self.h, dptr(w)))

    def upload_state(self, rho, u=None):
        r, v = f64(rho), f64(u)
        self._check(self.L.tx_upload_state(self.h, dptr(r), dptr(v)))

    def upload_species(self, conc, flux=None):
        c, f = f64(conc), f64(flux)
        self._check(self.L.tx_upload_species(self.h, dptr(c), dptr(f)))

    def upload_fi(self, fi):
        f = f64(fi)
        self._check(self.L.tx_upload_fi(self.h, dptr(f)))

    def upload_bc_values(self, face, vals):
        v = f64(vals)
        self._check(self.L.tx_upload_bc_values(self.h, int(face), dptr(v)))

    def init(self):
        self._check(self.L.tx_init(self.h))

    def step(self, n=1):
        self._check(self.L.tx_step(self.h, int(n)))

    def step_species(self, n=1):
        """Transport only: the steady-flow mode's step."""
        self._check(self.L.tx_step_species(self.h, int(n)))

    def sync(self):
        self._check(self.L.tx_sync(self.h))

    def download(self, field, out=None):
        n = self.L.tx_field_size(self.h, int(field))
        if out is None:
            out = np.empty(n, dtype=np.float64)
        assert out.size == n and out.dtype == np.float64 and out.flags.c_contiguous
        self._check(self.L.tx_download(self.h, int(field), dptr(out)))
        return out

    def delta_norm(self, field=P.FIELD_RHO):
        v = C.c_double()
        self._check(self.L.tx_delta_norm(self.h, int(field), C.byref(v)))
        return v.value

    def conservation(self):
        """Global (mass[s], momentum[s][ndims]) of the current state, FP64 sums on the device."""
        s, d = self.p.ncomponents, self.p.ndims
        out = np.empty(s + s * d, dtype=np.float64)
        self._check(self.L.tx_conservation(self.h, dptr(out)))
        return out[:s].copy(), out[s:].reshape(s, d).copy()

    def set_timing(self, on=True):
        self._check(self.L.tx_set_timing(self.h, 1 if on else 0))

    def timing(self):
        a, b, n = C.c_double(), C.c_double(), C.c_int64()
        self._check(self.L.tx_get_timing(self.h, C.byref(a), C.byref(b), C.byref(n)))
        return a.value, b.value, n.value

    def stream(self):
        return self.L.tx_get_stream(self.h)

    def kernel_name(self):
        return self.L.tx_kernel_name(self.h).decode()


class Batch:
    """One tx_batch: many lattices of one kernel form stepped together."""

    def __init__(self, form, hbm_budget_bytes=0):
        self.L = load()
        self.form = P.copy_params(form)
        b = C.c_void_p()
        rc = self.L.tx_batch_create(C.byref(self.form), int(hbm_budget_bytes), C.byref(b))
        if rc:
            raise TxError(rc, self.L.tx_last_error(None).decode())
        self.b = b

    def _check(self, rc):
        if rc:
            raise TxError(rc, self.L.tx_batch_last_error(self.b).decode())

    def close(self):
        if getattr(self, "b", None):
            self.L.tx_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def lattice_bytes(params):
        p = P.copy_params(params)
        return load().tx_batch_lattice_bytes(C.byref(p))

    def bytes_in_use(self):
        return self.L.tx_batch_bytes_in_use(self.b)

    def count(self):
        return self.L.tx_batch_count(self.b)

    def add(self, params, walls, rho, u=None, conc=None):
        p = P.copy_params(params)
        w, r, v, c = f64(walls), f64(rho), f64(u), f64(conc)
        lid = C.c_int32()
        self._check(self.L.tx_batch_add(self.b, C.byref(p), dptr(w), dptr(r), dptr(v), dptr(c), C.byref(lid)))
        return lid.value

    def remove(self, lid):
        self._check(self.L.tx_batch_remove(self.b, int(lid)))

    def step(self, n=1):
        self._check(self.L.tx_batch_step(self.b, int(n)))

    def launch(self, n=1):
        """Queue n steps on the batch's stream without waiting."""
        self._check(self.L.tx_batch_launch(self.b, int(n)))

    def sync(self):
        self._check(self.L.tx_batch_sync(self.b))

    def probe(self):
        """{id: TxProbe} for every lattice in the batch."""
        cap = max(1, self.count())
        arr = (TxProbe * cap)()
        n = C.c_int32()
        self._check(self.L.tx_batch_probe(self.b, cap, arr, C.byref(n)))
        return {arr[i].id: arr[i] for i in range(min(n.value, cap))}

    def download(self, lid, field, size):
        out = np.empty(size, dtype=np.float64)
        self._check(self.L.tx_batch_download(self.b, int(lid), int(field), dptr(out)))
        return out

    def set_tiles(self, bx, by, bz, blocks_per_sm):
        self._check(self.L.tx_batch_set_tiles(self.b, bx, by, bz, blocks_per_sm))

    def tune(self, steps_per_trial=4):
        ch = (C.c_int32 * 4)()
        self._check(self.L.tx_batch_tune(self.b, int(steps_per_trial), ch))
        return tuple(ch)

    def set_graph(self, steps_per_graph):
        self._check(self.L.tx_batch_set_graph(self.b, int(steps_per_graph)))

    def stream(self):
        return self.L.tx_batch_stream(self.b)
