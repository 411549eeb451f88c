"""Measured arithmetic-pipe ceilings of the GPU (libtx_peaks.so).

The FP64 step kernels are bound by the FP64 pipe, not by HBM, so their
roofline needs a measured FP64 instruction rate beside the measured copy
bandwidth.  ``pipe_rates`` times long chains of independent DFMA, DADD and
DMUL (and FP32 FFMA, scalar and packed pairs) over the whole GPU with CUDA
events and returns operations per second; ``per_sm_cycle`` converts a rate
to lanes per SM per clock with a sampled SM clock.
"""
import ctypes as C
import os

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_ROOT, "libtx_peaks.so")
OPS = {"dfma": 0, "dadd": 1, "dmul": 2, "ffma": 3, "ffma2": 4}

_lib = None


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libtx_peaks.so not found at %s: run __graft_entry__.build() first" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        L.txp_pipe_rate.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.txp_pipe_rate.restype = C.c_int
        _lib = L
    return _lib


def pipe_rate(op, blocks, iters, reps=5):
    """(ms per launch, operations per second) of one probe."""
    ms, ops = C.c_double(), C.c_double()
    rc = _load().txp_pipe_rate(OPS[op], int(blocks), int(iters), int(reps), C.byref(ms), C.byref(ops))
    if rc:
        raise RuntimeError("txp_pipe_rate(%s) failed with CUDA error %d" % (op, rc))
    return ms.value, ops.value / (ms.value * 1e-3)


def pipe_rates(sms, blocks_per_sm=8, target_ms=40.0):
    """Operations per second of every probe, each sized to run about
    ``target_ms`` per launch (first a short launch to calibrate)."""
    out = {}
    blocks = sms * blocks_per_sm
    for op in OPS:
        ms, _ = pipe_rate(op, blocks, 256, reps=2)
        iters = max(256, int(256 * target_ms / max(ms, 1e-3)))
        ms, rate = pipe_rate(op, blocks, iters, reps=5)
        out[op] = {"ops_per_s": rate, "ms_per_launch": ms, "iters": iters, "blocks": blocks}
    return out


def per_sm_cycle(rate, sms, sm_mhz):
    return rate / (sms * sm_mhz * 1e6)
