"""The lattice tables of the library and of the oracle against the reference source.

Direction velocities, weights, the MRT transform M^T, diag(M M^T), the moment
-> rate map and the isotropy weights of the Shan-Chen gradient are read from
the reference's DiscretizationSetup_D3Q19 / _D2Q9 and DiscretizationSetupRelax
(src/lbm/lbm_discretization_d3q19.F90:64-263, lbm_discretization_d2q9.F90:
53-166) and compared with the tables the library compiles (csrc/tx_lattice.cuh,
tx_host_params.h, dumped by the host emulation) and those of the oracle.  A
transposed moment row, a swapped rate or a mistyped weight fails here even
where no golden output of the reference covers that table (D3Q19, MRT,
isotropy 8).  Needs the reference tree; skipped without it.
"""
import ctypes as C
import json
import os
import re
import subprocess
import sys

import numpy as np
import pytest

import cases
from oracle import lib as oracle_lib
from taxila import params as P

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "hostemu"))
import build_emu  # noqa: E402

SRC = {3: os.path.join(cases.REF, "src/lbm/lbm_discretization_d3q19.F90"),
       2: os.path.join(cases.REF, "src/lbm/lbm_discretization_d2q9.F90")}
SETUP = {3: ("DiscretizationSetup_D3Q19", "DiscretizationSetupRelax_D3Q19"),
         2: ("DiscretizationSetUp_D2Q9", "DiscretizationSetUpRelax_D2Q9")}
RATE_VALUE = {"s_c": 1.01, "s_e": 1.02, "s_e2": 1.03, "s_q": 1.04, "s_nu": 1.05, "s_pi": 1.06, "s_m": 1.07}
ISOTROPY = {3: (4, 8), 2: (4, 8, 10)}


def _subroutine(text, name):
    start = re.search(r"subroutine\s+%s\b" % name, text, re.I).start()
    end = re.search(r"end\s+subroutine\s+%s\b" % name, text[start:], re.I).end() + start
    body = text[start:end]
    body = re.sub(r"!.*", "", body)           # comments
    return re.sub(r"&\s*\n\s*", " ", body)     # continuation lines


def _fnum(s):
    """A Fortran numeric expression of literals (1.d0/36.d0, 4.d0/45., 8)."""
    s = s.strip().lower().replace("d0", "e0")
    if not re.fullmatch(r"[-+0-9.e/ ]+", s):
        raise ValueError("unexpected expression %r" % s)
    return float(eval(s))  # literals and one division only (checked above)


def reference_tables(D):
    text = open(SRC[D]).read()
    setup, relax = (_subroutine(text, n) for n in SETUP[D])
    axes = "XYZ"[:D]
    ci = {}
    for a in axes:
        m = re.search(r"disc%%ci\(:,\s*%s_DIRECTION\)\s*=\s*\(/(.*?)/\)" % a, setup)
        ci[a] = [int(v) for v in m.group(1).split(",")]
    Q = len(ci["X"])
    c = np.zeros((Q, 3), dtype=int)
    for i, a in enumerate(axes):
        c[:, i] = ci[a]
    w = np.array([_fnum(v) for v in re.search(r"disc%weights\s*=\s*\(/(.*?)/\)", setup).group(1).split(",")])
    mt = np.zeros((Q, Q), dtype=int)
    for m in re.finditer(r"disc%mt_mrt\(:,\s*(\d+)\)\s*=\s*(\(/(.*?)/\)|disc%ci\(:,\s*([XYZ])_DIRECTION\))", setup):
        k = int(m.group(1))
        mt[:, k] = [int(v) for v in m.group(3).split(",")] if m.group(3) else ci[m.group(4)]
    mmt = np.array([int(v) for v in re.search(r"disc%mmt_mrt\s*=\s*\(/(.*?)/\)", setup).group(1).split(",")])
    ffw = {}
    for m in re.finditer(r"if\s*\(\s*disc%isotropy_order\s*\.eq\.\s*(\d+)\s*\)\s*then(.*?)end\s*if", setup, re.S | re.I):
        t = np.zeros(12)
        for a in re.finditer(r"disc%ffw\(\s*(\d+)\s*\)\s*=\s*([^\n]+)", m.group(2)):
            if int(a.group(1)) < 12:
                t[int(a.group(1))] = _fnum(a.group(2))
        ffw[int(m.group(1))] = t
    rate = np.zeros(Q)
    for m in re.finditer(r"relax%tau_mrt\((\d+)\)\s*=\s*relax%(s_\w+)", relax):
        rate[int(m.group(1))] = RATE_VALUE[m.group(2)]
    return {"ci": c, "w": w, "mt": mt, "mmt": mmt, "ffw": ffw, "rate": rate}


def library_tables(D, iso):
    exe = build_emu.build()
    r = subprocess.run([exe, "lattice", str(D), str(iso)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout)


def oracle_tables(D, iso):
    L = oracle_lib()
    L.orc_lattice.argtypes = [C.POINTER(P.TxParams)] + [C.c_void_p] * 6
    p = cases.base(P.D3Q19 if D == 3 else P.D2Q9, (4, 4, 4) if D == 3 else (1, 4, 4), ncomp=1, mode=P.MRT, iso=iso)
    for name, v in RATE_VALUE.items():
        getattr(p, name)[0] = v
    Q = 19 if D == 3 else 9
    ci, mt, mmt = (np.zeros(n, dtype=np.int32) for n in (Q * 3, Q * Q, Q))
    w, ffw, rate = np.zeros(Q), np.zeros(12), np.zeros(Q)
    assert L.orc_lattice(C.byref(p), *(a.ctypes.data for a in (ci, w, mt, mmt, ffw, rate))) == 0
    return {"ci": ci.reshape(Q, 3), "w": w, "mt": mt.reshape(Q, Q), "mmt": mmt, "ffw": ffw, "rate": rate}


@pytest.mark.parametrize("D", [3, 2], ids=["d3q19", "d2q9"])
def test_lattice_tables_match_reference(D):
    if not os.path.exists(SRC[D]):
        pytest.skip("reference tree not present")
    ref = reference_tables(D)
    assert len(ref["ffw"]) >= len(ISOTROPY[D])
    for iso in ISOTROPY[D]:
        for who, got in (("library", library_tables(D, iso)), ("oracle", oracle_tables(D, iso))):
            assert np.array_equal(np.array(got["ci"]), ref["ci"]), (who, "ci")
            assert np.array_equal(np.array(got["w"]), ref["w"]), (who, "weights")
            assert np.array_equal(np.array(got["mt"]), ref["mt"]), (who, "M^T")
            assert np.array_equal(np.array(got["mmt"]), ref["mmt"]), (who, "diag(M M^T)")
            assert np.array_equal(np.array(got["rate"]), ref["rate"]), (who, "rate map")
            assert np.array_equal(np.array(got["ffw"]), ref["ffw"][iso]), (who, "isotropy %d weights" % iso)


def test_mrt_basis_is_orthogonal():
    # without the reference: the committed M^T has orthogonal columns with the
    # committed diag(M M^T), and its moment 0 is the density
    for D in (3, 2):
        t = library_tables(D, 4)
        mt = np.array(t["mt"])
        assert np.array_equal(mt.T @ mt, np.diag(t["mmt"]))
        assert np.all(mt[:, 0] == 1)


def test_abi_constants_match_reference():
    # the boundary-condition kinds and relaxation modes cross the C ABI as the
    # reference's own integer codes (include/lbm_definitions.h)
    defs = os.path.join(cases.REF, "include/lbm_definitions.h")
    if not os.path.exists(defs):
        pytest.skip("reference tree not present")
    ref = {m.group(1): int(m.group(2))
           for m in re.finditer(r"PetscInt,\s*parameter\s*::\s*(\w+)\s*=\s*(-?\d+)", open(defs).read())}
    header = open(os.path.join(os.path.dirname(HERE), "include", "taxila_gb300.h")).read()
    ours = {m.group(1): int(m.group(2)) for m in re.finditer(r"#define\s+TX_(BC_\w+|RELAX_\w+)\s+(-?\d+)", header)}
    names = {k: ("RELAXATION_MODE_" + k[6:] if k.startswith("RELAX_") else k) for k in ours}
    assert len(ours) >= 14
    for k, v in ours.items():
        assert ref[names[k]] == v, (k, v, ref.get(names[k]))
