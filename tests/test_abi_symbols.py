"""The C-ABI library loads and exports every entry point include/*.h declares."""
import ctypes
import glob
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    names = []
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(tx_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared()
    for must in ("tx_create", "tx_destroy", "tx_upload_walls", "tx_upload_state", "tx_upload_fi",
                 "tx_init", "tx_step", "tx_download", "tx_delta_norm", "tx_last_error"):
        assert must in names


def test_library_exports_all_declared():
    from taxila import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("library not built (run __graft_entry__.build())")
    L = ctypes.CDLL(_lib.LIB_PATH)
    missing = [n for n in declared() if not hasattr(L, n)]
    assert not missing, missing


def test_params_struct_layout():
    # ctypes mirror matches the C struct (offset of the last field + its size)
    from taxila import params as P
    assert ctypes.sizeof(P.TxParams) == P.TxParams.species_rates.offset + 8 * 7 * P.MAXC


def test_params_default_matches_c():
    from taxila import _lib
    from taxila import params as P
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("library not built")
    L = _lib.load()
    a = P.TxParams()
    assert L.tx_params_default(ctypes.byref(a)) == 0
    b = P.default_params()
    assert bytes(a) == bytes(b)


def test_probe_struct_layout(tmp_path):
    # tx_probe as the C compiler lays it out, against the ctypes mirror
    import shutil
    import subprocess
    from taxila._lib import TxProbe
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    src = tmp_path / "probe.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "taxila_gb300.h"\n'
                   'int main(void) { printf("%zu %zu %zu %zu %zu %zu\\n", sizeof(tx_probe), offsetof(tx_probe, du_max),'
                   ' offsetof(tx_probe, u_sum), offsetof(tx_probe, pore_sites), offsetof(tx_probe, steps),'
                   ' offsetof(tx_probe, mass)); return 0; }\n')
    exe = tmp_path / "probe"
    subprocess.run([cc, "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert got == [ctypes.sizeof(TxProbe), TxProbe.du_max.offset, TxProbe.u_sum.offset,
                   TxProbe.pore_sites.offset, TxProbe.steps.offset, TxProbe.mass.offset]
