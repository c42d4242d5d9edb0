"""The C-ABI library loads and exports every symbol include/pcfd.h declares;
argument checks fail cleanly without touching the GPU."""
import ctypes as C
import re
from pathlib import Path

import pytest

from proteuscfd_gb300 import _native as N

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        for m in re.finditer(r"PCFD_API\s+[^;(]*?\b(pcfd_\w+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "pcfd_create" in names and "pcfd_residual" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(str(N.LIB_PATH))
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing


def test_bindings_cover_header():
    assert declared_symbols() <= set(N.PROTOTYPES), declared_symbols() - set(N.PROTOTYPES)


def test_build_info_and_errors_without_gpu():
    lib = N.load()
    assert b"sm_103a" in lib.pcfd_build_info()
    h = C.c_void_p()
    assert lib.pcfd_create(None, None, C.byref(h)) == 1  # PCFD_ERR_ARG
    assert b"null" in lib.pcfd_last_error()
    assert lib.pcfd_update_bcs(None) == 1
    assert lib.pcfd_residual(None, None, None) == 1


def test_create_rejects_out_of_range_maps():
    from proteuscfd_gb300 import Mesh, Param
    m = Mesh.box(3, 3, 3)
    v = N.MeshView()
    C.memmove(C.byref(v), C.byref(m.view), C.sizeof(v))
    import numpy as np
    bad = m.edges.copy()
    bad[0, 1] = m.nnode + 5
    bad = np.ascontiguousarray(bad.reshape(-1))
    v.edges = N.iptr(bad)
    p = Param(bc_type={t: N.BC_FARFIELD for t in range(1, 7)}).to_c()
    h = C.c_void_p()
    assert N.load().pcfd_create(C.byref(v), C.byref(p), C.byref(h)) == 1
    assert b"out of range" in N.load().pcfd_last_error()
