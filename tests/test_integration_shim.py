"""The reference-side binding (include/ucs_shim/pcfd_shim.h) compiles against
the reference's own headers, every function instantiated for its solver type,
and every C entry point it calls is exported by libpcfd.so.

The compile needs a checkout of the reference named by PCFD_REFERENCE_SRC;
the symbol check runs everywhere."""
import ctypes as C
import os
import re
import subprocess
from pathlib import Path

import pytest

from proteuscfd_gb300 import _native as N

ROOT = Path(__file__).resolve().parent.parent
SHIM = ROOT / "include" / "ucs_shim" / "pcfd_shim.h"
REF = os.environ.get("PCFD_REFERENCE_SRC")


def test_shim_calls_only_exported_entry_points():
    calls = set(re.findall(r"\b(pcfd_[a-z_0-9]+)\s*\(", SHIM.read_text()))
    assert {"pcfd_create", "pcfd_residual", "pcfd_newton_step"} <= calls
    lib = C.CDLL(str(N.LIB_PATH))
    assert not [c for c in sorted(calls) if not hasattr(lib, c)]


@pytest.mark.skipif(not (REF and (Path(REF) / "ucs" / "solutionSpace.h").exists()),
                    reason="PCFD_REFERENCE_SRC names no reference checkout")
def test_shim_compiles_against_reference_headers():
    r = subprocess.run(["make", "-C", str(ROOT / "oracle" / "refbuild"), "REF=%s" % REF, "shim-check"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
