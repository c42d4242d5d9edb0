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


@pytest.mark.skipif(not (REF and (Path(REF) / "ucs" / "chem.h").exists()),
                    reason="PCFD_REFERENCE_SRC names no reference checkout")
def test_shim_reacting_model_equals_product_model(tmp_path):
    """pcfd_shim::ChemModelFrom run on the reference's own ChemModel (built by
    its constructor from chemModels/5speciesAir.rxn and the species database
    its builder extracts, oracle/refbuild/chem_shim_dump.cpp) gives, field for
    field and bit for bit, the pcfd_chem_model the product builds from the
    mechanism fixture."""
    import sys
    sys.path.insert(0, str(ROOT / "tests" / "golden"))
    import make_ref_fixtures as MRF
    from chem_cases import FIXTURE
    from proteuscfd_gb300.chem import load_mechanism, model_struct
    r = subprocess.run(["make", "-C", str(ROOT / "oracle" / "refbuild"), "REF=%s" % REF, "chem-shim-dump"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    (tmp_path / "air.rxn").write_text((Path(REF) / "chemModels" / "5speciesAir.rxn").read_text())
    MRF.write_chem_db(tmp_path / "chemdb.txt", FIXTURE)
    out = subprocess.run([str(ROOT / "oracle" / "_ref" / "chem_shim_dump"), str(tmp_path), "air"], cwd=tmp_path,
                         capture_output=True, text=True)
    assert out.returncode == 0, out.stderr[-3000:]
    got = {}
    for line in out.stdout.splitlines():
        if line.startswith("PCFD "):
            f = line.split()[1:]
            got[(f[0],) + tuple(int(x) for x in f[1:-1])] = float(f[-1])
    m = model_struct(load_mechanism(FIXTURE))
    want = {("nspecies",): m.nspecies, ("nreactions",): m.nreactions}
    for k in range(m.nspecies):
        want[("mw", k)] = m.mw[k]
        want[("nmu", k)], want[("nk", k)] = m.nmu[k], m.nk[k]
        for i in range(7):
            want[("nasa_lo", k, i)], want[("nasa_hi", k, i)] = m.nasa_lo[k][i], m.nasa_hi[k][i]
        for r_ in range(m.nmu[k]):
            for i in range(6):
                want[("mu_fit", k, r_, i)] = m.mu_fit[k][r_][i]
        for r_ in range(m.nk[k]):
            for i in range(6):
                want[("k_fit", k, r_, i)] = m.k_fit[k][r_][i]
    for j in range(m.nreactions):
        c = m.rx[j]
        for key, v in (("type", c.type), ("A", c.A), ("EA", c.EA), ("n", c.n), ("third_bodies", c.third_bodies),
                       ("nlocal", c.nlocal)):
            want[(key, j)] = v
        for l in range(c.nlocal):
            want[("global", j, l)] = c.global_[l]
            want[("nup", j, l)], want[("nupp", j, l)], want[("tbeff", j, l)] = c.nup[l], c.nupp[l], c.tbeff[l]
    assert set(got) == set(want)
    bad = [(k, got[k], want[k]) for k in want if got[k] != float(want[k])]
    assert not bad, bad[:10]
