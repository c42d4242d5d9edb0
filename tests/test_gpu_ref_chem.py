"""The CUDA reacting path against the reference's own reacting solver: the
stages of tests/ref_chem_stages.py (boundary update, LSQ gradient, limiter,
residual with viscous terms, chemistry source, temporal term and no-slip
rows, and its norms) computed by the GPU kernels through the C ABI, each fed
the reference's input for that stage, against tests/golden/ref_fr_plate.npz.

Tolerances are those of the GPU-against-oracle tests: the GPU's exp, log and
pow differ from the host's libm by an ulp or so, and the GPU sums each
node's contributions in its own fixed order."""
import numpy as np
import pytest

import ref_chem_stages as RC

pytestmark = pytest.mark.gpu

TOL = {"state": 1e-13, "gradient": 1e-13, "limiter": 1e-12, "residual": 1e-11, "norms": 1e-11}


def test_gpu_stages_match_reference():
    f, bc, ref = RC.load()
    E = RC.ProductEngine(f, ref)
    try:
        seen = set()
        for name, kind, got, want in RC.stages(E, f, bc):
            seen.add(name)
            got = np.asarray(got, dtype=np.float64)
            if kind in ("state", "gradient"):
                # per column: each variable against its own scale
                scale = np.abs(want).max(axis=0, keepdims=True)
                scale[scale == 0] = 1.0
                err = (np.abs(got - want) / scale).max()
            elif kind == "limiter":
                err = np.abs(got - want).max()
            else:
                err = np.abs(got - want).max() / np.abs(want).max()
            assert err <= TOL[kind], (name, err)
        assert len(seen) == 9
    finally:
        E.close()
