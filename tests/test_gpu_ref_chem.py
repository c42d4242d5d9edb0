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


def clipped_nodes(f, bc, ref):
    """Nodes whose limiter the reference's pressure clip zeroed on step 2
    (the oracle's limiter with and without Kernel_PressureClip), and the
    oracle's limiter without the clip."""
    import ref_fixtures as R
    O = RC.OracleEngine(f, ref)
    n, nt = O.mesh.nnode, 2 * O.ns + 4
    q, g, chi = f["s2_q_bc"], f["s2_qgrad"].reshape(n, nt, 3), R.scalar(f, "chi")
    with_clip, without = O.limiter(q, g, chi), O.limiter_noclip(q, g, chi)
    rows = np.all(with_clip == 0.0, axis=1) & ~np.all(without == 0.0, axis=1)
    return rows, without


def test_gpu_stages_match_reference():
    f, bc, ref = RC.load()
    clipped, noclip = clipped_nodes(f, bc, ref)
    E = RC.ProductEngine(f, ref)
    try:
        seen = set()
        for name, kind, got, want in RC.stages(E, f, bc):
            seen.add(name)
            got = np.asarray(got, dtype=np.float64)
            if kind == "limiter":
                # the CUDA limiter has no reacting pressure clip: the reference's
                # limiter where the clip left a node alone, the oracle's
                # unclipped limiter where it did not
                assert np.abs(got[~clipped] - want[~clipped]).max() <= TOL[kind], name
                assert np.abs(got[clipped] - noclip[clipped]).max() <= TOL[kind], name
                continue
            if kind in ("state", "gradient"):
                # per column: each variable against its own scale
                scale = np.abs(want).max(axis=0, keepdims=True)
                scale[scale == 0] = 1.0
                err = (np.abs(got - want) / scale).max()
            else:
                err = np.abs(got - want).max() / np.abs(want).max()
            assert err <= TOL[kind], (name, err)
        assert len(seen) == 9
    finally:
        E.close()
