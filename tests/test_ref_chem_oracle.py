"""The reacting set's CPU oracle against the reference's own reacting solver.

tests/golden/ref_fr_plate.npz is written by tests/golden/make_ref_fixtures.py
from the reference itself (oracle/refbuild): the 5-species air mechanism of
chemModels/5speciesAir.rxn with the species data of the reference's database
builder, compressibleNSFR, second order with the modified Venkatakrishnan
limiter, finite-rate chemistry on, partly dissociated air at 3000 K (mass
fractions O2 0.2, O 0.01, N 0.01, N2 0.745, NO 0.035), on a jittered 7x6x5
box with sonic inflow,
outflow, an isothermal no-slip wall (1500 K) and mirror symmetry planes
(noCVBC).  Each stage of the first two Newton steps is fed the reference's
own input for that stage (tests/ref_chem_stages.py):

* UpdateBCs, the reacting LSQ gradient and the limiter with its pressure
  clip (Kernel_PressureClip zeroes 12 nodes' limiters here) - bit-identical;
* ComputeResiduals (HLLC at first and second order, viscous, chemistry
  source, the steady temporal term, the no-slip rows) and its norms - to
  1e-13 of their scale: the oracle sums each node's edge contributions, the
  reference scatters them edge by edge, so only the summation order differs."""
import numpy as np
import pytest

import ref_chem_stages as RC
import ref_fixtures as R
from proteuscfd_gb300 import Mesh

RES_TOL = 1e-13


@pytest.fixture(scope="module")
def case():
    f, bc, ref = RC.load()
    return f, bc, RC.OracleEngine(f, ref)


def test_case_shape(case):
    f, _, E = case
    assert R.scalar(f, "neqn") == E.ns + 4 == 9 and R.scalar(f, "nvars") == 6 + 3 * E.ns
    assert R.scalar(f, "sorder") == 2 and R.scalar(f, "param_limiter") == 3 and R.scalar(f, "viscous") == 1
    assert E.mesh.nnode == R.scalar(f, "nnode") and E.mesh.nedge == R.scalar(f, "nedge")


def test_mesh_matches_reference(case):
    """The oracle's preprocessing and the product's host preprocessing of the
    reference's element list equal the reacting case's maps and metrics."""
    f, _, E = case
    el = f["elements_pre"]
    t = el[:, 0]
    p = Mesh.from_elements(f["xyz_pre"], el[t == 0][:, 3:6], el[t == 0][:, 1], el[t == 2][:, 3:7], reorder=True)
    for mesh in (E.mesh, p):
        for k in ("xyz", "ipsp", "psp", "edges", "bedges", "bfactag", "edge_area", "bedge_area", "vol", "sw"):
            np.testing.assert_array_equal(getattr(mesh, k), f[k], err_msg=k)
    np.testing.assert_array_equal(p.ordering, f["ordering"])


def test_stages_match_reference(case):
    f, bc, E = case
    seen = set()
    for name, kind, got, want in RC.stages(E, f, bc):
        seen.add(name)
        if kind in ("state", "gradient", "limiter"):
            np.testing.assert_array_equal(got, want, err_msg=name)
        else:
            scale = np.abs(want).max()
            assert np.abs(got - want).max() <= RES_TOL * scale, (name, np.abs(got - want).max() / scale)
    assert {"s1_q_bc", "s1_qgrad", "s1_b", "s1_norms", "s2_q_bc", "s2_qgrad", "s2_limiter", "s2_b",
            "s2_norms"} <= seen
    lim = f["s2_limiter"]
    assert np.any((lim > 0.0) & (lim < 1.0))  # the limiter is active somewhere
    # and the pressure clip zeroed some nodes whole, which the unclipped limiter does not
    n, nt = E.mesh.nnode, 2 * E.ns + 4
    raw = E.limiter_noclip(f["s2_q_bc"], f["s2_qgrad"].reshape(n, nt, 3), R.scalar(f, "chi"))
    clipped = np.all(lim == 0.0, axis=1) & ~np.all(raw == 0.0, axis=1)
    assert clipped.sum() > 0


def test_boundary_update_is_idempotent_on_reference_state(case):
    f, bc, E = case
    for st in ("s1_", "s2_"):
        np.testing.assert_array_equal(E.update_bcs(f[st + "q_bc"], bc), f[st + "q_bc"], err_msg=st)


def test_timestep_matches_reference(case):
    """ComputeTimesteps of the reacting set (MaxEigenvalue with the mixture's
    frozen speed of sound, beta = 1 above Mach 1) with local time stepping:
    at PreIterate on the initial state, and at PreTimeAdvance on the state
    after the set-up's boundary pass - bit-identical, with dtmin."""
    f, bc, E = case
    cfl = R.scalar(f, "case_cfl")
    assert R.scalar(f, "velocity") > 1.0  # the reference's beta field is then 1 everywhere
    dt0, _ = E.S.timestep(E.mesh, f["q_init"], 1.0, cfl)
    np.testing.assert_array_equal(dt0, f["dt_preiterate"])
    dt1, dtmin = E.S.timestep(E.mesh, E.update_bcs(f["q_init"], bc), 1.0, cfl)
    np.testing.assert_array_equal(dt1, f["dt"])
    assert dtmin == R.scalar(f, "dtmin")
