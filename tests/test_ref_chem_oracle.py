"""The reacting set's CPU oracle against the reference's own reacting solver.

tests/golden/ref_fr_plate.npz is written by tests/golden/make_ref_fixtures.py
from the reference itself (oracle/refbuild): the 5-species air mechanism of
chemModels/5speciesAir.rxn with the species data of the reference's database
builder, compressibleNSFR, second order with the modified Venkatakrishnan
limiter, finite-rate chemistry on, on a jittered 7x6x5 box with sonic inflow,
outflow, an isothermal no-slip wall (1500 K) and mirror symmetry planes
(noCVBC).  Each stage of the first two Newton steps (ucs/solutionSpace.tcc:
573-818) is fed the reference's own input for that stage:

* UpdateBCs (ucs/bc.tcc:1400, the reacting boundary variables of
  ucs/compressibleFR.tcc) - bit-identical;
* the LSQ gradient of the reacting gradient list with the symmetry fix
  (ucs/gradient.tcc:57) - bit-identical;
* the modified Venkatakrishnan limiter on the native variables
  (ucs/limiters.tcc:534) - bit-identical;
* ComputeResiduals (ucs/residual.tcc:13): HLLC inviscid flux (first order,
  then second order with the limiter), the viscous flux (averaged gradient,
  then with the directional correction), the chemistry source, the temporal
  term a steady run still adds (vol x (conservative q - conservative q_old)),
  the no-slip rows zeroed (ModifyViscousWallResidual) - to 1e-13 of the
  residual's scale (the oracle sums edge contributions node by node, the
  reference scatters them edge by edge), and the norms to 1e-13."""
import numpy as np
import pytest

import ref_fixtures as R
from chem_cases import FIXTURE
from oracle_lib import OracleChemState, OracleMesh
from proteuscfd_gb300 import Mesh
from proteuscfd_gb300 import _native as N
from proteuscfd_gb300.chem import load_mechanism, model_struct

CASE = "fr_plate"
# boundary types of ucs/bc_defines.h
NOSLIP, SONIC_INFLOW, DIRICHLET, SYMMETRY = 4, 7, 1, 9
RES_TOL = 1e-13


@pytest.fixture(scope="module")
def case():
    f = R.load(CASE)
    # the reference's set-up reorder: node n becomes ordering[n]
    el = f["elements_pre"].copy()
    o = f["ordering"]
    nodes = el[:, 3:11]
    nodes[nodes >= 0] = o[nodes[nodes >= 0]]
    xyz = np.empty_like(f["xyz_pre"])
    xyz[o] = f["xyz_pre"]
    t = el[:, 0]
    m = OracleMesh.from_elements(xyz, el[t == 0][:, 3:6], el[t == 0][:, 1], el[t == 2][:, 3:7])
    refs = f["refs"].ravel()
    # (density, pressure, temperature, specific enthalpy, velocity, viscosity, conductivity)
    S = OracleChemState(model_struct(load_mechanism(FIXTURE)), N.ChemRef(*refs[:7]))
    bct = {int(a): int(b) for a, b in f["case_bc_types"]}
    qinf = f["qinf"].ravel()
    bc = dict(bc_type=bct, twall={int(a): float(b) for a, b in f["case_twall"]},
              qref={tg: qinf for tg, b in bct.items() if b in (SONIC_INFLOW, DIRICHLET)}, no_cvbc=1)
    return f, m, S, bc


def sym_tags(bc):
    return [t for t, b in bc["bc_type"].items() if b == SYMMETRY]


def wall_nodes(f, m):
    walls = [int(t) for t, k in f["case_bc_types"] if k == NOSLIP]
    return np.unique([m.bedges[k, 0] for k in range(m.nbedge) if int(m.bfactag[k]) in walls])


def conservative(S, q):
    """NativeToConservative (ucs/compressibleFR.tcc:2117) of node records."""
    ns = S.ns
    rhoi = q[:, :ns]
    return np.c_[rhoi, S.n2c(rhoi, q[:, ns:ns + 4], q[:, ns + 4])]


def l2_norms(b):
    """ParallelL2Norm and StridedParallelL2Norm (ucs/parallel.h:162,121)."""
    return np.r_[np.sqrt((b * b).sum()) / b.size, np.sqrt((b * b).sum(axis=0)) / b.shape[0]]


def test_case_shape(case):
    f, m, S, bc = case
    assert R.scalar(f, "neqn") == S.ns + 4 == 9 and R.scalar(f, "nvars") == 6 + 3 * S.ns
    assert R.scalar(f, "sorder") == 2 and R.scalar(f, "param_limiter") == 3 and R.scalar(f, "viscous") == 1
    assert m.nnode == R.scalar(f, "nnode") and m.nedge == R.scalar(f, "nedge")


def test_mesh_matches_reference(case):
    """The oracle's preprocessing and the product's host preprocessing of the
    reference's element list equal the reacting case's maps and metrics."""
    f, m, _, _ = case
    el = f["elements_pre"]
    t = el[:, 0]
    p = Mesh.from_elements(f["xyz_pre"], el[t == 0][:, 3:6], el[t == 0][:, 1], el[t == 2][:, 3:7], reorder=True)
    for mesh in (m, p):
        for k in ("xyz", "ipsp", "psp", "edges", "bedges", "bfactag", "edge_area", "bedge_area", "vol", "sw"):
            np.testing.assert_array_equal(getattr(mesh, k), f[k], err_msg=k)
    np.testing.assert_array_equal(p.ordering, f["ordering"])


def test_boundary_update_matches_reference(case):
    """UpdateBCs as the reference runs it before each step's residual: the
    boundary pass of the step's set-up, then NewtonIterate's own.  The
    update is also idempotent on the reference's result."""
    f, m, S, bc = case
    n = m.nnode
    starts = {"s1_": f["q_init"], "s2_": np.concatenate([f["s1_q"], f["s1_q_bc"][n:]])}
    for st, q in starts.items():
        for _ in range(2):
            q, rc = S.update_bcs(m, q, **bc)
            assert rc == 0
        np.testing.assert_array_equal(q, f[st + "q_bc"], err_msg=st)
        again, _ = S.update_bcs(m, f[st + "q_bc"], **bc)
        np.testing.assert_array_equal(again, f[st + "q_bc"], err_msg=st)


def test_gradient_and_limiter_match_reference(case):
    f, m, S, bc = case
    n, nt = m.nnode, 2 * S.ns + 4
    for st in ("s1_", "s2_"):
        g = S.gradient(m, f[st + "q_bc"], sym_tags(bc))
        np.testing.assert_array_equal(g.reshape(n, nt * 3), f[st + "qgrad"], err_msg=st)
    lim = S.limiter(m, f["s2_q_bc"], f["s2_qgrad"].reshape(n, nt, 3), R.scalar(f, "chi"))
    np.testing.assert_array_equal(lim, f["s2_limiter"])
    assert 0.0 < lim.min() < 1.0  # the limiter is active somewhere


@pytest.mark.parametrize("st", ["s1_", "s2_"])
def test_residual_matches_reference(case, st):
    """ComputeResiduals of the reacting set: SpatialResidual (inviscid HLLC
    at first order on step 1, second order with the limiter on step 2;
    viscous with the directional correction once second order is on; the
    chemistry source), TemporalResidual of a steady run, the no-slip rows
    zeroed, and the reported norms."""
    f, m, S, bc = case
    n, ns = m.nnode, S.ns
    qinf = f["qinf"].ravel()
    refs = f["refs"].ravel()
    opts = N.ChemFluxOpts(1.0, float(qinf[ns + 4]), 0)  # beta, GetPressure(Qinf), no 2-D symmetry
    ref_time = float(refs[7])
    q = f[st + "q_bc"]
    g = f[st + "qgrad"].reshape(n, 2 * ns + 4, 3)
    second = st == "s2_"
    if second:
        b, _ = S.residual_ho(opts, m, q, g, f["s2_limiter"], R.scalar(f, "chi"), ref_time, 1)
        qold = np.concatenate([f["s1_q"], f["s1_q_bc"][n:]])[:n]
    else:
        b, _ = S.residual(opts, m, q, ref_time, 1)
        qold = f["q_init"][:n]
    bv, bad = S.viscous_residual(opts, m, R.scalar(f, "Re"), int(second), q, g)
    assert bad == 0
    b = b + bv
    # TemporalResidual (ucs/residual.tcc:125) with Param::dt = -1: b -= (vol / -1) (Q - Q_old)
    b += m.vol[:, None] * (conservative(S, q[:n]) - conservative(S, qold))
    b[wall_nodes(f, m), ns:ns + 4] = 0.0
    ref_b = f[st + "b"]
    scale = np.abs(ref_b).max()
    assert np.abs(b - ref_b).max() <= RES_TOL * scale, np.abs(b - ref_b).max() / scale
    ref_n = f[st + "norms"].ravel()
    np.testing.assert_allclose(l2_norms(b), ref_n, rtol=RES_TOL, atol=0)
