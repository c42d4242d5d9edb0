"""CUDA residual path against the CPU oracle, through the C ABI.

Small seeded meshes of each workload family, compared stage by stage
(boundary update, LSQ gradient, limiter, residual and norms), plus
determinism and size-independent properties at full size."""
import numpy as np
import pytest

from oracle_lib import OracleSpace
from parity import assert_field_close, assert_residual_close
from proteuscfd_gb300 import Param, SolutionSpace, cases
from proteuscfd_gb300 import _native as N

pytestmark = pytest.mark.gpu

SMALL = [
    cases.euler_ramp(12, 8, 8, seed=4),
    cases.ns_flatplate(12, 10, 8, seed=5, venkat_K=1.0),   # the reference's hard-coded K
    cases.ns_flatplate(11, 9, 9, seed=6, venkat_K=5.0),    # K = 5 extension
]


def run_both(case, state="smooth", seed=0):
    m = cases.build_mesh(case)
    S = SolutionSpace(m, case.param)
    O = OracleSpace(m, case.param)
    nrows = m.nnode + m.nbedge
    if state == "smooth":
        q0 = cases.smooth_state(m, S.qinf(), nrows)
    else:
        q0 = cases.perturbed_state(S.qinf(), nrows, seed)
    return m, S, O, q0


@pytest.mark.parametrize("case", SMALL, ids=lambda c: c.name + "_K%g" % c.param.venkat_K)
@pytest.mark.parametrize("state", ["smooth", "perturbed"])
def test_stagewise_parity(case, state):
    m, S, O, q0 = run_both(case, state, seed=11)
    S.set_state(q0)
    S.update_bcs()
    qg = S.get_state()
    qo = O.update_bcs(q0)
    assert_field_close(qg, qo, 1e-13, "q after UpdateBCs")
    p = case.param
    g = l = None
    if p.sorder > 1 or p.viscous:
        gg = S.gradient()
        g = O.gradient(qo)
        assert_field_close(gg, g, 1e-12, "LSQ gradient")
    if p.sorder > 1:
        lg = S.limiter()
        l, nclip = O.limiter(qo, g)
        assert nclip == 0
        assert np.abs(lg - l).max() <= 1e-12
    bg, ng = S.compute_residuals()
    bo, no, kc = O.residual(qo, g, l, qold=q0)  # set_state makes q0 the step's q_old
    assert kc == 0
    assert_residual_close(bg, bo, O.last_babs)
    assert np.allclose(ng, no, rtol=1e-12, atol=0)
    h = S.health()
    assert h[0] == 0 and h[1] == 0 and h[6] == 0


@pytest.mark.parametrize("case", SMALL[:2], ids=lambda c: c.name)
def test_full_sequence_matches_oracle(case):
    """pcfd_residual_full = UpdateBCs + gradient + limiter + residual."""
    m, S, O, q0 = run_both(case, "perturbed", seed=3)
    S.set_state(q0)
    norms = S.residual_full()
    _, _, _, bo, no = O.full(q0)
    b = S.compute_residuals()[0]
    assert_residual_close(b, bo, O.last_babs)
    assert np.allclose(norms, no, rtol=1e-12, atol=0)


def test_residual_is_deterministic():
    case = cases.ns_flatplate(20, 16, 12, seed=7)
    m = cases.build_mesh(case)
    S = SolutionSpace(m, case.param)
    q0 = cases.perturbed_state(S.qinf(), m.nnode + m.nbedge, 2)
    out = []
    for _ in range(2):
        S.set_state(q0)
        S.residual_full()
        out.append(S.compute_residuals()[0])
    assert np.array_equal(out[0], out[1])


def test_full_size_freestream_and_determinism():
    """At the benchmark size (128x96x96 nodes, 8.1M edges): uniform freestream
    with far-field/symmetry boundaries is preserved to rounding, and two
    evaluations of a perturbed state agree bitwise."""
    case = cases.ns_flatplate(128, 96, 96)
    p = case.param
    p.bc_type = {1: N.BC_FARFIELD, 2: N.BC_FARFIELD, 3: N.BC_FARFIELD, 4: N.BC_FARFIELD,
                 5: N.BC_SYMMETRY, 6: N.BC_SYMMETRY, 7: N.BC_FARFIELD}
    m = cases.build_mesh(case)
    S = SolutionSpace(m, p)
    nrows = m.nnode + m.nbedge
    q = np.tile(S.qinf(), (nrows, 1))
    S.set_state(q)
    S.residual_full()
    b, norms = S.compute_residuals()
    area = np.zeros(m.nnode)
    np.add.at(area, m.edges[:, 0], m.edge_area[:, 3])
    np.add.at(area, m.edges[:, 1], m.edge_area[:, 3])
    assert (np.abs(b) / (area[:, None] * 5.0)).max() < 1e-12
    q2 = cases.perturbed_state(S.qinf(), nrows, 9)
    res = []
    for _ in range(2):
        S.set_state(q2)
        res.append(S.residual_full())
    assert np.array_equal(res[0], res[1])
    assert S.health()[0] == 0


def low_pressure_state(m, qinf, seed, npocket=6):
    """Freestream with a few interior nodes whose internal energy is nearly
    gone, so second-order extrapolations toward them go non-physical and the
    limiter's pressure clip (ucs/limiters.tcc:737) fires."""
    rng = np.random.default_rng(seed)
    q = np.tile(qinf, (m.nnode + m.nbedge, 1))
    idx = rng.choice(m.nnode, npocket, replace=False)
    ke = 0.5 * q[idx, 0] * ((q[idx, 1:4] / q[idx, 0:1]) ** 2).sum(1)
    q[idx, 4] = ke + rng.uniform(0.005, 0.05, npocket)
    return cases.with_aux(q)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_pressure_clip_matches_oracle(seed):
    case = cases.ns_flatplate(12, 10, 8, seed=5, venkat_K=1.0)
    m = cases.build_mesh(case)
    S = SolutionSpace(m, case.param)
    O = OracleSpace(m, case.param)
    q0 = low_pressure_state(m, S.qinf(), seed)
    qo = O.update_bcs(q0)
    g = O.gradient(qo)
    l, nclip = O.limiter(qo, g)
    assert nclip > 0
    # standalone limiter (explicit clip kernel)
    S.set_state(q0)
    S.update_bcs()
    S.gradient()
    lg = S.limiter()
    assert np.abs(lg - l).max() <= 1e-12
    bo, no, _ = O.residual(qo, g, l, qold=q0)
    bg, ng = S.compute_residuals()
    assert_residual_close(bg, bo, O.last_babs)
    # fused path: the clip detected inside the edge-flux pass
    S.set_state(q0)
    ng2 = S.residual_full()
    bg2, _ = S.compute_residuals()
    assert_residual_close(bg2, bo, O.last_babs)
    assert np.allclose(ng2, no, rtol=1e-12, atol=0)
    assert S.health()[1] > 0


@pytest.mark.parametrize("case", SMALL, ids=lambda c: c.name + "_K%g" % c.param.venkat_K)
@pytest.mark.parametrize("state", ["smooth", "perturbed"])
def test_double_float_residual_matches_oracle(case, state):
    """The double-float kernels (FP32 pipes, ~48-bit significands) meet the
    same 1e-12 residual parity bar as the FP64 kernels."""
    m, S, O, q0 = run_both(case, state, seed=13)
    S.set_residual_arithmetic(1)
    S.set_state(q0)
    norms = S.residual_full()
    b = S.get_residual()
    _, _, _, bo, no = O.full(q0)
    assert_residual_close(b, bo, O.last_babs)
    assert np.allclose(norms, no, rtol=1e-12, atol=0)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_double_float_pressure_clip(seed):
    case = cases.ns_flatplate(12, 10, 8, seed=5, venkat_K=1.0)
    m = cases.build_mesh(case)
    S = SolutionSpace(m, case.param)
    O = OracleSpace(m, case.param)
    q0 = low_pressure_state(m, S.qinf(), seed)
    S.set_residual_arithmetic(1)
    S.set_state(q0)
    ng = S.residual_full()
    bg = S.get_residual()
    _, _, _, bo, no = O.full(q0)
    assert_residual_close(bg, bo, O.last_babs)
    assert np.allclose(ng, no, rtol=1e-12, atol=0)
    assert S.health()[1] > 0


def test_double_float_full_size_freestream():
    case = cases.ns_flatplate(128, 96, 96)
    p = case.param
    p.bc_type = {1: N.BC_FARFIELD, 2: N.BC_FARFIELD, 3: N.BC_FARFIELD, 4: N.BC_FARFIELD,
                 5: N.BC_SYMMETRY, 6: N.BC_SYMMETRY, 7: N.BC_FARFIELD}
    m = cases.build_mesh(case)
    S = SolutionSpace(m, p)
    S.set_residual_arithmetic(1)
    q = np.tile(S.qinf(), (m.nnode + m.nbedge, 1))
    S.set_state(q)
    S.residual_full()
    b = S.get_residual()
    area = np.zeros(m.nnode)
    np.add.at(area, m.edges[:, 0], m.edge_area[:, 3])
    np.add.at(area, m.edges[:, 1], m.edge_area[:, 3])
    assert (np.abs(b) / (area[:, None] * 5.0)).max() < 1e-12


@pytest.mark.parametrize("kind", [1, 2], ids=["barth", "venkat"])
@pytest.mark.parametrize("arith", [0, 1], ids=["fp64", "df"])
def test_barth_and_venkat_limiters(kind, arith):
    """Barth (Kernel_Barth, ucs/limiters.tcc:194) and Venkatakrishnan
    (Kernel_Venkat, :372) limiters and the residual that uses them, against
    the oracle; the Venkatakrishnan case has negative raw values, so the
    pressure clip folded into the edge pass and the clamp to zero run too."""
    case = cases.ns_flatplate(12, 10, 8, seed=5, venkat_K=1.0)
    case.param.limiter = kind
    m, S, O, q0 = run_both(case, "perturbed", seed=11)
    S.set_residual_arithmetic(arith)
    S.set_state(q0)
    norms = S.residual_full()
    q, g, l, bo, no = O.full(q0)
    if arith == 0:
        b = S.compute_residuals()[0]
        assert_residual_close(b, bo, O.last_babs)
        assert np.allclose(norms, no, rtol=1e-12, atol=0)
        S.set_state(q0)
        S.update_bcs()
        S.gradient()
        assert np.abs(S.limiter() - O.limiter(q, g)[0]).max() <= 1e-12
    else:
        assert np.allclose(norms, no, rtol=1e-10, atol=0), (norms, no)
    if kind == 1:
        assert np.all((l >= 0) & (l <= 1))


@pytest.mark.parametrize("limiter", [3, 1], ids=["venkat_mod", "barth"])
@pytest.mark.parametrize("arith", [0, 1], ids=["fp64", "df"])
def test_muscl_with_nonzero_chi(limiter, arith):
    """The general MUSCL extrapolation q + (chi/2 dQ + (1 - chi) grad.dx) in
    the limiter and the edge flux (the chi = 0 kernels skip the dQ term),
    against the oracle with chi = 1/3."""
    case = cases.ns_flatplate(12, 10, 8, seed=5, venkat_K=1.0)
    case.param.chi = 1.0 / 3.0
    case.param.limiter = limiter
    m, S, O, q0 = run_both(case, "perturbed", seed=13)
    S.set_residual_arithmetic(arith)
    S.set_state(q0)
    norms = S.residual_full()
    q, g, l, bo, no = O.full(q0)
    if arith == 0:
        assert_residual_close(S.compute_residuals()[0], bo, O.last_babs)
        assert np.allclose(norms, no, rtol=1e-12, atol=0)
        S.set_state(q0)
        S.update_bcs()
        S.gradient()
        assert np.abs(S.limiter() - O.limiter(q, g)[0]).max() <= 1e-12
    else:
        assert np.allclose(norms, no, rtol=1e-10, atol=0), (norms, no)
