"""Implicit part on the GPU against the oracle, through the C ABI: local
time step, finite-difference Jacobian in block CRS, the multicolour block
Gauss-Seidel kernel, and whole Newton iterations."""
import numpy as np
import pytest

from oracle_lib import OracleImplicit
from parity import assert_field_close
from proteuscfd_gb300 import Mesh, Param, SolutionSpace, cases
from proteuscfd_gb300 import _native as N

pytestmark = pytest.mark.gpu


def euler_case(beval=1):
    c = cases.euler_ramp(14, 9, 7, seed=4)
    c.param.jac_boundary_eval = beval
    return c


def ns_case(beval=0):
    c = cases.ns_flatplate(11, 9, 7, seed=5, venkat_K=1.0)
    c.param.jac_boundary_eval = beval
    return c


CASES = [euler_case(0), euler_case(1), ns_case(0), ns_case(3)]
IDS = ["euler_beval0", "euler_beval1", "ns_beval0", "ns_beval3"]


def row_block_error(M, Mref, ia):
    """Largest |M - Mref| per CRS block row, relative to that row's largest
    reference entry."""
    blockmax = np.abs(Mref).max(axis=1)
    rowmax = np.maximum.reduceat(blockmax, ia[:-1])
    rows = np.repeat(np.arange(len(ia) - 1), np.diff(ia))
    return (np.abs(M - Mref).max(axis=1) / rowmax[rows]).max()


def setup(case, seed=1):
    m = cases.build_mesh(case)
    S = SolutionSpace(m, case.param)
    O = OracleImplicit(m, case.param)
    q0 = cases.perturbed_state(S.qinf(), m.nnode + m.nbedge, seed)
    return m, S, O, q0


@pytest.mark.parametrize("case", CASES[::2], ids=IDS[::2])
def test_timestep_parity(case):
    m, S, O, q0 = setup(case)
    S.set_state(q0)
    dt, dtmin = S.compute_timesteps(7.5)
    dto, dtmino = O.timestep(q0, 7.5)
    assert np.allclose(dt, dto, rtol=1e-13, atol=0)
    assert abs(dtmin - dtmino) <= 1e-13 * dtmino


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_jacobian_parity_fp64(case):
    m, S, O, q0 = setup(case)
    S.set_state(q0)
    S.update_bcs()
    q1 = S.get_state()
    dt, _ = S.compute_timesteps(5.0)
    S.compute_jacobians()
    Mg = S.get_jacobian()
    ia, ja, nc = S.crs_structure()
    assert np.array_equal(ia, O.ia) and np.array_equal(ja, O.ja)
    qo = O.update_bcs(q0)
    dto, _ = O.timestep(qo, 5.0)
    Mo, qo2 = O.jacobian(qo, dto)
    # the state after the Jacobian's boundary pass matches
    assert_field_close(S.get_state(), qo2, 1e-12, "state after Jacobian BC pass")
    # finite differences with h = 1e-8 turn flux rounding into ~1e-8
    # relative noise (a block the upwinding makes zero in exact arithmetic
    # holds only that noise), so each block row agrees to 1e-6 of its largest
    # entry
    err = row_block_error(Mg, Mo, O.ia)
    assert err < 1e-6, err
    assert S.health()[7] == 0


def test_jacobian_storage_precisions():
    case = ns_case(3)
    m, S, O, q0 = setup(case)
    S.set_state(q0)
    S.compute_timesteps(5.0)
    out = {}
    for prec in (0, 1, 2):
        S.set_state(q0)
        S.set_jacobian_precision(prec)
        S.compute_jacobians()
        out[prec] = S.get_jacobian()
    ref = out[0]
    # FP32 and BF16 storage difference the fluxes in double-float: flux
    # rounding ~2^-48 over h = 1e-8 leaves up to ~1e-5 relative noise per
    # block row, then the storage rounding
    assert row_block_error(out[1], ref, O.ia) < 5e-5    # FP32 storage
    assert row_block_error(out[2], ref, O.ia) < 1e-2    # BF16 storage


@pytest.mark.parametrize("arith", [0, 1])
def test_limiter_get_set_roundtrip(arith):
    case = ns_case(3)
    m, S, O, q0 = setup(case)
    S.set_state(q0)
    S.set_residual_arithmetic(arith)
    S.newton_iterate(1, cfl=5.0, nsgs=2)
    lim = S.get_limiter()
    assert lim.shape == (m.nnode, 5) and np.all(lim >= 0.0) and np.all(lim <= 1.0)
    lim2 = np.clip(lim * 0.5 + 0.25, 0.0, 1.0)
    S.set_limiter(lim2)
    # the double-float arithmetic holds the limiter as an FP32 pair (~48 bits)
    rtol = 0.0 if arith == 0 else 2.0 ** -46
    assert np.allclose(S.get_limiter(), lim2, rtol=rtol, atol=0.0)
    # a frozen limiter is what the next residual uses
    r1 = S.newton_iterate(2, cfl=5.0, nsgs=2, limiter_freeze=1)
    assert np.isfinite(r1["res"][0])
    assert np.allclose(S.get_limiter(), lim2, rtol=rtol, atol=0.0)


def test_jacobian_double_float_fluxes():
    """Residual arithmetic 1 evaluates the finite-difference fluxes in
    double-float: flux rounding ~2^-48 over h = 1e-8 leaves ~1e-6 relative
    noise per block row against the FP64 Jacobian."""
    case = ns_case(3)
    m, S, O, q0 = setup(case)
    S.set_state(q0)
    S.compute_timesteps(5.0)
    out = {}
    for arith in (0, 1):
        S.set_state(q0)
        S.set_residual_arithmetic(arith)
        S.compute_jacobians()
        out[arith] = S.get_jacobian()
    assert row_block_error(out[1], out[0], O.ia) < 2e-5
    # FP32 storage: quotients and viscous blocks formed in FP32
    S.set_state(q0)
    S.set_jacobian_precision(1)
    S.compute_jacobians()
    assert row_block_error(S.get_jacobian(), out[0], O.ia) < 5e-5
    assert S.health()[0] == 0


@pytest.mark.parametrize("case", [CASES[1], CASES[3]], ids=[IDS[1], IDS[3]])
def test_sgs_kernel_matches_colored_oracle(case):
    """The GPU sweep kernel is the oracle's row update in the GPU's colour
    order (same arithmetic, different order from the reference's
    lexicographic sweep)."""
    m, S, O, q0 = setup(case)
    S.set_state(q0)
    S.compute_timesteps(5.0)
    S.compute_jacobians()
    S.residual_full()
    b = S.compute_residuals()[0]
    x, _ = S.sgs(4)
    M = S.get_jacobian()
    Mlu, pv = O.lu(M)
    cptr, rows = S.coloring()
    xo = O.sgs_colored(Mlu, pv, b, 4, cptr, rows)
    assert_field_close(x, xo, 1e-11, "SGS solution")
    # and it is a good approximate solve of the same system
    xl, _ = O.sgs(Mlu, pv, b, 4)
    assert np.linalg.norm(x - xl) < 0.5 * np.linalg.norm(xl)


@pytest.mark.parametrize("case", [CASES[1], CASES[3]], ids=[IDS[1], IDS[3]])
def test_newton_iterates_match_oracle(case):
    """Three outer iterations on the GPU against the oracle's iteration with
    the same colour order; FD Jacobian noise (~1e-8) bounds the agreement."""
    m, S, O, q0 = setup(case)
    # start from a state the boundary conditions have already been applied
    # to, as after any earlier iteration
    q0 = O.update_bcs(q0)
    S.set_state(q0)
    hist = []
    for it in range(3):  # the reference's counter starts at 0
        rep = S.newton_iterate(it, cfl=5.0, nsgs=6)
        hist.append(rep["res"][0])
    qg = S.get_state()
    qo, ho = O.newton(q0, 3, cfl=5.0, nsgs=6, coloring=S.coloring())
    assert np.allclose(hist, ho, rtol=1e-7, atol=0), (hist, ho)
    n = m.nnode
    assert_field_close(qg[:n, :5], qo[:n, :5], 1e-6, "q after 3 Newton iterations")


def test_fgmres_reduces_linear_residual():
    case = ns_case(3)
    m, S, O, q0 = setup(case)
    S.set_state(q0)
    for prec in (0, 1):
        S.set_state(q0)
        rep = S.newton_iterate(1, cfl=20.0, nsgs=1, linear_solver=1, fgmres_m=20, fgmres_restarts=2,
                               fgmres_rtol=1e-6, jac_precision=prec)
        assert rep["lin_res"] < 1e-6, rep
        assert np.isfinite(rep["dqnorm"]) and rep["dqnorm"] > 0


def star_mesh(npts=40):
    """A ball of tets around one centre node joined to npts hull vertices:
    its Jacobian row has npts off-diagonal blocks, past the block counts the
    row kernels stage or shuffle (16 and 32)."""
    from scipy.spatial import ConvexHull
    k = np.arange(npts) + 0.5
    phi = np.arccos(1 - 2 * k / npts)
    th = np.pi * (1 + 5 ** 0.5) * k
    pts = np.c_[np.cos(th) * np.sin(phi), np.sin(th) * np.sin(phi), np.cos(phi)]
    xyz = np.vstack([[0.0, 0.0, 0.0], pts])
    tris, tets = [], []
    for a, b, c in ConvexHull(pts).simplices:
        tris.append([a + 1, b + 1, c + 1])
        v = np.dot(np.cross(pts[b] - pts[a], pts[c] - pts[a]), -pts[a])
        tets.append([0, a + 1, c + 1, b + 1] if v > 0 else [0, a + 1, b + 1, c + 1])
    return Mesh.from_elements(xyz, np.array(tris), np.ones(len(tris), int), np.array(tets))


@pytest.mark.parametrize("which", ["star", "box"])
def test_matvec_matches_crs_product(which):
    """pcfd_matvec (CRSMatrix::MatVecMultiply, ucs/crs.tcc:484) against the
    CRS product of the assembled matrix, for FP64/FP32/BF16 block storage and
    FP64 or FP32 vectors; the star row (40 blocks) covers the rows longer than
    the staged and shuffled block counts, the 40x32x32 box many rows per warp."""
    if which == "star":
        m = star_mesh(40)
        prm = Param(gamma=1.4, mach=0.7, bc_type={1: N.BC_FARFIELD})
    else:
        c = cases.ns_flatplate(40, 32, 32, seed=3)
        m = cases.build_mesh(c)
        prm = c.param
    S = SolutionSpace(m, prm)
    S.set_state(cases.perturbed_state(S.qinf(), m.nnode + m.nbedge, 2))
    rng = np.random.default_rng(4)
    x = rng.normal(size=(m.nnode, 5))
    for prec in (0, 1, 2):
        S.set_jacobian_precision(prec)
        S.compute_timesteps(5.0)
        S.compute_jacobians()
        M = S.get_jacobian().reshape(-1, 5, 5)
        ia, ja, _ = S.crs_structure()
        ref = np.add.reduceat(np.einsum("kij,kj->ki", M, x[ja]), ia[:-1], axis=0)
        scale = np.add.reduceat(np.einsum("kij,kj->ki", np.abs(M), np.abs(x[ja])), ia[:-1], axis=0)
        err = np.abs(S.matvec(x) - ref) / scale
        assert err.max() < (1e-13 if prec == 0 else 2e-6), (prec, err.max())
        if prec > 0:
            err = np.abs(S.matvec(x, fp32=True) - ref) / scale
            assert err.max() < 2e-6, (prec, err.max())
        else:
            with pytest.raises(N.PcfdError):
                S.matvec(x, fp32=True)
    S.close()


@pytest.mark.parametrize("prec", [0, 1, 2], ids=["fp64", "fp32", "bf16"])
def test_sgs_rhs_matches_colored_oracle(prec):
    """pcfd_sgs_rhs against the oracle's row update in the GPU's colour order
    on the same stored matrix: FP64 vectors to rounding, and the FP32
    Krylov preconditioner's sweep (FP32 vectors and diagonal inverse, FP32
    accumulation) to FP32 accuracy, on a box with many rows per warp."""
    c = cases.ns_flatplate(40, 32, 32, seed=3)
    m = cases.build_mesh(c)
    S = SolutionSpace(m, c.param)
    O = OracleImplicit(m, c.param)
    S.set_state(cases.perturbed_state(S.qinf(), m.nnode + m.nbedge, 2))
    S.set_jacobian_precision(prec)
    S.compute_timesteps(5.0)
    S.compute_jacobians()
    b = np.random.default_rng(6).normal(size=(m.nnode, 5))
    Mlu, pv = O.lu(S.get_jacobian())
    cptr, rows = S.coloring()
    xo = O.sgs_colored(Mlu, pv, b, 3, cptr, rows)
    x = S.sgs_rhs(b, 3)
    tol = 1e-10 if prec == 0 else 2e-4   # FP64 vectors over an FP32/BF16 matrix accumulate in FP32
    assert np.abs(x - xo).max() <= tol * np.abs(xo).max(), np.abs(x - xo).max() / np.abs(xo).max()
    if prec > 0:
        xf = S.sgs_rhs(b, 3, fp32=True)
        assert np.abs(xf - xo).max() <= 2e-4 * np.abs(xo).max(), np.abs(xf - xo).max() / np.abs(xo).max()
    S.close()
