"""The CPU oracle against the reference solver's own outputs.

Each stage of the reference's first two Newton steps (ucs/solutionSpace.tcc:
573-818) is fed the reference's own input for that stage, so a stage is
judged on its own: the boundary update, the LSQ gradient, the limiter, the
residual with its norms (including the temporal term the reference always
adds), the finite-difference Jacobian, the block-SGS sweeps and ApplyDQ.
The whole Newton iteration is then run from the seeded initial state.

Bar: bit-identical.  Every stage, the CRS structure and the Newton iterates
and residual histories equal the reference's to the last bit.
"""
import numpy as np
import pytest

import ref_fixtures as R
from oracle_lib import OracleImplicit


def stage_inputs(f, n):
    """(stage prefix, state at the start of that step) for steps 1 and 2."""
    yield "s1_", f["q_init"]
    yield "s2_", np.concatenate([f["s1_q"], f["s1_q_bc"][n:]])


@pytest.mark.parametrize("case", R.CASES)
def test_oracle_stages_match_reference(case):
    f = R.load(case)
    m = R.mesh(f)
    p = R.param(f)
    O = OracleImplicit(m, p)
    n = m.nnode
    np.testing.assert_allclose(O.qinf(), f["qinf"].ravel(), rtol=1e-14, atol=0)
    for st, qstart in stage_inputs(f, n):
        it = R.scalar(f, st + "iter")
        ho = p.sorder > 1 and it > 0
        qb = f[st + "q_bc"]
        g = lim = None
        if ho or p.viscous:
            g = O.gradient(qb)
            np.testing.assert_array_equal(g, f[st + "qgrad"], err_msg=st + "qgrad")
        if ho and p.limiter:
            lim, _ = O.limiter(qb, f[st + "qgrad"])
            np.testing.assert_array_equal(lim, f[st + "limiter"], err_msg=st + "limiter")
        Ob = O if ho else O._first_order()
        b, norms, _ = Ob.residual(qb, f.get(st + "qgrad"), f.get(st + "limiter") if ho else None,
                                  qold=qstart[:n, :5])
        np.testing.assert_array_equal(b, f[st + "b"], err_msg=st + "b")
        np.testing.assert_array_equal(norms, f[st + "norms"].ravel(), err_msg=st + "norms")
        q, _ = O.apply_dq(f[st + "x_sgs"], qb)
        np.testing.assert_array_equal(q[:n], f[st + "q"], err_msg=st + "q")


@pytest.mark.parametrize("case", R.CASES)
def test_oracle_jacobian_sgs_and_boundary_update(case):
    f = R.load(case)
    m = R.mesh(f)
    O = OracleImplicit(m, R.param(f))
    np.testing.assert_array_equal(O.ia, f["ia"])
    np.testing.assert_array_equal(O.ja, f["ja"])
    cfl = R.scalar(f, "case_cfl")
    dt, _ = O.timestep(f["q_init"], cfl)
    np.testing.assert_array_equal(dt, f["dt_preiterate"])
    # the Jacobian assembly also rewrites the boundary nodes' states
    M, qj = O.jacobian(f["q_init"], f["dt_preiterate"])
    np.testing.assert_array_equal(M, f["jacobian"])
    dt2, _ = O.timestep(qj, cfl)
    np.testing.assert_array_equal(dt2, f["dt"])
    qb = O.update_bcs(qj)
    np.testing.assert_array_equal(qb, f["s1_q_bc"])
    Mlu, pv = O.lu(f["jacobian"])
    x, d = O.sgs(Mlu, pv, f["s1_b"], R.scalar(f, "case_nsgs"))
    np.testing.assert_array_equal(x, f["s1_x_sgs"])
    assert d == R.scalar(f, "s1_sgs_delta")


@pytest.mark.parametrize("case", R.CASES)
def test_oracle_newton_iterates_match_reference(case):
    f = R.load(case)
    m = R.mesh(f)
    O = OracleImplicit(m, R.param(f))
    n = m.nnode
    steps = R.scalar(f, "case_steps")
    q, hist = O.newton(f["q_init"], steps, cfl=R.scalar(f, "case_cfl"), nsgs=R.scalar(f, "case_nsgs"))
    ref_final = f["q_final"] if "q_final" in f else f["s%d_q" % steps]
    np.testing.assert_array_equal(q[:n], ref_final)
    ref_hist = [R.scalar(f, "s1_norms"), f["s2_norms"].ravel()[0]] + list(f.get("resglobal_steps3on", []))
    assert hist == ref_hist[:len(hist)]


@pytest.mark.parametrize("case", [c for c in R.CASES if "s1_forces" in R.load(c)])
def test_oracle_forces_match_reference(case):
    """The body forces Forces::Compute reports after each step (FORCE_Kernel
    on the no-slip wall: pressure and viscous parts), bit for bit."""
    f = R.load(case)
    m = R.mesh(f)
    O = OracleImplicit(m, R.param(f))
    n = m.nnode
    walls = [int(t) for t, k in f["case_bc_types"] if k == 4]
    for st in ("s1_", "s2_"):
        q = np.concatenate([f[st + "q"], f[st + "q_bc"][n:]])
        fp, fv = O.forces(q, f[st + "qgrad"], walls)
        np.testing.assert_array_equal(np.r_[fp, fv], f[st + "forces"].ravel())
