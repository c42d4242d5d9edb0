"""The CUDA path against the reference solver's own outputs, through the C ABI.

The fixtures (tests/golden/ref_<case>.npz) were written by the reference
solver itself on small cases of the two benchmark families (Mach 2 Euler
ramp, Mach 0.8 laminar flat plate with the modified Venkatakrishnan and the
Barth limiters).  The product mesh is built from the reference's element
list with the reference's set-up reorder, so every array below is in the
reference's numbering.  Each stage is fed the reference's own input:

* block CRS structure: bit-exact;
* boundary update, gradient, limiter, one FP64 residual and its norms:
  within 1e-12 relative (the bar for one FP64 residual evaluation), taken per
  component against the magnitudes of the terms summed into it
  (tests/parity.py), per column against the column's largest magnitude for
  states and gradients;
* finite-difference Jacobian: within 1e-6 of each block row's scale - the
  flux rounding of GPU fused multiply-adds, ~1e-16, over the reference's
  h = 1e-8;
* ApplyDQ: within 1e-13.

The block SGS sweep is not compared with the reference's: the reference
sweeps rows lexicographically, one after another; the GPU sweeps colour by
colour (tests/test_gpu_implicit.py checks it against the oracle's sweep in
the same colour order), so after a fixed number of sweeps the two updates
differ while solving the same system.
"""
import numpy as np
import pytest

import ref_fixtures as R
from oracle_lib import OracleImplicit
from parity import assert_residual_close
from proteuscfd_gb300 import SolutionSpace

pytestmark = pytest.mark.gpu


def close(x, ref, rtol, what):
    """Per column relative to the column's largest magnitude, floored at 1e-2
    of the array's largest (a column the reference holds at zero, such as a
    velocity component of a two-dimensional flow, is judged on that floor)."""
    x = np.asarray(x).reshape(len(ref), -1)
    ref = np.asarray(ref).reshape(len(ref), -1)
    scale = np.maximum(np.abs(ref).max(axis=0, keepdims=True), 1e-2 * np.abs(ref).max())
    err = np.abs(x - ref) / scale
    worst = np.unravel_index(np.argmax(err), err.shape)
    assert err.max() <= rtol, "%s mismatch %.3e at %s: gpu %r ref %r" % (what, err.max(), worst, x[worst], ref[worst])


def space(case, first_order=False):
    """A solution space on the reference's mesh and parameters.  The
    reference's first step runs first order (its counter starts at 0 and
    NewtonIterate tests iter > nFirstOrderSteps); first_order=True stands
    for that step with spatialOrder 1, which switches off the same terms."""
    f = R.load(case)
    m = R.mesh(f)
    p = R.param(f)
    if first_order:
        p.sorder = 1
    return f, m, p, SolutionSpace(m, p)


@pytest.mark.parametrize("case", R.CASES)
def test_crs_structure_and_freestream(case):
    f, m, p, S = space(case)
    ia, ja, _ = S.crs_structure()
    np.testing.assert_array_equal(ia, f["ia"])
    np.testing.assert_array_equal(ja, f["ja"])
    np.testing.assert_allclose(S.qinf(), f["qinf"].ravel(), rtol=1e-15, atol=0)


@pytest.mark.parametrize("case", R.CASES)
def test_boundary_update_matches_reference(case):
    f, m, p, S = space(case)
    O = OracleImplicit(m, p)
    # the reference's UpdateBCs input: the state after the Jacobian assembly
    # rewrote the boundary nodes (reproduced bit for bit by the oracle)
    _, qj = O.jacobian(f["q_init"], f["dt_preiterate"])
    S.set_state(qj)
    S.update_bcs()
    close(S.get_state(), f["s1_q_bc"], 1e-13, "state after UpdateBCs")


@pytest.mark.parametrize("case", R.CASES)
@pytest.mark.parametrize("step", ["s1_", "s2_"])
def test_residual_stages_match_reference(case, step):
    f = R.load(case)
    ho = R.scalar(f, "sorder") > 1 and R.scalar(f, step + "iter") > 0
    f, m, p, S = space(case, first_order=not ho)
    n = m.nnode
    qstart = f["q_init"] if step == "s1_" else f["s1_q"]
    S.set_state(f[step + "q_bc"])
    S.set_qold(qstart[:n, :5])
    if ho or p.viscous:
        g = S.gradient()
        close(g, f[step + "qgrad"], 1e-12, step + "gradient")
    if ho and p.limiter:
        lim = S.limiter()
        close(lim, f[step + "limiter"], 1e-12, step + "limiter")
    # the scale of each residual entry: the magnitudes of the terms summed into it
    O = OracleImplicit(m, p)
    O.residual(f[step + "q_bc"], f.get(step + "qgrad"), f.get(step + "limiter") if ho else None,
               qold=qstart[:n, :5])
    b, norms = S.compute_residuals()
    assert_residual_close(b, f[step + "b"], O.last_babs)
    np.testing.assert_allclose(norms, f[step + "norms"].ravel(), rtol=1e-12, atol=0)


@pytest.mark.parametrize("case", R.CASES)
def test_jacobian_matches_reference(case):
    f, m, p, S = space(case)
    S.set_state(f["q_init"])
    dt, _ = S.compute_timesteps(R.scalar(f, "case_cfl"))
    close(dt, f["dt_preiterate"], 1e-13, "local time step")
    S.compute_jacobians()
    M = S.get_jacobian()
    ia = f["ia"]
    ref = f["jacobian"]
    blockmax = np.abs(ref).max(axis=1)
    rowmax = np.maximum.reduceat(blockmax, ia[:-1])
    rows = np.repeat(np.arange(len(ia) - 1), np.diff(ia))
    err = (np.abs(M - ref).max(axis=1) / rowmax[rows]).max()
    assert err < 1e-6, err
    # and the boundary nodes' states the assembly rewrote
    O = OracleImplicit(m, p)
    _, qj = O.jacobian(f["q_init"], f["dt_preiterate"])
    close(S.get_state(), qj, 1e-13, "state after the Jacobian assembly")


@pytest.mark.parametrize("case", R.CASES)
def test_apply_dq_matches_reference(case):
    f, m, p, S = space(case)
    n = m.nnode
    S.set_state(f["s1_q_bc"])
    S.apply_dq(f["s1_x_sgs"])
    close(S.get_state()[:n], f["s1_q"], 1e-13, "state after ApplyDQ")


@pytest.mark.parametrize("case", [c for c in R.CASES if "s1_forces" in R.load(c)])
def test_forces_match_oracle(case):
    """pcfd_forces against the oracle's FORCE_Kernel (itself bit-identical to
    the reference's reported forces) on the reference's state and gradient."""
    f, m, p, S = space(case)
    walls = [int(t) for t, k in f["case_bc_types"] if k == 4]
    S.set_state(f["s1_q_bc"])
    g = S.gradient()
    fp, fv = S.forces(walls)
    O = OracleImplicit(m, p)
    op, ov = O.forces(f["s1_q_bc"], g, walls)
    np.testing.assert_allclose(fp, op, rtol=1e-13, atol=1e-16 * np.abs(op).max())
    np.testing.assert_allclose(fv, ov, rtol=1e-12, atol=1e-12 * np.abs(ov).max())
