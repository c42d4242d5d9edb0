"""The linear-solve entry points on their own, through the C ABI: pcfd_fgmres
(CRS<T>::GMRES's role, ucs/crs.tcc:176, in its flexible SGS-preconditioned
form) on the system pcfd_jacobian and the last residual leave."""
import numpy as np
import pytest

from proteuscfd_gb300 import SolutionSpace, cases
from proteuscfd_gb300 import _native as N

pytestmark = pytest.mark.gpu


def setup():
    c = cases.ns_flatplate(11, 9, 7, seed=5, venkat_K=1.0)
    c.param.jac_boundary_eval = 3
    m = cases.build_mesh(c)
    S = SolutionSpace(m, c.param)
    q0 = cases.perturbed_state(S.qinf(), m.nnode + m.nbedge, 1)
    return m, S, q0


def test_fgmres_entry_point_solves_the_assembled_system():
    """pcfd_fgmres on the system pcfd_jacobian and the residual left: the
    library's own product of its solution meets the right-hand side to the
    requested tolerance (FP64 storage), or to the FP32 Krylov solver's
    accuracy (FP32 storage); and a call before any Jacobian is refused."""
    m, S, q0 = setup()
    S.set_state(q0)
    with pytest.raises(N.PcfdError):
        S.fgmres(10, 1, 1e-3, 1)
    for prec, rtol, bar in ((0, 1e-8, 1e-7), (1, 1e-4, 1e-3)):
        S.set_state(q0)
        S.set_jacobian_precision(prec)
        S.compute_timesteps(5.0)
        S.compute_jacobians()
        S.residual_full()
        b = S.compute_residuals()[0]
        x, rel, its = S.fgmres(20, 10, rtol, 1)
        assert rel < rtol and its > 0, (prec, rel, its)
        true_rel = np.linalg.norm(S.matvec(x) - b) / np.linalg.norm(b)
        assert true_rel < bar, (prec, true_rel)
    S.set_jacobian_precision(0)
