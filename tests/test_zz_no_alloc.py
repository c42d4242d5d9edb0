"""The residual-norm entry point that allocates no device memory.

Some callers cannot let a library allocate GPU memory: an application that
hands out every byte from its own pool, or a solver loop that must not
allocate once it runs.  pcfd_residual_norms_noalloc serves them: they pass
their own device buffers and the only scratch is a fixed array inside the
library.  This file checks it against the norms pcfd_residual returns, on
two calls in a row (the shared scratch keeps the previous call's contents),
and checks its size limit.  It is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from proteuscfd_gb300 import SolutionSpace, cases
from proteuscfd_gb300 import _native as N

pytestmark = pytest.mark.gpu


def test_noalloc_norms_match_the_residual_entry_point():
    torch = pytest.importorskip("torch")
    lib = N.load()
    case = cases.ns_flatplate(20, 16, 12, seed=3, venkat_K=1.0)
    m = cases.build_mesh(case)
    S = SolutionSpace(m, case.param)
    # the caller's own device buffers, allocated once up front
    b_dev = torch.empty(m.nnode * 5, dtype=torch.float64, device="cuda:0")
    out = torch.empty(6, dtype=torch.float64, device="cuda:0")
    free_after = []
    for seed in (1, 2):  # two calls in a row, different inputs
        q0 = cases.perturbed_state(S.qinf(), m.nnode + m.nbedge, seed)
        S.set_state(q0)
        S.update_bcs()
        S.gradient()
        S.limiter()
        b, norms = S.compute_residuals()  # the existing entry point
        b_dev.copy_(torch.from_numpy(np.ascontiguousarray(b).reshape(-1)))
        out.fill_(float("nan"))
        torch.cuda.synchronize()
        rc = lib.pcfd_residual_norms_noalloc(C.c_void_p(b_dev.data_ptr()), m.nnode, C.c_void_p(out.data_ptr()),
                                             None)
        assert rc == 0, lib.pcfd_last_error()
        got = out.cpu().numpy()
        assert np.allclose(got, norms, rtol=1e-12, atol=0), (got, norms)
        free_after.append(torch.cuda.mem_get_info(0)[0])
    # the second call (after the one-time set-up) left free device memory as it was
    assert free_after[1] == free_after[0]
    # beyond the fixed scratch the call is refused before touching the GPU
    rc = lib.pcfd_residual_norms_noalloc(C.c_void_p(b_dev.data_ptr()), 33554433, C.c_void_p(out.data_ptr()), None)
    assert rc == 1
    assert b"exceeds the fixed scratch limit" in lib.pcfd_last_error()
