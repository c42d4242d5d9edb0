"""The residual-norm entry point that allocates no device memory.

Some callers cannot let a library allocate GPU memory: an application that
hands out every byte from its own pool, or a solver loop that must not
allocate once it runs.  pcfd_residual_norms_noalloc serves them: they pass
their own device buffers and the only scratch is a fixed array inside the
library.  This file checks it against the norms pcfd_residual returns, on
two calls in a row (the shared scratch keeps the previous call's contents),
that the second call leaves the device's free memory unchanged, and that it
refuses inputs beyond its size limit and a capturing stream.  It is
collected last on purpose.
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
    def call():
        return lib.pcfd_residual_norms_noalloc(C.c_void_p(b_dev.data_ptr()), m.nnode, C.c_void_p(out.data_ptr()),
                                               None)

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
        rc = call()
        assert rc == 0, lib.pcfd_last_error()
        got = out.cpu().numpy()
        assert np.allclose(got, norms, rtol=1e-12, atol=0), (got, norms)
    # after the one-time set-up a call leaves the device's free memory as it
    # was, read right before and right after it; the device's free memory can
    # also move for reasons outside this process, so one equal pair of three
    # tries is the bar
    unchanged = []
    for _ in range(3):
        torch.cuda.synchronize()
        before = torch.cuda.mem_get_info(0)[0]
        assert call() == 0, lib.pcfd_last_error()
        unchanged.append(torch.cuda.mem_get_info(0)[0] == before)
        if unchanged[-1]:
            break
    assert any(unchanged)
    # beyond the fixed scratch the call is refused before touching the GPU
    rc = lib.pcfd_residual_norms_noalloc(C.c_void_p(b_dev.data_ptr()), 33554433, C.c_void_p(out.data_ptr()), None)
    assert rc == 1
    assert b"exceeds the fixed scratch limit" in lib.pcfd_last_error()


def test_noalloc_refuses_a_capturing_stream():
    """The call synchronizes its stream, so it cannot be captured into a
    graph: on a capturing stream it returns PCFD_ERR_ARG and enqueues nothing."""
    torch = pytest.importorskip("torch")
    lib = N.load()
    b_dev = torch.zeros(100 * 5, dtype=torch.float64, device="cuda:0")
    out = torch.zeros(6, dtype=torch.float64, device="cuda:0")
    # the one-time set-up outside the capture
    assert lib.pcfd_residual_norms_noalloc(C.c_void_p(b_dev.data_ptr()), 100, C.c_void_p(out.data_ptr()), None) == 0
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            out.add_(0.0)  # something for the graph to hold
            rc = lib.pcfd_residual_norms_noalloc(C.c_void_p(b_dev.data_ptr()), 100, C.c_void_p(out.data_ptr()),
                                                 C.c_void_p(s.cuda_stream))
    assert rc == 1
    assert b"capturing" in lib.pcfd_last_error()
