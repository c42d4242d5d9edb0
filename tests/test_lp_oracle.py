"""The learned preconditioner's network on the CPU oracle: the backward pass
against central differences of the forward pass, the graph against the mesh,
and the BF16 rounding (test infrastructure checks; no GPU)."""
import numpy as np
import pytest

from proteuscfd_gb300 import cases
from oracle_lib import OracleNet, lib, lp_random_params


@pytest.fixture(scope="module")
def small():
    c = cases.euler_ramp(6, 5, 4)
    m = cases.build_mesh(c)
    return m, OracleNet(m)


def test_nparam_matches_header():
    from proteuscfd_gb300 import _native as N
    assert lib().oracle_lp_nparam() == N.LP_NPARAM == 26821


def test_bf16_rounding():
    L = lib()
    assert L.oracle_bf16(1.0) == 1.0
    # 1 + 2^-8 is halfway between 1 and 1 + 2^-7: ties to even -> 1
    assert L.oracle_bf16(1.0 + 2.0 ** -8) == 1.0
    assert L.oracle_bf16(1.0 + 3 * 2.0 ** -8) == 1.0 + 2.0 ** -6
    assert L.oracle_bf16(-3.0) == -3.0


def test_graph(small):
    m, net = small
    deg = np.diff(net.nptr)
    assert deg.sum() == 2 * m.nedge
    e = np.asarray(m.edges).reshape(-1, 2)
    assert np.array_equal(np.bincount(e.ravel(), minlength=m.nnode), deg)
    # every neighbour entry's normal is the edge normal, flipped for the second node
    ea = np.asarray(m.edge_area).reshape(-1, 4)
    i = 0
    p = net.nptr[i]
    j = net.nbr[p]
    k = np.nonzero(((e[:, 0] == i) & (e[:, 1] == j)) | ((e[:, 0] == j) & (e[:, 1] == i)))[0][0]
    sgn = 1.0 if e[k, 0] == i else -1.0
    assert np.allclose(net.ef[p, :3], sgn * ea[k, :3], atol=1e-7)
    assert np.all(net.ef[:, 3] > 0)


def test_backward_matches_central_differences(small):
    m, net = small
    rng = np.random.default_rng(3)
    n = m.nnode
    x = rng.uniform(-1, 1, (n, 11)).astype(np.float32)
    t = rng.uniform(-1, 1, (n, 5)).astype(np.float32)
    w = lp_random_params(5)
    loss, g = net.loss_grad(x, t, w, emulate=0)
    assert loss > 0
    # a spread of parameters from every block
    idx = list(range(0, 704, 97)) + [704 + 3]
    for l in range(3):
        b = 768 + l * 8576
        idx += [b + 5, b + 130, b + 256 + 7, b + 320 + 1000, b + 320 + 4096 + 2000, b + 8512 + 9]
    idx += [26496 + 17, 26496 + 300, 26816 + 2]
    h = 1e-3
    for k in idx:
        wp = w.astype(np.float64).copy()
        wm = wp.copy()
        wp[k] += h
        wm[k] -= h
        # perturb through a float32 copy: use the exact perturbed values
        lp_, _ = net.loss_grad(x, t, wp.astype(np.float32), emulate=0)
        lm_, _ = net.loss_grad(x, t, wm.astype(np.float32), emulate=0)
        hp = float(np.float32(wp[k])) - float(np.float32(wm[k]))
        fd = (lp_ - lm_) / hp
        assert abs(fd - g[k]) <= 2e-3 * max(1.0, abs(g[k])) + 1e-6, (k, fd, g[k])


def test_emulated_forward_close_to_exact(small):
    m, net = small
    rng = np.random.default_rng(4)
    x = rng.uniform(-1, 1, (m.nnode, 11)).astype(np.float32)
    w = lp_random_params(6)
    a = net.forward(x, w, emulate=0)
    b = net.forward(x, w, emulate=1)
    rel = np.linalg.norm(a - b) / np.linalg.norm(a)
    assert 0 < rel < 5e-2
