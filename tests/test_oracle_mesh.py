"""The oracle's own mesh generator and preprocessing (oracle/mesh.c), which
the CPU baseline builds its workload with, against the reference's maps and
metrics and against the product's box generator - bit for bit."""
import numpy as np
import pytest

import ref_fixtures as R
from oracle_lib import OracleMesh
from proteuscfd_gb300 import Mesh

FIELDS = ["xyz", "ipsp", "psp", "edges", "bedges", "bfactag", "edge_area", "bedge_area", "vol", "sw"]


@pytest.mark.parametrize("case", R.CASES)
def test_oracle_preprocessing_matches_reference(case):
    f = R.load(case)
    el = f["elements_pre"].copy()
    xyz = f["xyz_pre"]
    if R.scalar(f, "case_reorder"):
        # the reference's set-up reorder: node n becomes ordering[n] (ReorderC2nMap)
        o = f["ordering"]
        nodes = el[:, 3:11]
        nodes[nodes >= 0] = o[nodes[nodes >= 0]]
        x2 = np.empty_like(xyz)
        x2[o] = xyz
        xyz = x2
    t = el[:, 0]
    m = OracleMesh.from_elements(xyz, el[t == 0][:, 3:6], el[t == 0][:, 1], el[t == 2][:, 3:7])
    for k in FIELDS:
        np.testing.assert_array_equal(getattr(m, k), f[k], err_msg="%s: %s" % (case, k))


@pytest.mark.parametrize("kw", [dict(nx=9, ny=7, nz=6, lx=1.3, jitter=0.2, seed=4, y_ratio=1.1),
                                dict(nx=9, ny=8, nz=5, lx=1.1, jitter=0.2, seed=5, y_ratio=1.2, jitter_mode=1),
                                dict(nx=10, ny=6, nz=5, lx=2.0, jitter=0.2, seed=9, ramp_deg=15.0, ramp_x0=0.5),
                                dict(nx=14, ny=12, nz=4, lx=13 / 11, jitter=0.2, seed=6, y_ratio=1.1, wall_ar_max=3.0,
                                     wall_start_i=2, upstream_tag=7),
                                # large enough (98,560 nodes, 74k half-edges) for the product's
                                # preprocessing to run its loops on several host threads
                                dict(nx=56, ny=44, nz=40, lx=55 / 43, jitter=0.2, seed=3, y_ratio=1.1, jitter_mode=1,
                                     wall_ar_max=50.0, wall_start_i=12, upstream_tag=7)])
def test_oracle_box_matches_product_box(kw):
    o = OracleMesh.box(**kw)
    p = Mesh.box(**kw)
    for k in FIELDS:
        np.testing.assert_array_equal(getattr(o, k), getattr(p, k), err_msg=k)


def test_wall_cell_floor_and_run_in():
    """The first wall cell is floored at the x spacing / wall_ar_max, the
    spacing grows by y_ratio and stops at the spacing that fills the height;
    y=0 faces ahead of wall_start_i carry the upstream tag."""
    nx, ny = 40, 30
    kw = dict(nx=nx, ny=ny, nz=3, lx=(nx - 1) / (ny - 1), y_ratio=1.1)
    plain = OracleMesh.box(**kw)
    capped = OracleMesh.box(wall_ar_max=5.0, wall_start_i=10, upstream_tag=7, **kw)
    y0 = np.unique(plain.xyz[:, 1])
    y1 = np.unique(capped.xyz[:, 1])
    h0, h1 = np.diff(y0), np.diff(y1)
    hx = 1.0 / (ny - 1)
    assert h0[0] < hx / 5.0 and abs(h1[0] - hx / 5.0) < 1e-15
    ratio = h1[1:] / h1[:-1]
    grow = ratio > 1.0 + 1e-9
    k = int(np.argmin(grow))  # first spacing that stops growing
    assert np.allclose(ratio[:k - 1], 1.1, rtol=1e-12)  # geometric up to the cap ...
    assert np.allclose(h1[k + 1:-1], h1[k + 1], rtol=1e-12)  # ... constant after it
    assert h1[k] <= h1[k + 1] * (1 + 1e-12) and abs(y1[-1] - 1.0) < 1e-15
    # the y=0 half-edges ahead of x = 10 hx carry tag 7, the rest tag 3
    b = capped.bedges[:, 0]
    yb, xb, tag = capped.xyz[b, 1], capped.xyz[b, 0], capped.bfactag
    bottom = (yb == 0.0) & ((tag == 3) | (tag == 7))
    assert set(tag[bottom & (xb < 10 * hx - 1e-12)]) == {7}
    assert set(tag[bottom & (xb > 10 * hx + 1e-12)]) == {3}
