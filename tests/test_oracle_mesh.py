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
                                dict(nx=10, ny=6, nz=5, lx=2.0, jitter=0.2, seed=9, ramp_deg=15.0, ramp_x0=0.5)])
def test_oracle_box_matches_product_box(kw):
    o = OracleMesh.box(**kw)
    p = Mesh.box(**kw)
    for k in FIELDS:
        np.testing.assert_array_equal(getattr(o, k), getattr(p, k), err_msg=k)
