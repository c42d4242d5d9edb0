"""Host mesh preprocessing against the reference's own maps and metrics.

The fixtures were written by the reference solver itself
(tests/golden/make_ref_fixtures.py): the element list its solver read, the
reverse Cuthill-McKee ordering of its set-up, and every map and metric it
built from them.  Integer work must match bit for bit (ordering, psp, edges,
boundary half-edges, CRS structure); the dual metrics and LSQ matrices are
computed in the reference's operation order and must match exactly too.

Reference: ucs/mesh.tcc:517 (BuildPsp), :1056 (BuildEdges), :1653
(CalcAreasVolumes), :2412 (ReorderMeshCuthillMcKee), :224 (ReorderC2nMap);
ucs/gradient.tcc:115,461 (LSQ normal matrices).
"""
import numpy as np
import pytest

import ref_fixtures as R

FIELDS_EXACT = ["xyz", "ipsp", "psp", "edges", "bedges", "bfactag", "edge_area", "bedge_area", "vol", "sw"]


@pytest.mark.parametrize("case", R.CASES)
def test_maps_and_metrics_bit_exact(case):
    f = R.load(case)
    m = R.mesh(f)
    assert m.nnode == R.scalar(f, "nnode")
    assert m.nedge == R.scalar(f, "nedge")
    assert m.nbedge == R.scalar(f, "nbedge")
    for k in FIELDS_EXACT:
        np.testing.assert_array_equal(getattr(m, k), f[k], err_msg="%s: %s" % (case, k))


@pytest.mark.parametrize("case", [c for c in R.CASES if R.scalar(R.load(c), "case_reorder")])
def test_cuthill_mckee_ordering_bit_exact(case):
    f = R.load(case)
    m = R.mesh(f)
    np.testing.assert_array_equal(m.ordering, f["ordering"])


def test_reorder_changes_numbering_and_keeps_geometry():
    """The reorder is a permutation: same node set, same total volume."""
    f = R.load("ns_plate")
    el = f["elements_pre"]
    t = el[:, 0]
    from proteuscfd_gb300 import Mesh
    plain = Mesh.from_elements(f["xyz_pre"], el[t == 0][:, 3:6], el[t == 0][:, 1], el[t == 2][:, 3:7])
    m = R.mesh(f)
    assert sorted(m.ordering.tolist()) == list(range(m.nnode))
    np.testing.assert_array_equal(m.xyz[m.ordering], plain.xyz)
    assert abs(m.vol.sum() - plain.vol.sum()) < 1e-14 * plain.vol.sum()
    assert m.nedge == plain.nedge
