"""Host mesh preprocessing: the reference's maps and dual metrics
(ucs/mesh.tcc BuildPsp/BuildEdges/CalcAreasVolumes/CheckForClosure)."""
import json
from pathlib import Path

import numpy as np
import pytest

from proteuscfd_gb300 import Mesh, cases

GOLDEN = Path(__file__).resolve().parent / "golden"


def kuhn_counts(nx, ny, nz):
    """Node, interior-edge, half-edge and CRS-block counts of a 6-tet Kuhn box."""
    n = nx * ny * nz
    axis = (nx - 1) * ny * nz + nx * (ny - 1) * nz + nx * ny * (nz - 1)
    face = (nx - 1) * (ny - 1) * nz + (nx - 1) * ny * (nz - 1) + nx * (ny - 1) * (nz - 1)
    body = (nx - 1) * (ny - 1) * (nz - 1)
    e = axis + face + body
    quads = 2 * ((nx - 1) * (ny - 1) + (nx - 1) * (nz - 1) + (ny - 1) * (nz - 1))
    b = 3 * 2 * quads
    return n, e, b, n + 2 * e


@pytest.mark.parametrize("dims,expect", [
    ((64, 32, 32), (65536, 438527, 58404, 942590)),     # euler ramp box
])
def test_box_counts_match_closed_forms(dims, expect):
    assert kuhn_counts(*dims) == expect
    m = Mesh.box(*dims, lx=2.0, jitter=0.2, ramp_deg=15.0)
    assert (m.nnode, m.nedge, m.nbedge, m.nnode + 2 * m.nedge) == expect


def test_full_size_counts_closed_form():
    assert kuhn_counts(128, 96, 96) == (1179648, 8123007, 397860, 17425662)
    assert kuhn_counts(256, 176, 176) == (7929856, 55025855, 1438500, 117981566)


@pytest.mark.parametrize("case", [cases.euler_ramp(12, 8, 6), cases.ns_flatplate(10, 9, 7)])
def test_maps_and_closure(case):
    m = cases.build_mesh(case)
    st = m.stats()
    assert st["unclosed"] == 0 and st["max_open"] < 1e-12
    assert st["rewound"] == 0
    e = m.edges
    # BuildEdges: left node ascending, left < right
    assert np.all(np.diff(e[:, 0]) >= 0) and np.all(e[:, 0] < e[:, 1])
    # psp symmetric, no self or duplicate entries
    ipsp, psp = m.ipsp, m.psp
    pairs = set()
    for i in range(m.nnode):
        nb = psp[ipsp[i]:ipsp[i + 1]]
        assert len(set(nb.tolist())) == len(nb) and i not in nb
        pairs.update((i, int(j)) for j in nb)
    assert all((j, i) in pairs for (i, j) in pairs)
    assert len(pairs) == 2 * m.nedge
    # phantom ids
    be = m.bedges
    assert np.array_equal(be[:, 1], np.arange(m.nnode, m.nnode + m.nbedge))
    assert np.all(m.vol > 0)
    # unit normals
    assert np.allclose(np.linalg.norm(m.edge_area[:, :3], axis=1), 1.0, atol=1e-14)
    assert np.allclose(np.linalg.norm(m.bedge_area[:, :3], axis=1), 1.0, atol=1e-14)


def test_unit_cube_known_answer():
    """unitTest/meshTest.h:97-109: the GMSH unit cube has 14 nodes, 48
    elements and total dual volume 1 (tolerance 1e-7 as in the reference)."""
    d = json.loads((GOLDEN / "cube_msh.json").read_text())
    xyz = np.array(d["xyz"])
    tets = []
    for t in d["tets"]:
        a, b, c, q = xyz[t]
        if np.dot(np.cross(b - a, c - a), q - a) < 0:  # right-handed node order
            t = [t[0], t[2], t[1], t[3]]
        tets.append(t)
    m = Mesh.from_elements(xyz, d["tris"], d["tri_tags"], tets)
    st = m.stats()
    assert m.nnode == d["expect"]["nnode"]
    assert st["ntri"] + st["ntet"] == d["expect"]["nelem"]
    assert abs(st["total_vol"] - d["expect"]["volume"]) < 1e-7
    assert st["unclosed"] == 0


def test_box_volume_equals_geometry():
    m = Mesh.box(9, 7, 5, lx=2.0, ly=1.0, lz=0.5, jitter=0.2, seed=3)
    assert abs(m.vol.sum() - 1.0) < 1e-13
    m = Mesh.box(9, 7, 5, lx=1.0, ly=1.0, lz=1.0, jitter=0.0, y_ratio=1.1)
    assert abs(m.vol.sum() - 1.0) < 1e-13


def test_rcm_order_is_the_reference_sequence_applied_as_old_to_new():
    """pcfd_mesh_rcm_order returns Mesh::ordering as ReorderMeshCuthillMcKee(1)
    leaves it: the reversed Cuthill-McKee sequence (position -> node), whose
    neighbours in the sequence are neighbours in the mesh, so read that way it
    has a small bandwidth.  The reference's ReorderC2nMap then applies it as an
    old-to-new map (node n becomes ordering[n]); the reordered mesh built with
    reorder=True follows that."""
    m = Mesh.box(10, 9, 8, jitter=0.2)
    order = m.rcm_order()
    assert sorted(order.tolist()) == list(range(m.nnode))
    assert order[-1] == 0  # the sequence starts at node 0 and is reversed
    pos = np.empty_like(order)
    pos[order] = np.arange(m.nnode)
    e = m.edges
    assert np.abs(pos[e[:, 0]] - pos[e[:, 1]]).max() < 0.3 * m.nnode
    r = Mesh.box(10, 9, 8, jitter=0.2, reorder=True)
    np.testing.assert_array_equal(r.ordering, order)
    np.testing.assert_array_equal(r.xyz[order], m.xyz)


def test_rcm_numbering_reduces_bandwidth():
    """reorder="rcm" numbers nodes in the reverse Cuthill-McKee sequence
    (new node k is old node ordering[k]); the reference's set-up reorder
    uses the same list as an old-to-new map, which scatters neighbours.  On
    a structured box the natural numbering is already near the minimum
    bandwidth (one x-y plane); the sequence from corner node 0 sweeps
    diagonal planes, a little wider."""
    from proteuscfd_gb300 import Mesh

    def bandwidth(m):
        e = np.asarray(m.edges).reshape(-1, 2)
        return int(np.abs(e[:, 0] - e[:, 1]).max())

    kw = dict(nx=14, ny=11, nz=9, jitter=0.2, seed=3)
    plain = Mesh.box(**kw)
    rcm = Mesh.box(reorder="rcm", **kw)
    ref = Mesh.box(reorder=True, **kw)
    assert sorted(rcm.ordering.tolist()) == list(range(plain.nnode))
    np.testing.assert_array_equal(rcm.xyz, plain.xyz[rcm.ordering])
    assert np.array_equal(rcm.ordering, ref.ordering)
    assert bandwidth(rcm) < 1.5 * bandwidth(plain)
    assert bandwidth(ref) > 4 * bandwidth(rcm)
