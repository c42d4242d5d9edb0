"""Generates the committed golden fixtures in this directory from the
reference source tree (run in a checkout that has it; the fixtures then
travel without it):

* cube_msh.json - the 14-node / 48-element unit cube of the reference's mesh
  unit test (unitTest/meshResources/cube.msh, checked at
  unitTest/meshTest.h:97-109: 14 nodes, 48 elements, total volume 1).
* ref_pin_vectors.json - outputs of the reference's own ucs/matrix.h (LU,
  LuSolve, MatVecMult) and ucs/geometry.h (CalcTriArea, CalcTetVol) on
  seeded inputs, computed through oracle/_ref/libref_pin.so.

Usage: python tests/golden/make_golden.py [/path/to/reference]
"""
import ctypes as C
import json
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent


def read_gmsh2(path):
    lines = Path(path).read_text().split("\n")
    i = lines.index("$Nodes")
    nn = int(lines[i + 1])
    xyz = [[float(v) for v in lines[i + 2 + k].split()[1:4]] for k in range(nn)]
    j = lines.index("$Elements")
    ne = int(lines[j + 1])
    tris, tags, tets = [], [], []
    for k in range(ne):
        f = [int(v) for v in lines[j + 2 + k].split()]
        etype, ntag = f[1], f[2]
        nodes = [v - 1 for v in f[3 + ntag:]]
        if etype == 2:
            tris.append(nodes)
            tags.append(f[3 + 1])  # elementary entity tag as the boundary tag
        elif etype == 4:
            tets.append(nodes)
    return xyz, tris, tags, tets


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PCFD_REFERENCE_SRC")
    if not ref:
        sys.exit("usage: make_golden.py <reference checkout> (or set PCFD_REFERENCE_SRC)")
    ref = Path(ref)
    xyz, tris, tags, tets = read_gmsh2(ref / "unitTest" / "meshResources" / "cube.msh")
    (HERE / "cube_msh.json").write_text(json.dumps(
        {"source": "unitTest/meshResources/cube.msh", "expect": {"nnode": 14, "nelem": 48, "volume": 1.0},
         "xyz": xyz, "tris": tris, "tri_tags": tags, "tets": tets}))

    sys.path.insert(0, str(ROOT))
    os.environ["PCFD_REFERENCE_SRC"] = str(ref)
    from proteuscfd_gb300 import build as B
    lib_path = B.build_ref_pin()
    L = C.CDLL(str(lib_path))
    DP = C.POINTER(C.c_double)
    IP = C.POINTER(C.c_int)
    rng = np.random.default_rng(20261203)
    cases = []
    for k in range(24):
        a = rng.normal(size=(5, 5)) + (np.eye(5) * (3.0 if k % 3 else 0.0))
        if k % 4 == 0:
            a[:, 0] *= 1e-3  # force pivoting
        b = rng.normal(size=5)
        a_lu = np.ascontiguousarray(a.copy())
        p = np.zeros(5, dtype=np.int32)
        err = L.ref_lu(a_lu.ctypes.data_as(DP), p.ctypes.data_as(IP), 5)
        bb = b.copy()
        x = np.zeros(5)
        L.ref_lusolve(a_lu.ctypes.data_as(DP), bb.ctypes.data_as(DP), p.ctypes.data_as(IP), x.ctypes.data_as(DP), 5)
        y = np.zeros(5)
        L.ref_matvec(np.ascontiguousarray(a).ctypes.data_as(DP), np.ascontiguousarray(b).ctypes.data_as(DP),
                     y.ctypes.data_as(DP), 5)
        cases.append({"a": a.tolist(), "b": b.tolist(), "lu": a_lu.tolist(), "piv": p.tolist(), "err": err,
                      "solve": bb.tolist(), "matvec": y.tolist()})
    geo = []
    L.ref_tet_vol.restype = C.c_double
    for k in range(24):
        pts = rng.normal(size=(4, 3))
        r = np.zeros(3)
        L.ref_tri_area(*[np.ascontiguousarray(pts[i]).ctypes.data_as(DP) for i in range(3)], r.ctypes.data_as(DP))
        v = L.ref_tet_vol(*[np.ascontiguousarray(pts[i]).ctypes.data_as(DP) for i in range(4)])
        geo.append({"pts": pts.tolist(), "tri_area": r.tolist(), "tet_vol": v})
    (HERE / "ref_pin_vectors.json").write_text(json.dumps(
        {"source": "ucs/matrix.h LU/LuSolve/MatVecMult, ucs/geometry.h CalcTriArea/CalcTetVol",
         "matrix": cases, "geometry": geo}))
    print("wrote", HERE / "cube_msh.json", HERE / "ref_pin_vectors.json")


if __name__ == "__main__":
    main()
