"""Loading of the reference-output fixtures (tests/golden/ref_<case>.npz,
written by tests/golden/make_ref_fixtures.py from the reference solver
itself) and the product-side objects for the same case: the mesh built from
the reference's own element list with the reference's reorder, and the
parameters the reference derived from its input deck."""
from pathlib import Path

import numpy as np

from proteuscfd_gb300 import Mesh, Param

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = ("euler_ramp", "ns_plate", "ns_plate_barth")


def load(case):
    f = np.load(GOLDEN / ("ref_%s.npz" % case))
    return {k: f[k] for k in f.files}


def scalar(f, k):
    return f[k].ravel()[0].item()


def mesh(f):
    """Product mesh from the element list the reference's solver read (its
    partitioned mesh, before set-up), reordered the way the reference's
    set-up does when the case asks for it."""
    el = f["elements_pre"]
    t = el[:, 0]
    tris, tags, tets = el[t == 0][:, 3:6], el[t == 0][:, 1], el[t == 2][:, 3:7]
    reorder = bool(scalar(f, "case_reorder"))
    return Mesh.from_elements(f["xyz_pre"], tris, tags, tets, reorder=reorder)


def param(f):
    bct = {int(a): int(b) for a, b in f["case_bc_types"]}
    twall = {int(a): float(b) for a, b in f["case_twall"]}
    return Param(gamma=scalar(f, "gamma"), mach=scalar(f, "velocity"), Re=scalar(f, "Re"), Pr=scalar(f, "Pr"),
                 ref_temperature=scalar(f, "ref_temperature"), sorder=scalar(f, "sorder"), chi=scalar(f, "chi"),
                 viscous=scalar(f, "viscous"), limiter=scalar(f, "param_limiter"), venkat_K=1.0,
                 tinf=scalar(f, "qinf_T"), pinf=scalar(f, "qinf_p"),
                 bc_type=bct, bc_twall=twall)
