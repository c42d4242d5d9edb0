"""Generates the reference-output fixtures ``ref_<case>.npz`` in this directory
by running the reference solver itself (oracle/refbuild, built from the
reference's own sources) on small synthetic cases.  Run it in a checkout that
has the reference; the fixtures then travel without it.

For each case this script
  1. writes a jittered Kuhn-split tetrahedral box as UGRID (the reference's
     ASCII reader, ucs/mesh.tcc:6740) with boundary tags 1..6 on the faces
     x=0, x=max, y=0, y=max, z=0, z=max, a ``.param`` and a ``.bc`` file, and a
     seeded ``.qinit`` state (freestream x (1 + U[-amp, amp]) per stored
     variable); a reacting case also gets its mechanism file and the species
     datasets as ``chemdb.txt``, which the harness stores as the case's
     chemical database;
  2. runs ``oracle/_ref/ref_dump``, which decomposes the mesh into one
     partition (udecomp.x), sets the solver up as ucs.x does (reverse
     Cuthill-McKee reorder, maps, metrics, CRS) and runs Newton steps stage by
     stage;
  3. packs every array it wrote into ``ref_<case>.npz``.

Usage: python tests/golden/make_ref_fixtures.py <reference checkout>
       (or set PCFD_REFERENCE_SRC)
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent

# boundary types by name (ucs/bc_defines.h)
CASES = {
    # the Euler ramp family: Mach 2 Euler over a sheared ramp, first order
    "euler_ramp": dict(
        n=(9, 6, 5), lx=2.0, ly=1.0, lz=1.0, jitter=0.2, seed=11, ramp_deg=15.0, ramp_x0=0.5, y_ratio=1.0,
        eqn="compressibleEuler", mach=2.0, sorder=1, limiter=0, nsgs=10, cfl=5.0, steps=3, amp=0.01,
        bc={1: "sonicInflow", 2: "sonicOutflow", 3: "impermeableWall", 4: "impermeableWall",
            5: "symmetry", 6: "symmetry"}),
    # the flat-plate family: Mach 0.8 laminar NS over an adiabatic no-slip wall, second order
    "ns_plate": dict(
        n=(8, 7, 5), lx=7.0 / 6.0, ly=1.0, lz=1.0, jitter=0.2, seed=12, ramp_deg=0.0, ramp_x0=0.5, y_ratio=1.1,
        eqn="compressibleNS", mach=0.8, sorder=2, limiter=3, nsgs=10, cfl=5.0, steps=3, amp=0.01,
        bc={1: "farField", 2: "farField", 3: "noSlip", 4: "farField", 5: "symmetry", 6: "symmetry"},
        twall={3: -1.0}),
    # the same physics with the Barth limiter and a second seed; no reorder
    "ns_plate_barth": dict(
        n=(7, 6, 6), lx=1.2, ly=1.0, lz=1.0, jitter=0.2, seed=13, ramp_deg=0.0, ramp_x0=0.5, y_ratio=1.1,
        eqn="compressibleNS", mach=0.8, sorder=2, limiter=1, nsgs=6, cfl=3.0, steps=2, amp=0.02,
        bc={1: "farField", 2: "farField", 3: "noSlip", 4: "farField", 5: "symmetry", 6: "symmetry"},
        twall={3: -1.0}, reorder=0),
    # the reacting set: 5-species air (the reference's chemModels/5speciesAir.rxn), laminar NS,
    # second order, an isothermal no-slip wall, finite-rate chemistry on
    "fr_plate": dict(
        n=(7, 6, 5), lx=1.2, ly=1.0, lz=1.0, jitter=0.2, seed=14, ramp_deg=0.0, ramp_x0=0.5, y_ratio=1.1,
        eqn="compressibleNSFR", mach=2.0, sorder=2, limiter=3, nsgs=4, cfl=2.0, steps=2, amp=0.01,
        bc={1: "sonicInflow", 2: "sonicOutflow", 3: "noSlip", 4: "sonicOutflow", 5: "symmetry", 6: "symmetry"},
        twall={3: 1500.0}, reorder=1, chem="5speciesAir", temperature=3000.0, no_cvbc=1,
        # mass fractions in the model's species order (O2, O, N, N2, NO: first appearance over the
        # mechanism's reactions, ChemModel::BuildGlobalSpeciesList): partly dissociated air
        massfractions=[0.2, 0.01, 0.01, 0.745, 0.035]),
}


def write_chem_db(path, fixture):
    """The species datasets Species::GetDBInfo reads (ucs/species.tcc:140),
    from the fixture the reference's own database builder produced, as the
    text the harness writes into the stand-in HDF5 store."""
    import json
    d = json.loads(Path(fixture).read_text())
    lines = []
    for sp in d["species"]:
        lines.append("species %s" % sp["name"])
        lines.append("MW %r" % (sp["MW"] * 1000.0))
        lines.append("NASA7_burcat_coeff15 %r" % sp["hf298"])
        for key, v in (("NASA7_burcat1", sp["lo"]), ("NASA7_burcat2", sp["hi"])):
            lines.append("%s %d 1 %s" % (key, len(v), " ".join(repr(float(x)) for x in v)))
        for key in ("mu", "k"):
            rows = sp[key]
            lines.append("%s %d %d %s" % (key, len(rows), len(rows[0]),
                                          " ".join(repr(float(x)) for r in rows for x in r)))
    Path(path).write_text("\n".join(lines) + "\n")


def kuhn_box(nx, ny, nz, lx, ly, lz, jitter, seed, ramp_deg, ramp_x0, y_ratio):
    """Node box split into 6 tets per hex along the (0,0,0)-(1,1,1) diagonal;
    interior nodes jittered by U[-jitter*h, jitter*h] per axis; optional y
    shear ramp and geometric y clustering toward y=0."""
    cx = lx * np.arange(nx) / (nx - 1)
    cz = lz * np.arange(nz) / (nz - 1)
    if y_ratio > 1.0:
        h = (y_ratio - 1.0) / (y_ratio ** (ny - 1) - 1.0) * y_ratio ** np.arange(ny - 1)
        cy = ly * np.concatenate([[0.0], np.cumsum(h)])
        cy[-1] = ly
    else:
        cy = ly * np.arange(ny) / (ny - 1)

    def local_h(c):
        d = np.diff(c)
        left = np.concatenate([[np.inf], d])
        right = np.concatenate([d, [np.inf]])
        return np.minimum(left, right)

    hx, hy, hz = local_h(cx), local_h(cy), local_h(cz)
    rng = np.random.default_rng(seed)
    K, J, I = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    I, J, K = I.ravel(), J.ravel(), K.ravel()
    x, y, z = cx[I].copy(), cy[J].copy(), cz[K].copy()
    interior = (I > 0) & (I < nx - 1) & (J > 0) & (J < ny - 1) & (K > 0) & (K < nz - 1)
    r = rng.uniform(-1.0, 1.0, size=(len(x), 3))
    x[interior] += jitter * hx[I[interior]] * r[interior, 0]
    y[interior] += jitter * hy[J[interior]] * r[interior, 1]
    z[interior] += jitter * hz[K[interior]] * r[interior, 2]
    if ramp_deg:
        t = np.tan(np.radians(ramp_deg))
        m = x > ramp_x0
        y[m] = y[m] + t * (x[m] - ramp_x0) * (ly - y[m]) / ly
    xyz = np.stack([x, y, z], axis=1)

    def nid(i, j, k):
        return i + nx * (j + ny * k)

    tets = []
    perms = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]
    for k in range(nz - 1):
        for j in range(ny - 1):
            for i in range(nx - 1):
                for p in perms:
                    off = [0, 0, 0]
                    v = [nid(i, j, k)]
                    off[p[0]] = 1
                    v.append(nid(i + off[0], j + off[1], k + off[2]))
                    off[p[1]] = 1
                    v.append(nid(i + off[0], j + off[1], k + off[2]))
                    v.append(nid(i + 1, j + 1, k + 1))
                    a, b, c, d = (xyz[q] for q in v)
                    if np.dot(d - a, np.cross(b - a, c - a)) < 0.0:
                        v[1], v[2] = v[2], v[1]
                    tets.append(v)
    tris, tags = [], []
    for f in range(6):
        axis, side = f // 2, f % 2
        out = np.zeros(3)
        out[axis] = 1.0 if side else -1.0
        dims = [nx, ny, nz]
        a_ax, b_ax = [d for d in range(3) if d != axis]
        fixed = dims[axis] - 1 if side else 0
        for b in range(dims[b_ax] - 1):
            for a in range(dims[a_ax] - 1):
                def corner(da, db):
                    ijk = [0, 0, 0]
                    ijk[axis] = fixed
                    ijk[a_ax] = a + da
                    ijk[b_ax] = b + db
                    return nid(*ijk)
                q0, q1, q2, q3 = corner(0, 0), corner(1, 0), corner(1, 1), corner(0, 1)
                for t in ((q0, q1, q2), (q0, q2, q3)):
                    t = list(t)
                    nrm = np.cross(xyz[t[1]] - xyz[t[0]], xyz[t[2]] - xyz[t[0]])
                    if np.dot(nrm, out) < 0.0:
                        t[0], t[2] = t[2], t[0]
                    tris.append(t)
                    tags.append(f + 1)
    return xyz, np.array(tris, dtype=np.int64), np.array(tags, dtype=np.int64), np.array(tets, dtype=np.int64)


def write_ugrid(path, xyz, tris, tags, tets):
    with open(path, "w") as f:
        f.write("%d %d 0 %d 0 0 0\n" % (len(xyz), len(tris), len(tets)))
        for p in xyz:
            f.write("%r %r %r\n" % (float(p[0]), float(p[1]), float(p[2])))
        for t in tris:
            f.write("%d %d %d\n" % tuple(int(v) + 1 for v in t))
        for g in tags:
            f.write("%d\n" % int(g))
        for t in tets:
            f.write("%d %d %d %d\n" % tuple(int(v) + 1 for v in t))


def write_param(path, name, c):
    lines = [
        "<<<BEGIN TEMPORAL CONTROL>>>",
        "numTimeSteps = %d" % c["steps"],
        "newtonIterations = 1",
        "<<<END TEMPORAL CONTROL>>>",
        "<<<BEGIN SPACE %s>>>" % name,
        "equationSet = %s" % c["eqn"],
        "fluxType = roeFlux",
        "reorderMesh = %d" % c.get("reorder", 1),
        "localTimeStepping = 1",
        "startingCFL = %r" % c["cfl"],
        "CFL = %r" % c["cfl"],
        "rampCFL = 0",
        "spatialOrder = %d" % c["sorder"],
        "limiter = %d" % c["limiter"],
        "numberSGS = %d" % c["nsgs"],
        "jacobianUpdateFrequency = 1",
        "velocity = %r" % c["mach"],
        "flowDirection = [1.0, 0.0, 0.0]",
        "refPressure = 101325.0",
        "initialPressure = 101325.0",
        "initialTemperature = %r" % c.get("temperature", 300.0),
        "refLength = 1.0",
        # laminar viscosity giving Re close to 1e5 on unit length (the
        # reference derives Re from it, ucs/compressible.tcc:86-89)
        "refViscosity = 0.0032686",
        "prandtlNumber = 0.72",
        "solutionWrite = 0",
        "turbulenceModel = 0",
    ]
    if "chem" in c:
        lines += ["chemicalDatabase = chemdb.h5",
                  "massFractions = [%s]" % ", ".join(repr(float(v)) for v in c["massfractions"]),
                  "reactionsOn = 1",
                  "noCVBC = %d" % c.get("no_cvbc", 0)]
    lines.append("<<<END SPACE>>>")
    Path(path).write_text("\n".join(lines) + "\n")


def write_bc(path, c):
    lines = []
    for tag, kind in sorted(c["bc"].items()):
        extra = ""
        if tag in c.get("twall", {}):
            extra = " twall = [%r]" % c["twall"][tag]
        lines.append('surface #%d = %s "face%d"%s' % (tag, kind, tag, extra))
    # the no-slip walls as composite body 1, whose forces the reference reports
    walls = [t for t, k in sorted(c["bc"].items()) if k == "noSlip"]
    if walls:
        lines.append("body #1 = [%s]" % ", ".join(str(t) for t in walls))
    Path(path).write_text("\n".join(lines) + "\n")


def run_case(exe, name, c, workdir, ref=None):
    nx, ny, nz = c["n"]
    xyz, tris, tags, tets = kuhn_box(nx, ny, nz, c["lx"], c["ly"], c["lz"], c["jitter"], c["seed"],
                                     c["ramp_deg"], c["ramp_x0"], c["y_ratio"])
    d = Path(workdir) / name
    d.mkdir(parents=True, exist_ok=True)
    write_ugrid(d / (name + ".ugrid"), xyz, tris, tags, tets)
    write_param(d / (name + ".param"), name, c)
    write_bc(d / (name + ".bc"), c)
    if "chem" in c:
        # the mechanism file beside the case (ChemModel reads <case>.rxn) and the species data
        (d / (name + ".rxn")).write_text((Path(ref) / "chemModels" / (c["chem"] + ".rxn")).read_text())
        write_chem_db(d / "chemdb.txt", HERE / "chem_5species_air.json")
    # freestream (non-dimensional: rho = gamma, p = 1, |u| = Mach) with a seeded perturbation
    rng = np.random.default_rng(1000 + c["seed"])
    out = d / "dump"
    out.mkdir(exist_ok=True)
    # the reference's own gamma (Cp / Cv with its default Cp and MW) sets rho_inf
    r_univ = 8.314459848  # ucs/chem_constants.h R_UNIV is checked against the dump below
    del r_univ
    # Pass 1 without .qinit: learn qinf; pass 2 with the perturbed state.
    for p in d.glob("*.qinit"):
        p.unlink()
    subprocess.run([str(exe), str(d), name, str(out), "1"], check=True, cwd=d,
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    qinf = np.fromfile(out / "qinf.bin", dtype="<f8")
    neqn = int(np.fromfile(out / "neqn.bin", dtype="<i4")[0])
    q0 = np.tile(qinf[:neqn], (len(xyz), 1)) * (1.0 + rng.uniform(-c["amp"], c["amp"], size=(len(xyz), neqn)))
    if "chem" in c:
        # native variables (rhoi, u, v, w, T): give v and w a seeded non-zero part too
        ns = neqn - 4
        q0[:, ns + 1:ns + 3] += c["amp"] * qinf[ns] * rng.uniform(-1.0, 1.0, size=(len(xyz), 2))
    q0.astype("<f8").tofile(d / (name + ".qinit"))
    for p in out.glob("*"):
        p.unlink()
    subprocess.run([str(exe), str(d), name, str(out), str(c["steps"])], check=True, cwd=d,
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    arrays = {}
    for line in (out / "index.txt").read_text().split("\n"):
        if not line.strip():
            continue
        nm, dt, n0, n1 = line.split()
        if nm == "s2_jacobian":  # the step-1 matrix already pins the assembly
            continue
        a = np.fromfile(out / (nm + ".bin"), dtype="<" + dt)
        arrays[nm] = a.reshape(int(n0), int(n1)) if int(n1) > 1 else a
    arrays["ugrid_xyz"] = xyz
    arrays["ugrid_tris"] = tris.astype(np.int32)
    arrays["ugrid_tri_tags"] = tags.astype(np.int32)
    arrays["ugrid_tets"] = tets.astype(np.int32)
    arrays["qinit_file_order"] = q0
    arrays["case_bc_types"] = np.array([[t, ["dirichlet", "neumann", "impermeableWall", "noSlip", "farFieldViscous",
                                              "farField", "sonicInflow", "sonicOutflow", "symmetry"].index(k) + 1]
                                        for t, k in sorted(c["bc"].items())], dtype=np.int32)
    arrays["case_twall"] = np.array([[t, v] for t, v in sorted(c.get("twall", {}).items())] or np.zeros((0, 2)))
    arrays["case_nsgs"] = np.array(c["nsgs"])
    arrays["case_reorder"] = np.array(c.get("reorder", 1))
    arrays["case_cfl"] = np.array(c["cfl"])
    arrays["case_steps"] = np.array(c["steps"])
    np.savez_compressed(HERE / ("ref_%s.npz" % name), **arrays)
    return arrays


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PCFD_REFERENCE_SRC")
    if not ref:
        sys.exit("usage: make_ref_fixtures.py <reference checkout> (or set PCFD_REFERENCE_SRC)")
    subprocess.run(["make", "-C", str(ROOT / "oracle" / "refbuild"), "REF=%s" % ref, "-j8"], check=True,
                   stdout=subprocess.DEVNULL)
    exe = ROOT / "oracle" / "_ref" / "ref_dump"
    names = sys.argv[2:] if len(sys.argv) > 2 else list(CASES)
    with tempfile.TemporaryDirectory() as tmp:
        for name in names:
            a = run_case(exe, name, CASES[name], tmp, ref)
            print(name, "nnode", int(a["nnode"][0]), "nedge", int(a["nedge"][0]), "norms", a["s1_norms"].ravel())


if __name__ == "__main__":
    main()
