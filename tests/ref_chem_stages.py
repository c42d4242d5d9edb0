"""The reacting case the reference's own reacting solver ran
(tests/golden/ref_fr_plate.npz, written by tests/golden/make_ref_fixtures.py)
and the stages of its first two Newton steps, each recomputed from the
reference's own input for that stage by an engine: the oracle on the CPU or
the CUDA path through the C ABI.

Stages (ucs/solutionSpace.tcc:573-818): UpdateBCs as the reference runs it
before a step's residual (the boundary pass of the step's set-up, then
NewtonIterate's own); the LSQ gradient with the symmetry fix; the modified
Venkatakrishnan limiter with the reacting pressure clip (step 2; the CUDA
path has no clip, so its limiter is compared where the clip left a node
alone); ComputeResiduals (ucs/residual.tcc:13) -
inviscid HLLC (first order on step 1, second order with the limiter on step
2), viscous (the directional correction once second order is on), the
chemistry source, the temporal term a steady run still adds (Param::dt = -1:
b -= (vol / -1) (Q - Q_old), conservative), the no-slip momentum and energy
rows zeroed (ModifyViscousWallResidual, ucs/compressibleFR.tcc:2101) - and
the norms (ParallelL2Norm / StridedParallelL2Norm, ucs/parallel.h:162,121)."""
import numpy as np

import ref_fixtures as R
from chem_cases import FIXTURE
from proteuscfd_gb300 import _native as N
from proteuscfd_gb300.chem import load_mechanism

CASE = "fr_plate"
# boundary types of ucs/bc_defines.h
NOSLIP, SONIC_INFLOW, DIRICHLET, SYMMETRY = 4, 7, 1, 9


def load():
    """(fixture arrays, boundary conditions, reference scales)."""
    f = R.load(CASE)
    bct = {int(a): int(b) for a, b in f["case_bc_types"]}
    qinf = f["qinf"].ravel()
    bc = dict(bc_type=bct, twall={int(a): float(b) for a, b in f["case_twall"]},
              qref={tg: qinf for tg, b in bct.items() if b in (SONIC_INFLOW, DIRICHLET)}, no_cvbc=1)
    # (density, pressure, temperature, specific enthalpy, velocity, viscosity, conductivity)
    ref = N.ChemRef(*f["refs"].ravel()[:7])
    return f, bc, ref


def reordered_elements(f):
    """The reference's element list after its set-up reorder (node n becomes
    ordering[n]): (xyz, triangles, triangle tags, tets)."""
    el = f["elements_pre"].copy()
    o = f["ordering"]
    nodes = el[:, 3:11]
    nodes[nodes >= 0] = o[nodes[nodes >= 0]]
    xyz = np.empty_like(f["xyz_pre"])
    xyz[o] = f["xyz_pre"]
    t = el[:, 0]
    return xyz, el[t == 0][:, 3:6], el[t == 0][:, 1], el[t == 2][:, 3:7]


class OracleEngine:
    """The oracle (oracle/chem.c, oracle/mesh.c)."""

    def __init__(self, f, ref):
        from oracle_lib import OracleChemState, OracleMesh
        from proteuscfd_gb300.chem import model_struct
        self.mesh = OracleMesh.from_elements(*reordered_elements(f))
        self.S = OracleChemState(model_struct(load_mechanism(FIXTURE)), ref)
        self.ns = self.S.ns

    def update_bcs(self, q, bc):
        q, rc = self.S.update_bcs(self.mesh, q, **bc)
        assert rc == 0
        return q

    def gradient(self, q, sym):
        return self.S.gradient(self.mesh, q, sym)

    def limiter(self, q, g, chi):
        """with the reacting pressure clip, as Limiter::Compute runs it"""
        return self.S.limiter_clip(self.mesh, q, g, chi)

    def limiter_noclip(self, q, g, chi):
        return self.S.limiter(self.mesh, q, g, chi)

    def residual(self, opts, q, ref_time):
        return self.S.residual(opts, self.mesh, q, ref_time, 1)[0]

    def residual_ho(self, opts, q, g, lim, chi, ref_time):
        return self.S.residual_ho(opts, self.mesh, q, g, lim, chi, ref_time, 1)[0]

    def viscous(self, opts, Re, directional, q, g):
        b, bad = self.S.viscous_residual(opts, self.mesh, Re, directional, q, g)
        assert bad == 0
        return b

    def n2c(self, rhoi, native, P):
        return self.S.n2c(rhoi, native, P)

    def flux_opts(self, beta, pref):
        return N.ChemFluxOpts(beta, pref, 0)


class ProductEngine:
    """The CUDA path through the C ABI (proteuscfd_gb300.chem.ChemModel) on
    the product's host preprocessing of the reference's element list."""

    def __init__(self, f, ref):
        from proteuscfd_gb300 import Mesh
        from proteuscfd_gb300.chem import ChemModel
        el = f["elements_pre"]
        t = el[:, 0]
        self.mesh = Mesh.from_elements(f["xyz_pre"], el[t == 0][:, 3:6], el[t == 0][:, 1], el[t == 2][:, 3:7],
                                       reorder=True)
        self.C = ChemModel(load_mechanism(FIXTURE))
        self.C.attach_mesh(self.mesh)
        self.ref = ref
        self.ns = self.C.nspecies

    def close(self):
        self.C.close()

    def update_bcs(self, q, bc):
        return self.C.update_bcs(self.ref, q, bc["bc_type"], twall=bc["twall"], qref=bc["qref"],
                                 no_cvbc=bc["no_cvbc"])

    def gradient(self, q, sym):
        return self.C.gradient(q, sym_tags=sym)

    def limiter(self, q, g, chi):
        return self.C.limiter(chi, q, g)

    def residual(self, opts, q, ref_time):
        return self.C.residual(self.ref, opts, ref_time, 1, q)[0]

    def residual_ho(self, opts, q, g, lim, chi, ref_time):
        return self.C.residual_ho(self.ref, opts, chi, ref_time, 1, q, g, lim)[0]

    def viscous(self, opts, Re, directional, q, g):
        return self.C.viscous_residual(self.ref, opts, Re, directional, q, g)

    def n2c(self, rhoi, native, P):
        return self.C.native_to_conservative(self.ref, rhoi, native, P)

    def flux_opts(self, beta, pref):
        return self.C.flux_opts(beta, pref, 0)


def l2_norms(b):
    return np.r_[np.sqrt((b * b).sum()) / b.size, np.sqrt((b * b).sum(axis=0)) / b.shape[0]]


def stages(E, f, bc):
    """Yields (stage name, kind, computed, reference's) for every stage of
    the two steps; kind is "state" (boundary update), "gradient",
    "limiter", "residual" or "norms"."""
    n, ns = int(R.scalar(f, "nnode")), E.ns
    nt = 2 * ns + 4
    sym = [t for t, b in bc["bc_type"].items() if b == SYMMETRY]
    walls = [t for t, b in bc["bc_type"].items() if b == NOSLIP]
    bedges, bfactag = f["bedges"], f["bfactag"]
    wall_nodes = np.unique([bedges[k, 0] for k in range(len(bfactag)) if int(bfactag[k]) in walls])
    qinf = f["qinf"].ravel()
    opts = E.flux_opts(1.0, float(qinf[ns + 4]))  # beta, GetPressure(Qinf)
    ref_time = float(f["refs"].ravel()[7])
    vol = f["vol"]
    chi = R.scalar(f, "chi")

    def conservative(q):
        rhoi = np.ascontiguousarray(q[:, :ns])
        return np.c_[rhoi, E.n2c(rhoi, np.ascontiguousarray(q[:, ns:ns + 4]), np.ascontiguousarray(q[:, ns + 4]))]

    starts = {"s1_": f["q_init"], "s2_": np.concatenate([f["s1_q"], f["s1_q_bc"][n:]])}
    for st, q0 in starts.items():
        second = st == "s2_"
        q = q0
        for _ in range(2):
            q = E.update_bcs(q, bc)
        yield st + "q_bc", "state", q, f[st + "q_bc"]
        qb = f[st + "q_bc"]
        yield st + "qgrad", "gradient", E.gradient(qb, sym).reshape(n, nt * 3), f[st + "qgrad"]
        g = f[st + "qgrad"].reshape(n, nt, 3)
        if second:
            yield st + "limiter", "limiter", E.limiter(qb, g, chi), f[st + "limiter"]
            b = E.residual_ho(opts, qb, g, f[st + "limiter"], chi, ref_time)
        else:
            b = E.residual(opts, qb, ref_time)
        b = b + E.viscous(opts, R.scalar(f, "Re"), int(second), qb, g)
        b = b + vol[:, None] * (conservative(qb[:n]) - conservative(q0[:n]))
        b[wall_nodes, ns:ns + 4] = 0.0
        yield st + "b", "residual", b, f[st + "b"]
        yield st + "norms", "norms", l2_norms(b), f[st + "norms"].ravel()
