"""Host-side interface mirroring the reference's operator API for the hot path.

The names follow the reference's classes and functions, with the device work
behind the C ABI of libpcfd.so:

=====================================  =====================================================
this module                            reference (ngcurrier/ProteusCFD)
=====================================  =====================================================
``Mesh.box`` / ``Mesh.from_elements``  mesh readers + ``Mesh::BuildMaps``/``CalcMetrics``
                                       (ucs/mesh.tcc:265,1576)
``Param``                              ``Param<T>`` (ucs/param.h:31), hot-path subset
``SolutionSpace.update_bcs``           ``UpdateBCs`` (ucs/bc.tcc:1400)
``SolutionSpace.gradient``             ``Gradient<T>::Compute`` (ucs/gradient.tcc:57)
``SolutionSpace.limiter``              ``Limiter<T>::Compute`` (ucs/limiters.tcc:53)
``SolutionSpace.compute_residuals``    ``ComputeResiduals`` (ucs/residual.tcc:13)
``SolutionSpace.compute_timesteps``    ``ComputeTimesteps`` (ucs/timestep.tcc:7)
``SolutionSpace.compute_jacobians``    ``ComputeJacobians`` (ucs/jacobian.tcc:13)
``SolutionSpace.sgs``                  ``CRS::SGS`` (ucs/crs.tcc:62)
``SolutionSpace.apply_dq``             ``CompressibleEqnSet::ApplyDQ`` (ucs/compressible.tcc:929)
``SolutionSpace.newton_iterate``       ``PreTimeAdvance`` + ``NewtonIterate``
                                       (ucs/solutionSpace.tcc:573,640)
``solve``                              ``Solve`` (ucs/solve.tcc:24)
=====================================  =====================================================

Errors raise ``PcfdError`` (the reference aborts through ``Abort <<``,
ucs/exceptions.h:30-49).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _native as N

NEQN = 5
NVARS = 10
NTERMS = 9


class Mesh:
    """Host mesh with the reference's maps and dual metrics."""

    def __init__(self, handle, reorder=False, nnode=0):
        """Takes ownership of a mesh handle and builds its maps and metrics.
        ``reorder`` True first applies the reference's set-up reorder
        (reverse Cuthill-McKee from node 0, ``Param::reorder``, on by default
        in the reference; ucs/solutionSpace.tcc:61-66); ``ordering`` then
        holds the reference's ``Mesh::ordering`` (old node n is now
        ordering[n]).  ``reorder="rcm"`` numbers the nodes in that reverse
        Cuthill-McKee sequence instead (new node k is old node ordering[k]),
        the bandwidth-reducing use of the same list."""
        self._lib = N.load()
        self._h = None
        self.ordering = None
        if not handle:
            raise N.PcfdError(4, "mesh create", self._lib.pcfd_mesh_last_error().decode())
        self._h = handle
        if reorder == "rcm":
            order = np.zeros(nnode, dtype=np.int32)
            rc = self._lib.pcfd_mesh_rcm_order(self._h, N.iptr(order))
            if rc == 0:
                rc = self._lib.pcfd_mesh_renumber(self._h, N.iptr(order))
            if rc != 0:
                msg = self._lib.pcfd_mesh_last_error().decode()
                self._lib.pcfd_mesh_destroy(self._h)
                self._h = None
                raise N.PcfdError(rc, "pcfd_mesh_renumber", msg)
            self.ordering = order
        elif reorder:
            order = np.zeros(nnode, dtype=np.int32) if nnode > 0 else None
            rc = self._lib.pcfd_mesh_reorder_rcm(self._h, N.iptr(order) if order is not None else None)
            if rc != 0:
                msg = self._lib.pcfd_mesh_last_error().decode()
                self._lib.pcfd_mesh_destroy(self._h)
                self._h = None
                raise N.PcfdError(rc, "pcfd_mesh_reorder_rcm", msg)
            self.ordering = order
        rc = self._lib.pcfd_mesh_build(self._h)
        if rc != 0:
            msg = self._lib.pcfd_mesh_last_error().decode()
            self._lib.pcfd_mesh_destroy(self._h)
            self._h = None
            raise N.PcfdError(rc, "pcfd_mesh_build", msg)
        self.view = N.MeshView()
        N.check(self._lib.pcfd_mesh_view_get(self._h, C.byref(self.view)), "pcfd_mesh_view_get")

    @classmethod
    def box(cls, nx, ny, nz, lx=1.0, ly=1.0, lz=1.0, jitter=0.0, seed=1, ramp_deg=0.0, ramp_x0=0.5,
            y_ratio=1.0, tags=(1, 2, 3, 4, 5, 6), reorder=False, jitter_mode=0, wall_start_i=0, upstream_tag=7,
            wall_ar_max=0.0):
        p = N.BoxParams(nx, ny, nz, lx, ly, lz, jitter, seed, ramp_deg, ramp_x0, y_ratio, (C.c_int * 6)(*tags),
                        jitter_mode, wall_start_i, upstream_tag, wall_ar_max)
        return cls(N.load().pcfd_mesh_box_create(C.byref(p)), reorder, nx * ny * nz)

    @classmethod
    def from_elements(cls, xyz, tris, tri_tags, tets, reorder=False):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        tris = np.ascontiguousarray(tris, dtype=np.int32)
        tri_tags = np.ascontiguousarray(tri_tags, dtype=np.int32)
        tets = np.ascontiguousarray(tets, dtype=np.int32)
        h = N.load().pcfd_mesh_from_elements(len(xyz), N.dptr(xyz), len(tris), N.iptr(tris), N.iptr(tri_tags),
                                             len(tets), N.iptr(tets))
        return cls(h, reorder, len(xyz))

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.pcfd_mesh_destroy(self._h)
            self._h = None

    # numpy views of the host arrays (valid while the Mesh lives)
    def _arr(self, ptr, n, dtype):
        return np.ctypeslib.as_array(ptr, shape=(n,)).view(dtype) if n else np.zeros(0, dtype)

    @property
    def nnode(self):
        return self.view.nnode

    @property
    def nedge(self):
        return self.view.nedge

    @property
    def nbedge(self):
        return self.view.nbedge

    @property
    def edges(self):
        return self._arr(self.view.edges, 2 * self.nedge, np.int32).reshape(-1, 2)

    @property
    def edge_area(self):
        return self._arr(self.view.edge_area, 4 * self.nedge, np.float64).reshape(-1, 4)

    @property
    def bedges(self):
        return self._arr(self.view.bedges, 2 * self.nbedge, np.int32).reshape(-1, 2)

    @property
    def bedge_area(self):
        return self._arr(self.view.bedge_area, 4 * self.nbedge, np.float64).reshape(-1, 4)

    @property
    def bfactag(self):
        return self._arr(self.view.bfactag, self.nbedge, np.int32)

    @property
    def xyz(self):
        return self._arr(self.view.xyz, 3 * self.nnode, np.float64).reshape(-1, 3)

    @property
    def vol(self):
        return self._arr(self.view.vol, self.nnode, np.float64)

    @property
    def sw(self):
        return self._arr(self.view.sw, 6 * self.nnode, np.float64).reshape(-1, 6)

    @property
    def ipsp(self):
        return self._arr(self.view.ipsp, self.nnode + 1, np.int32)

    @property
    def psp(self):
        n = int(self.ipsp[-1])
        return self._arr(self.view.psp, n, np.int32)

    def stats(self):
        a = [C.c_int() for _ in range(4)]
        d = [C.c_double() for _ in range(2)]
        N.check(self._lib.pcfd_mesh_stats(self._h, *[C.byref(x) for x in a], *[C.byref(x) for x in d]),
                "pcfd_mesh_stats")
        keys = ("ntri", "ntet", "rewound", "unclosed")
        out = {k: x.value for k, x in zip(keys, a)}
        out["max_open"] = d[0].value
        out["total_vol"] = d[1].value
        return out

    def rcm_order(self):
        order = np.zeros(self.nnode, dtype=np.int32)
        N.check(self._lib.pcfd_mesh_rcm_order(self._h, N.iptr(order)), "pcfd_mesh_rcm_order")
        return order


@dataclass
class Param:
    """Hot-path subset of ``Param<T>`` (ucs/param.h:31); non-dimensional values."""

    gamma: float = 1.4
    mach: float = 0.5
    flowdir: tuple = (1.0, 0.0, 0.0)
    Re: float = 1.0
    Pr: float = 0.72
    PrT: float = 0.85
    ref_temperature: float = 300.0
    sorder: int = 1
    chi: float = 0.0
    viscous: int = 0
    limiter: int = 0
    venkat_K: float = 1.0
    no_cvbc: int = 0
    jac_boundary_eval: int = 0
    torder: int = 1            # Param::torder: the temporal residual is always on in the reference
    time_step: float = -1.0    # Param::dt: steady (the reference's default)
    tinf: float = 1.0          # freestream T / ref_temperature (UpdateQinf)
    pinf: float = 1.0          # freestream p / ref_pressure
    bc_type: dict = field(default_factory=dict)   # factag -> BC type
    bc_twall: dict = field(default_factory=dict)  # factag -> wall temperature [K] (<0 adiabatic)

    def to_c(self):
        ntags = max(self.bc_type) + 1 if self.bc_type else 1
        bct = np.zeros(ntags, dtype=np.int32)
        btw = np.full(ntags, 1.0, dtype=np.float64)  # BCObj default twall = 1 K
        for k, v in self.bc_type.items():
            bct[k] = v
        for k, v in self.bc_twall.items():
            btw[k] = v
        p = N.Params()
        p.gamma, p.mach = self.gamma, self.mach
        p.flowdir = (C.c_double * 3)(*self.flowdir)
        p.Re, p.Pr, p.PrT, p.ref_temperature = self.Re, self.Pr, self.PrT, self.ref_temperature
        p.sorder, p.chi, p.viscous, p.limiter = self.sorder, self.chi, self.viscous, self.limiter
        p.venkat_K, p.no_cvbc, p.ntags = self.venkat_K, self.no_cvbc, ntags
        p.jac_boundary_eval = self.jac_boundary_eval
        p.torder, p.time_step = self.torder, self.time_step
        p.tinf, p.pinf = self.tinf, self.pinf
        p.bc_type = N.iptr(bct)
        p.bc_twall = N.dptr(btw)
        p._keep = (bct, btw)
        return p


class SolutionSpace:
    """Device-resident solution space for one mesh (``SolutionSpace<T>``,
    ucs/solutionSpace.h), driven through the C ABI."""

    def __init__(self, mesh: Mesh, param: Param):
        self._lib = N.load()
        self.mesh = mesh
        self.param = param
        self._cp = param.to_c()
        h = C.c_void_p()
        N.check(self._lib.pcfd_create(C.byref(mesh.view), C.byref(self._cp), C.byref(h)), "pcfd_create")
        self._h = h
        self.nrows = mesh.nnode + mesh.view.nbnode

    def close(self):
        if getattr(self, "_h", None):
            self._lib.pcfd_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    @property
    def handle(self):
        return self._h

    def set_state(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(self.nrows, NVARS)
        N.check(self._lib.pcfd_set_state(self._h, N.dptr(q), NVARS, self.nrows), "pcfd_set_state")

    def set_qold(self, q):
        """The start-of-step state of the temporal residual ([nnode][5] or
        [nrows][10]); set_state and newton_iterate set it themselves."""
        q = np.ascontiguousarray(q, dtype=np.float64)
        q2 = q.reshape(q.shape[0], -1)
        N.check(self._lib.pcfd_set_qold(self._h, N.dptr(q2), q2.shape[1], q2.shape[0]), "pcfd_set_qold")

    def forces(self, tags):
        """(pressure force, viscous force) on the body made of the given
        boundary tags (Forces::Compute's FORCE_Kernel)."""
        t = np.ascontiguousarray(list(tags), dtype=np.int32)
        out = np.empty(6, dtype=np.float64)
        N.check(self._lib.pcfd_forces(self._h, N.iptr(t), len(t), N.dptr(out)), "pcfd_forces")
        return out[:3], out[3:]

    def get_state(self):
        q = np.empty((self.nrows, NVARS), dtype=np.float64)
        N.check(self._lib.pcfd_get_state(self._h, N.dptr(q), NVARS, self.nrows), "pcfd_get_state")
        return q

    def qinf(self):
        q = np.empty(NVARS, dtype=np.float64)
        N.check(self._lib.pcfd_get_qinf(self._h, N.dptr(q)), "pcfd_get_qinf")
        return q

    def update_bcs(self):
        N.check(self._lib.pcfd_update_bcs(self._h), "pcfd_update_bcs")

    def gradient(self):
        g = np.empty((self.mesh.nnode, NTERMS * 3), dtype=np.float64)
        N.check(self._lib.pcfd_gradient(self._h, N.dptr(g)), "pcfd_gradient")
        return g

    def limiter(self):
        lim = np.empty((self.mesh.nnode, NEQN), dtype=np.float64)
        N.check(self._lib.pcfd_limiter(self._h, N.dptr(lim)), "pcfd_limiter")
        return lim

    def compute_residuals(self, want_b=True):
        """Returns (b, norms); norms = [resGlobal, per-equation] (ComputeResiduals)."""
        b = np.empty((self.mesh.nnode, NEQN), dtype=np.float64) if want_b else None
        norms = np.empty(6, dtype=np.float64)
        N.check(self._lib.pcfd_residual(self._h, N.dptr(b) if want_b else None, N.dptr(norms)), "pcfd_residual")
        return b, norms

    def get_residual(self, out=None):
        """The residual [nnode][5]; out, when given, is a C-contiguous FP64
        array of that shape to fill (for instance in pinned host memory)."""
        b = np.empty((self.mesh.nnode, NEQN), dtype=np.float64) if out is None else out
        if b.shape != (self.mesh.nnode, NEQN) or b.dtype != np.float64 or not b.flags["C_CONTIGUOUS"]:
            raise ValueError("get_residual: out must be a C-contiguous float64 array of shape (nnode, 5)")
        N.check(self._lib.pcfd_get_residual(self._h, N.dptr(b)), "pcfd_get_residual")
        return b

    def residual_full(self):
        norms = np.empty(6, dtype=np.float64)
        N.check(self._lib.pcfd_residual_full(self._h, N.dptr(norms)), "pcfd_residual_full")
        return norms

    def bench_residual_full(self, nsteps):
        """Device time (ms) of nsteps back-to-back residual evaluations."""
        ms = C.c_double()
        norms = np.empty(6, dtype=np.float64)
        N.check(self._lib.pcfd_bench_residual_full(self._h, int(nsteps), C.byref(ms), N.dptr(norms)),
                "pcfd_bench_residual_full")
        return ms.value, norms

    def bench_spmv(self, nrep, fp32=True):
        """Device time (ms) of nrep back-to-back products with the assembled
        matrix (FP32 vectors through the FP32 Krylov product, or FP64)."""
        ms = C.c_double()
        N.check(self._lib.pcfd_bench_spmv(self._h, int(nrep), 1 if fp32 else 0, C.byref(ms)), "pcfd_bench_spmv")
        return ms.value

    def bench_sgs(self, nrep, nsweeps=1, fp32=True):
        """Device time (ms) of nrep calls of nsweeps block-SGS sweeps on the
        assembled matrix (FP32 vectors, the Krylov preconditioner's sweep, or
        FP64 vectors)."""
        ms = C.c_double()
        N.check(self._lib.pcfd_bench_sgs(self._h, int(nrep), int(nsweeps), 1 if fp32 else 0, C.byref(ms)),
                "pcfd_bench_sgs")
        return ms.value

    def set_residual_arithmetic(self, mode):
        """0 FP64, 1 double-float on the FP32 pipes (composite calls only)."""
        N.check(self._lib.pcfd_set_residual_arithmetic(self._h, int(mode)), "pcfd_set_residual_arithmetic")

    def get_limiter(self):
        """Limiter<T>::l as the next residual uses it (no recomputation)."""
        lim = np.empty((self.mesh.nnode, NEQN), dtype=np.float64)
        N.check(self._lib.pcfd_get_limiter(self._h, N.dptr(lim)), "pcfd_get_limiter")
        return lim

    def set_limiter(self, lim):
        lim = np.ascontiguousarray(lim, dtype=np.float64)
        assert lim.shape == (self.mesh.nnode, NEQN)
        N.check(self._lib.pcfd_set_limiter(self._h, N.dptr(lim)), "pcfd_set_limiter")

    # ---- learned right preconditioner (pcfd_lp_*; no reference counterpart,
    # it sits where CRS<T>::PrecondBackSolve sits, ucs/crs.tcc:591) --------
    def lp_init(self, seed=1):
        N.check(self._lib.pcfd_lp_init(self._h, int(seed)), "pcfd_lp_init")

    def lp_get_params(self):
        w = np.empty(N.LP_NPARAM, dtype=np.float32)
        N.check(self._lib.pcfd_lp_get_params(self._h, N.fptr(w)), "pcfd_lp_get_params")
        return w

    def lp_set_params(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        assert w.size == N.LP_NPARAM
        N.check(self._lib.pcfd_lp_set_params(self._h, N.fptr(w)), "pcfd_lp_set_params")

    def lp_forward(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32)
        assert x.shape == (self.mesh.nnode, N.LP_NIN)
        out = np.empty((self.mesh.nnode, N.LP_NOUT), dtype=np.float32)
        N.check(self._lib.pcfd_lp_forward(self._h, N.fptr(x), N.fptr(out)), "pcfd_lp_forward")
        return out

    def lp_loss_grad(self, x, t):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        g = np.empty(N.LP_NPARAM, dtype=np.float32)
        loss = C.c_double()
        N.check(self._lib.pcfd_lp_loss_grad(self._h, N.fptr(x), N.fptr(t), N.fptr(g), C.byref(loss)), "pcfd_lp_loss_grad")
        return loss.value, g

    def lp_features(self, y):
        y = np.ascontiguousarray(y, dtype=np.float64)
        x = np.empty((self.mesh.nnode, N.LP_NIN), dtype=np.float32)
        sg = C.c_double()
        N.check(self._lib.pcfd_lp_features(self._h, N.dptr(y), N.fptr(x), C.byref(sg)), "pcfd_lp_features")
        return x, sg.value

    def lp_apply(self, v, nsgs=1):
        v = np.ascontiguousarray(v, dtype=np.float64)
        z = np.empty((self.mesh.nnode, 5), dtype=np.float64)
        N.check(self._lib.pcfd_lp_apply(self._h, int(nsgs), N.dptr(v), N.dptr(z)), "pcfd_lp_apply")
        return z

    def lp_collect(self, nsgs=1, rtol=1e-6, krylov_pairs=0):
        ns = C.c_int()
        N.check(self._lib.pcfd_lp_collect(self._h, int(nsgs), float(rtol), int(krylov_pairs), C.byref(ns)),
                "pcfd_lp_collect")
        return ns.value

    def lp_clear_samples(self):
        N.check(self._lib.pcfd_lp_clear_samples(self._h), "pcfd_lp_clear_samples")

    def lp_train(self, epochs, lr=1e-3):
        a, b = C.c_double(), C.c_double()
        N.check(self._lib.pcfd_lp_train(self._h, int(epochs), float(lr), C.byref(a), C.byref(b)), "pcfd_lp_train")
        return a.value, b.value

    def compute_timesteps(self, cfl):
        dt = np.empty(self.mesh.nnode, dtype=np.float64)
        dtmin = C.c_double()
        N.check(self._lib.pcfd_timestep(self._h, float(cfl), N.dptr(dt), C.byref(dtmin)), "pcfd_timestep")
        return dt, dtmin.value

    def set_jacobian_precision(self, prec):
        """0 FP64, 1 FP32, 2 BF16 storage of the off-diagonal blocks."""
        N.check(self._lib.pcfd_set_jacobian_precision(self._h, int(prec)), "pcfd_set_jacobian_precision")

    def compute_jacobians(self):
        N.check(self._lib.pcfd_jacobian(self._h), "pcfd_jacobian")

    def nblocks(self):
        return int(self._lib.pcfd_nblocks(self._h))

    def get_jacobian(self):
        nb = self.nblocks()
        M = np.empty((nb, 25), dtype=np.float64)
        N.check(self._lib.pcfd_get_jacobian(self._h, N.dptr(M), nb), "pcfd_get_jacobian")
        return M

    def crs_structure(self):
        ia = np.empty(self.mesh.nnode + 1, dtype=np.int32)
        ja = np.empty(self.nblocks(), dtype=np.int32)
        nc = C.c_int()
        N.check(self._lib.pcfd_crs_structure(self._h, N.iptr(ia), N.iptr(ja), C.byref(nc)), "pcfd_crs_structure")
        return ia, ja, nc.value

    def coloring(self):
        _, _, nc = self.crs_structure()
        cptr = np.empty(nc + 1, dtype=np.int32)
        rows = np.empty(self.mesh.nnode, dtype=np.int32)
        N.check(self._lib.pcfd_coloring(self._h, N.iptr(cptr), N.iptr(rows)), "pcfd_coloring")
        return cptr, rows

    def sgs(self, nsweeps):
        x = np.empty((self.mesh.nnode, NEQN), dtype=np.float64)
        dn = C.c_double()
        N.check(self._lib.pcfd_sgs(self._h, int(nsweeps), N.dptr(x), C.byref(dn)), "pcfd_sgs")
        return x, dn.value

    def fgmres(self, m=30, restarts=1, rtol=1e-3, nsgs=1):
        """Flexible GMRES(m), right-preconditioned by nsgs SGS sweeps, on the
        assembled system with the last residual as right-hand side, from
        x = 0: returns (x, relative residual, Krylov iterations)."""
        x = np.empty((self.mesh.nnode, NEQN), dtype=np.float64)
        rel = C.c_double()
        its = C.c_int()
        N.check(self._lib.pcfd_fgmres(self._h, int(m), int(restarts), float(rtol), int(nsgs), N.dptr(x),
                                      C.byref(rel), C.byref(its)), "pcfd_fgmres")
        return x, rel.value, its.value

    def matvec(self, x, fp32=False):
        """y = A x with the assembled matrix (FP64 vectors, or FP32 vectors
        through the FP32 Krylov solver's product)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty((self.mesh.nnode, NEQN), dtype=np.float64)
        N.check(self._lib.pcfd_matvec(self._h, N.dptr(x), N.dptr(y), 1 if fp32 else 0), "pcfd_matvec")
        return y

    def sgs_rhs(self, b, nsweeps, fp32=False):
        """nsweeps SGS sweeps from x = 0 for the right-hand side b (FP64
        vectors, or the FP32 Krylov preconditioner's sweep)."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.empty((self.mesh.nnode, NEQN), dtype=np.float64)
        N.check(self._lib.pcfd_sgs_rhs(self._h, int(nsweeps), N.dptr(b), N.dptr(x), 1 if fp32 else 0),
                "pcfd_sgs_rhs")
        return x

    def apply_dq(self, x=None):
        dn = C.c_double()
        xp = N.dptr(np.ascontiguousarray(x, dtype=np.float64)) if x is not None else None
        N.check(self._lib.pcfd_apply_dq(self._h, xp, C.byref(dn)), "pcfd_apply_dq")
        return dn.value

    def newton_iterate(self, it, cfl=5.0, nsgs=10, cfl_start=0.0, cfl_ramp_steps=0, jac_precision=0,
                       linear_solver=0, fgmres_m=30, fgmres_restarts=1, fgmres_rtol=1e-2, jac_update_freq=1,
                       limiter_refresh=1, limiter_freeze=0, first_order_steps=0, lp_directions=0):
        o = N.NewtonOpts(int(it), float(cfl), float(cfl_start), int(cfl_ramp_steps), int(nsgs), int(jac_update_freq),
                         int(jac_precision), int(linear_solver), int(fgmres_m), int(fgmres_restarts),
                         float(fgmres_rtol), int(limiter_refresh), int(limiter_freeze), int(first_order_steps),
                         int(lp_directions))
        r = N.NewtonReport()
        N.check(self._lib.pcfd_newton_step(self._h, C.byref(o), C.byref(r)), "pcfd_newton_step")
        return {"res": list(r.res), "dqnorm": r.dqnorm, "dtmin": r.dtmin, "lin_res": r.lin_res,
                "lin_iters": r.lin_iters, "cfl": r.cfl, "lp_fallbacks": r.lp_fallbacks}

    def health(self):
        c = (C.c_longlong * 8)()
        N.check(self._lib.pcfd_get_health(self._h, c), "pcfd_get_health")
        return list(c)

    def profile(self, on=True):
        N.check(self._lib.pcfd_profile_enable(self._h, 1 if on else 0), "pcfd_profile_enable")

    def profile_reset(self):
        N.check(self._lib.pcfd_profile_reset(self._h), "pcfd_profile_reset")

    def timers(self):
        out = {}
        i = 0
        buf = C.create_string_buffer(64)
        while True:
            ms, n = C.c_double(), C.c_longlong()
            if self._lib.pcfd_profile_get(self._h, i, buf, 64, C.byref(ms), C.byref(n)) != 0:
                break
            out[buf.value.decode()] = (ms.value, n.value)
            i += 1
        return out

    def launch_count(self):
        return int(self._lib.pcfd_launch_count(self._h))


def solve(space: SolutionSpace, nsteps: int, drop: float = 0.0, **opts):
    """Outer iterations (``Solve``, ucs/solve.tcc:24) with the reference's
    counter (0 on the first step).  Runs ``nsteps`` iterations, or stops
    early once resGlobal has dropped by ``drop`` relative to the first
    iteration (the reference itself never stops early).  Returns the
    per-iteration reports."""
    hist = []
    r0 = None
    for it in range(nsteps):
        rep = space.newton_iterate(it, **opts)
        hist.append(rep)
        if r0 is None:
            r0 = rep["res"][0]
        if drop > 0.0 and r0 > 0.0 and rep["res"][0] <= drop * r0:
            break
    return hist
