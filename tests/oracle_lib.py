"""ctypes access to the CPU oracle (oracle/liboracle.so) - test infrastructure."""
import ctypes as C
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int)
_LLP = C.POINTER(C.c_longlong)
_FP = C.POINTER(C.c_float)
_lib = None


def lib():
    global _lib
    if _lib is None:
        from proteuscfd_gb300 import _native as N
        from proteuscfd_gb300 import build as B
        B.build_oracle()
        L = C.CDLL(str(ROOT / "oracle" / "liboracle.so"))
        MV = C.POINTER(N.MeshView)
        PP = C.POINTER(N.Params)
        protos = {
            "oracle_aux": (None, [C.c_double, _DP]),
            "oracle_qinf": (None, [PP, _DP]),
            "oracle_init_state": (None, [PP, C.c_int, _DP]),
            "oracle_roe_flux": (None, [_DP, _DP, _DP, C.c_double, C.c_double, _DP]),
            "oracle_viscous_flux": (None, [PP, _DP, _DP, _DP, C.c_double, _DP]),
            "oracle_normal_node": (C.c_int, [MV, C.c_int, _DP]),
            "oracle_update_bcs": (C.c_int, [MV, PP, _DP]),
            "oracle_gradient": (C.c_int, [MV, PP, _DP, _DP]),
            "oracle_limiter": (C.c_int, [MV, PP, _DP, _DP, _DP, _LLP]),
            "oracle_residual": (C.c_int, [MV, PP, _DP, _DP, _DP, _DP, _DP, _LLP]),
            "oracle_residual_scaled": (C.c_int, [MV, PP, _DP, _DP, _DP, _DP, _DP, _DP, _LLP]),
            "oracle_residual_full": (C.c_int, [MV, PP, _DP, _DP, _DP, _DP, _DP, _DP, _DP, _LLP]),
            "oracle_lu": (C.c_int, [_DP, _IP, C.c_int]),
            "oracle_timestep": (C.c_double, [MV, PP, _DP, C.c_double, _DP]),
            "oracle_crs_init": (None, [MV, _IP, _IP]),
            "oracle_prepare_sgs": (None, [C.c_int, _IP, _DP, _IP]),
            "oracle_jacobian": (C.c_int, [MV, PP, _DP, _DP, _IP, _IP, _DP]),
            "oracle_sgs": (C.c_double, [C.c_int, _IP, _IP, _DP, _IP, _DP, _DP, C.c_int]),
            "oracle_sgs_colored": (None, [C.c_int, _IP, _IP, _DP, _IP, _DP, _DP, C.c_int, C.c_int, _IP, _IP]),
            "oracle_apply_dq": (C.c_double, [MV, PP, _DP, _DP]),
            "oracle_lusolve": (None, [_DP, _DP, _IP, _DP, C.c_int]),
            "oracle_matvec": (None, [_DP, _DP, _DP, C.c_int]),
            "oracle_tri_area": (None, [_DP, _DP, _DP, _DP]),
            "oracle_tet_vol": (C.c_double, [_DP, _DP, _DP, _DP]),
            "oracle_bf16": (C.c_double, [C.c_double]),
            "oracle_chem_rates_n": (None, [C.POINTER(N.ChemModelC), C.c_longlong, _DP, _DP, _DP]),
            "oracle_chem_kf": (C.c_double, [C.POINTER(N.ChemReaction), C.c_double]),
            "oracle_chem_kc": (C.c_double, [C.POINTER(N.ChemModelC), C.POINTER(N.ChemReaction), C.c_double]),
            "oracle_chem_find_T": (C.c_int, [C.POINTER(N.ChemModelC), C.POINTER(N.ChemRef), _DP, C.c_double,
                                             C.c_double, _DP]),
            "oracle_chem_c2n": (C.c_int, [C.POINTER(N.ChemModelC), C.POINTER(N.ChemRef), _DP, C.c_double, _DP]),
            "oracle_chem_c2n_n": (C.c_longlong, [C.POINTER(N.ChemModelC), C.POINTER(N.ChemRef), C.c_longlong, _DP,
                                                 _DP, _DP]),
            "oracle_chem_hllc": (C.c_int, [C.POINTER(N.ChemModelC), C.POINTER(N.ChemRef), C.POINTER(N.ChemFluxOpts),
                                           _DP, _DP, _DP, _DP]),
            "oracle_chem_hllc_n": (C.c_longlong, [C.POINTER(N.ChemModelC), C.POINTER(N.ChemRef),
                                                  C.POINTER(N.ChemFluxOpts), _DP, C.c_longlong, _IP, _DP, _DP]),
            "oracle_chem_residual": (None, [C.POINTER(N.ChemModelC), C.POINTER(N.ChemRef), C.POINTER(N.ChemFluxOpts),
                                            C.POINTER(N.MeshView), _DP, C.c_double, C.c_int, _DP, _DP]),
            "oracle_chem_source_jacobian_n": (None, [C.POINTER(N.ChemModelC), C.POINTER(N.ChemRef), C.c_double,
                                                     C.c_longlong, _DP, _DP, _DP]),
            "oracle_chem_temporal_n": (None, [C.POINTER(N.ChemModelC), C.POINTER(N.ChemRef), C.c_longlong, _DP, _DP,
                                              _DP, _DP, C.c_double, C.c_double, C.c_int, _DP]),
            "oracle_chem_n2c": (None, [C.POINTER(N.ChemModelC), C.POINTER(N.ChemRef), _DP, _DP, C.c_double, _DP]),
            "oracle_chem_aux": (None, [C.POINTER(N.ChemModelC), C.POINTER(N.ChemRef), _DP, C.c_double, _DP, _DP,
                                       _DP]),
            "oracle_chem_transport_n": (C.c_longlong, [C.POINTER(N.ChemModelC), C.POINTER(N.ChemRef), C.c_longlong,
                                                       _DP, _DP, _DP, _DP]),
            "oracle_chem_gradient": (C.c_int, [C.POINTER(N.ChemModelC), C.POINTER(N.MeshView), _DP, _IP, C.c_int,
                                               _DP]),
            "oracle_chem_limiter": (None, [C.POINTER(N.ChemModelC), C.POINTER(N.MeshView), _DP, _DP, C.c_double,
                                           _DP]),
            "oracle_chem_limiter_clip": (None, [C.POINTER(N.ChemModelC), C.POINTER(N.ChemRef), C.POINTER(N.MeshView),
                                                _DP, _DP, C.c_double, _DP]),
            "oracle_chem_timestep": (C.c_double, [C.POINTER(N.ChemModelC), C.POINTER(N.ChemRef),
                                                  C.POINTER(N.MeshView), _DP, C.c_double, C.c_double, _DP]),
            "oracle_chem_residual_ho": (None, [C.POINTER(N.ChemModelC), C.POINTER(N.ChemRef),
                                               C.POINTER(N.ChemFluxOpts), C.POINTER(N.MeshView), _DP, _DP, _DP,
                                               C.c_double, C.c_double, C.c_int, _DP, _DP]),
            "oracle_chem_update_bcs": (C.c_int, [C.POINTER(N.ChemModelC), C.POINTER(N.ChemRef), C.POINTER(N.MeshView),
                                                 C.c_int, _IP, _DP, _DP, C.c_int, _DP]),
            "oracle_chem_viscous_residual": (C.c_int, [C.POINTER(N.ChemModelC), C.POINTER(N.ChemRef),
                                                       C.POINTER(N.ChemFluxOpts), C.POINTER(N.MeshView), C.c_double,
                                                       C.c_int, _DP, _DP, _DP]),
            "oracle_forces": (None, [MV, PP, _DP, _DP, _IP, _DP]),
            "oracle_mesh_box": (C.c_void_p, [C.POINTER(N.BoxParams)]),
            "oracle_mesh_elements": (C.c_void_p, [C.c_int, _DP, C.c_int, _IP, _IP, C.c_int, _IP]),
            "oracle_mesh_build": (C.c_int, [C.c_void_p]),
            "oracle_mesh_view": (C.c_int, [C.c_void_p, MV]),
            "oracle_mesh_free": (None, [C.c_void_p]),
            "oracle_lp_nparam": (C.c_int, []),
            "oracle_lp_graph": (None, [MV, _IP, _IP, _FP]),
            "oracle_lp_features": (C.c_double, [C.c_int, _DP, _DP, _DP, _DP, C.c_double, _FP]),
            "oracle_lp_forward": (None, [C.c_int, _IP, _IP, _FP, _FP, _FP, C.c_int, _DP]),
            "oracle_lp_loss_grad": (C.c_double, [C.c_int, _IP, _IP, _FP, _FP, _FP, _FP, C.c_int, _DP]),
        }
        for n, (r, a) in protos.items():
            f = getattr(L, n)
            f.restype = r
            f.argtypes = a
        _lib = L
    return _lib


def dp(a):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_DP)


def ip(a):
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_IP)


def fp(a):
    assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_FP)


class OracleMesh:
    """A mesh generated and preprocessed by the oracle alone (oracle/mesh.c),
    with the attributes the oracle's solution spaces read from a mesh."""

    def __init__(self, handle):
        self.L = lib()
        if not handle:
            raise RuntimeError("oracle mesh: bad input")
        self._h = handle
        rc = self.L.oracle_mesh_build(self._h)
        if rc != 0:
            self.L.oracle_mesh_free(self._h)
            self._h = None
            raise RuntimeError("oracle_mesh_build failed (%d)" % rc)
        from proteuscfd_gb300 import _native as N
        self.view = N.MeshView()
        assert self.L.oracle_mesh_view(self._h, C.byref(self.view)) == 0

    @classmethod
    def box(cls, nx, ny, nz, lx=1.0, ly=1.0, lz=1.0, jitter=0.0, seed=1, ramp_deg=0.0, ramp_x0=0.5, y_ratio=1.0,
            tags=(1, 2, 3, 4, 5, 6), jitter_mode=0, wall_start_i=0, upstream_tag=7, wall_ar_max=0.0):
        from proteuscfd_gb300 import _native as N
        p = N.BoxParams(nx, ny, nz, lx, ly, lz, jitter, seed, ramp_deg, ramp_x0, y_ratio, (C.c_int * 6)(*tags),
                        jitter_mode, wall_start_i, upstream_tag, wall_ar_max)
        return cls(lib().oracle_mesh_box(C.byref(p)))

    @classmethod
    def from_elements(cls, xyz, tris, tri_tags, tets):
        xyz = np.ascontiguousarray(xyz, np.float64)
        tris = np.ascontiguousarray(tris, np.int32)
        tri_tags = np.ascontiguousarray(tri_tags, np.int32)
        tets = np.ascontiguousarray(tets, np.int32)
        return cls(lib().oracle_mesh_elements(len(xyz), dp(xyz), len(tris), ip(tris), ip(tri_tags), len(tets),
                                              ip(tets)))

    def __del__(self):
        if getattr(self, "_h", None):
            self.L.oracle_mesh_free(self._h)
            self._h = None

    def _a(self, ptr, n, dtype, cols=1):
        a = np.ctypeslib.as_array(ptr, shape=(n * cols,)).view(dtype)
        return a.reshape(-1, cols) if cols > 1 else a

    nnode = property(lambda self: self.view.nnode)
    nedge = property(lambda self: self.view.nedge)
    nbedge = property(lambda self: self.view.nbedge)
    edges = property(lambda self: self._a(self.view.edges, self.nedge, np.int32, 2))
    edge_area = property(lambda self: self._a(self.view.edge_area, self.nedge, np.float64, 4))
    bedges = property(lambda self: self._a(self.view.bedges, self.nbedge, np.int32, 2))
    bedge_area = property(lambda self: self._a(self.view.bedge_area, self.nbedge, np.float64, 4))
    bfactag = property(lambda self: self._a(self.view.bfactag, self.nbedge, np.int32))
    xyz = property(lambda self: self._a(self.view.xyz, self.nnode, np.float64, 3))
    vol = property(lambda self: self._a(self.view.vol, self.nnode, np.float64))
    sw = property(lambda self: self._a(self.view.sw, self.nnode, np.float64, 6))
    ipsp = property(lambda self: self._a(self.view.ipsp, self.nnode + 1, np.int32))
    psp = property(lambda self: self._a(self.view.psp, int(self.ipsp[-1]), np.int32))


class OracleNet:
    """The learned preconditioner's network on the oracle (CPU, double)."""

    def __init__(self, mesh):
        self.L = lib()
        self.n = mesh.nnode
        nnz = 2 * mesh.nedge
        self.nptr = np.zeros(self.n + 1, np.int32)
        self.nbr = np.zeros(nnz, np.int32)
        self.ef = np.zeros((nnz, 4), np.float32)
        self.L.oracle_lp_graph(C.byref(mesh.view), ip(self.nptr), ip(self.nbr), fp(self.ef))

    def forward(self, x, w, emulate=1):
        x = np.ascontiguousarray(x, np.float32)
        w = np.ascontiguousarray(w, np.float32)
        out = np.zeros((self.n, 5))
        self.L.oracle_lp_forward(self.n, ip(self.nptr), ip(self.nbr), fp(self.ef), fp(x), fp(w), emulate, dp(out))
        return out

    def loss_grad(self, x, t, w, emulate=1):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        w = np.ascontiguousarray(w, np.float32)
        g = np.zeros(self.L.oracle_lp_nparam())
        loss = self.L.oracle_lp_loss_grad(self.n, ip(self.nptr), ip(self.nbr), fp(self.ef), fp(x), fp(t), fp(w),
                                          emulate, dp(g))
        return loss, g


def lp_features(y, q, vol, qinf, gamma):
    n = vol.shape[0]
    x = np.zeros((n, 11), np.float32)
    y = np.ascontiguousarray(y, np.float64)
    q = np.ascontiguousarray(q, np.float64)
    vol = np.ascontiguousarray(vol, np.float64)
    qinf = np.ascontiguousarray(qinf, np.float64)
    sigma = lib().oracle_lp_features(n, dp(y), dp(q), dp(vol), dp(qinf), gamma, fp(x))
    return x, sigma


def lp_random_params(seed, scale=1.0):
    """Seeded parameters with every block non-zero (for checks of the backward pass)."""
    rng = np.random.default_rng(seed)
    nin, h, ne, nout, nl = 11, 64, 4, 5, 3
    parts = [rng.uniform(-1, 1, h * nin) * np.sqrt(3.0 / nin), rng.uniform(-0.1, 0.1, h)]
    for _ in range(nl):
        parts += [rng.uniform(-0.5, 0.5, h * ne), 1.0 + rng.uniform(-0.1, 0.1, h),
                  rng.uniform(-1, 1, h * h) * np.sqrt(3.0 / h), rng.uniform(-1, 1, h * h) * np.sqrt(3.0 / h),
                  rng.uniform(-0.1, 0.1, h)]
    parts += [rng.uniform(-1, 1, nout * h) * np.sqrt(3.0 / h), rng.uniform(-0.1, 0.1, nout)]
    return (np.concatenate(parts) * scale).astype(np.float32)


class OracleSpace:
    """The oracle run on the same mesh view and parameters as a SolutionSpace."""

    def __init__(self, mesh, param):
        self.mesh = mesh
        self.param = param
        self.cp = param.to_c()
        self.L = lib()

    def qinf(self):
        q = np.zeros(10)
        self.L.oracle_qinf(C.byref(self.cp), dp(q))
        return q

    def update_bcs(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64).copy()
        rc = self.L.oracle_update_bcs(C.byref(self.mesh.view), C.byref(self.cp), dp(q))
        assert rc == 0
        return q

    def gradient(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64)
        g = np.zeros((self.mesh.nnode, 27))
        assert self.L.oracle_gradient(C.byref(self.mesh.view), C.byref(self.cp), dp(q), dp(g)) == 0
        return g

    def limiter(self, q, g):
        q = np.ascontiguousarray(q, dtype=np.float64)
        l = np.zeros((self.mesh.nnode, 5))
        nclip = C.c_longlong()
        assert self.L.oracle_limiter(C.byref(self.mesh.view), C.byref(self.cp), dp(q), dp(g), dp(l),
                                     C.byref(nclip)) == 0
        return l, nclip.value

    def residual(self, q, g=None, l=None, qold=None):
        """ComputeResiduals; qold ([nnode][5], the state at the start of the
        step) adds the reference's temporal residual."""
        n = self.mesh.nnode
        q = np.ascontiguousarray(q, dtype=np.float64)
        g = np.zeros((n, 27)) if g is None else np.ascontiguousarray(g)
        l = np.ones((n, 5)) if l is None else np.ascontiguousarray(l)
        qo = None if qold is None else np.ascontiguousarray(np.asarray(qold, dtype=np.float64)[:n, :5])
        b = np.zeros((n, 5))
        babs = np.zeros((n, 5))
        norms = np.zeros(6)
        kc = C.c_longlong()
        assert self.L.oracle_residual_full(C.byref(self.mesh.view), C.byref(self.cp), dp(q),
                                           dp(qo) if qo is not None else None, dp(g), dp(l), dp(b),
                                           dp(babs), dp(norms), C.byref(kc)) == 0
        self.last_babs = babs
        return b, norms, kc.value

    def forces(self, q, g, tags):
        """FORCE_Kernel over the half-edges with the given tags: (pressure
        force, viscous force)."""
        mask = np.zeros(self.cp.ntags, np.int32)
        mask[list(tags)] = 1
        out = np.zeros(6)
        g = np.zeros((self.mesh.nnode, 27)) if g is None else np.ascontiguousarray(g, np.float64)
        self.L.oracle_forces(C.byref(self.mesh.view), C.byref(self.cp), dp(np.ascontiguousarray(q, np.float64)),
                             dp(g), ip(mask), dp(out))
        return out[:3], out[3:]

    def full(self, q):
        """UpdateBCs, gradient, limiter, residual - the NewtonIterate order;
        the state given is the step's q_old of the temporal residual."""
        q_in = np.asarray(q, dtype=np.float64)
        q = self.update_bcs(q)
        p = self.param
        g = l = None
        if p.sorder > 1 or p.viscous:
            g = self.gradient(q)
        if p.sorder > 1:
            l, _ = self.limiter(q, g)
        b, norms, _ = self.residual(q, g, l, qold=q_in)
        return q, g, l, b, norms


class OracleImplicit(OracleSpace):
    """The reference's implicit iteration on the CPU: time step, FD Jacobian,
    diagonal LU, lexicographic block SGS, ApplyDQ (test infrastructure)."""

    def __init__(self, mesh, param):
        super().__init__(mesh, param)
        n = mesh.nnode
        self.ia = np.zeros(n + 1, dtype=np.int32)
        self.ja = np.zeros(n + 2 * mesh.nedge, dtype=np.int32)
        self.L.oracle_crs_init(C.byref(mesh.view), ip(self.ia), ip(self.ja))
        self.dt = None

    def timestep(self, q, cfl):
        dt = np.zeros(self.mesh.nnode)
        dtmin = self.L.oracle_timestep(C.byref(self.mesh.view), C.byref(self.cp), dp(np.ascontiguousarray(q)),
                                       float(cfl), dp(dt))
        return dt, dtmin

    def jacobian(self, q, dt):
        """Returns (M, q) - the reference's Jacobian modifies the state."""
        q = np.ascontiguousarray(q, dtype=np.float64).copy()
        M = np.zeros((len(self.ja), 25))
        assert self.L.oracle_jacobian(C.byref(self.mesh.view), C.byref(self.cp), dp(q), dp(np.ascontiguousarray(dt)),
                                      ip(self.ia), ip(self.ja), dp(M)) == 0
        return M, q

    def lu(self, M):
        M = M.copy()
        pv = np.zeros(self.mesh.nnode * 5, dtype=np.int32)
        self.L.oracle_prepare_sgs(self.mesh.nnode, ip(self.ia), dp(M), ip(pv))
        return M, pv

    def sgs(self, Mlu, pv, b, nsweeps):
        x = np.zeros((self.mesh.nnode, 5))
        d = self.L.oracle_sgs(self.mesh.nnode, ip(self.ia), ip(self.ja), dp(Mlu), ip(pv),
                              dp(np.ascontiguousarray(b)), dp(x), int(nsweeps))
        return x, d

    def sgs_colored(self, Mlu, pv, b, nsweeps, cptr, rows):
        x = np.zeros((self.mesh.nnode, 5))
        self.L.oracle_sgs_colored(self.mesh.nnode, ip(self.ia), ip(self.ja), dp(Mlu), ip(pv),
                                  dp(np.ascontiguousarray(b)), dp(x), int(nsweeps), len(cptr) - 1,
                                  ip(np.ascontiguousarray(cptr, dtype=np.int32)),
                                  ip(np.ascontiguousarray(rows, dtype=np.int32)))
        return x

    def apply_dq(self, x, q):
        x = np.ascontiguousarray(x, dtype=np.float64).copy()
        q = np.ascontiguousarray(q, dtype=np.float64).copy()
        dn = self.L.oracle_apply_dq(C.byref(self.mesh.view), C.byref(self.cp), dp(x), dp(q))
        return q, dn

    def newton(self, q, nsteps, cfl=5.0, nsgs=10, cfl_start=0.0, cfl_ramp_steps=0, coloring=None,
               first_order_steps=0, limiter_refresh=1, limiter_freeze=999999):
        """Solve's loop (ucs/solve.tcc:24-60): PreIterate, then per step
        PreTimeAdvance (q_old, Jacobian, time steps) and NewtonIterate
        (boundary update, gradient, limiter, residual with the temporal term,
        SGS, ApplyDQ) in the reference's order and with its iteration
        counter, which starts at 0 (so the first step is first order).
        Returns the final q and the resGlobal history."""
        def ramp(it):
            cs = cfl_start if cfl_start > 0 else cfl
            if cfl_ramp_steps > 0 and it < cfl_ramp_steps:
                return (cfl - cs) / cfl_ramp_steps * it + cs
            return cfl
        q = np.ascontiguousarray(q, dtype=np.float64).copy()
        dt, _ = self.timestep(q, ramp(0))
        hist = []
        p = self.param
        for it in range(nsteps):
            qold = q[:self.mesh.nnode, :5].copy()
            M, q = self.jacobian(q, dt)
            dt, _ = self.timestep(q, ramp(it))
            q = self.update_bcs(q)
            ho = p.sorder > 1 and it > first_order_steps
            g = l = None
            if ho or p.viscous:
                g = self.gradient(q)
            if ho and p.limiter and it % limiter_refresh == 0 and it < limiter_freeze:
                l, _ = self.limiter(q, g)
                self._lim = l
            elif ho and p.limiter:
                l = self._lim
            if ho:
                b, norms, _ = self.residual(q, g, l, qold=qold)
            else:
                b, norms, _ = OracleImplicit._first_order(self).residual(q, g, None, qold=qold)
            hist.append(norms[0])
            Mlu, pv = self.lu(M)
            if coloring is None:
                x, _ = self.sgs(Mlu, pv, b, nsgs)
            else:
                x = self.sgs_colored(Mlu, pv, b, nsgs, *coloring)
            x[~np.isfinite(x).all(axis=1)] = 0.0
            q, _ = self.apply_dq(x, q)
        return q, hist

    def _first_order(self):
        if getattr(self, "_fo", None) is None:
            import dataclasses
            self._fo = OracleSpace(self.mesh, dataclasses.replace(self.param, sorder=1))
        return self._fo


def chem_rates(model_struct, rhoi, T):
    """Oracle production rates for a pcfd_chem_model ctypes structure."""
    rhoi = np.ascontiguousarray(rhoi, np.float64)
    T = np.ascontiguousarray(T, np.float64)
    w = np.zeros_like(rhoi)
    lib().oracle_chem_rates_n(C.byref(model_struct), T.shape[0], dp(rhoi), dp(T), dp(w))
    return w


class OracleChemState:
    """The oracle's node state of the reacting equation set, node by node."""

    def __init__(self, model_struct, ref):
        self.m, self.ref, self.L = model_struct, ref, lib()
        self.ns = model_struct.nspecies

    def find_T(self, rhoi, P, T_init):
        T, its = np.empty(len(P)), np.empty(len(P), dtype=int)
        for k in range(len(P)):
            t = C.c_double()
            its[k] = self.L.oracle_chem_find_T(C.byref(self.m), C.byref(self.ref),
                                               dp(np.ascontiguousarray(rhoi[k], np.float64)), float(P[k]),
                                               float(T_init[k]), C.byref(t))
            T[k] = t.value
        return T, its

    def c2n(self, q, P):
        out, its = np.empty((len(P), 4)), np.empty(len(P), dtype=int)
        for k in range(len(P)):
            o = np.empty(4)
            its[k] = self.L.oracle_chem_c2n(C.byref(self.m), C.byref(self.ref),
                                            dp(np.ascontiguousarray(q[k], np.float64)), float(P[k]), dp(o))
            out[k] = o
        return out, its

    def c2n_batch(self, q, P):
        """c2n over all nodes in one oracle call; returns (native, nodes not converged)."""
        q = np.ascontiguousarray(q, np.float64)
        P = np.ascontiguousarray(P, np.float64)
        out = np.empty((len(P), 4))
        bad = self.L.oracle_chem_c2n_n(C.byref(self.m), C.byref(self.ref), len(P), dp(q), dp(P), dp(out))
        return out, bad

    def n2c(self, rhoi, native, P):
        out = np.empty((len(P), 4))
        for k in range(len(P)):
            o = np.empty(4)
            self.L.oracle_chem_n2c(C.byref(self.m), C.byref(self.ref), dp(np.ascontiguousarray(rhoi[k], np.float64)),
                                   dp(np.ascontiguousarray(native[k], np.float64)), float(P[k]), dp(o))
            out[k] = o
        return out

    def aux(self, rhoi, T):
        n = len(T)
        P, cvi, mol = np.empty(n), np.empty((n, self.ns)), np.empty((n, self.ns))
        for k in range(n):
            p, c, mo = C.c_double(), np.empty(self.ns), np.empty(self.ns)
            self.L.oracle_chem_aux(C.byref(self.m), C.byref(self.ref), dp(np.ascontiguousarray(rhoi[k], np.float64)),
                                   float(T[k]), C.byref(p), dp(c), dp(mo))
            P[k], cvi[k], mol[k] = p.value, c, mo
        return P, cvi, mol

    def transport(self, rhoi, T):
        """(mu [n], k [n], nodes above every fit's range)."""
        rhoi = np.ascontiguousarray(rhoi, np.float64)
        T = np.ascontiguousarray(T, np.float64)
        mu, k = np.empty(len(T)), np.empty(len(T))
        bad = self.L.oracle_chem_transport_n(C.byref(self.m), C.byref(self.ref), len(T), dp(rhoi), dp(T), dp(mu),
                                             dp(k))
        return mu, k, bad

    def hllc(self, opts, q, edges, avec):
        """HLLCFlux edge by edge; returns (flux [E][ns + 4], failures)."""
        ne = len(edges)
        flux = np.empty((ne, self.ns + 4))
        bad = 0
        for e in range(ne):
            f = np.empty(self.ns + 4)
            bad += self.L.oracle_chem_hllc(C.byref(self.m), C.byref(self.ref), C.byref(opts),
                                           dp(np.ascontiguousarray(q[edges[e][0]], np.float64)),
                                           dp(np.ascontiguousarray(q[edges[e][1]], np.float64)),
                                           dp(np.ascontiguousarray(avec[e], np.float64)), dp(f))
            flux[e] = f
        return flux, bad

    def hllc_batch(self, opts, q, edges, avec):
        """HLLCFlux over the edge list in one oracle call."""
        q = np.ascontiguousarray(q, np.float64)
        edges = np.ascontiguousarray(edges, np.int32)
        avec = np.ascontiguousarray(avec, np.float64)
        flux = np.empty((len(edges), self.ns + 4))
        bad = self.L.oracle_chem_hllc_n(C.byref(self.m), C.byref(self.ref), C.byref(opts), dp(q), len(edges),
                                        ip(edges), dp(avec), dp(flux))
        return flux, bad

    def source_jacobian(self, q, vol, ref_time):
        """SourceTermJacobian per node -> [n][ns + 4][ns + 4]."""
        q = np.ascontiguousarray(q, np.float64)
        vol = np.ascontiguousarray(vol, np.float64)
        A = np.empty((len(vol), self.ns + 4, self.ns + 4))
        self.L.oracle_chem_source_jacobian_n(C.byref(self.m), C.byref(self.ref), float(ref_time), len(vol), dp(q),
                                             dp(vol), dp(A))
        return A

    def temporal(self, q, vol, dtau, beta, cnp1, dt, local_ts, A=None):
        """ContributeTemporalTerms per node, added into A [n][ns + 4][ns + 4]
        (zeros when not given); returns A."""
        n = len(vol)
        A = np.zeros((n, self.ns + 4, self.ns + 4)) if A is None else np.ascontiguousarray(A, np.float64).copy()
        arr = lambda x: np.ascontiguousarray(x, np.float64)
        self.L.oracle_chem_temporal_n(C.byref(self.m), C.byref(self.ref), n, dp(arr(q)), dp(arr(vol)), dp(arr(dtau)),
                                      dp(arr(beta)), float(cnp1), float(dt), int(local_ts), dp(A))
        return A

    def update_bcs(self, mesh, q, bc_type, twall=None, qref=None, no_cvbc=1):
        """(updated records, first half-edge of an unbuilt type + 1 or 0)."""
        from proteuscfd_gb300.chem import ChemModel
        q = np.array(q, dtype=np.float64, copy=True)
        bt, tw, qr = ChemModel.bc_tables(q.shape[1], bc_type, twall, qref)
        rc = self.L.oracle_chem_update_bcs(C.byref(self.m), C.byref(self.ref), C.byref(mesh.view), len(bt), ip(bt),
                                           dp(tw), dp(np.ascontiguousarray(qr)), int(no_cvbc), dp(q))
        return q, rc

    def gradient(self, mesh, q, sym_tags=()):
        q = np.ascontiguousarray(q, np.float64)
        tags = np.ascontiguousarray(list(sym_tags) or [0], dtype=np.int32)
        grad = np.empty((mesh.nnode, 2 * self.ns + 4, 3))
        self.L.oracle_chem_gradient(C.byref(self.m), C.byref(mesh.view), dp(q), ip(tags), len(sym_tags), dp(grad))
        return grad

    def viscous_residual(self, opts, mesh, Re, directional, q, grad):
        """The viscous part of the reacting residual; returns (b, faces above
        every transport fit)."""
        q = np.ascontiguousarray(q, np.float64)
        grad = np.ascontiguousarray(grad, np.float64)
        b = np.empty((mesh.nnode, self.ns + 4))
        bad = self.L.oracle_chem_viscous_residual(C.byref(self.m), C.byref(self.ref), C.byref(opts), C.byref(mesh.view),
                                                  float(Re), int(directional), dp(q), dp(grad), dp(b))
        return b, bad

    def limiter(self, mesh, q, grad, chi):
        q = np.ascontiguousarray(q, np.float64)
        grad = np.ascontiguousarray(grad, np.float64)
        lim = np.empty((mesh.nnode, self.ns + 4))
        self.L.oracle_chem_limiter(C.byref(self.m), C.byref(mesh.view), dp(q), dp(grad), float(chi), dp(lim))
        return lim

    def timestep(self, mesh, q, beta, cfl):
        """Local time steps of the reacting set -> (dt [nnode], smallest)."""
        q = np.ascontiguousarray(q, np.float64)
        dt = np.empty(mesh.nnode)
        dtmin = self.L.oracle_chem_timestep(C.byref(self.m), C.byref(self.ref), C.byref(mesh.view), dp(q),
                                            float(beta), float(cfl), dp(dt))
        return dt, dtmin

    def limiter_clip(self, mesh, q, grad, chi):
        """The limiter with the reacting pressure clip (Kernel_PressureClip)."""
        q = np.ascontiguousarray(q, np.float64)
        grad = np.ascontiguousarray(grad, np.float64)
        lim = np.empty((mesh.nnode, self.ns + 4))
        self.L.oracle_chem_limiter_clip(C.byref(self.m), C.byref(self.ref), C.byref(mesh.view), dp(q), dp(grad),
                                        float(chi), dp(lim))
        return lim

    def residual_ho(self, opts, mesh, q, grad, lim, chi, ref_time, reactions):
        """SpatialResidual of the reacting set at second order (inviscid)."""
        q = np.ascontiguousarray(q, np.float64)
        grad = np.ascontiguousarray(grad, np.float64)
        lim = np.ascontiguousarray(lim, np.float64)
        b = np.empty((mesh.nnode, self.ns + 4))
        norms = np.empty(1 + self.ns + 4)
        self.L.oracle_chem_residual_ho(C.byref(self.m), C.byref(self.ref), C.byref(opts), C.byref(mesh.view), dp(q),
                                       dp(grad), dp(lim), float(chi), float(ref_time), int(reactions), dp(b),
                                       dp(norms))
        return b, norms

    def residual(self, opts, mesh, q, ref_time, reactions):
        """SpatialResidual of the reacting set (first order, inviscid)."""
        q = np.ascontiguousarray(q, np.float64)
        b = np.empty((mesh.nnode, self.ns + 4))
        norms = np.empty(1 + self.ns + 4)
        self.L.oracle_chem_residual(C.byref(self.m), C.byref(self.ref), C.byref(opts), C.byref(mesh.view), dp(q),
                                    float(ref_time), int(reactions), dp(b), dp(norms))
        return b, norms
