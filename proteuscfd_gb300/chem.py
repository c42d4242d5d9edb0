"""Finite-rate chemistry on the GPU: the mass production rates of a reacting
air mechanism per node (ChemModel<T>::GetMassProductionRates,
ucs/chem.tcc:575), through the C ABI (pcfd_chem_*)."""
from __future__ import annotations

import ctypes as C
import json
from pathlib import Path

import numpy as np

from . import _native as N


def model_struct(spec: dict) -> "N.ChemModelC":
    """pcfd_chem_model from a mechanism description: {"species": [{"MW" (kg/mol),
    "lo", "hi" (NASA-7)}], "reactions": [{"type", "A", "EA", "n",
    "third_bodies", "global", "nup", "nupp", "tbeff"}]}."""
    m = N.ChemModelC()
    sp = spec["species"]
    rx = spec["reactions"]
    if not 0 < len(sp) <= N.CHEM_MAX_SPECIES or len(rx) > N.CHEM_MAX_REACTIONS:
        raise ValueError("mechanism too large")
    m.nspecies = len(sp)
    for k, s in enumerate(sp):
        m.mw[k] = s["MW"]
        for i in range(7):
            m.nasa_lo[k][i] = s["lo"][i]
            m.nasa_hi[k][i] = s["hi"][i]
    for k, s in enumerate(sp):
        for key, cnt, fit in (("mu", m.nmu, m.mu_fit), ("k", m.nk, m.k_fit)):
            rows = s.get(key, [])
            if len(rows) > N.CHEM_MAX_TRANSPORT_FITS:
                raise ValueError("too many transport fits")
            cnt[k] = len(rows)
            for r, row in enumerate(rows):
                for i in range(6):
                    fit[k][r][i] = row[i]
    m.nreactions = len(rx)
    for j, r in enumerate(rx):
        c = m.rx[j]
        c.type, c.A, c.EA, c.n, c.third_bodies = r["type"], r["A"], r["EA"], r["n"], r["third_bodies"]
        c.nlocal = len(r["global"])
        if c.nlocal > N.CHEM_MAX_LOCAL:
            raise ValueError("reaction with too many species")
        for l in range(c.nlocal):
            c.global_[l] = r["global"][l]
            c.nup[l] = r["nup"][l]
            c.nupp[l] = r["nupp"][l]
            c.tbeff[l] = r["tbeff"][l]
    return m


def load_mechanism(path) -> dict:
    return json.loads(Path(path).read_text())


class ChemModel:
    """Handle of a mechanism on the GPU."""

    def __init__(self, spec: dict):
        self._lib = N.load()
        self.spec = spec
        self.nspecies = len(spec["species"])
        self._m = model_struct(spec)
        h = C.c_void_p()
        N.check(self._lib.pcfd_chem_create(C.byref(self._m), C.byref(h)), "pcfd_chem_create")
        self._h = h

    def production_rates(self, rhoi, T, out=None):
        """rhoi [n][nspecies] kg/m^3, T [n] K -> wdot [n][nspecies] kg/(m^3 s);
        out, when given, is the C-contiguous FP64 result array to fill."""
        rhoi = np.ascontiguousarray(rhoi, dtype=np.float64)
        T = np.ascontiguousarray(T, dtype=np.float64)
        n = T.shape[0]
        assert rhoi.shape == (n, self.nspecies)
        w = np.empty_like(rhoi) if out is None else out
        if w.shape != rhoi.shape or w.dtype != np.float64 or not w.flags["C_CONTIGUOUS"]:
            raise ValueError("production_rates: out must be a C-contiguous float64 array shaped like rhoi")
        N.check(self._lib.pcfd_chem_production_rates(self._h, n, N.dptr(rhoi), N.dptr(T), N.dptr(w)),
                "pcfd_chem_production_rates")
        return w

    def production_rates_dev(self, n, rhoi_ptr, T_ptr, wdot_ptr):
        """Device pointers; returns the kernel's device time in ms."""
        ms = C.c_double()
        N.check(self._lib.pcfd_chem_production_rates_dev(self._h, int(n), rhoi_ptr, T_ptr, wdot_ptr, C.byref(ms)),
                "pcfd_chem_production_rates_dev")
        return ms.value

    # ---- node state of the reacting equation set (non-dimensional variables) ----

    @staticmethod
    def ref(density, pressure, temperature, specific_enthalpy, velocity):
        """Reference scales (Param::ref_*) of the non-dimensional variables."""
        return N.ChemRef(density, pressure, temperature, specific_enthalpy, velocity)

    def _arr(self, a, shape):
        a = np.ascontiguousarray(a, dtype=np.float64)
        if a.shape != shape:
            raise ValueError("expected shape %s, got %s" % (shape, a.shape))
        return a

    def find_T_given_P(self, ref, rhoi, P, T_init):
        """NewtonFindTGivenP per node: returns (T, nodes not converged)."""
        n = len(P)
        rhoi = self._arr(rhoi, (n, self.nspecies))
        P, T_init = self._arr(P, (n,)), self._arr(T_init, (n,))
        T = np.empty(n)
        bad = C.c_longlong()
        N.check(self._lib.pcfd_chem_find_T_given_P(self._h, C.byref(ref), n, N.dptr(rhoi), N.dptr(P), N.dptr(T_init),
                                                   N.dptr(T), C.byref(bad), 0), "pcfd_chem_find_T_given_P")
        return T, bad.value

    def conservative_to_native(self, ref, q, P):
        """q [n][ns+4] = (rhoi, rho u, rho v, rho w, rho Et), P [n] -> [n][4] = (u, v, w, T)."""
        n = len(P)
        q, P = self._arr(q, (n, self.nspecies + 4)), self._arr(P, (n,))
        out = np.empty((n, 4))
        N.check(self._lib.pcfd_chem_conservative_to_native(self._h, C.byref(ref), n, N.dptr(q), N.dptr(P),
                                                           N.dptr(out), 0), "pcfd_chem_conservative_to_native")
        return out

    def conservative_to_native_dev(self, ref, n, q_ptr, P_ptr, out_ptr):
        """The same on device addresses."""
        N.check(self._lib.pcfd_chem_conservative_to_native(self._h, C.byref(ref), int(n), q_ptr, P_ptr, out_ptr, 1),
                "pcfd_chem_conservative_to_native")

    def native_to_conservative(self, ref, rhoi, native, P):
        """rhoi [n][ns], native [n][4] = (u, v, w, T), P [n] -> [n][4] = (rho u, rho v, rho w, rho Et)."""
        n = len(P)
        rhoi = self._arr(rhoi, (n, self.nspecies))
        native, P = self._arr(native, (n, 4)), self._arr(P, (n,))
        out = np.empty((n, 4))
        N.check(self._lib.pcfd_chem_native_to_conservative(self._h, C.byref(ref), n, N.dptr(rhoi), N.dptr(native),
                                                           N.dptr(P), N.dptr(out), 0),
                "pcfd_chem_native_to_conservative")
        return out

    def aux(self, ref, rhoi, T):
        """ComputeAuxiliaryVariables: returns (P [n], cvi [n][ns], concentrations [n][ns])."""
        n = len(T)
        rhoi, T = self._arr(rhoi, (n, self.nspecies)), self._arr(T, (n,))
        P, cvi, mol = np.empty(n), np.empty((n, self.nspecies)), np.empty((n, self.nspecies))
        N.check(self._lib.pcfd_chem_aux(self._h, C.byref(ref), n, N.dptr(rhoi), N.dptr(T), N.dptr(P), N.dptr(cvi),
                                        N.dptr(mol), 0), "pcfd_chem_aux")
        return P, cvi, mol

    def transport(self, ref, rhoi, T):
        """GetMolecularViscosity / GetThermalConductivity of the reacting set
        (Wilke's rule): non-dimensional rhoi [n][ns] and T [n] -> (mu [n], k [n]),
        over ref.viscosity and ref.conductivity."""
        n = len(T)
        rhoi, T = self._arr(rhoi, (n, self.nspecies)), self._arr(T, (n,))
        mu, k = np.empty(n), np.empty(n)
        N.check(self._lib.pcfd_chem_transport(self._h, C.byref(ref), n, N.dptr(rhoi), N.dptr(T), N.dptr(mu),
                                              N.dptr(k), 0), "pcfd_chem_transport")
        return mu, k

    def node_records(self, ref, rhoi, vel, T):
        """The reacting node record [n][6 + 3 ns] (rhoi, u, v, w, T, P, rho,
        cvi, concentrations) that ComputeAuxiliaryVariables completes."""
        n = len(T)
        P, cvi, mol = self.aux(ref, rhoi, T)
        rhoi = self._arr(rhoi, (n, self.nspecies))
        return np.ascontiguousarray(np.c_[rhoi, np.asarray(vel, np.float64), T, P, rhoi.sum(axis=1), cvi, mol])

    @staticmethod
    def flux_opts(beta=1.0, pref=0.0, symmetry2D=0):
        return N.ChemFluxOpts(beta, pref, symmetry2D)

    def hllc_flux(self, ref, opts, q, edges, avec):
        """HLLCFlux over an edge list: q [n][6 + 3 ns] node records, edges
        [E][2] (left, right), avec [E][4] (unit normal, area) -> flux [E][ns + 4]."""
        q = np.ascontiguousarray(q, dtype=np.float64)
        edges = np.ascontiguousarray(edges, dtype=np.int32)
        avec = np.ascontiguousarray(avec, dtype=np.float64)
        ne = len(edges)
        if q.shape[1] != 6 + 3 * self.nspecies or edges.shape != (ne, 2) or avec.shape != (ne, 4):
            raise ValueError("hllc_flux: bad shapes")
        flux = np.empty((ne, self.nspecies + 4))
        bad = C.c_longlong()
        N.check(self._lib.pcfd_chem_hllc_flux(self._h, C.byref(ref), C.byref(opts), len(q), N.dptr(q), ne,
                                              edges.ctypes.data_as(C.c_void_p), N.dptr(avec), N.dptr(flux),
                                              C.byref(bad), 0), "pcfd_chem_hllc_flux")
        return flux

    def hllc_flux_dev(self, ref, opts, nnode, q_ptr, nedge, edges_ptr, avec_ptr, flux_ptr):
        """The same on device addresses; returns the failure count."""
        bad = C.c_longlong()
        N.check(self._lib.pcfd_chem_hllc_flux(self._h, C.byref(ref), C.byref(opts), int(nnode), q_ptr, int(nedge),
                                              edges_ptr, avec_ptr, flux_ptr, C.byref(bad), 1), "pcfd_chem_hllc_flux")
        return bad.value

    def source_jacobian(self, ref, ref_time, q, vol):
        """SourceTermJacobian per node: q [n][6 + 3 ns] records, vol [n] ->
        A [n][ns + 4][ns + 4], A[p, j, i] = dS_j / dQ_i by one-sided
        differences (h = 1e-8)."""
        n = len(vol)
        q, vol = self._arr(q, (n, 6 + 3 * self.nspecies)), self._arr(vol, (n,))
        neqn = self.nspecies + 4
        A = np.empty((n, neqn, neqn))
        N.check(self._lib.pcfd_chem_source_jacobian(self._h, C.byref(ref), float(ref_time), n, N.dptr(q), N.dptr(vol),
                                                    N.dptr(A), 0), "pcfd_chem_source_jacobian")
        return A

    def source_jacobian_dev(self, ref, ref_time, n, q_ptr, vol_ptr, A_ptr):
        """The same on device addresses."""
        N.check(self._lib.pcfd_chem_source_jacobian(self._h, C.byref(ref), float(ref_time), int(n), q_ptr, vol_ptr,
                                                    A_ptr, 1), "pcfd_chem_source_jacobian")

    def temporal_terms(self, ref, q, vol, dtau, beta, cnp1=1.0, dt=0.0, local_ts=0, A=None):
        """ContributeTemporalTerms per node: q [n][6 + 3 ns] records, vol,
        dtau, beta [n] -> A [n][ns + 4][ns + 4] + the temporal terms (A zero
        when not given)."""
        n = len(vol)
        neqn = self.nspecies + 4
        q = self._arr(q, (n, 6 + 3 * self.nspecies))
        vol, dtau, beta = self._arr(vol, (n,)), self._arr(dtau, (n,)), self._arr(beta, (n,))
        A = np.zeros((n, neqn, neqn)) if A is None else np.array(A, dtype=np.float64, order="C", copy=True)
        if A.shape != (n, neqn, neqn):
            raise ValueError("temporal_terms: A must be [n][ns + 4][ns + 4]")
        N.check(self._lib.pcfd_chem_temporal_terms(self._h, C.byref(ref), n, N.dptr(q), N.dptr(vol), N.dptr(dtau),
                                                   N.dptr(beta), float(cnp1), float(dt), int(local_ts), N.dptr(A), 0),
                "pcfd_chem_temporal_terms")
        return A

    def temporal_terms_dev(self, ref, n, q_ptr, vol_ptr, dtau_ptr, beta_ptr, cnp1, dt, local_ts, A_ptr):
        """The same on device addresses; adds into the blocks at A_ptr."""
        N.check(self._lib.pcfd_chem_temporal_terms(self._h, C.byref(ref), int(n), q_ptr, vol_ptr, dtau_ptr, beta_ptr,
                                                   float(cnp1), float(dt), int(local_ts), A_ptr, 1),
                "pcfd_chem_temporal_terms")

    def attach_mesh(self, mesh):
        """Copies the mesh's edges, areas, boundary half-edges and dual
        volumes to the device for residual()."""
        N.check(self._lib.pcfd_chem_attach_mesh(self._h, C.byref(mesh.view)), "pcfd_chem_attach_mesh")
        self._mesh = mesh

    def residual(self, ref, opts, ref_time, reactions, q):
        """First-order inviscid residual of the reacting set on the attached
        mesh: q [nnode + nbedge][6 + 3 ns] records -> (b [nnode][ns + 4], norms [1 + ns + 4])."""
        m = self._mesh
        q = self._arr(q, (m.nnode + m.nbedge, 6 + 3 * self.nspecies))
        b = np.empty((m.nnode, self.nspecies + 4))
        norms = np.empty(1 + self.nspecies + 4)
        N.check(self._lib.pcfd_chem_residual(self._h, C.byref(ref), C.byref(opts), float(ref_time), int(reactions),
                                             N.dptr(q), N.dptr(b), N.dptr(norms), 0), "pcfd_chem_residual")
        return b, norms

    @staticmethod
    def bc_tables(nrec, bc_type, twall=None, qref=None):
        """Per-tag tables of update_bcs from dicts tag -> type / K / record."""
        ntags = max(bc_type) + 1
        bt = np.full(ntags, -1, dtype=np.int32)
        tw = np.zeros(ntags)
        qr = np.zeros((ntags, nrec))
        for t, v in bc_type.items():
            bt[t] = v
        for t, v in (twall or {}).items():
            tw[t] = v
        for t, v in (qref or {}).items():
            qr[t] = v
        return bt, tw, qr

    def update_bcs(self, ref, q, bc_type, twall=None, qref=None, no_cvbc=1):
        """UpdateBCs of the reacting set on the attached mesh: returns the
        updated records (q [nnode + nbedge][6 + 3 ns] is not changed)."""
        m = self._mesh
        nrec = 6 + 3 * self.nspecies
        q = np.array(self._arr(q, (m.nnode + m.nbedge, nrec)), copy=True)
        bt, tw, qr = self.bc_tables(nrec, bc_type, twall, qref)
        N.check(self._lib.pcfd_chem_update_bcs(self._h, C.byref(ref), len(bt), N.iptr(bt), N.dptr(tw), N.dptr(qr),
                                               int(no_cvbc), q.ctypes.data, 0), "pcfd_chem_update_bcs")
        return q

    def gradient(self, q, sym_tags=()):
        """The reacting set's LSQ gradient on the attached mesh: q [nnode + nbedge][6 + 3 ns]
        -> grad [nnode][2 ns + 4][3], with the symmetry fix on the given tags."""
        m = self._mesh
        q = self._arr(q, (m.nnode + m.nbedge, 6 + 3 * self.nspecies))
        tags = np.ascontiguousarray(list(sym_tags) or [0], dtype=np.int32)
        grad = np.empty((m.nnode, 2 * self.nspecies + 4, 3))
        N.check(self._lib.pcfd_chem_gradient(self._h, q.ctypes.data, N.iptr(tags), len(sym_tags), grad.ctypes.data, 0),
                "pcfd_chem_gradient")
        return grad

    def viscous_residual(self, ref, opts, Re, directional, q, grad):
        """The viscous part of the reacting residual on the attached mesh:
        q [nnode + nbedge][6 + 3 ns] records, grad [nnode][2 ns + 4][3] ->
        b [nnode][ns + 4]."""
        m = self._mesh
        q = self._arr(q, (m.nnode + m.nbedge, 6 + 3 * self.nspecies))
        grad = self._arr(grad, (m.nnode, 2 * self.nspecies + 4, 3))
        b = np.empty((m.nnode, self.nspecies + 4))
        N.check(self._lib.pcfd_chem_viscous_residual(self._h, C.byref(ref), C.byref(opts), float(Re), int(directional),
                                                     q.ctypes.data, grad.ctypes.data, b.ctypes.data, 0),
                "pcfd_chem_viscous_residual")
        return b

    def limiter(self, chi, q, grad):
        """The modified Venkatakrishnan limiter of the native variables (no
        pressure clip): -> lim [nnode][ns + 4]."""
        m = self._mesh
        q = self._arr(q, (m.nnode + m.nbedge, 6 + 3 * self.nspecies))
        grad = self._arr(grad, (m.nnode, 2 * self.nspecies + 4, 3))
        lim = np.empty((m.nnode, self.nspecies + 4))
        N.check(self._lib.pcfd_chem_limiter(self._h, float(chi), q.ctypes.data, grad.ctypes.data, lim.ctypes.data, 0),
                "pcfd_chem_limiter")
        return lim

    def residual_ho(self, ref, opts, chi, ref_time, reactions, q, grad, lim):
        """The reacting residual at second order: q records, grad [nnode][2 ns + 4][3],
        lim [nnode][ns + 4] -> (b [nnode][ns + 4], norms [1 + ns + 4])."""
        m = self._mesh
        q = self._arr(q, (m.nnode + m.nbedge, 6 + 3 * self.nspecies))
        grad = self._arr(grad, (m.nnode, 2 * self.nspecies + 4, 3))
        lim = self._arr(lim, (m.nnode, self.nspecies + 4))
        b = np.empty((m.nnode, self.nspecies + 4))
        norms = np.empty(1 + self.nspecies + 4)
        N.check(self._lib.pcfd_chem_residual_ho(self._h, C.byref(ref), C.byref(opts), float(chi), float(ref_time),
                                                int(reactions), q.ctypes.data, grad.ctypes.data, lim.ctypes.data,
                                                b.ctypes.data, N.dptr(norms), 0), "pcfd_chem_residual_ho")
        return b, norms

    def residual_dev(self, ref, opts, ref_time, reactions, q_ptr, b_ptr=None):
        """The same with q (and b, optional) as device addresses; returns the norms."""
        norms = np.empty(1 + self.nspecies + 4)
        N.check(self._lib.pcfd_chem_residual(self._h, C.byref(ref), C.byref(opts), float(ref_time), int(reactions),
                                             q_ptr, b_ptr, N.dptr(norms), 1), "pcfd_chem_residual")
        return norms

    def close(self):
        if getattr(self, "_h", None):
            self._lib.pcfd_chem_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
