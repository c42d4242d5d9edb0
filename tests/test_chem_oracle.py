"""The finite-rate chemistry restatement on the CPU oracle: the mechanism
fixture against the reference's own files, and conservation properties of
the production rates (test infrastructure checks; no GPU)."""
import json
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from chem_cases import FIXTURE, conservation, mechanism, states
from oracle_lib import chem_rates
from proteuscfd_gb300.chem import model_struct

# the reference checkout, when PCFD_REFERENCE_SRC names one
REF = Path(os.environ.get("PCFD_REFERENCE_SRC") or "/nonexistent")


def test_fixture_shape():
    spec = mechanism()
    assert [s["name"] for s in spec["species"]] == ["O2", "O", "N", "N2", "NO"]
    assert len(spec["reactions"]) == 6
    # O2 + M <==> 2O + M with the file's third-body efficiencies
    r = spec["reactions"][0]
    assert r["type"] == 2 and r["third_bodies"] == 1
    assert r["species"] == ["O2", "O", "N", "N2", "NO"] and r["tbeff"] == [9.0, 25.0, 1.0, 2.0, 1.0]
    assert r["nup"][:2] == [1.0, 0.0] and r["nupp"][:2] == [0.0, 2.0]
    # N2 + N <==> 2N + N merges N on the right
    r = spec["reactions"][2]
    assert r["species"] == ["N2", "N"] and r["nup"] == [1.0, 1.0] and r["nupp"] == [0.0, 3.0]


@pytest.mark.skipif(not (REF / "chemdata" / "chemDB.py").exists(), reason="reference tree absent")
def test_fixture_regenerates_from_reference(tmp_path):
    out = subprocess.run([sys.executable, str(FIXTURE.parent / "make_chem_fixture.py"), str(REF)],
                         capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    assert json.loads(FIXTURE.read_text()) == mechanism()


def test_oracle_conserves_mass_and_elements():
    spec = mechanism()
    m = model_struct(spec)
    rho, T = states(4000, seed=2)
    w = chem_rates(m, rho, T)
    assert np.all(np.isfinite(w))
    mass, elem = conservation(spec, w)
    # atoms are conserved exactly; mass only to the rounding of the database's
    # molecular weights (2 MW(N) - MW(N2) = 8e-8 kg/mol in the Burcat data)
    assert elem < 1e-12
    assert mass < 1e-5


def test_oracle_dissociation_direction():
    """Pure O2 at 6000 K dissociates; pure O at 300 K recombines."""
    spec = mechanism()
    m = model_struct(spec)
    rho = np.zeros((2, 5))
    rho[0, 0] = 1e-2   # O2
    rho[1, 1] = 1e-2   # O
    w = chem_rates(m, rho, np.array([6000.0, 300.0]))
    assert w[0, 0] < 0 and w[0, 1] > 0
    assert w[1, 1] < 0 and w[1, 0] > 0


def test_find_T_given_P_reference_known_answer():
    """The reference's own test (unitTest/compressibleFRTest.h:6-29): 21 % of
    1.161 kg/m^3 in species 0 and 79 % in species 2 (O2 and N in the 5-species
    mechanism's order) at 101,200 Pa gives 166.5 K +- 0.01, and 83.25 K at
    half the pressure, from a 150 K start."""
    from chem_cases import reference_scales
    from oracle_lib import OracleChemState
    spec = mechanism()
    assert [s["name"] for s in spec["species"]][0] == "O2" and spec["species"][2]["name"] == "N"
    ref = reference_scales()
    O = OracleChemState(model_struct(spec), ref)
    rho = 1.161 / ref.density
    rhoi = np.array([[0.21 * rho, 0.0, 0.79 * rho, 0.0, 0.0]] * 2)
    T, its = O.find_T(rhoi, np.array([101200.0, 50600.0]) / ref.pressure, np.full(2, 150.0 / ref.temperature))
    T *= ref.temperature
    assert abs(T[0] - 166.5) < 0.01 and abs(T[1] - 166.5 / 2.0) < 0.01, T
    assert np.all(its < 28)


def test_fr_native_conservative_round_trip():
    """NativeToConservative followed by ConservativeToNative (the FP64
    temperature Newton from total energy) returns the temperature and
    velocities; ComputeAuxiliaryVariables' pressure is Dalton's law."""
    from chem_cases import fr_states
    from oracle_lib import OracleChemState
    ref, rhoi, vel, T = fr_states(200)
    O = OracleChemState(model_struct(mechanism()), ref)
    P, cvi, mol = O.aux(rhoi, T)
    mw = np.array([s["MW"] for s in mechanism()["species"]])
    R = 8.31447215 / mw
    assert np.allclose(P * ref.pressure, (rhoi * ref.density * R).sum(axis=1) * T * ref.temperature, rtol=1e-14)
    assert np.all(cvi > 0)
    assert np.allclose(mol, rhoi / mw / 1000.0, rtol=0)
    native = np.c_[vel, T]
    qm = O.n2c(rhoi, native, P)
    back, its = O.c2n(np.c_[rhoi, qm], P * 1.3)   # a stale pressure as the initial guess
    assert np.all(its < 20)
    assert np.allclose(back[:, 3], T, rtol=1e-11, atol=0)
    assert np.allclose(back[:, :3], vel, rtol=1e-14, atol=1e-15)


def test_fr_hllc_consistency():
    """HLLCFlux(Q, Q) is the physical flux: rho_i theta, rho u theta +
    (p - Pref) n (the reference carries the gauge pressure in the momentum
    flux), theta (rho Et + p), times the area; symmetry2D zeroes one momentum
    component."""
    from chem_cases import fr_records, fr_states
    from oracle_lib import OracleChemState
    from proteuscfd_gb300 import _native as N
    ref, rhoi, vel, T = fr_states(20, seed=11)
    q = fr_records(ref, rhoi, vel, T)
    O = OracleChemState(model_struct(mechanism()), ref)
    ns = O.ns
    rng = np.random.default_rng(1)
    nrm = rng.normal(size=(20, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    avec = np.c_[nrm, rng.uniform(0.5, 2.0, 20)]
    pref = 0.7
    for beta in (1.0, 0.3):
        f, bad = O.hllc(N.ChemFluxOpts(beta, pref, 0), q, np.c_[np.arange(20), np.arange(20)], avec)
        assert bad == 0
        th = (vel * nrm).sum(axis=1)
        rho = rhoi.sum(axis=1)
        P = q[:, ns + 4]
        X = rhoi / rho[:, None]
        Et = O.n2c(rhoi, np.c_[vel, T], P)[:, 3]
        ref_f = np.c_[rhoi * th[:, None], rho[:, None] * vel * th[:, None] + (P - pref)[:, None] * nrm,
                      th * (Et + P)] * avec[:, 3:4]
        scale = np.abs(ref_f).max(axis=1, keepdims=True)
        assert np.abs(f - ref_f).max() <= 1e-12 * scale.max(), np.abs(f - ref_f).max()
    f2, _ = O.hllc(N.ChemFluxOpts(1.0, pref, 2), q, np.c_[np.arange(20), np.arange(20)], avec)
    assert np.all(f2[:, ns + 1] == 0.0)


def test_fr_residual_freestream_preserved():
    """A uniform reacting state on every node and phantom of a closed
    jittered box leaves a zero residual with reactions off (the dual faces
    close and HLLC(Q, Q) is the physical flux)."""
    from chem_cases import fr_records, fr_states
    from oracle_lib import OracleChemState
    from proteuscfd_gb300 import Mesh
    from proteuscfd_gb300 import _native as N
    m = Mesh.box(7, 6, 5, jitter=0.2, seed=3)
    ref, rhoi, vel, T = fr_states(1, seed=4)
    q = np.tile(fr_records(ref, rhoi, vel, T), (m.nnode + m.nbedge, 1))
    O = OracleChemState(model_struct(mechanism()), ref)
    b, norms = O.residual(N.ChemFluxOpts(1.0, 0.3, 0), m, q, 1e-3, 0)
    ns = O.ns
    scale = np.abs(q[0, :ns]).max() * np.abs(vel).max() * np.asarray(m.edge_area)[:, 3].max()
    assert np.abs(b).max() < 1e-13 * max(scale, 1.0), np.abs(b).max()


def test_fr_source_jacobian_against_central_differences():
    """The oracle's SourceTermJacobian (one-sided, h = 1e-8) against central
    differences of the oracle's own source term with a larger step: equal to
    the one-sided truncation and rounding error.  Velocity columns and the
    momentum and energy rows are zero, and the species rows of every column
    sum to zero (mass is conserved by every reaction)."""
    from chem_cases import fr_records, fr_states
    from oracle_lib import OracleChemState
    ref, rhoi, vel, T = fr_states(40, seed=21)
    T = np.clip(T, 1500.0 / ref.temperature, None)
    q = fr_records(ref, rhoi, vel, T)
    vol = np.random.default_rng(5).uniform(0.5, 2.0, size=len(T))
    ref_time = 2.5e-4
    O = OracleChemState(model_struct(mechanism()), ref)
    A = O.source_jacobian(q, vol, ref_time)
    ns = O.ns
    neqn = ns + 4
    assert A.shape == (len(T), neqn, neqn)
    assert np.all(A[:, ns:, :] == 0.0) and np.all(A[:, :, ns:ns + 3] == 0.0)

    def source(Q):
        w = chem_rates(model_struct(mechanism()), (Q[:, :ns] * ref.density).copy(), Q[:, ns + 3] * ref.temperature)
        return vol[:, None] * (w / (ref.density / ref_time))

    S0 = source(q)
    smax = np.abs(S0).max(axis=1)
    cols = list(range(ns)) + [ns + 3]
    for i in cols:
        hc = 1e-5 * np.abs(q[:, i]).max()
        qp, qm = q.copy(), q.copy()
        qp[:, i] += hc
        qm[:, i] -= hc
        Ac = (source(qp) - source(qm)) / (2 * hc)
        scale = np.abs(Ac).max(axis=1) + smax
        err = np.abs(A[:, :ns, i] - Ac).max(axis=1) / scale
        assert err.max() < 1e-5, (i, err.max())
        colsum = np.abs(A[:, :ns, i].sum(axis=1)) / scale
        assert colsum.max() < 5e-5, (i, colsum.max())


def test_fr_temporal_terms_are_conservative_over_native():
    """ContributeTemporalTerms with beta = 1 (no preconditioning) adds
    vol/dtau times the Jacobian of the conservative variables (rhoi, rho u,
    rho v, rho w, rho Et) over the native ones (rhoi, u, v, w, T); checked
    against central differences of the oracle's NativeToConservative, with
    the pressure of each perturbed state from ComputeAuxiliaryVariables.
    With beta < 1 only the temperature column changes, and adding into a
    block adds."""
    from chem_cases import fr_records, fr_states
    from oracle_lib import OracleChemState
    ref, rhoi, vel, T = fr_states(12, seed=31)
    q = fr_records(ref, rhoi, vel, T)
    n = len(T)
    vol = np.linspace(0.5, 2.0, n)
    dtau = np.linspace(0.01, 0.2, n)
    O = OracleChemState(model_struct(mechanism()), ref)
    ns = O.ns
    A1 = O.temporal(q, vol, dtau, np.ones(n), 1.0, 0.0, 0)

    def cons(nat):
        r, vv, t = nat[:, :ns], nat[:, ns:ns + 3], nat[:, ns + 3]
        P, _, _ = O.aux(r, t)
        return np.c_[r, O.n2c(r, np.c_[vv, t], P)]

    nat = np.c_[rhoi, vel, T]
    J = np.empty((n, ns + 4, ns + 4))
    for i in range(ns + 4):
        hc = 1e-6 * max(np.abs(nat[:, i]).max(), 1e-3)
        p, m = nat.copy(), nat.copy()
        p[:, i] += hc
        m[:, i] -= hc
        J[:, :, i] = (cons(p) - cons(m)) / (2 * hc)
    want = (vol / dtau)[:, None, None] * J
    scale = np.abs(want).max(axis=2, keepdims=True)
    err = (np.abs(A1 - want) / scale).max()
    assert err < 1e-6, err
    base = np.random.default_rng(2).normal(size=A1.shape)
    Ab = O.temporal(q, vol, dtau, np.full(n, 0.3), 1.0, 0.0, 0, A=base)
    A3 = O.temporal(q, vol, dtau, np.full(n, 0.3), 1.0, 0.0, 0)
    assert np.allclose(Ab - base, A3, rtol=1e-12, atol=1e-12 * np.abs(A3).max())
    assert np.array_equal(A3[:, :, :ns + 3], A1[:, :, :ns + 3])
    assert not np.allclose(A3[:, :, ns + 3], A1[:, :, ns + 3])


def _numpy_transport(spec, rhoi_dim, Td):
    """Species and mixture viscosity and conductivity restated with NumPy
    (White's forms at or below 1000 K, the last matching RP-1311 fit above,
    Wilke's rule with mole fractions whose last is 1 - the sum of the
    others), dimensional."""
    sp = spec["species"]
    mw = np.array([s["MW"] for s in sp])

    def fit(rows, T, conv):
        r = [row for row in rows if row[0] <= T <= row[1]][-1]
        return np.exp(r[2] * np.log(T) + r[3] / T + r[4] / T ** 2 + r[5]) * conv

    def props(T):
        if T <= 1000.0:
            mu = 1.716e-5 * (T / 273.0) ** 1.5 * (384.0 / (T + 111.0))
            k = 0.0241 * (T / 273.0) ** 1.5 * (467.0 / (T + 194.0))
            return np.full(len(sp), mu), np.full(len(sp), k)
        return (np.array([fit(s["mu"], T, 1e-7) for s in sp]), np.array([fit(s["k"], T, 1e-4) for s in sp]))

    mu_out, k_out = [], []
    for r, T in zip(rhoi_dim, Td):
        X = (r / r.sum()) / mw
        X = X / X.sum()
        X[-1] = 1.0 - X[:-1].sum()
        vi, ki = props(T)
        temp = 1.0 + np.sqrt(vi[:, None] / vi[None, :]) * (mw[None, :] / mw[:, None]) ** 0.25
        phi = (1.0 + mw[:, None] / mw[None, :]) ** -0.5 * temp ** 2 / np.sqrt(8.0)
        w = (phi * X[None, :]).sum(axis=1)
        mu_out.append((X / w * vi).sum())
        k_out.append((X / w * ki).sum())
    return np.array(mu_out), np.array(k_out)


def test_transport_properties():
    """Mixture viscosity and conductivity (GetMolecularViscosity /
    GetThermalConductivity with Wilke's rule) against a NumPy restatement,
    White's air values at 300 K for a pure species, and the fits' own
    range limit."""
    from oracle_lib import OracleChemState
    from chem_cases import reference_scales
    spec = mechanism()
    ref = reference_scales()
    ref.viscosity, ref.conductivity = 1.0e-5, 0.02
    ns = len(spec["species"])
    rng = np.random.default_rng(4)
    rhoi = 10.0 ** rng.uniform(-4, 0, size=(200, ns))
    Td = np.concatenate([[300.0, 1000.0, 1000.5, 5000.0, 5000.5, 14999.0], rng.uniform(250.0, 14000.0, 194)])
    O = OracleChemState(model_struct(spec), ref)
    mu, k, bad = O.transport(rhoi / ref.density, Td / ref.temperature)
    assert bad == 0
    mu_np, k_np = _numpy_transport(spec, rhoi, Td)
    np.testing.assert_allclose(mu * ref.viscosity, mu_np, rtol=1e-12)
    np.testing.assert_allclose(k * ref.conductivity, k_np, rtol=1e-12)
    # a pure species takes its own values: White's air viscosity at 300 K
    pure = np.zeros((1, ns))
    pure[0, 3] = 1.0
    mu1, k1, _ = O.transport(pure / ref.density, np.array([300.0]) / ref.temperature)
    assert abs(mu1[0] * ref.viscosity - 1.716e-5 * (300 / 273.0) ** 1.5 * 384.0 / 411.0) < 1e-20
    assert abs(k1[0] * ref.conductivity - 0.0241 * (300 / 273.0) ** 1.5 * 467.0 / 494.0) < 1e-17
    # N2 at 2000 K from its RP-1311 fit: about 6.3e-5 Pa s
    mu2, _, _ = O.transport(pure / ref.density, np.array([2000.0]) / ref.temperature)
    assert 6.0e-5 < mu2[0] * ref.viscosity < 6.7e-5
    # above every fit's range the reference aborts; the oracle counts it
    assert O.transport(pure / ref.density, np.array([16000.0]) / ref.temperature)[2] == 1


def test_viscous_residual_properties():
    """The oracle's reacting viscous residual: zero for a uniform state with
    zero gradients; for a linear velocity u = a y with its exact gradient
    the momentum flux through a face of unit normal y is -(area / Re) mu a,
    and the interior faces' contributions cancel in the sum over nodes."""
    from chem_cases import fr_records, fr_states, reference_scales
    from oracle_lib import OracleChemState
    from proteuscfd_gb300 import Mesh
    from proteuscfd_gb300.chem import ChemModel
    spec = mechanism()
    ns = len(spec["species"])
    m = Mesh.box(6, 5, 4, jitter=0.2, seed=3)
    nrows = m.nnode + m.nbedge
    ref, rhoi, vel, T = fr_states(nrows, seed=3)
    rhoi[:] = rhoi[0]
    vel[:] = vel[0]
    T[:] = T[0]
    q = fr_records(ref, rhoi, vel, T)
    O = OracleChemState(model_struct(spec), ref)
    opts = ChemModel.flux_opts(1.0, 0.4, 0)
    grad = np.zeros((m.nnode, 2 * ns + 4, 3))
    b, bad = O.viscous_residual(opts, m, 1.0e4, 1, q, grad)
    assert bad == 0 and np.abs(b).max() == 0.0
    # u = a y at every node and phantom, exact gradient
    a = 0.3
    y = np.r_[m.xyz[:, 1], m.xyz[m.bedges[:, 0], 1]]
    q2 = q.copy()
    q2[:, ns] = a * y
    grad[:, ns, 1] = a
    b2, _ = O.viscous_residual(opts, m, 1.0e4, 1, q2, grad)
    # only the x-momentum and energy rows see the shear, and the interior
    # faces cancel in the total: what remains is the boundary faces' sum
    assert np.abs(b2[:, :ns]).max() == 0.0
    mu, _, _ = O.transport(rhoi[:1], T[:1])
    ba = m.bedge_area
    expect = -(-(mu[0] / 1.0e4) * a * (ba[:, 1] * ba[:, 3])).sum()
    assert abs(b2[:, ns].sum() - expect) < 1e-12 * abs(expect) + 1e-18


def test_gradient_linear_exactness():
    """The oracle's reacting LSQ gradient reproduces fields linear in x, y, z
    exactly at every node (the weighted least squares is exact for them),
    and the symmetry fix removes the normal part on the listed tags."""
    from chem_cases import fr_records, fr_states
    from oracle_lib import OracleChemState
    from proteuscfd_gb300 import Mesh
    spec = mechanism()
    ns = len(spec["species"])
    m = Mesh.box(7, 6, 5, jitter=0.2, seed=4)
    nrows = m.nnode + m.nbedge
    ref, rhoi, vel, T = fr_states(nrows, seed=5)
    x = np.r_[m.xyz, m.xyz[m.bedges[:, 0]]]
    a = np.array([0.3, -0.2, 0.1])
    lin = x @ a
    rhoi[:] = rhoi[0] * (1.0 + 0.1 * lin[:, None])
    vel[:, 0] = 0.2 + 0.5 * lin
    T[:] = T[0] * (1.0 + 0.05 * lin)
    q = fr_records(ref, rhoi, vel, T)
    O = OracleChemState(model_struct(spec), ref)
    g = O.gradient(m, q)
    assert np.allclose(g[:, ns, :], 0.5 * a, rtol=0, atol=1e-12)         # u
    assert np.allclose(g[:, ns + 3, :], 0.05 * T[0] * a, rtol=0, atol=1e-12)  # T
    assert np.allclose(g[:, 0, :], 0.1 * rhoi[0, 0] * a, rtol=0, atol=1e-9 * rhoi[0, 0])
    gs = O.gradient(m, q, sym_tags=[5, 6])
    zmin = m.bfactag == 5
    nodes = np.unique(m.bedges[zmin, 0])
    assert np.allclose(gs[nodes, ns, 2], 0.0, atol=1e-12)


def test_boundary_conditions():
    """The oracle's reacting UpdateBCs: inflow nodes and phantoms take the
    reference record, outflow phantoms copy their node, the isothermal wall
    rests at its temperature, and the mirror flips the normal velocity and
    keeps the tangential one; an unbuilt type (far field) is reported."""
    from chem_cases import fr_records, fr_states
    from oracle_lib import OracleChemState
    from proteuscfd_gb300 import Mesh
    from proteuscfd_gb300 import _native as N
    spec = mechanism()
    ns = len(spec["species"])
    m = Mesh.box(7, 6, 5, jitter=0.2, seed=4)
    nrows = m.nnode + m.nbedge
    ref, rhoi, vel, T = fr_states(nrows, seed=6)
    q = fr_records(ref, rhoi, vel, T)
    O = OracleChemState(model_struct(spec), ref)
    types = {1: N.BC_SONIC_INFLOW, 2: N.BC_SONIC_OUTFLOW, 3: N.BC_NOSLIP, 4: N.BC_SYMMETRY, 5: N.BC_SYMMETRY,
             6: N.BC_IMPERMEABLE_WALL}
    qin = q[0].copy()
    q2, rc = O.update_bcs(m, q, types, twall={3: 2000.0}, qref={1: qin})
    assert rc == 0
    be, tag, ba = m.bedges, m.bfactag, m.bedge_area
    order = np.arange(m.nbedge)
    last = {}
    for k in order:          # the last half-edge of each node decides its state
        last[be[k, 0]] = k
    for k in order:
        node, ph = be[k]
        if tag[k] == 1:
            assert np.allclose(q2[ph, :ns + 4], qin[:ns + 4], rtol=0, atol=0)
        if tag[k] == 3 and last[node] == k:
            assert np.all(q2[node, ns:ns + 3] == 0.0) and q2[node, ns + 3] == 2000.0 / ref.temperature
        if tag[k] in (4, 6) and last[node] == k:
            vn = q2[node, ns:ns + 3] @ ba[k, :3]
            assert np.allclose(q2[ph, ns:ns + 3] @ ba[k, :3], -vn, atol=1e-13)
    # far field is not restated: reported, records left as they were
    _, rc = O.update_bcs(m, q, {**types, 2: N.BC_FARFIELD}, twall={3: 2000.0}, qref={1: qin})
    assert rc > 0 and tag[rc - 1] == 2


def test_second_order_residual_reduces_to_first_order():
    """The oracle's second-order reacting residual equals the first-order one
    when the corrections vanish (zero gradient and chi = 0, or a zero
    limiter), and differs when they do not."""
    from chem_cases import fr_records, fr_states
    from oracle_lib import OracleChemState
    from proteuscfd_gb300 import Mesh
    from proteuscfd_gb300.chem import ChemModel
    spec = mechanism()
    ns = len(spec["species"])
    m = Mesh.box(6, 5, 4, jitter=0.2, seed=8)
    nrows = m.nnode + m.nbedge
    ref, rhoi, vel, T = fr_states(nrows, seed=8)
    q = fr_records(ref, rhoi, vel, T)
    O = OracleChemState(model_struct(spec), ref)
    opts = ChemModel.flux_opts(1.0, 0.4, 0)
    b1, n1 = O.residual(opts, m, q, 2.5e-4, 1)
    zero_g = np.zeros((m.nnode, 2 * ns + 4, 3))
    ones = np.ones((m.nnode, ns + 4))
    b2, _ = O.residual_ho(opts, m, q, zero_g, ones, 0.0, 2.5e-4, 1)
    assert np.array_equal(b1, b2)
    g = np.random.default_rng(1).normal(size=zero_g.shape) * 1e-3
    b3, _ = O.residual_ho(opts, m, q, g, np.zeros_like(ones), 0.0, 2.5e-4, 1)
    assert np.array_equal(b1, b3)
    b4, _ = O.residual_ho(opts, m, q, g, ones, 0.0, 2.5e-4, 1)
    assert not np.array_equal(b1, b4)


def test_limiter_properties():
    """The oracle's reacting limiter: values in [0, 1], exactly 1 for a
    uniform field (no extrapolated change), and below 1 where the
    extrapolation overshoots the neighbour bounds."""
    from chem_cases import fr_records, fr_states
    from oracle_lib import OracleChemState
    from proteuscfd_gb300 import Mesh
    spec = mechanism()
    ns = len(spec["species"])
    m = Mesh.box(7, 6, 5, jitter=0.2, seed=9)
    nrows = m.nnode + m.nbedge
    ref, rhoi, vel, T = fr_states(nrows, seed=9)
    q = fr_records(ref, rhoi, vel, T)
    O = OracleChemState(model_struct(spec), ref)
    g = O.gradient(m, q)
    lim = O.limiter(m, q, g, 0.0)
    assert lim.min() >= 0.0 and lim.max() <= 1.0 and lim.min() < 1.0
    qu = q.copy()
    qu[:] = q[0]
    lu = O.limiter(m, qu, np.zeros_like(g), 0.0)
    assert np.all(lu == 1.0)
