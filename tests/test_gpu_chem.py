"""Finite-rate chemistry on the GPU against the oracle, through the C ABI:
production rates of the 5-species air mechanism at seeded states across
both curve fits and the pinned temperature ranges, and conservation of the
elements at the reacting workload's size (2,007,040 nodes)."""
import numpy as np
import pytest

from chem_cases import conservation, mechanism, states
from oracle_lib import chem_rates
from proteuscfd_gb300 import _native as N
from proteuscfd_gb300.chem import ChemModel, model_struct

pytestmark = pytest.mark.gpu


def test_rates_parity():
    spec = mechanism()
    c = ChemModel(spec)
    rho, T = states(20000, seed=3)
    w = c.production_rates(rho, T)
    ref = chem_rates(model_struct(spec), rho, T)
    # the same operations; exp, log and pow differ between CUDA's and the
    # host's libm by an ulp or so, which the largest term of each node
    # bounds (1e-12 of the node's largest rate)
    scale = np.abs(ref).max(axis=1, keepdims=True)
    err = np.abs(w - ref) / scale
    assert err.max() < 1e-12, err.max()
    c.close()


def test_rates_full_size_conservation():
    spec = mechanism()
    c = ChemModel(spec)
    rho, T = states(2007040, seed=4, tmin=300.0, tmax=8000.0)
    w = c.production_rates(rho, T)
    assert np.all(np.isfinite(w))
    mass, elem = conservation(spec, w)
    assert elem < 1e-12 and mass < 1e-5
    c.close()


def test_bad_model_rejected():
    spec = mechanism()
    bad = dict(spec, reactions=[dict(spec["reactions"][0], **{"global": [0, 1, 2, 3, 99]})])
    with pytest.raises(N.PcfdError):
        ChemModel(bad)


def test_fr_find_T_given_P_known_answer_gpu():
    """unitTest/compressibleFRTest.h:6-29 on the GPU: 166.5 K and 83.25 K
    (+- 0.01), and the same values as the oracle."""
    from chem_cases import reference_scales
    from oracle_lib import OracleChemState
    spec = mechanism()
    ref = reference_scales()
    C = ChemModel(spec)
    rho = 1.161 / ref.density
    rhoi = np.array([[0.21 * rho, 0.0, 0.79 * rho, 0.0, 0.0]] * 2)
    P = np.array([101200.0, 50600.0]) / ref.pressure
    T0 = np.full(2, 150.0 / ref.temperature)
    T, bad = C.find_T_given_P(ref, rhoi, P, T0)
    assert bad == 0
    Td = T * ref.temperature
    assert abs(Td[0] - 166.5) < 0.01 and abs(Td[1] - 83.25) < 0.01, Td
    To, _ = OracleChemState(model_struct(spec), ref).find_T(rhoi, P, T0)
    assert np.allclose(T, To, rtol=1e-14, atol=0)
    C.close()


def test_fr_node_state_parity():
    """ComputeAuxiliaryVariables, NativeToConservative and the FP64
    temperature Newton of ConservativeToNative against the oracle on 3,000
    seeded states (250 to 6000 K), host arrays and device arrays."""
    import torch
    from chem_cases import fr_states
    from oracle_lib import OracleChemState
    spec = mechanism()
    ref, rhoi, vel, T = fr_states(3000, seed=5)
    C = ChemModel(spec)
    O = OracleChemState(model_struct(spec), ref)
    P, cvi, mol = C.aux(ref, rhoi, T)
    Po, cvo, mo = O.aux(rhoi, T)
    assert np.allclose(P, Po, rtol=1e-14, atol=0)
    assert np.allclose(cvi, cvo, rtol=1e-13, atol=0)
    assert np.allclose(mol, mo, rtol=1e-15, atol=0)
    native = np.c_[vel, T]
    qm = C.native_to_conservative(ref, rhoi, native, P)
    qo = O.n2c(rhoi, native, Po)
    assert np.allclose(qm, qo, rtol=1e-13, atol=1e-15)
    q = np.c_[rhoi, qm]
    Pst = P * 1.3   # a stale stored pressure as the initial guess
    back = C.conservative_to_native(ref, q, Pst)
    bo, its = O.c2n(q, Pst)
    assert np.all(its < 20)
    assert np.allclose(back, bo, rtol=1e-12, atol=1e-15)
    assert np.allclose(back[:, 3], T, rtol=1e-11, atol=0)
    # device arrays, in place on the handle's stream
    dq = torch.from_numpy(q).cuda()
    dP = torch.from_numpy(Pst).cuda()
    dout = torch.empty((len(T), 4), dtype=torch.float64, device="cuda")
    C.conservative_to_native_dev(ref, len(T), dq.data_ptr(), dP.data_ptr(), dout.data_ptr())
    assert np.array_equal(dout.cpu().numpy(), back)
    C.close()


def test_fr_conservative_to_native_reports_nonconvergence():
    """A total energy below every temperature's (negative internal energy)
    leaves the Newton iteration unconverged after 20 iterations: the call
    returns PCFD_ERR_NUMERIC, as the reference aborts."""
    from chem_cases import fr_states
    from proteuscfd_gb300 import _native as N
    spec = mechanism()
    ref, rhoi, vel, T = fr_states(4, seed=9)
    C = ChemModel(spec)
    P, _, _ = C.aux(ref, rhoi, T)
    qm = C.native_to_conservative(ref, rhoi, np.c_[vel, T], P)
    qm[1, 3] = -1.0e3 * abs(qm[1, 3])
    with pytest.raises(N.PcfdError) as e:
        C.conservative_to_native(ref, np.c_[rhoi, qm], P)
    assert e.value.code == N.PCFD_ERR_NUMERIC
    C.close()


@pytest.mark.parametrize("beta", [1.0, 0.25])
def test_fr_hllc_parity(beta):
    """The reacting HLLC flux on the GPU against the oracle on 4,000 random
    edges between 1,000 seeded node records (all four HLLC regions occur),
    host and device arrays, with the reference's gauge pressure."""
    import torch
    from chem_cases import fr_edges, fr_records, fr_states
    from oracle_lib import OracleChemState
    spec = mechanism()
    ref, rhoi, vel, T = fr_states(1000, seed=12)
    vel = vel * 4.0   # supersonic and subsonic pairs
    q = fr_records(ref, rhoi, vel, T)
    edges, avec = fr_edges(1000, 4000, seed=4)
    C = ChemModel(spec)
    opts = C.flux_opts(beta, 0.5, 0)
    f = C.hllc_flux(ref, opts, q, edges, avec)
    fo, bad = OracleChemState(model_struct(spec), ref).hllc_batch(opts, q, edges, avec)
    assert bad == 0
    scale = np.abs(fo).max(axis=1, keepdims=True)
    err = np.abs(f - fo) / scale
    assert err.max() < 1e-12, err.max()
    # which HLLC region each edge took: both supersonic sides and both star regions occur
    ns = C.nspecies
    th = lambda k: (q[edges[:, k], ns:ns + 3] * avec[:, :3]).sum(axis=1)
    assert (th(0) > 2.0).any() and (th(1) < -2.0).any()
    dq = torch.from_numpy(q).cuda()
    de = torch.from_numpy(edges).cuda()
    da = torch.from_numpy(np.ascontiguousarray(avec)).cuda()
    dfx = torch.empty((len(edges), ns + 4), dtype=torch.float64, device="cuda")
    assert C.hllc_flux_dev(ref, opts, len(q), dq.data_ptr(), len(edges), de.data_ptr(), da.data_ptr(),
                           dfx.data_ptr()) == 0
    assert np.array_equal(dfx.cpu().numpy(), f)
    C.close()


def test_fr_hllc_rejects_bad_node_ids():
    """Host arrays with an out-of-range node id are refused before any copy;
    on device arrays the kernel's own bounds check skips the edge and the
    call reports it."""
    import torch
    from chem_cases import fr_edges, fr_records, fr_states
    spec = mechanism()
    ref, rhoi, vel, T = fr_states(50, seed=13)
    q = fr_records(ref, rhoi, vel, T)
    edges, avec = fr_edges(50, 10, seed=5)
    edges[3, 1] = 50
    C = ChemModel(spec)
    opts = C.flux_opts()
    with pytest.raises(N.PcfdError) as e:
        C.hllc_flux(ref, opts, q, edges, avec)
    assert e.value.code == N.PCFD_ERR_ARG
    dq = torch.from_numpy(q).cuda()
    de = torch.from_numpy(edges).cuda()
    da = torch.from_numpy(np.ascontiguousarray(avec)).cuda()
    dfx = torch.empty((10, C.nspecies + 4), dtype=torch.float64, device="cuda")
    with pytest.raises(N.PcfdError) as e:
        C.hllc_flux_dev(ref, opts, len(q), dq.data_ptr(), 10, de.data_ptr(), da.data_ptr(), dfx.data_ptr())
    assert e.value.code == N.PCFD_ERR_NUMERIC
    assert np.all(dfx.cpu().numpy()[3] == 0.0)
    C.close()


@pytest.mark.parametrize("reactions", [0, 1])
def test_fr_residual_parity(reactions):
    """The reacting first-order residual (HLLC fluxes on edges and boundary
    half-edges, deterministic gather, chemistry source) and its norms against
    the oracle on a jittered box with seeded states on every node and
    phantom; host arrays, then device arrays."""
    import torch
    from chem_cases import fr_records, fr_states
    from oracle_lib import OracleChemState
    from proteuscfd_gb300 import Mesh
    spec = mechanism()
    m = Mesh.box(12, 9, 8, jitter=0.2, seed=5)
    nrows = m.nnode + m.nbedge
    ref, rhoi, vel, T = fr_states(nrows, seed=14)
    q = fr_records(ref, rhoi, vel, T)
    C = ChemModel(spec)
    C.attach_mesh(m)
    opts = C.flux_opts(1.0, 0.4, 0)
    ref_time = 2.5e-4
    b, norms = C.residual(ref, opts, ref_time, reactions, q)
    bo, no = OracleChemState(model_struct(spec), ref).residual(opts, m, q, ref_time, reactions)
    scale = np.abs(bo).max(axis=0, keepdims=True)
    assert (np.abs(b - bo) / scale).max() < 1e-11, (np.abs(b - bo) / scale).max()
    assert np.allclose(norms, no, rtol=1e-11, atol=0)
    dq = torch.from_numpy(q).cuda()
    db = torch.empty((m.nnode, C.nspecies + 4), dtype=torch.float64, device="cuda")
    nd = C.residual_dev(ref, opts, ref_time, reactions, dq.data_ptr(), db.data_ptr())
    assert np.array_equal(db.cpu().numpy(), b) and np.array_equal(nd, norms)
    C.close()


def test_source_jacobian_parity():
    """SourceTermJacobian on the GPU against the oracle's, node by node, on
    seeded reacting states (host arrays, then device arrays).  The one-sided
    difference divides the rates' last-ulp differences between CUDA's and
    the host's libm by h = 1e-8, so entries are compared to 1e-5 of the
    node's scale (largest entry of the column plus the largest source
    value); the zero rows and columns are exact."""
    import torch
    from chem_cases import fr_records, fr_states
    from oracle_lib import OracleChemState
    spec = mechanism()
    ref, rhoi, vel, T = fr_states(3000, seed=23)
    q = fr_records(ref, rhoi, vel, T)
    vol = np.random.default_rng(6).uniform(0.5, 2.0, size=len(T))
    ref_time = 2.5e-4
    C = ChemModel(spec)
    A = C.source_jacobian(ref, ref_time, q, vol)
    Ao = OracleChemState(model_struct(spec), ref).source_jacobian(q, vol, ref_time)
    ns = C.nspecies
    assert np.all(A[:, ns:, :] == 0.0) and np.all(A[:, :, ns:ns + 3] == 0.0)
    w = chem_rates(model_struct(spec), (q[:, :ns] * ref.density).copy(), q[:, ns + 3] * ref.temperature)
    smax = np.abs(vol[:, None] * w / (ref.density / ref_time)).max(axis=1)
    scale = np.abs(Ao).max(axis=1) + smax[:, None]
    err = (np.abs(A - Ao) / scale[:, None, :]).max()
    assert err < 1e-5, err
    dq = torch.from_numpy(q).cuda()
    dv = torch.from_numpy(vol).cuda()
    dA = torch.empty(A.shape, dtype=torch.float64, device="cuda")
    C.source_jacobian_dev(ref, ref_time, len(vol), dq.data_ptr(), dv.data_ptr(), dA.data_ptr())
    assert np.array_equal(dA.cpu().numpy(), A)
    C.close()


def test_source_jacobian_full_size_mass_conservation():
    """At the reacting box's size (2,007,040 nodes) the species rows of every
    column of the source Jacobian sum to zero up to the difference quotient's
    rounding, as every reaction conserves mass."""
    from chem_cases import fr_states
    spec = mechanism()
    C = ChemModel(spec)
    ref, rhoi, vel, T = fr_states(2007040, seed=24)
    P, cvi, mol = C.aux(ref, rhoi, T)
    q = np.ascontiguousarray(np.c_[rhoi, vel, T, P, rhoi.sum(axis=1), cvi, mol])
    vol = np.full(len(T), 1.0)
    ref_time = 2.5e-4
    A = C.source_jacobian(ref, ref_time, q, vol)
    ns = C.nspecies
    assert np.all(np.isfinite(A))
    # the quotient's rounding scales with the source itself where the
    # reactions are frozen (low T), so the bound includes it
    w = C.production_rates(rhoi * ref.density, T * ref.temperature)
    smax = np.abs(w / (ref.density / ref_time)).max(axis=1)
    colsum = np.abs(A[:, :ns, :].sum(axis=1))
    scale = np.abs(A[:, :ns, :]).max(axis=1) + smax[:, None]
    assert (colsum / scale).max() < 1e-4, (colsum / scale).max()
    C.close()


@pytest.mark.parametrize("local_ts", [0, 1])
def test_temporal_terms_parity(local_ts):
    """ContributeTemporalTerms on the GPU against the oracle on seeded
    reacting records with per-node volumes, pseudo-time steps and beta in
    (0.2, 1], added into a random block (host arrays), then in place on
    device arrays."""
    import torch
    from chem_cases import fr_records, fr_states
    from oracle_lib import OracleChemState
    spec = mechanism()
    ref, rhoi, vel, T = fr_states(4000, seed=33)
    q = fr_records(ref, rhoi, vel, T)
    n = len(T)
    rng = np.random.default_rng(8)
    vol = rng.uniform(0.5, 2.0, size=n)
    dtau = rng.uniform(1e-3, 1e-1, size=n)
    beta = rng.uniform(0.2, 1.0, size=n)
    C = ChemModel(spec)
    ns = C.nspecies
    base = rng.normal(size=(n, ns + 4, ns + 4))
    A = C.temporal_terms(ref, q, vol, dtau, beta, 1.5, 0.05, local_ts, A=base)
    Ao = OracleChemState(model_struct(spec), ref).temporal(q, vol, dtau, beta, 1.5, 0.05, local_ts, A=base)
    scale = np.abs(Ao).max(axis=2, keepdims=True)
    err = (np.abs(A - Ao) / scale).max()
    assert err < 1e-13, err
    dq = torch.from_numpy(q).cuda()
    dv, dt_, db = (torch.from_numpy(x).cuda() for x in (vol, dtau, beta))
    dA = torch.from_numpy(base.copy()).cuda()
    C.temporal_terms_dev(ref, n, dq.data_ptr(), dv.data_ptr(), dt_.data_ptr(), db.data_ptr(), 1.5, 0.05, local_ts,
                         dA.data_ptr())
    assert np.array_equal(dA.cpu().numpy(), A)
    C.close()


def test_transport_parity():
    """Mixture viscosity and conductivity (Wilke's rule over White's forms
    and the RP-1311 fits) on the GPU against the oracle; above every fit's
    range the call is refused, as the reference aborts."""
    from chem_cases import reference_scales
    from oracle_lib import OracleChemState
    spec = mechanism()
    c = ChemModel(spec)
    ref = reference_scales()
    ref.viscosity, ref.conductivity = 1.0e-5, 0.02
    rng = np.random.default_rng(9)
    ns = len(spec["species"])
    n = 20000
    rhoi = 10.0 ** rng.uniform(-4, 0, size=(n, ns)) / ref.density
    Td = rng.uniform(250.0, 14900.0, size=n)
    Td[:6] = [300.0, 1000.0, 1000.5, 5000.0, 5000.5, 14999.0]
    T = Td / ref.temperature
    mu, k = c.transport(ref, rhoi, T)
    O = OracleChemState(model_struct(spec), ref)
    mo, ko, bad = O.transport(rhoi, T)
    assert bad == 0
    # the same operations; exp, log, pow and sqrt differ between CUDA's and
    # the host's libm by an ulp or so
    np.testing.assert_allclose(mu, mo, rtol=1e-13, atol=0)
    np.testing.assert_allclose(k, ko, rtol=1e-13, atol=0)
    with pytest.raises(N.PcfdError):
        c.transport(ref, rhoi[:1], np.array([16000.0 / ref.temperature]))
    c.close()


@pytest.mark.parametrize("directional", [0, 1])
def test_fr_viscous_residual_parity(directional):
    """The viscous part of the reacting residual (face-averaged states and
    gradients, the directional correction, mixture transport, boundary
    faces) on the GPU against the oracle, on a jittered box with seeded
    records and gradients."""
    from chem_cases import fr_records, fr_states
    from oracle_lib import OracleChemState
    from proteuscfd_gb300 import Mesh
    spec = mechanism()
    ns = len(spec["species"])
    m = Mesh.box(12, 9, 8, jitter=0.2, seed=5)
    nrows = m.nnode + m.nbedge
    ref, rhoi, vel, T = fr_states(nrows, seed=21)
    q = fr_records(ref, rhoi, vel, T)
    grad = np.random.default_rng(22).normal(size=(m.nnode, 2 * ns + 4, 3))
    C = ChemModel(spec)
    C.attach_mesh(m)
    opts = C.flux_opts(1.0, 0.4, 0)
    b = C.viscous_residual(ref, opts, 2.0e4, directional, q, grad)
    bo, bad = OracleChemState(model_struct(spec), ref).viscous_residual(opts, m, 2.0e4, directional, q, grad)
    assert bad == 0
    # the same operations in the same order; the transport's exp, log and
    # pow differ from the host's libm by an ulp or so
    scale = np.abs(bo).max(axis=0, keepdims=True)
    scale[scale == 0] = 1.0
    assert (np.abs(b - bo) / scale).max() < 1e-12, (np.abs(b - bo) / scale).max()
    assert np.abs(b[:, :ns]).max() == 0.0
    C.close()


def test_fr_gradient_parity_and_viscous_chain():
    """The reacting LSQ gradient on the GPU against the oracle (the same
    operations in the same order per node), with the symmetry fix on two
    tags; then the viscous residual fed the GPU's own gradient."""
    from chem_cases import fr_records, fr_states
    from oracle_lib import OracleChemState
    from proteuscfd_gb300 import Mesh
    spec = mechanism()
    m = Mesh.box(12, 9, 8, jitter=0.2, seed=6)
    nrows = m.nnode + m.nbedge
    ref, rhoi, vel, T = fr_states(nrows, seed=23)
    q = fr_records(ref, rhoi, vel, T)
    C = ChemModel(spec)
    C.attach_mesh(m)
    O = OracleChemState(model_struct(spec), ref)
    g = C.gradient(q, sym_tags=[5, 6])
    go = O.gradient(m, q, sym_tags=[5, 6])
    scale = np.abs(go).reshape(m.nnode, -1).max(axis=0)
    scale[scale == 0] = 1.0
    assert (np.abs(g - go).reshape(m.nnode, -1) / scale).max() < 1e-13
    opts = C.flux_opts(1.0, 0.4, 0)
    b = C.viscous_residual(ref, opts, 2.0e4, 1, q, g)
    bo, _ = O.viscous_residual(opts, m, 2.0e4, 1, q, go)
    sc = np.abs(bo).max(axis=0, keepdims=True)
    sc[sc == 0] = 1.0
    assert (np.abs(b - bo) / sc).max() < 1e-11
    C.close()


def test_fr_boundary_conditions_parity():
    """The reacting UpdateBCs on the GPU against the oracle (inflow, outflow,
    isothermal wall, mirror), node by node in half-edge order; an unbuilt
    type is refused."""
    from chem_cases import fr_records, fr_states
    from oracle_lib import OracleChemState
    from proteuscfd_gb300 import Mesh
    spec = mechanism()
    m = Mesh.box(12, 9, 8, jitter=0.2, seed=7)
    nrows = m.nnode + m.nbedge
    ref, rhoi, vel, T = fr_states(nrows, seed=24)
    q = fr_records(ref, rhoi, vel, T)
    C = ChemModel(spec)
    C.attach_mesh(m)
    O = OracleChemState(model_struct(spec), ref)
    types = {1: N.BC_SONIC_INFLOW, 2: N.BC_SONIC_OUTFLOW, 3: N.BC_NOSLIP, 4: N.BC_SYMMETRY, 5: N.BC_SYMMETRY,
             6: N.BC_IMPERMEABLE_WALL}
    kw = dict(twall={3: 2000.0}, qref={1: q[0]})
    q2 = C.update_bcs(ref, q, types, **kw)
    qo, rc = O.update_bcs(m, q, types, **kw)
    assert rc == 0
    scale = np.abs(qo).max(axis=0, keepdims=True)
    scale[scale == 0] = 1.0
    assert (np.abs(q2 - qo) / scale).max() < 1e-13
    with pytest.raises(N.PcfdError):
        C.update_bcs(ref, q, {**types, 2: N.BC_FARFIELD}, **kw)
    C.close()


def test_fr_second_order_residual_parity():
    """The second-order reacting residual (midpoint extrapolation with the
    gradient and a limiter, the pressure and density of the extrapolated
    states, HLLC, first-order boundary faces, chemistry source) on the GPU
    against the oracle, with the GPU's own gradient and a seeded limiter."""
    from chem_cases import fr_records, fr_states
    from oracle_lib import OracleChemState
    from proteuscfd_gb300 import Mesh
    spec = mechanism()
    ns = len(spec["species"])
    m = Mesh.box(12, 9, 8, jitter=0.2, seed=9)
    nrows = m.nnode + m.nbedge
    ref, rhoi, vel, T = fr_states(nrows, seed=25)
    # a smooth field, so the extrapolated states stay physical
    x = np.r_[m.xyz, m.xyz[m.bedges[:, 0]]]
    s = np.sin(2.0 * x[:, 0] + 0.3) * np.cos(1.5 * x[:, 1])
    rhoi[:] = rhoi[0] * (1.0 + 0.05 * s[:, None])
    vel[:] = vel[0] * (1.0 + 0.1 * s[:, None])
    T[:] = T[0] * (1.0 + 0.05 * s)
    q = fr_records(ref, rhoi, vel, T)
    C = ChemModel(spec)
    C.attach_mesh(m)
    g = C.gradient(q)
    lim = np.random.default_rng(26).uniform(0.0, 1.0, size=(m.nnode, ns + 4))
    opts = C.flux_opts(1.0, 0.4, 0)
    for chi in (0.0, 0.5):
        b, norms = C.residual_ho(ref, opts, chi, 2.5e-4, 1, q, g, lim)
        bo, no = OracleChemState(model_struct(spec), ref).residual_ho(opts, m, q, g, lim, chi, 2.5e-4, 1)
        scale = np.abs(bo).max(axis=0, keepdims=True)
        assert (np.abs(b - bo) / scale).max() < 1e-11, (np.abs(b - bo) / scale).max()
        assert np.allclose(norms, no, rtol=1e-11, atol=0)
    C.close()


def test_fr_limiter_parity():
    """The reacting modified Venkatakrishnan limiter on the GPU against the
    oracle's edge-by-edge minimum, on seeded records with their gradient."""
    from chem_cases import fr_records, fr_states
    from oracle_lib import OracleChemState
    from proteuscfd_gb300 import Mesh
    spec = mechanism()
    m = Mesh.box(12, 9, 8, jitter=0.2, seed=10)
    nrows = m.nnode + m.nbedge
    ref, rhoi, vel, T = fr_states(nrows, seed=27)
    q = fr_records(ref, rhoi, vel, T)
    C = ChemModel(spec)
    C.attach_mesh(m)
    O = OracleChemState(model_struct(spec), ref)
    g = C.gradient(q)
    for chi in (0.0, 0.5):
        lim = C.limiter(chi, q, g)
        lo = O.limiter(m, q, g, chi)
        assert np.abs(lim - lo).max() < 1e-12, np.abs(lim - lo).max()
    C.close()
