"""Shared inputs of the chemistry tests: the 5-species air mechanism and
seeded thermochemical states."""
from pathlib import Path

import numpy as np

from proteuscfd_gb300.chem import load_mechanism

FIXTURE = Path(__file__).resolve().parent / "golden" / "chem_5species_air.json"
# atoms of N and O per molecule, by species name
ATOMS = {"N": (1, 0), "O": (0, 1), "N2": (2, 0), "O2": (0, 2), "NO": (1, 1)}


def mechanism():
    return load_mechanism(FIXTURE)


def states(n, seed=1, tmin=150.0, tmax=9000.0):
    """Densities log-uniform over 1e-8..1e-1 kg/m^3 per species and
    temperatures spanning both curve fits and both pinned ranges."""
    rng = np.random.default_rng(seed)
    spec = mechanism()
    ns = len(spec["species"])
    rho = 10.0 ** rng.uniform(-8, -1, size=(n, ns))
    T = rng.uniform(tmin, tmax, size=n)
    T[: min(n, 8)] = [150.0, 199.0, 200.0, 999.0, 1000.0, 1001.0, 6000.0, 7500.0][: min(n, 8)]
    return rho, T


def conservation(spec, w):
    """Relative mass and element imbalance of production rates w [n][ns]."""
    mw = np.array([s["MW"] for s in spec["species"]])
    names = [s["name"] for s in spec["species"]]
    scale = np.abs(w).sum(axis=1) + 1e-300
    mass = np.abs(w.sum(axis=1)) / scale
    mol = w / mw
    elem = []
    for e in range(2):
        a = np.array([ATOMS[nm][e] for nm in names])
        elem.append(np.abs((mol * a).sum(axis=1)) / ((np.abs(mol) * a).sum(axis=1) + 1e-300))
    return mass.max(), max(x.max() for x in elem)


def reference_scales():
    """Reference scales in the reference's style (ucs/param.tcc:372-397):
    air at 300 K and 101325 Pa, velocity = speed of sound, density =
    p / velocity^2, specific enthalpy = velocity^2."""
    from proteuscfd_gb300.chem import ChemModel
    v = (1.4 * 287.0 * 300.0) ** 0.5
    return ChemModel.ref(101325.0 / v ** 2, 101325.0, 300.0 / 1.4, v * v, v)


def fr_states(n, seed=2):
    """Non-dimensional reacting node states: species densities, velocities,
    T from 250 to 6000 K (scaled), and the pressure aux variable."""
    rng = np.random.default_rng(seed)
    ref = reference_scales()
    ns = len(mechanism()["species"])
    rhoi = (10.0 ** rng.uniform(-4, 0, size=(n, ns))) / ref.density
    vel = rng.normal(size=(n, 3)) * 0.5
    T = rng.uniform(250.0, 6000.0, size=n) / ref.temperature
    return ref, rhoi, vel, T


def fr_edges(nnode, nedge, seed=3):
    """Random node pairs with unit normals and areas."""
    rng = np.random.default_rng(seed)
    e = rng.integers(0, nnode, size=(nedge, 2)).astype(np.int32)
    nrm = rng.normal(size=(nedge, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    return e, np.c_[nrm, rng.uniform(0.1, 2.0, size=nedge)]


def fr_records(ref, rhoi, vel, T):
    """Node records through the oracle's ComputeAuxiliaryVariables."""
    from oracle_lib import OracleChemState
    from proteuscfd_gb300.chem import model_struct
    P, cvi, mol = OracleChemState(model_struct(mechanism()), ref).aux(rhoi, T)
    return np.ascontiguousarray(np.c_[rhoi, vel, T, P, rhoi.sum(axis=1), cvi, mol])
