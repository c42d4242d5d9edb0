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
