"""Shared comparison helpers for the GPU-versus-oracle parity tests."""
import numpy as np

# One FP64 residual must match within 1e-12 relative per component.  The
# residual is a sum of face fluxes that cancel, so "relative" is taken
# against the sum of the magnitudes of the terms added into each entry
# (the oracle reports it), floored at 1e-3 of the largest such sum.
RESIDUAL_RTOL = 1e-12
FIELD_RTOL = 1e-12


def assert_residual_close(b_gpu, b_ref, babs, rtol=RESIDUAL_RTOL):
    scale = np.maximum(babs, 1e-3 * babs.max(axis=0, keepdims=True))
    err = np.abs(b_gpu - b_ref) / scale
    worst = np.unravel_index(np.argmax(err), err.shape)
    assert err.max() <= rtol, "residual mismatch %.3e at %s: gpu %r ref %r scale %r" % (
        err.max(), worst, b_gpu[worst], b_ref[worst], scale[worst])


def assert_field_close(x_gpu, x_ref, rtol=FIELD_RTOL, what="field"):
    """Per column, relative to the column's largest magnitude."""
    x_gpu = np.asarray(x_gpu).reshape(len(x_ref), -1)
    x_ref = np.asarray(x_ref).reshape(len(x_ref), -1)
    scale = np.maximum(np.abs(x_ref).max(axis=0, keepdims=True), 1e-300)
    err = np.abs(x_gpu - x_ref) / scale
    worst = np.unravel_index(np.argmax(err), err.shape)
    assert err.max() <= rtol, "%s mismatch %.3e at %s: gpu %r ref %r" % (
        what, err.max(), worst, x_gpu[worst], x_ref[worst])
