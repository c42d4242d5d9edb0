"""GB300 (sm_103a) implementation of ProteusCFD's implicit edge-based
finite-volume hot path: CUDA kernels behind a C ABI (include/pcfd.h), with a
host-side mirror of the reference's operator interface in ``api``.

The native library ``libpcfd.so`` is loaded on first use; any use without it
raises ImportError (build it with ``python -m proteuscfd_gb300.build``).
There is no CPU fallback.
"""
from .api import Mesh, Param, SolutionSpace  # noqa: F401
from . import cases  # noqa: F401

__all__ = ["Mesh", "Param", "SolutionSpace", "cases"]
