"""Synthetic workloads: the meshes, boundary conditions and physics of the
three ideal-gas cases this path is measured on, at full size or scaled down
for tests.

Boundary tags of the generated box: 1 x=0, 2 x=max, 3 y=0, 4 y=max, 5 z=0,
6 z=max, and 7 for the part of y=0 ahead of a wall's leading edge.  Values are the reference's non-dimensional ones (velocity scale =
freestream speed of sound, p_inf = 1, rho_inf = gamma).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import _native as N
from .api import Mesh, Param


@dataclass
class Case:
    name: str
    nx: int
    ny: int
    nz: int
    mesh_kw: dict
    param: Param


def euler_ramp(nx=64, ny=32, nz=32, seed=1):
    """Mach 2 Euler over a 15 degree ramp: first-order Roe, supersonic inflow
    and outflow, slip walls at y=0/1, symmetry at z=0/1; box [0,2]x[0,1]x[0,1]."""
    p = Param(gamma=1.4, mach=2.0, sorder=1, viscous=0, limiter=0,
              bc_type={1: N.BC_SONIC_INFLOW, 2: N.BC_SONIC_OUTFLOW, 3: N.BC_IMPERMEABLE_WALL,
                       4: N.BC_IMPERMEABLE_WALL, 5: N.BC_SYMMETRY, 6: N.BC_SYMMETRY})
    kw = dict(lx=2.0, ly=1.0, lz=1.0, jitter=0.2, seed=seed, ramp_deg=15.0, ramp_x0=0.5, y_ratio=1.0)
    return Case("euler_ramp_%dx%dx%d" % (nx, ny, nz), nx, ny, nz, kw, p)


def ns_flatplate(nx=128, ny=96, nz=96, seed=2, venkat_K=1.0):
    """Mach 0.8 laminar Navier-Stokes, Re 1e5 on unit length, Pr 0.72,
    Sutherland viscosity; second order with LSQ gradients and the modified
    Venkatakrishnan limiter; adiabatic no-slip wall at y=0 with geometric
    y-clustering (ratio 1.1), far field at x=0, x=max and y=max, symmetry
    at z=0/1.  Box [0,(nx-1)/(ny-1)]x[0,1]x[0,1].

    The limiter constant defaults to the reference's: Kernel_VenkatMod
    hard-codes K = 1 (ucs/limiters.tcc:563) whatever the case asks for;
    venkat_K=5 runs the K = 5 variant.

    Three choices make the family one the reference's method converges on:
    * the jitter moves each interior node by up to 0.2 of its smallest local
      spacing on every axis (jittering each axis by that axis's spacing moves
      the first wall layer by ~50 wall-normal spacings at 128x96x96 and
      leaves near-wall LSQ systems with condition numbers up to 7e5);
    * the first wall cell is at least 1/50 of the x spacing high (a single
      geometric series with ratio 1.1 over the whole height makes it
      1/900 at 128x96x96 and 1/1,000,000 at 256x176x176); the spacing grows
      by 1.1 from there and stops growing at the spacing that fills the box;
    * the wall starts at x = (nx-ny)/(ny-1), so the plate is one unit long
      (the Reynolds number's length), behind a symmetry run-in (tag 7) that
      keeps its leading edge off the far-field inflow boundary.
    """
    p = Param(gamma=1.4, mach=0.8, Re=1.0e5, Pr=0.72, PrT=0.85, ref_temperature=300.0,
              sorder=2, chi=0.0, viscous=1, limiter=3, venkat_K=venkat_K,
              bc_type={1: N.BC_FARFIELD, 2: N.BC_FARFIELD, 3: N.BC_NOSLIP, 4: N.BC_FARFIELD,
                       5: N.BC_SYMMETRY, 6: N.BC_SYMMETRY, 7: N.BC_SYMMETRY},
              bc_twall={3: -1.0})
    kw = dict(lx=(nx - 1) / (ny - 1), ly=1.0, lz=1.0, jitter=0.2, seed=seed, ramp_deg=0.0, y_ratio=1.1,
              jitter_mode=1, wall_start_i=nx - ny if nx > ny else (nx - 1) // 4, upstream_tag=7,
              wall_ar_max=50.0)
    return Case("ns_flatplate_%dx%dx%d" % (nx, ny, nz), nx, ny, nz, kw, p)


def build_mesh(case: Case) -> Mesh:
    return Mesh.box(case.nx, case.ny, case.nz, **case.mesh_kw)


def perturbed_state(qinf: np.ndarray, nrows: int, seed: int, amp: float = 0.01, gamma: float = 1.4) -> np.ndarray:
    """Freestream times (1 + U[-amp, amp]) per conserved component, with the
    auxiliary variables recomputed - the seeded initial state of the cases."""
    rng = np.random.default_rng(seed)
    q = np.tile(qinf, (nrows, 1))
    q[:, :5] *= 1.0 + rng.uniform(-amp, amp, size=(nrows, 5))
    return with_aux(q, gamma)


def with_aux(q: np.ndarray, gamma: float = 1.4) -> np.ndarray:
    """ComputeAuxiliaryVariables (ucs/compressible.tcc:1230) on every row."""
    q = np.array(q, dtype=np.float64, copy=True)
    u = q[:, 1] / q[:, 0]
    v = q[:, 2] / q[:, 0]
    w = q[:, 3] / q[:, 0]
    P = (gamma - 1.0) * (q[:, 4] - 0.5 * q[:, 0] * (u * u + v * v + w * w))
    q[:, 6] = P
    q[:, 5] = gamma * P / q[:, 0]
    q[:, 7], q[:, 8], q[:, 9] = u, v, w
    return q


def smooth_state(mesh: Mesh, qinf: np.ndarray, nrows: int, amp: float = 0.05, gamma: float = 1.4) -> np.ndarray:
    """A smooth, non-uniform state (sinusoidal modulation of the freestream)
    so gradients, limiters and viscous terms are all active."""
    q = np.tile(qinf, (nrows, 1))
    x = mesh.xyz
    n = mesh.nnode
    s = np.sin(2.1 * x[:, 0] + 0.3) * np.cos(1.7 * x[:, 1] - 0.2) * np.sin(1.3 * x[:, 2] + 0.5)
    q[:n, 0] *= 1.0 + amp * s
    q[:n, 1] *= 1.0 + amp * np.cos(1.9 * x[:, 1])
    q[:n, 2] += amp * qinf[0] * 0.3 * np.sin(2.3 * x[:, 0])
    q[:n, 3] += amp * qinf[0] * 0.2 * np.cos(1.1 * x[:, 2] + x[:, 0])
    q[:n, 4] *= 1.0 + 0.5 * amp * s
    return with_aux(q, gamma)
