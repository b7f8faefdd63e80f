"""Grids, seeded initial fields and host-side ghost fills for channel snapshots.

The reference builds its face grids in ``init_flow`` (input_output.f90:150-172)
or reads them from a snapshot (input_output.f90:231-384).  The channels this
package runs are 2*pi x 2 x pi by default with a tanh-stretched wall-normal
grid; they enter the solver exactly as a snapshot would, as face coordinates
x(nx), y(ny), z(nz).

Array layout everywhere (host and device) is the reference's Fortran layout:
U (nx, ny+1, nz+1), V (nx+1, ny, nz+1), W (nx+1, ny+1, nz),
P and nu_t (nx+1, ny+1, nz+1), column-major, ghosts and periodic duplicates
included.
"""
from __future__ import annotations

import math

import numpy as np


def face_grid_periodic(n_faces: int, length: float) -> np.ndarray:
    """Uniform periodic face grid: face 1 and face n-1 are one period apart,
    as in input_output.f90:150-158 (x(nx-1) - x(1) = L)."""
    nper = n_faces - 2
    return np.arange(n_faces, dtype=np.float64) * (length / nper)


def face_grid_wall(n_faces: int, stretch: float = 1.5, height: float = 2.0) -> np.ndarray:
    """Wall-normal faces on [0, height]; tanh clustering as in
    input_output.f90:160-172 (stretch <= 0 gives a uniform grid)."""
    y = np.arange(n_faces, dtype=np.float64) * 0.3
    y = 2.0 * y / y.max() - 1.0
    if stretch > 0:
        y = np.tanh(stretch * y) / math.tanh(stretch)
    y = y - y.min()
    y = y * height / y.max()
    return y


def channel_grid(nx: int, ny: int, nz: int, Lx: float = 2 * math.pi, Lz: float = math.pi,
                 stretch: float = 1.5):
    """Face grids for a channel of nx, ny, nz faces (input_parameters counts)."""
    return face_grid_periodic(nx, Lx), face_grid_wall(ny, stretch), face_grid_periodic(nz, Lz)


def centres(f: np.ndarray) -> np.ndarray:
    """Cell centres with one ghost each side (initialization.f90:169-195)."""
    m = 0.5 * (f[:-1] + f[1:])
    g = np.empty(len(f) + 1)
    g[1:-1] = m
    g[0] = m[0] - 2.0 * (m[0] - f[0])
    g[-1] = m[-1] + 2.0 * (f[-1] - m[-1])
    return g


def field_shapes(nx: int, ny: int, nz: int) -> dict:
    return dict(U=(nx, ny + 1, nz + 1), V=(nx + 1, ny, nz + 1), W=(nx + 1, ny + 1, nz),
                P=(nx + 1, ny + 1, nz + 1), nu_t=(nx + 1, ny + 1, nz + 1))


def apply_bcs_noslip(U: np.ndarray, V: np.ndarray, W: np.ndarray) -> None:
    """Host mirror of apply_boundary_conditions for iwall_model=0
    (boundary_conditions.f90:20-75): x/z periodic wraps, then no-slip walls.
    0-based: a Fortran index f is Python index f-1."""
    nx = U.shape[0]
    nxg = nx + 1
    nz = W.shape[2]
    nzg = nz + 1
    # periodic x: faces (U), centres (V, W)
    U[0] = U[nx - 2]; U[nx - 1] = U[1]
    for F in (V, W):
        F[0] = F[nxg - 3]; F[nxg - 2] = F[1]; F[nxg - 1] = F[2]
    # periodic z: centres (U, V), faces (W)
    for F in (U, V):
        a, b, c = F[:, :, nzg - 3].copy(), F[:, :, 1].copy(), F[:, :, 2].copy()
        F[:, :, 0] = a; F[:, :, nzg - 2] = b; F[:, :, nzg - 1] = c
    a, b = W[:, :, nz - 2].copy(), W[:, :, 1].copy()
    W[:, :, 0] = a; W[:, :, nz - 1] = b
    # walls
    U[:, 0, :] = -U[:, 1, :]; U[:, -1, :] = -U[:, -2, :]
    V[:, 0, :] = 0.0; V[:, -1, :] = 0.0
    W[:, 0, :] = -W[:, 1, :]; W[:, -1, :] = -W[:, -2, :]


def seeded_fields(x, y, z, seed: int = 1, amp: float = 0.1, profile: str = "laminar",
                  bulk: float = 1.0):
    """Perturbed initial velocity in the reference layout.

    profile 'laminar': U = 1.5*bulk*y(2-y) at the U centres; 'plug': U = bulk;
    'turbulent': the 1/7 power-law profile of bulk velocity `bulk` plus
    large-scale wall-vanishing Fourier modes (see turbulent_modes), a field
    that becomes turbulent within a few tens of time units.
    Uniform i.i.d. noise in [-amp, amp]*bulk on U, V, W (PCG64, seeded), then
    the periodic and no-slip ghost fills.  A projection (done by the solver)
    makes the field divergence-free."""
    nx, ny, nz = len(x), len(y), len(z)
    s = field_shapes(nx, ny, nz)
    rng = np.random.Generator(np.random.PCG64(seed))
    yg = centres(np.asarray(y))
    if profile == "laminar":
        prof = 1.5 * bulk * yg * (2.0 - yg)
    elif profile == "turbulent":
        eta = np.clip(1.0 - np.abs(1.0 - yg / (0.5 * (y[-1] - y[0]))), 0.0, 1.0)
        prof = bulk * (8.0 / 7.0) * eta ** (1.0 / 7.0)
    else:
        prof = np.full_like(yg, bulk)
    U = np.asfortranarray(np.broadcast_to(prof[None, :, None], s["U"]).copy())
    U += amp * bulk * (2.0 * rng.random(s["U"]) - 1.0)
    V = np.asfortranarray(amp * bulk * (2.0 * rng.random(s["V"]) - 1.0))
    W = np.asfortranarray(amp * bulk * (2.0 * rng.random(s["W"]) - 1.0))
    U = np.asfortranarray(U)
    if profile == "turbulent":
        dU, dV, dW = turbulent_modes(x, y, z, rng, bulk)
        U += dU; V += dV; W += dW
    apply_bcs_noslip(U, V, W)
    return U, V, W


def turbulent_modes(x, y, z, rng, bulk: float = 1.0, amp_u: float = 0.25, amp_vw: float = 0.12):
    """Large-scale perturbations that trip a channel into turbulence: a sum of
    Fourier modes with streamwise wavenumbers 0..3 and spanwise 1..4 (and
    oblique ones), random phases, wall-normal shape (1 - eta^2)^2 (eta the
    distance from the centre plane over the half height), so that every mode
    vanishes at both walls.  Streamwise rolls (kx = 0) in V, W lift up streaks
    in U; the oblique modes break them.  Returned on the U, V, W staggered
    positions; the projection that follows removes their divergence."""
    x, y, z = (np.asarray(a, dtype=np.float64) for a in (x, y, z))
    nx, ny, nz = len(x), len(y), len(z)
    Lx, Lz = x[nx - 2] - x[0], z[nz - 2] - z[0]
    h = 0.5 * (y[-1] - y[0])
    xg, yg, zg = centres(x), centres(y), centres(z)

    def shape(yy):
        eta = (yy - y[0]) / h - 1.0
        return np.where(np.abs(eta) < 1.0, (1.0 - eta * eta) ** 2, 0.0)

    modes = [(kx, kz) for kx in range(0, 4) for kz in range(1, 5)] + [(kx, 0) for kx in range(1, 4)]
    out = []
    for (xs, ys, zs), a in (((x, yg, zg), amp_u), ((xg, y, zg), amp_vw), ((xg, yg, z), amp_vw)):
        f = np.zeros((len(xs), len(ys), len(zs)))
        wy = shape(ys)
        for kx, kz in modes:
            c = rng.standard_normal() / math.sqrt(len(modes))
            ph = rng.random() * 2 * math.pi
            ax = 2 * math.pi * kx * (xs - x[0]) / Lx
            az = 2 * math.pi * kz * (zs - z[0]) / Lz
            f += c * np.cos(ax[:, None, None] + az[None, None, :] + ph) * wy[None, :, None]
        out.append(np.asfortranarray(a * bulk * f))
    return out


def dean_nu(retau: float) -> float:
    """Viscosity for bulk velocity 1 and half-height 1 from Dean's correlation
    Re_tau = 0.09 Re_b^0.88 with Re_b = 2 h U_b / nu."""
    re_b = (retau / 0.09) ** (1.0 / 0.88)
    return 2.0 / re_b
