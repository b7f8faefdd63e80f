import math
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "channel-flow_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def rel_err(a, b):
    """max|a-b| / max|b| (normwise relative error of one array)."""
    dt = np.complex128 if (np.iscomplexobj(a) or np.iscomplexobj(b)) else np.float64
    a = np.asarray(a, dtype=dt)
    b = np.asarray(b, dtype=dt)
    den = np.max(np.abs(b))
    if den == 0:
        return float(np.max(np.abs(a - b)))
    return float(np.max(np.abs(a - b)) / den)


def assert_close(a, b, tol, what=""):
    e = rel_err(a, b)
    assert e <= tol, f"{what}: relative error {e:.3e} > {tol:.1e}"
    return e


def pointwise_rel_err(a, b, floor=1e-4):
    """max over points of |a-b| / max(|b|, floor*max|b|): the relative error
    of every value, values below `floor` of the array's largest measured
    against that floor (an exact zero has no relative error).  With the
    default floor a 1e-10 bound holds every value of magnitude >= 1e-4 max|b|
    to 1e-10 relative and every smaller one (zero crossings, wall values) to
    1e-14 max|b| absolute."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.maximum(np.abs(b), floor * np.max(np.abs(b)))
    if not np.any(den > 0):
        return float(np.max(np.abs(a - b)))
    den = np.where(den > 0, den, 1.0)
    return float(np.max(np.abs(a - b) / den))


def assert_pointwise(a, b, tol, what="", floor=1e-4):
    e = pointwise_rel_err(a, b, floor)
    assert e <= tol, f"{what}: pointwise relative error {e:.3e} > {tol:.1e} (floor {floor:.0e} of max)"
    return e


def channel_case(nx, ny, nz, retau=180.0, stretch=1.5, les=2, wall=0, dt=2e-3, seed=1, mass=1, jref=3,
                 profile="laminar", ncv=100):
    """A seeded channel: face grids, oracle/library parameter dicts, fields."""
    from channelflow import grids
    x, y, z = grids.channel_grid(nx, ny, nz, stretch=stretch)
    nu = grids.dean_nu(retau)
    U, V, W = grids.seeded_fields(x, y, z, seed=seed, profile=profile)
    prm = dict(nu=nu, CFL=-dt, dPdx=(retau * nu) ** 2, LES_model=les, iwall_model=wall, x_mass_cte=mass,
               jref_eqwm=jref, eqwm_ncv=ncv, eqwm_stretch=1.10)
    return dict(x=x, y=y, z=z, U=U, V=V, W=W, prm=prm, dt=dt)


@pytest.fixture(scope="session")
def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
