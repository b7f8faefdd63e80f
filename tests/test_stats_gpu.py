"""Long-run statistics of the split path against the FP64 path on developed
turbulence (the accuracy gate of the split-precision form): a 64 x 64 x 64
Re_tau 180 channel (dynamic Smagorinsky, no-slip, constant mass flow) is
developed from the turbulent initial field with the split path, then the FP64
and split paths advance the same developed field 2000 steps each, and the
time averages of compute_statistics (statistics.f90:43-118) over the last
1000 steps are compared: mean U+, u, v, w RMS and the uv Reynolds stress
within 1 % (max|split - FP64| / max|FP64| per profile).  The developed state
is checked to be turbulent (Re_tau near 180, wall-normal and Reynolds-stress
fluctuations of the turbulent size) so that the gate is not met trivially by
a laminar flow."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DEVELOP, STEPS, EVERY = 12000, 2000, 10


def _channel(x, y, z, fields, precision, prm, dPdx=None):
    import channelflow as cf
    ch = cf.Channel(x, y, z, precision=precision, **prm)
    ch.upload(*fields)
    ch.init_mass_flow()
    ch.apply_boundary_conditions()
    if dPdx is not None:
        ch.set_scalars(dt=5e-3, rk_step=1, dPdx=dPdx)
    return ch


def _averaged(ch, ny):
    acc, tail, n, done = np.zeros(9 * ny), np.zeros(8), 0, 0
    while done < STEPS:
        ch.time_step_rk3(EVERY)
        done += EVERY
        if done > STEPS // 2:
            s = ch.statistics()
            acc += s[:9 * ny]
            tail += s[9 * ny:]
            n += 1
    m, t = acc / n, tail / n
    U, V, W, U2, V2, W2, UV = (m[q * ny:(q + 1) * ny] for q in range(7))
    return dict(Uplus=U / t[0], urms=np.sqrt(np.maximum(U2 - U * U, 0)), vrms=np.sqrt(np.maximum(V2 - V * V, 0)),
                wrms=np.sqrt(np.maximum(W2 - W * W, 0)), uv=UV - U * V, utau=t[0], retau=t[1])


def test_split_statistics_on_developed_turbulence():
    import channelflow as cf
    from channelflow import grids
    nx, ny, nz = 66, 65, 66
    x, y, z = grids.channel_grid(nx, ny, nz, stretch=1.5)
    nu = grids.dean_nu(180.0)
    prm = dict(nu=nu, CFL=0.5, dPdx=(180.0 * nu) ** 2, LES_model=2, iwall_model=0, x_mass_cte=1)
    U, V, W = grids.seeded_fields(x, y, z, seed=11, profile="turbulent")
    dev = _channel(x, y, z, (U, V, W), cf.PREC_SPLIT, prm)
    dev.set_scalars(dt=5e-3, rk_step=2)
    dev.compute_projection_step()
    dev.apply_boundary_conditions()
    dev.time_step_rk3(DEVELOP)
    f, dPdx = dev.download(), dev.scalars()["dPdx"]
    dev.close()
    out = {}
    for name, prec in (("fp64", cf.PREC_FP64), ("split", cf.PREC_SPLIT)):
        ch = _channel(x, y, z, (f["U"], f["V"], f["W"]), prec, prm, dPdx=dPdx)
        out[name] = _averaged(ch, ny)
        assert np.isfinite(ch.download()["U"]).all()
        ch.close()
    b = out["fp64"]
    # developed turbulence, not a laminar or transitional flow
    assert 150.0 < b["retau"] < 210.0, b["retau"]
    assert 2.0 < b["urms"].max() / b["utau"] < 3.5
    assert 0.6 < b["vrms"].max() / b["utau"] < 1.3
    assert 0.5 < np.abs(b["uv"]).max() / b["utau"] ** 2 < 1.0
    errs = {k: float(np.max(np.abs(out["split"][k] - b[k])) / np.max(np.abs(b[k])))
            for k in ("Uplus", "urms", "vrms", "wrms", "uv")}
    print("Re_tau", b["retau"], "errors", errs)
    for k, e in errs.items():
        assert e <= 1e-2, (k, e)
