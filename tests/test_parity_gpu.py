"""FP64 parity of the CUDA path (through the C ABI) against the CPU oracle.

Tolerances: per-routine results within 1e-12 (normwise relative); 10 RK3
steps within 1e-10 normwise and, for U, V and W, within 1e-10 pointwise
(|a-b| / max(|b|, 1e-4 max|b|) at every point: values of at least 1e-4 of
the field's largest to 1e-10 relative, smaller ones to 1e-14 of the largest
absolute), with max|div u| <= 1e-10 -- the FP64 gate of the reference-port
contract.  The pointwise error against a 1e-6 floor is printed beside it.
Bit-exact where the operation is a copy (boundary ghosts).
"""
import numpy as np
import pytest

from conftest import assert_close, assert_pointwise, channel_case, pointwise_rel_err, rel_err

pytestmark = pytest.mark.gpu


def make_pair(case, precision=0, **extra):
    from oracle import Oracle
    import channelflow as cf
    o = Oracle(case["x"], case["y"], case["z"], case["prm"])
    o.set_fields(case["U"], case["V"], case["W"])
    kw = dict(case["prm"])
    kw.update(extra)
    ch = cf.Channel(case["x"], case["y"], case["z"], precision=precision, **kw)
    ch.upload(case["U"], case["V"], case["W"])
    q0 = ch.init_mass_flow()
    o.init_mass_flow()
    # FP64: the same sums; split: the FP32 state (hi word) against FP64
    assert abs(q0 - o.scalar("Qflow_x_0")) <= (1e-14 if precision == 0 else 1e-7) * abs(q0)
    return o, ch


def compare_fields(o, ch, tol, names=("U", "V", "W"), what=""):
    g = ch.download()
    f = o.fields()
    errs = {}
    for n in names:
        errs[n] = assert_close(g[n], f[n], tol, f"{what} {n}")
    return errs


def compare_pointwise(o, ch, tol, names=("U", "V", "W"), report=("P", "nu_t"), what=""):
    """Pointwise relative errors (floor 1e-4 of each array's largest value):
    `names` within tol; `report` only reported (the pseudo-pressure
    P = phi/(dt 8/15) carries the cancellation of div u* = O(dt), so its
    values near zero have no meaningful relative error -- it is held to its
    normwise bound -- and nu_t the clipping max(., 0) next to zero)."""
    g = ch.download()
    f = o.fields()
    errs = {}
    for n in names:
        errs[n] = assert_pointwise(g[n], f[n], tol, f"{what} {n}")
        errs[n + "@1e-6"] = pointwise_rel_err(g[n], f[n], floor=1e-6)
    for n in report:
        errs[n] = pointwise_rel_err(g[n], f[n])
    return errs


CASES = {
    "small": (18, 17, 18),
    "config1": (66, 65, 66),
    "config2": (194, 129, 194),
}


@pytest.mark.parametrize("which", ["small"])
def test_boundary_conditions_exact(which):
    case = channel_case(*CASES[which])
    rng = np.random.default_rng(5)
    # raw (non-periodic) fields so that every ghost is rewritten
    for k in ("U", "V", "W"):
        case[k] = np.asfortranarray(rng.standard_normal(case[k].shape))
    o, ch = make_pair(case)
    o.apply_boundary_conditions()
    ch.apply_boundary_conditions()
    g, f = ch.download(), o.fields()
    for n in ("U", "V", "W"):
        assert np.array_equal(g[n], f[n]), n


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("dims,wall", [((34, 33, 34), 0), ((18, 17, 22), 0), ((66, 65, 66), 0), ((34, 33, 34), 3),
                                       ((26, 17, 22), 3)])
def test_step_ghosts_are_the_boundary_conditions(precision, dims, wall):
    """After graph-captured steps (the projection writes every ghost copy of
    its canonical cells instead of a separate apply_boundary_conditions: the
    no-slip rule, or with the equilibrium wall model its Neumann rule with
    alpha at each ghost; no mass-flow forcing in the wall-model cases, so that
    the step ends with the projection), the ghosts hold exactly what
    apply_boundary_conditions would put there: the fields do not change when
    it is applied once more (low words included in the split path)."""
    import channelflow as cf
    extra = dict(stretch=0.0, wall=3, retau=2000.0, profile="plug", mass=0) if wall else {}
    case = channel_case(*dims, seed=11, **extra)
    ch = cf.Channel(case["x"], case["y"], case["z"], precision=precision, **case["prm"])
    ch.upload(case["U"], case["V"], case["W"])
    ch.init_mass_flow()
    ch.apply_boundary_conditions()
    ch.set_fixed_dt(case["dt"])
    ch.time_step_rk3(3)
    a = ch.download()
    ch.apply_boundary_conditions()
    b = ch.download()
    for n in ("U", "V", "W"):
        assert np.array_equal(a[n], b[n]), n
    ch.close()


@pytest.mark.parametrize("which", ["small", "config1"])
def test_eddy_viscosity_and_rhs(which):
    case = channel_case(*CASES[which])
    o, ch = make_pair(case)
    for a in (o, ch):
        a.apply_boundary_conditions()
    o.set_scalar("dt", case["dt"])
    ch.set_scalars(dt=case["dt"])
    o.compute_eddy_viscosity()
    ch.compute_eddy_viscosity()
    f, g = o.fields(), ch.download()
    assert_close(g["nu_t"], f["nu_t"], 1e-12, "nu_t")
    assert_close(ch.avg_nu_t()[1:-1], o.array("avg_nu_t").ravel()[1:-1], 1e-12, "avg_nu_t")
    for s in (1,):
        o.compute_rhs_u(s); o.compute_rhs_v(s); o.compute_rhs_w(s)
        ch.compute_rhs_u(s); ch.compute_rhs_v(s); ch.compute_rhs_w(s)
        nx, ny, nz = ch.nx, ch.ny, ch.nz
        gu = ch.download_rhs(0, s)[1:nx - 1, 1:ny, 1:nz]
        gv = ch.download_rhs(1, s)[1:nx, 1:ny - 1, 1:nz]
        gw = ch.download_rhs(2, s)[1:nx, 1:ny, 1:nz - 1]
        assert_close(gu, o.array(f"Fu{s}"), 1e-12, "Fu")
        assert_close(gv, o.array(f"Fv{s}"), 1e-12, "Fv")
        assert_close(gw, o.array(f"Fw{s}"), 1e-12, "Fw")


@pytest.mark.parametrize("which", ["small", "config1"])
def test_projection(which):
    case = channel_case(*CASES[which])
    o, ch = make_pair(case)
    for a in (o, ch):
        a.apply_boundary_conditions()
    o.set_scalar("dt", case["dt"]); o.set_scalar("rk_step", 1)
    ch.set_scalars(dt=case["dt"], rk_step=1)
    o.compute_projection_step(); ch.compute_projection_step()
    o.apply_boundary_conditions(); ch.apply_boundary_conditions()
    compare_fields(o, ch, 1e-12, names=("U", "V", "W", "P"), what="projection")
    d, dabs = ch.check_divergence()
    assert dabs <= 1e-12, dabs
    od, odabs = o.check_divergence()
    assert abs(d - od) <= 1e-12


def test_dt_and_mass_flow():
    case = channel_case(*CASES["small"])
    case["prm"]["CFL"] = 0.5
    o, ch = make_pair(case)
    for a in (o, ch):
        a.apply_boundary_conditions()
    o.compute_dt()
    assert ch.compute_dt() == o.scalar("dt")
    assert abs(ch.compute_dPx_for_constant_mass_flow() - o.compute_dPx_for_constant_mass_flow()) <= 1e-15


@pytest.mark.parametrize("which", ["small", "config1"])
def test_wall_model_eqwm(which):
    """eqwm alphas, stress and counters, the boundary conditions they give,
    and then the eddy viscosity of that state, whose wall ghost rows are not
    periodic at the seams (the one-pass kernel with the seam band)."""
    case = channel_case(*CASES[which], stretch=0.0, wall=3, retau=2000.0, profile="plug", jref=3)
    o, ch = make_pair(case)
    for a in (o, ch):
        a.apply_boundary_conditions()
    o.compute_eddy_viscosity(); ch.compute_eddy_viscosity()
    o.compute_wall_model(); ch.compute_wall_model()
    w = ch.download_wall()
    assert_close(w["alpha_x"], o.array("alpha_x"), 1e-12, "alpha_x")
    assert_close(w["alpha_z"], o.array("alpha_z"), 1e-12, "alpha_z")
    assert_close(w["tau_eqwm_initial"], o.array("tau_eqwm_initial"), 1e-12, "tau")
    assert ch.eqwm_counters() == (int(o.scalar("n_nan_eqwm")), int(o.scalar("n_iter_eqwm")))
    o.apply_boundary_conditions(); ch.apply_boundary_conditions()
    compare_fields(o, ch, 1e-12, what="eqwm BC")
    o.compute_eddy_viscosity(); ch.compute_eddy_viscosity()
    assert_close(ch.download()["nu_t"], o.fields()["nu_t"], 1e-12, "nu_t after the eqwm BC")
    assert_close(ch.avg_nu_t()[1:-1], o.array("avg_nu_t").ravel()[1:-1], 1e-12, "avg_nu_t after the eqwm BC")


@pytest.mark.parametrize("which,wall", [("small", 0), ("config1", 0), ("small", 3)])
def test_ten_steps(which, wall):
    extra = dict(stretch=0.0, wall=3, retau=2000.0, profile="plug") if wall else {}
    case = channel_case(*CASES[which], **extra)
    o, ch = make_pair(case)
    for a in (o, ch):
        a.apply_boundary_conditions()
    o.set_scalar("dt", case["dt"]); o.set_scalar("rk_step", 2)
    ch.set_scalars(dt=case["dt"], rk_step=2)
    for a in (o, ch):
        a.compute_projection_step()
        a.apply_boundary_conditions()
    ch.set_fixed_dt(case["dt"])
    for _ in range(10):
        o.compute_dt()
        o.time_step_rk3()
    ch.time_step_rk3(10)
    errs = compare_fields(o, ch, 1e-10, names=("U", "V", "W", "P", "nu_t"), what="10 steps")
    perr = compare_pointwise(o, ch, 1e-10, what="10 steps")
    _, dabs = ch.check_divergence()
    assert dabs <= 1e-10, dabs
    # dPdx = (Q0 - Q)/dt is a cancellation: compare the correction Q0 - Q
    # against the mass flow it corrects
    assert abs(ch.scalars()["dPdx"] - o.scalar("dPdx")) * case["dt"] <= 1e-12 * abs(o.scalar("Qflow_x_0"))
    print(which, wall, "normwise", errs, "pointwise", perr)


def test_two_steps_config2():
    """The headline grid itself (Re_tau 550, 192 x 128 x 192 cells, faces
    194 129 194, tanh-stretched y, dynamic Smagorinsky), FP64 path against the
    oracle after two RK3 steps at the reference rule's dt = 5e-3: normwise
    and pointwise within 1e-10, max|div u| <= 1e-10."""
    case = channel_case(*CASES["config2"], retau=550.0, dt=5e-3)
    o, ch = make_pair(case)
    for a in (o, ch):
        a.apply_boundary_conditions()
    o.set_scalar("dt", case["dt"]); o.set_scalar("rk_step", 2)
    ch.set_scalars(dt=case["dt"], rk_step=2)
    for a in (o, ch):
        a.compute_projection_step()
        a.apply_boundary_conditions()
    ch.set_fixed_dt(case["dt"])
    for _ in range(2):
        o.compute_dt()
        o.time_step_rk3()
    ch.time_step_rk3(2)
    errs = compare_fields(o, ch, 1e-10, names=("U", "V", "W", "P", "nu_t"), what="config 2, 2 steps")
    perr = compare_pointwise(o, ch, 1e-10, what="config 2, 2 steps")
    _, dabs = ch.check_divergence()
    assert dabs <= 1e-10, dabs
    assert abs(ch.scalars()["dPdx"] - o.scalar("dPdx")) * case["dt"] <= 1e-12 * abs(o.scalar("Qflow_x_0"))
    print("config2 normwise", errs, "pointwise", perr)
    ch.close()
    o.close()


def test_mirror_matches_fast_path():
    import channelflow as cf
    case = channel_case(*CASES["small"])
    chs = []
    for mode in ("mirror", "fast"):
        ch = cf.Channel(case["x"], case["y"], case["z"], **case["prm"])
        ch.upload(case["U"], case["V"], case["W"])
        ch.init_mass_flow()
        ch.apply_boundary_conditions()
        ch.set_scalars(dt=case["dt"], rk_step=1)
        ch.set_fixed_dt(case["dt"])
        if mode == "mirror":
            for _ in range(2):
                ch.compute_dt()
                ch.compute_time_step_rk3_mirror()
        else:
            ch.time_step_rk3(2)
        chs.append(ch.download())
    for n in ("U", "V", "W", "nu_t"):
        assert_close(chs[0][n], chs[1][n], 1e-13, n)
    # P = phi/(dt*8/15) carries the cancellation of div(u*) = O(dt)
    assert_close(chs[0]["P"], chs[1]["P"], 1e-11, "P")


def test_split_precision_short_horizon():
    """FP32 state/stencils/SGS with the compensated update stays within 1e-4
    of the FP64 path over 20 steps (pointwise, normwise relative)."""
    import channelflow as cf
    case = channel_case(*CASES["config1"])
    out = []
    for prec in (0, 1):
        ch = cf.Channel(case["x"], case["y"], case["z"], precision=prec, **case["prm"])
        ch.upload(case["U"], case["V"], case["W"])
        ch.init_mass_flow()
        ch.apply_boundary_conditions()
        ch.set_fixed_dt(case["dt"])
        ch.time_step_rk3(20)
        out.append(ch.download())
    for n in ("U", "V", "W"):
        e = rel_err(out[1][n], out[0][n])
        assert e < 1e-4, (n, e)


@pytest.mark.parametrize("dims", [(66, 65, 66), (98, 65, 98), (34, 33, 130), (194, 129, 194), (18, 17, 258),
                                  (34, 33, 386), (18, 17, 514), (386, 17, 18), (514, 17, 34)])
def test_split_projection_matches_fp64(dims):
    """The split-path projection (FP32 transforms of 16-512 points, FP32 tridiagonal replays,
    the pivoting modes refined against the FP64 residual) against the FP64
    projection of the same fields: U, V, W within 1e-5 normwise relative,
    P within 1e-3, and the split result divergence-free to 1e-4 max|U|/dx."""
    import channelflow as cf
    case = channel_case(*dims, seed=7)
    out, div = [], []
    for prec in (cf.PREC_FP64, cf.PREC_SPLIT):
        ch = cf.Channel(case["x"], case["y"], case["z"], precision=prec, **case["prm"])
        ch.upload(case["U"], case["V"], case["W"])
        ch.apply_boundary_conditions()
        ch.set_scalars(0.0, case["dt"], 1)
        ch.compute_projection_step()
        ch.apply_boundary_conditions()
        out.append(ch.download())
        div.append(ch.check_divergence()[1])
        ch.close()
    for n in ("U", "V", "W"):
        assert_close(out[1][n], out[0][n], 1e-5, n)
    assert_close(out[1]["P"], out[0]["P"], 1e-3, "P")
    dx = case["x"][1] - case["x"][0]
    assert div[1] <= 1e-4 * np.max(np.abs(out[1]["U"])) / dx, div
    assert div[0] <= 1e-10 * np.max(np.abs(out[0]["U"])) / dx, div


@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (1, 2e-4)])
def test_dsm_fused_matches_multipass(precision, tol):
    """The one-pass dynamic Smagorinsky kernel (periodic state) against the
    multi-pass kernels on the same fields."""
    import channelflow as cf
    case = channel_case(*CASES["config1"])
    out = []
    for unfused in (0, 1):
        ch = cf.Channel(case["x"], case["y"], case["z"], precision=precision, dsm_unfused=unfused, **case["prm"])
        ch.upload(case["U"], case["V"], case["W"])
        ch.apply_boundary_conditions()
        ch.compute_eddy_viscosity()
        out.append((ch.download()["nu_t"], ch.avg_nu_t()))
    assert_close(out[0][0], out[1][0], tol, "nu_t")
    assert_close(out[0][1][1:-1], out[1][1][1:-1], tol, "avg_nu_t")


@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (1, 2e-4)])
@pytest.mark.parametrize("dims", [(18, 17, 18), (34, 33, 34), (102, 25, 74), (66, 65, 66)])
def test_dsm_fused_wall_model_matches_multipass(dims, precision, tol):
    """The one-pass dynamic Smagorinsky kernel on a wall-model state (the
    seam band computed by k_dsm_seam with the reference's readings of the
    non-periodic wall ghosts) against the multi-pass kernels, after an eqwm
    call and the boundary conditions it implies; the state's wall ghost rows
    are checked to differ from their periodic twins at the seams."""
    import channelflow as cf
    case = channel_case(*dims, seed=11, stretch=0.0, wall=3, retau=2000.0, profile="plug")
    out = []
    for unfused in (0, 1):
        ch = cf.Channel(case["x"], case["y"], case["z"], precision=precision, dsm_unfused=unfused, **case["prm"])
        ch.upload(case["U"], case["V"], case["W"])
        ch.apply_boundary_conditions()
        ch.compute_eddy_viscosity()
        ch.compute_wall_model()
        ch.apply_boundary_conditions()
        f = ch.download()
        # U's ghost column 1 and ghost plane 1 against their periodic twins, in the wall rows
        gap = max(np.abs(f["U"][0, [0, -1], :] - f["U"][-2, [0, -1], :]).max(),
                  np.abs(f["U"][:, [0, -1], 0] - f["U"][:, [0, -1], -3]).max())
        assert gap > 1e-12 * np.abs(f["U"]).max(), gap
        ch.compute_eddy_viscosity()
        out.append((ch.download()["nu_t"], ch.avg_nu_t()))
        ch.close()
    assert_close(out[0][0], out[1][0], tol, "nu_t")
    assert_close(out[0][1][1:-1], out[1][1][1:-1], tol, "avg_nu_t")


@pytest.mark.parametrize("dims,wall", [((66, 65, 66), 0), ((50, 33, 34), 0), ((42, 11, 18), 0), ((102, 17, 42), 3),
                                       ((194, 129, 194), 3)])
def test_dsm_tensor_copy_gather_matches_element_gather(dims, wall):
    """The FP32 multi-pass filter kernel with its tensor-copy (TMA) plane
    gather against the per-element gather (dsm_unfused 2), bit for bit in
    nu_t and avg_nu_t: nxp a multiple of 32 (64, 192), of 4 only (48, 100),
    the smallest box-sized plane (40 x 10), and the wall model's
    non-periodic ghost rows (after one wall-model call)."""
    import channelflow as cf
    extra = dict(stretch=0.0, wall=3, retau=2000.0, profile="plug") if wall else {}
    case = channel_case(*dims, seed=7, **extra)
    out = []
    for mode in (1, 2):
        ch = cf.Channel(case["x"], case["y"], case["z"], precision=cf.PREC_SPLIT, dsm_unfused=mode, **case["prm"])
        ch.upload(case["U"], case["V"], case["W"])
        ch.apply_boundary_conditions()
        ch.compute_eddy_viscosity()
        if wall:
            ch.compute_wall_model()
            ch.apply_boundary_conditions()
            ch.compute_eddy_viscosity()
        assert ch.copy_wait_expired() == 0
        out.append((ch.download()["nu_t"], ch.avg_nu_t()))
        ch.close()
    assert np.array_equal(out[0][0], out[1][0]), rel_err(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1]), rel_err(out[0][1], out[1][1])


def test_dsm_plane_copy_wait_expires():
    """A plane copy that never arrives (test hook: the first copy of every
    block is left out): the blocks' bounded waits expire, the eddy viscosity
    call reports it (CF_ERR_CUDA) and clears the count, and with the hook off
    the same context gives the nu_t of a clean one."""
    import channelflow as cf
    case = channel_case(66, 65, 66, seed=3)
    ref = None
    for hook in (False, True):
        ch = cf.Channel(case["x"], case["y"], case["z"], precision=cf.PREC_SPLIT, dsm_unfused=1, **case["prm"])
        ch.upload(case["U"], case["V"], case["W"])
        ch.apply_boundary_conditions()
        if hook:
            ch.test_skip_plane_copy(True)
            with pytest.raises(cf.CfError, match="plane copy"):
                ch.compute_eddy_viscosity()
            assert ch.copy_wait_expired() == 0  # cleared by the failed call
            ch.test_skip_plane_copy(False)
        ch.compute_eddy_viscosity()
        nut = ch.download()["nu_t"]
        ch.close()
        if ref is None:
            ref = nut
        else:
            assert np.array_equal(nut, ref)


def test_pinned_host_buffers_match_pageable():
    """Uploads and downloads through page-locked host arrays (converted by the
    kernels over the host link) give the same bits as pageable arrays
    (staged copies), in both precisions."""
    torch = pytest.importorskip("torch")
    import channelflow as cf
    case = channel_case(34, 33, 34, seed=4)
    for prec in (cf.PREC_SPLIT, cf.PREC_FP64):
        ch = cf.Channel(case["x"], case["y"], case["z"], precision=prec, **case["prm"])
        ch.upload(case["U"], case["V"], case["W"])
        ref = ch.download()
        pinned = {}
        for k in ("U", "V", "W"):
            shp = ch.shapes[k]
            t = torch.empty(int(np.prod(shp)), dtype=torch.float64, pin_memory=True)
            pinned[k] = t.numpy().reshape(shp, order="F")
            pinned[k][...] = case[k]
        ch.upload(pinned["U"], pinned["V"], pinned["W"])
        for k in ("U", "V", "W"):
            pinned[k][...] = np.nan
        ch.download_into(U=pinned["U"], V=pinned["V"], W=pinned["W"])
        for k in ("U", "V", "W"):
            assert np.array_equal(pinned[k], ref[k]), (prec, k)
        ch.close()


@pytest.mark.parametrize("which,wall,precision,tol", [("small", 0, 0, 1e-11), ("config1", 0, 0, 1e-11),
                                                       ("small", 3, 0, 1e-11), ("config1", 0, 1, 1e-4)])
def test_actual_pressure(which, wall, precision, tol):
    """compute_pressure (pressure.f90:21) on the fields left by a projection
    of rk_step 1: P everywhere, ghost columns included (those keep the
    projection's values on both sides).  The oracle follows the reference's
    boundary terms; the CUDA path drops the two that cancel."""
    extra = dict(stretch=0.0, wall=3, retau=2000.0, profile="plug") if wall else {}
    case = channel_case(*CASES[which], **extra)
    o, ch = make_pair(case, precision=precision)
    for a in (o, ch):
        a.apply_boundary_conditions()
    o.set_scalar("dt", case["dt"]); o.set_scalar("rk_step", 1)
    ch.set_scalars(dt=case["dt"], rk_step=1)
    o.compute_eddy_viscosity(); ch.compute_eddy_viscosity()
    if wall:
        o.compute_wall_model(); ch.compute_wall_model()
    o.compute_projection_step(); ch.compute_projection_step()
    o.apply_boundary_conditions(); ch.apply_boundary_conditions()
    o.compute_pressure(); ch.compute_pressure()
    g, f = ch.download(), o.fields()
    P0 = f["P"]
    # the wall rows carry the boundary condition: they must differ from the
    # first interior row, or the check of the ghost formula is empty
    assert abs(P0[1:-1, 0, 1:-1] - P0[1:-1, 1, 1:-1]).max() > 1e-6 * abs(P0).max()
    assert_close(g["P"], P0, tol, "P")
    # rows 1 and nyg alone, relative to the size of the wall jump
    for j0, j1 in ((0, 1), (-1, -2)):
        jg, jo = g["P"][1:-1, j0, 1:-1] - g["P"][1:-1, j1, 1:-1], P0[1:-1, j0, 1:-1] - P0[1:-1, j1, 1:-1]
        assert_close(jg, jo, max(tol, 1e-10) * 10, f"wall jump {j0}")


def test_statistics_and_text_file(tmp_path):
    """compute_statistics (statistics.f90:22-171) after five steps against the
    oracle, and the text file of output_statistics written from it."""
    import channelflow as cf
    case = channel_case(*CASES["config1"])
    o, ch = make_pair(case)
    for a in (o, ch):
        a.apply_boundary_conditions()
    ch.set_fixed_dt(case["dt"])
    for _ in range(5):
        o.compute_dt()
        o.time_step_rk3()
    ch.time_step_rk3(5)
    sg, so = ch.statistics(), o.statistics()
    ny = ch.ny
    for q in range(9):  # profiles, normwise
        assert_close(sg[q * ny:(q + 1) * ny], so[q * ny:(q + 1) * ny], 1e-11, f"profile {q}")
    assert_close(sg[9 * ny:], so[9 * ny:], 1e-9, "scalars")
    path = ch.output_statistics(str(tmp_path / "run"), istep=5, nstep_init=100)
    assert path.endswith("run.105.stats.txt")
    lines = open(path).read().split("\n")
    assert len(lines) == ny + 2 and lines[-1] == ""
    hdr = lines[0]
    assert hdr[0] == "%" and len(hdr) == 1 + 4 * 15 + 4 * 12
    assert [int(hdr[61 + 12 * q:73 + 12 * q]) for q in range(4)] == [ch.nx, ny, ch.nz, 5]
    assert abs(float(hdr[16:31]) - so[9 * ny + 1]) <= 1e-8  # Retau
    rows = np.array([[float(l[15 * c:15 * (c + 1)]) for c in range(7)] for l in lines[1:-1]])
    want = np.stack([o.array("y")] + [so[q * ny:(q + 1) * ny] for q in (0, 3, 4, 5, 6, 8)], axis=1)
    assert abs(rows - want).max() <= 5.1e-9


@pytest.mark.parametrize("which,dirichlet,wall", [("small", 0, 0), ("small", 1, 0), ("small", 2, 0),
                                                  ("config1", 0, 0), ("small", 0, 3)])
def test_eddy_viscosity_amd(which, dirichlet, wall):
    """sgs_AMD (subgrid.f90:639-881): nu_t everywhere (ghosts included) and the
    plane means avg_nu_t(2..nyg-1) against the oracle."""
    extra = dict(stretch=0.0, wall=3, retau=2000.0, profile="plug") if wall else {}
    case = channel_case(*CASES[which], les=3, **extra)
    case["prm"]["Dirichlet_nu_t"] = dirichlet
    o, ch = make_pair(case)
    for a in (o, ch):
        a.apply_boundary_conditions()
    o.compute_eddy_viscosity(); ch.compute_eddy_viscosity()
    assert o.scalar("amd_nan_canonical") == 0
    f, g = o.fields(), ch.download()
    assert_close(g["nu_t"], f["nu_t"], 1e-12, "nu_t")
    assert (f["nu_t"] > 0).mean() > 0.2
    assert_close(ch.avg_nu_t()[1:-1], o.array("avg_nu_t").ravel()[1:-1], 1e-12, "avg_nu_t")


@pytest.mark.parametrize("which,wall", [("small", 0), ("config1", 0), ("small", 3)])
def test_ten_steps_amd(which, wall):
    """Ten RK3 steps with the AMD model, fast path against the oracle."""
    extra = dict(stretch=0.0, wall=3, retau=2000.0, profile="plug") if wall else {}
    case = channel_case(*CASES[which], les=3, **extra)
    o, ch = make_pair(case)
    for a in (o, ch):
        a.apply_boundary_conditions()
    ch.set_fixed_dt(case["dt"])
    for _ in range(10):
        o.compute_dt()
        o.time_step_rk3()
    ch.time_step_rk3(10)
    errs = compare_fields(o, ch, 1e-10, names=("U", "V", "W", "P", "nu_t"), what="10 AMD steps")
    perr = compare_pointwise(o, ch, 1e-10, what="10 AMD steps")
    _, dabs = ch.check_divergence()
    assert dabs <= 1e-10, dabs
    print(which, wall, "normwise", errs, "pointwise", perr)


def test_amd_split_precision_short_horizon():
    """AMD in the split (FP32 + compensated state) path against FP64 after ten
    steps."""
    import channelflow as cf
    case = channel_case(*CASES["config1"], les=3)
    out = []
    for prec in (cf.PREC_FP64, cf.PREC_SPLIT):
        ch = cf.Channel(case["x"], case["y"], case["z"], precision=prec, **case["prm"])
        ch.upload(case["U"], case["V"], case["W"])
        ch.init_mass_flow()
        ch.apply_boundary_conditions()
        ch.set_fixed_dt(case["dt"])
        ch.time_step_rk3(10)
        out.append(ch.download())
        ch.close()
    for n in ("U", "V", "W", "nu_t"):
        e = rel_err(out[1][n], out[0][n])
        assert e < (1e-4 if n != "nu_t" else 1e-3), (n, e)


def test_monitor_reductions(capsys):
    """output_monitor (monitor.f90:20-150) after five steps: means to
    round-off, maxima exactly, and the printed block."""
    case = channel_case(*CASES["config1"])
    o, ch = make_pair(case)
    for a in (o, ch):
        a.apply_boundary_conditions()
    ch.set_fixed_dt(case["dt"])
    for _ in range(5):
        o.compute_dt()
        o.time_step_rk3()
    ch.time_step_rk3(5)
    mo = o.output_monitor()
    mg = ch.output_monitor(5)
    g = [mg[k] for k in ("meanU", "meanV", "meanW", "maxU", "maxV", "maxW", "meanNut", "maxNut", "max_divergence")]
    for q in (0, 1, 2, 6):
        assert abs(g[q] - mo[q]) <= 1e-12 * max(abs(mo[q]), 1e-3), (q, g[q], mo[q])
    f = o.fields()
    for q, n in ((3, "U"), (4, "V"), (5, "W"), (7, "nu_t")):
        assert abs(g[q] - mo[q]) <= 1e-10 * abs(f[n]).max(), (q, g[q], mo[q])
    assert abs(g[8] - mo[8]) <= 1e-10
    text = capsys.readouterr().out
    assert "Maximum nu_t:" in text and "Maximum divergence" in text and "step number :5" in text
    assert ch.scalars()["t"] == o.scalar("t") > 0  # t = to + dt per step, summed alike


@pytest.mark.parametrize("precision,tol", [(0, 1e-15), (1, 1e-6)])
def test_corrected_cfl_option(precision, tol):
    """cfl_corrected = 1: dt = min(CFL min over cells of spacing/|u|, the
    viscous limit, 5e-3), computed here with numpy on the same fields with
    the ranges of time_integration.f90:191-197; the default keeps the
    reference's rule (viscous limit or cap)."""
    import channelflow as cf
    case = channel_case(*CASES["config1"])
    ch0 = cf.Channel(case["x"], case["y"], case["z"], precision=precision, **dict(case["prm"], CFL=0.5))
    ch0.upload(case["U"], case["V"], case["W"])
    ch0.apply_boundary_conditions()
    dt_ref = ch0.compute_dt()
    g = ch0.download()
    ch0.close()
    xg = np.r_[np.nan, grids_centres(case["x"])]
    yg = np.r_[np.nan, grids_centres(case["y"])]
    zg = np.r_[np.nan, grids_centres(case["z"])]
    nx, ny, nz = len(case["x"]), len(case["y"]), len(case["z"])
    nxg, nyg, nzg = nx + 1, ny + 1, nz + 1

    def conv(U, V, W):
        with np.errstate(divide="ignore"):
            lu = ((xg[3:nxg + 1] - xg[2:nxg])[:, None, None] / np.abs(U[1:nxg - 1, 1:nyg - 1, 1:nzg - 1])).min()
            lv = ((yg[3:nyg + 1] - yg[2:nyg])[None, :, None] / np.abs(V[1:nxg - 1, 1:nyg - 1, 1:nzg - 1])).min()
            lw = ((zg[3:nzg + 1] - zg[2:nzg])[None, None, :] / np.abs(W[1:nxg - 1, 1:nyg - 1, 1:nzg - 1])).min()
        return 0.5 * min(lu, lv, lw)

    scale = conv(g["U"], g["V"], g["W"]) / (0.5 * dt_ref)  # convective limit at half the reference's dt
    U, V, W = (case[k] * scale for k in ("U", "V", "W"))
    ch = cf.Channel(case["x"], case["y"], case["z"], precision=precision, **dict(case["prm"], CFL=0.5, cfl_corrected=1))
    ch.upload(U, V, W)
    ch.apply_boundary_conditions()
    for _ in range(2):  # the second call checks the reset of the per-index maxima
        dt = ch.compute_dt()
        f = ch.download()
        want = min(conv(f["U"], f["V"], f["W"]), dt_ref)
        assert abs(dt - want) <= tol * want, (dt, want)
    assert dt < 0.6 * dt_ref
    ch.close()


def grids_centres(f):
    """Ghost-extended centre grid of initialization.f90:169-195 (nf + 1 values)."""
    from channelflow import grids
    return grids.centres(np.asarray(f))


@pytest.mark.parametrize("batched,stencils", [(False, False), (True, False), (False, True), (True, True)])
def test_ensemble_members_match_single_runs(batched, stencils):
    """Four channels of different grids, models and wall treatments advanced
    as one ensemble give bit for bit the fields of each advanced alone, with
    their fused DSM passes and right-hand sides in member branches or as one
    launch over all members (stencils) -- the split-path members of the
    batched stencil launches to within 1e-6 in U, V, W (measured 1e-11 to
    1e-9: the batched kernel's FP32 contractions; P, which carries the
    cancellation of div u*, and nu_t as below); with the batched FP64 tridiagonal
    solve the FP64 members still do (the same replay), the split-path members
    agree to the precision of their FP32 solves."""
    import channelflow as cf
    specs = [dict(dims=(18, 17, 18), seed=3), dict(dims=(34, 33, 26), seed=4, les=3),
             dict(dims=(26, 17, 22), seed=5, stretch=0.0, wall=3, retau=2000.0, profile="plug"),
             dict(dims=(42, 25, 34), seed=6)]
    cases = []
    for sp in specs:
        kw = {k: v for k, v in sp.items() if k not in ("dims",)}
        cases.append(channel_case(*sp["dims"], **kw))

    def make(case, prec):
        ch = cf.Channel(case["x"], case["y"], case["z"], precision=prec, **case["prm"])
        ch.upload(case["U"], case["V"], case["W"])
        ch.init_mass_flow()
        ch.apply_boundary_conditions()
        ch.set_fixed_dt(case["dt"])
        return ch

    for prec in (cf.PREC_FP64, cf.PREC_SPLIT):
        alone = []
        for case in cases:
            ch = make(case, prec)
            ch.time_step_rk3(6)
            alone.append(ch.download())
            ch.close()
        members = [make(case, prec) for case in cases]
        ens = cf.Ensemble(members, batched_tri=batched, batched_stencils=stencils)
        ens.step(2)
        ens.step(4)
        assert ens.launches_per_step() > 3 * 20
        for m, ref in zip(members, alone):
            got = m.download()
            for n in ("U", "V", "W", "P", "nu_t"):
                if prec == cf.PREC_FP64 or not (batched or stencils):
                    assert np.array_equal(got[n], ref[n]), (prec, n)
                elif not batched and n in ("U", "V", "W"):
                    # the batched stencil kernels compile the same FP32 arithmetic
                    # with their own contraction choices: rounding-level changes
                    # (the compensated state keeps them near 1e-9)
                    assert rel_err(got[n], ref[n]) < 1e-6, (prec, n, rel_err(got[n], ref[n]))
                else:  # the pseudo-pressure carries the FP32 solve's error directly
                    tol = {"P": 2e-3, "nu_t": 1e-4}.get(n, 1e-5)
                    assert rel_err(got[n], ref[n]) < tol, (prec, n, rel_err(got[n], ref[n]))
        ens.close()
        for m in members:
            m.close()


@pytest.mark.parametrize("les", [2, 3])
def test_autotune_keeps_the_state(les):
    """cf_autotune on a running channel: the chosen chunk counts are
    admissible, the timed launches leave the state as it was, and the run
    continues to the same fields up to the order of the plane sums."""
    import channelflow as cf
    case = channel_case(*CASES["config1"], les=les)
    runs = []
    for tune in (False, True):
        ch = cf.Channel(case["x"], case["y"], case["z"], precision=cf.PREC_FP64, **case["prm"])
        ch.upload(case["U"], case["V"], case["W"])
        ch.init_mass_flow()
        ch.apply_boundary_conditions()
        ch.set_fixed_dt(case["dt"])
        ch.time_step_rk3(2)
        if tune:
            before = ch.download()
            rep = ch.autotune(reps=2)
            after = ch.download()
            for n in ("U", "V", "W"):
                assert np.array_equal(before[n], after[n]), n
            assert rep["rhs_chunks"] >= 1 and rep["rhs_us"] > 0
            if les == 2:
                assert 1 <= rep["dsm_chunk_len"] <= 64 and rep["dsm_us"] > 0
            else:
                assert rep["amd_chunks"] >= 1 and rep["amd_us"] > 0
        ch.time_step_rk3(3)
        runs.append(ch.download())
        ch.close()
    for n in ("U", "V", "W", "nu_t"):
        assert rel_err(runs[1][n], runs[0][n]) < 1e-12, n


def test_ensemble_autotune_keeps_a_valid_choice():
    """cf_ensemble_autotune times every candidate and keeps the fastest; the
    ensemble then still advances its members as single runs would (FP64: to
    the order of the DSM plane sums, which the candidates' z chunks change)."""
    import channelflow as cf
    specs = [dict(dims=(18, 17, 18), seed=3), dict(dims=(34, 25, 26), seed=4)]
    cases = [channel_case(*sp["dims"], seed=sp["seed"]) for sp in specs]

    def make(case):
        ch = cf.Channel(case["x"], case["y"], case["z"], precision=cf.PREC_FP64, **case["prm"])
        ch.upload(case["U"], case["V"], case["W"])
        ch.init_mass_flow()
        ch.apply_boundary_conditions()
        ch.set_fixed_dt(case["dt"])
        return ch

    members = [make(c) for c in cases]
    ens = cf.Ensemble(members)
    ens.step(1)
    rep = ens.autotune(steps=2)
    assert rep["choice"] in rep["ms_per_step"] and all(v > 0 for v in rep["ms_per_step"].values())
    ens.step(3)
    done = 1 + cf.ENS_TUNE_CANDIDATES * 3 + 3
    for m, case in zip(members, cases):
        ref = make(case)
        ref.time_step_rk3(done)
        a, b = m.download(), ref.download()
        for n in ("U", "V", "W", "nu_t"):
            assert rel_err(a[n], b[n]) < 1e-11, (n, rel_err(a[n], b[n]))
        ref.close()
    ens.close()
    for m in members:
        m.close()
