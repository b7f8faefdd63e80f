"""CPU tests of the oracle: its third-party arithmetic pinned to numpy/scipy
(FFTW's DFT, LAPACK zgtsv) and known-answer tests derived from the
discretisation.  The Fortran reference ships no tests or golden vectors and
cannot be compiled here, so these are the pins available.
"""
import numpy as np
import pytest

from conftest import assert_close, channel_case, rel_err


def oracle_for(case, **kw):
    from oracle import Oracle
    p = dict(case["prm"])
    p.update(kw)
    o = Oracle(case["x"], case["y"], case["z"], p)
    o.set_fields(case["U"], case["V"], case["W"])
    return o


# --------------------------------------------------------------------- FFT
@pytest.mark.parametrize("n", [16, 30, 60, 64, 96, 128, 192, 256, 512])
def test_fft_matches_numpy(n):
    from oracle import lib
    L = lib()
    rng = np.random.default_rng(n)
    z = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    for sign, ref in ((-1, np.fft.fft(z)), (+1, np.fft.ifft(z) * n)):
        a = np.ascontiguousarray(z.copy())
        L.cfo_fft(a.view(np.float64).ctypes.data_as(__import__("ctypes").POINTER(__import__("ctypes").c_double)), n, sign)
        assert rel_err(a, ref) < 1e-13, (n, sign)


# ------------------------------------------------------------------ zgtsv
def _zgtsv_oracle(dl, d, du, b):
    import ctypes as C
    from oracle import lib
    L = lib()
    arrs = [np.ascontiguousarray(x.astype(np.complex128)) for x in (dl, d, du, b)]
    ptr = [a.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)) for a in arrs]
    info = L.cfo_zgtsv(len(d), *ptr)
    return arrs[3], info


def test_zgtsv_matches_lapack_random_pivoting():
    from scipy.linalg.lapack import zgtsv
    rng = np.random.default_rng(3)
    for n in (5, 17, 64, 128):
        for trial in range(4):
            d = rng.standard_normal(n) * (0.1 if trial % 2 else 3.0)  # weak diagonal forces row interchanges
            dl = rng.standard_normal(n - 1)
            du = rng.standard_normal(n - 1)
            b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
            x, info = _zgtsv_oracle(dl, d, du, b)
            _, _, _, xr, infor = zgtsv(dl.astype(complex), d.astype(complex), du.astype(complex), b[:, None])
            assert info == infor == 0
            assert rel_err(x, xr[:, 0]) < 1e-12


def test_zgtsv_on_channel_matrices():
    """The per-mode matrices of projection.f90:97-107 (including the (0,0)
    mode with D(2)*1.5) solved by the restated zgtsv and by LAPACK."""
    from scipy.linalg.lapack import zgtsv
    case = channel_case(66, 65, 66)
    o = oracle_for(case)
    Dyy = o.array("Dyy")
    kxx, kzz = o.array("kxx"), o.array("kzz")
    n = Dyy.shape[0]
    rng = np.random.default_rng(1)
    for kx, kz in ((0, 0), (1, 0), (0, 1), (5, 7), (32, 32), (63, 10)):
        d = np.diag(Dyy) + kxx[kx] + kzz[kz]
        if kx == 0 and kz == 0:
            d[0] *= 1.5
        dl = np.array([Dyy[j + 1, j] for j in range(n - 1)])
        du = np.array([Dyy[j, j + 1] for j in range(n - 1)])
        b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        x, info = _zgtsv_oracle(dl, d, du, b)
        _, _, _, xr, _ = zgtsv(dl.astype(complex), d.astype(complex), du.astype(complex), b[:, None])
        assert info == 0
        assert rel_err(x, xr[:, 0]) < 1e-12, (kx, kz)


# ---------------------------------------------------------- known answers
def test_modified_wavenumbers_are_eigenvalues():
    """kxx(k) is the eigenvalue of the periodic second difference on e^{2 pi i k x / L}
    (initialization.f90:284-296)."""
    case = channel_case(34, 17, 34)
    o = oracle_for(case)
    kxx = o.array("kxx")
    nxp = len(kxx)
    dx = o.scalar("dxmin")
    idx = np.arange(nxp)
    for k in (0, 1, 3, nxp // 2, nxp - 2):
        f = np.exp(2j * np.pi * k * idx / nxp)
        lap = (np.roll(f, -1) - 2 * f + np.roll(f, 1)) / dx ** 2
        assert np.allclose(lap, kxx[k] * f, rtol=1e-12, atol=1e-12 * abs(kxx).max())


def test_projection_recovers_manufactured_potential():
    """u* = grad(phi0) with dphi0/dy = 0 at the walls: the projection returns
    phi0 (up to the mean-mode gauge of D(2)*1.5) and u = 0."""
    case = channel_case(18, 17, 18)
    o = oracle_for(case)
    nx, ny, nz = 18, 17, 18
    nxg, nyg, nzg = nx + 1, ny + 1, nz + 1
    xg, yg, zg = o.array("xg"), o.array("yg"), o.array("zg")
    rng = np.random.default_rng(2)
    nxp, nym, nzp = nx - 2, ny - 1, nz - 2
    can = rng.standard_normal((nxp, nym, nzp))
    phi = np.zeros((nxg, nyg, nzg))
    wx = lambda i: 2 + ((i - 2) % nxp)
    for i in range(1, nxg + 1):
        for k in range(1, nzg + 1):
            phi[i - 1, 1:nyg - 1, k - 1] = can[wx(i) - 2, :, wx(k) - 2] if False else can[(i - 2) % nxp, :, (k - 2) % nzp]
    phi[:, 0, :] = phi[:, 1, :]
    phi[:, -1, :] = phi[:, -2, :]
    U = np.zeros((nx, nyg, nzg), order="F")
    V = np.zeros((nxg, ny, nzg), order="F")
    W = np.zeros((nxg, nyg, nz), order="F")
    for i in range(1, nx + 1):
        U[i - 1] = (phi[i] - phi[i - 1]) / (xg[i] - xg[i - 1])
    for j in range(1, ny + 1):
        V[:, j - 1] = (phi[:, j] - phi[:, j - 1]) / (yg[j] - yg[j - 1])
    for k in range(1, nz + 1):
        W[:, :, k - 1] = (phi[:, :, k] - phi[:, :, k - 1]) / (zg[k] - zg[k - 1])
    o.set_fields(U, V, W)
    o.set_scalar("dt", 1.0)
    o.set_scalar("rk_step", 2)
    o.compute_projection_step()
    f = o.fields()
    scale = max(abs(U).max(), abs(V).max(), abs(W).max())
    assert abs(f["U"][1:nx - 1, 1:nyg - 1, 1:nzg - 1]).max() < 1e-11 * scale
    assert abs(f["V"][1:nxg - 1, 1:ny - 1, 1:nzg - 1]).max() < 1e-11 * scale
    assert abs(f["W"][1:nxg - 1, 1:nyg - 1, 1:nz - 1]).max() < 1e-11 * scale


def test_projection_leaves_divergence_at_round_off():
    case = channel_case(34, 33, 34)
    o = oracle_for(case)
    o.apply_boundary_conditions()
    o.set_scalar("dt", 2e-3)
    o.set_scalar("rk_step", 2)
    o.compute_projection_step()
    o.apply_boundary_conditions()
    _, m = o.check_divergence()
    assert m < 1e-12


def test_poiseuille_discrete_steady_state():
    """The discrete laminar profile with nu_t = 0 and a fixed dPdx has a zero
    right-hand side (equations.f90:108-166)."""
    nx, ny, nz = 10, 33, 10
    case = channel_case(nx, ny, nz)
    nu, dpdx = 1e-2, 2e-2
    o = oracle_for(case, LES_model=0, x_mass_cte=0, nu=nu, dPdx=dpdx)
    y, yg = o.array("y"), o.array("yg")
    nyg = ny + 1
    # unknowns U(2..nyg-1); ghost U(1) = -U(2), U(nyg) = -U(nyg-1)
    n = nyg - 2
    A = np.zeros((n, n))
    rhs = np.full(n, -dpdx / nu)
    for m in range(n):
        j = m + 2
        dy3 = y[j - 1] - y[j - 2]
        ap = 1.0 / (yg[j] - yg[j - 1]) / dy3
        am = 1.0 / (yg[j - 1] - yg[j - 2]) / dy3
        A[m, m] -= ap + am
        if m + 1 < n:
            A[m, m + 1] += ap
        else:
            A[m, m] -= ap
        if m > 0:
            A[m, m - 1] += am
        else:
            A[m, m] -= am
    prof = np.linalg.solve(A, rhs)
    U = np.zeros((nx, nyg, nz + 1), order="F")
    U[:, 1:nyg - 1, :] = prof[None, :, None]
    U[:, 0, :] = -U[:, 1, :]
    U[:, -1, :] = -U[:, -2, :]
    V = np.zeros((nx + 1, ny, nz + 1), order="F")
    W = np.zeros((nx + 1, nyg, nz), order="F")
    o.set_fields(U, V, W)
    o.compute_eddy_viscosity()
    o.compute_rhs_u(1)
    o.compute_rhs_v(1)
    o.compute_rhs_w(1)
    assert abs(o.array("Fu1")).max() < 1e-10 * dpdx * 1e3
    assert abs(o.array("Fv1")).max() == 0.0
    assert abs(o.array("Fw1")).max() == 0.0


def test_rk3_coefficients_are_third_order():
    """Stages of time_integration.f90:108-145 with the coefficients of
    initialization.f90:407-417 on u' = z u give 1 + z + z^2/2 + z^3/6."""
    c11, c21, c22, c31, c32, c33 = 8 / 15, 1 / 4, 5 / 12, 1 / 4, 0.0, 3 / 4
    P = np.polynomial.Polynomial
    z = P([0, 1])
    u0 = P([1])
    u1 = u0 + c11 * z * u0
    u2 = u0 + z * (c21 * u0 + c22 * u1)
    u3 = u0 + z * (c31 * u0 + c32 * u1 + c33 * u2)
    assert np.allclose(u3.coef, [1, 1, 0.5, 1 / 6])


def test_boundary_conditions_idempotent_and_periodic():
    case = channel_case(18, 17, 18)
    rng = np.random.default_rng(4)
    for k in ("U", "V", "W"):
        case[k] = np.asfortranarray(rng.standard_normal(case[k].shape))
    o = oracle_for(case)
    o.apply_boundary_conditions()
    a = o.fields()
    o.apply_boundary_conditions()
    b = o.fields()
    for n in ("U", "V", "W"):
        assert np.array_equal(a[n], b[n])
    U = a["U"]
    assert np.array_equal(U[0], U[-2]) and np.array_equal(U[-1], U[1])      # faces, x
    assert np.array_equal(U[:, :, 0], U[:, :, -3])                           # centres, z
    assert np.array_equal(U[:, 0, :], -U[:, 1, :])                           # no slip
    assert not a["V"][:, 0, :].any() and not a["V"][:, -1, :].any()


def test_dsm_galilean_invariance():
    """L_ij and M_ij are unchanged by a uniform shift of U (the filter weights
    sum to one in every row, one-sided rows included)."""
    case = channel_case(34, 33, 34)
    o = oracle_for(case)
    o.apply_boundary_conditions()
    f = o.fields()
    o.compute_eddy_viscosity()
    nt0 = o.array("nu_t")
    o.set_fields(f["U"] + 0.75, f["V"], f["W"])
    o.compute_eddy_viscosity()
    nt1 = o.array("nu_t")
    assert rel_err(nt1, nt0) < 1e-9


def test_bounds_checked_oracle_runs_a_step():
    """The oracle with every array index range-checked (the reference's
    -check all) runs a full RK3 step with the wall model."""
    from oracle import Oracle
    case = channel_case(14, 13, 14, stretch=0.0, wall=3, retau=2000.0, profile="plug")
    o = Oracle(case["x"], case["y"], case["z"], case["prm"], check=True)
    o.set_fields(case["U"], case["V"], case["W"])
    o.init_mass_flow()
    o.apply_boundary_conditions()
    o.compute_dt()
    o.time_step_rk3()
    assert np.isfinite(o.array("U")).all()


@pytest.mark.parametrize("check", [False, True])
def test_pressure_solves_discrete_poisson(check):
    """compute_pressure (pressure.f90:21): with its wall rows, the 3-point
    Laplacian of P (x and z through the periodic wrap) equals div(rhs) on
    every interior row; on row 2 up to one constant, the gauge of the (0,0)
    mode (D(2)*3/2).  The periodic copies are exact."""
    from oracle import Oracle
    nx, ny, nz = 18, 17, 14
    case = channel_case(nx, ny, nz, stretch=1.5)
    o = Oracle(case["x"], case["y"], case["z"], case["prm"], check=check)
    o.set_fields(case["U"], case["V"], case["W"])
    o.apply_boundary_conditions()
    o.compute_eddy_viscosity()
    o.compute_pressure()
    P, rp = o.array("P"), o.array("rhs_p")
    nxg, nyg, nzg, nxp, nzp = nx + 1, ny + 1, nz + 1, nx - 2, nz - 2
    x, y, z, yg = o.array("x"), o.array("y"), o.array("z"), o.array("yg")
    dx, dz = x[1] - x[0], z[1] - z[0]
    Pc = P[1:nxp + 1, :, 1:nzp + 1]
    lap = (np.roll(Pc, -1, 0) - 2 * Pc + np.roll(Pc, 1, 0)) / dx ** 2 + \
          (np.roll(Pc, -1, 2) - 2 * Pc + np.roll(Pc, 1, 2)) / dz ** 2
    res = np.zeros((nxp, nyg - 2, nzp))
    for j in range(2, nyg):  # Fortran row j; arrays are 0-based
        a = 1 / (y[j - 1] - y[j - 2]) / (yg[j] - yg[j - 1])
        c = 1 / (y[j - 1] - y[j - 2]) / (yg[j - 1] - yg[j - 2])
        res[:, j - 2, :] = lap[:, j - 1, :] + c * Pc[:, j - 2, :] - (a + c) * Pc[:, j - 1, :] + a * Pc[:, j, :]
    res -= rp[:nxp, :, :nzp]
    scale = abs(rp).max()
    assert abs(res[:, 1:, :]).max() < 1e-12 * scale
    assert abs(res[:, 0, :] - res[:, 0, :].mean()).max() < 1e-12 * scale
    assert np.array_equal(P[nxg - 2], P[1])
    assert np.array_equal(P[1:nxg - 1, :, nzg - 2], P[1:nxg - 1, :, 1])
    assert abs(P[1:-1, 0, 1:-1] - P[1:-1, 1, 1:-1]).max() > 1e-6 * abs(P).max()
