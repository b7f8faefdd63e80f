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


def amd_point_formula(o, U, V, W):
    """sgs_AMD (subgrid.f90:639-871) at the canonical cells as one formula per
    cell: the reference's section operations (interpolate_x/y/z of squared or
    plain differences of partly set temporaries) reduced by hand to the cell's
    3x3x3 neighbourhood.  Returns (-C num/den clipped, den)."""
    nxg, nyg, nzg = U.shape[0] + 1, U.shape[1], U.shape[2]
    P = lambda a: np.r_[np.nan, a]  # 1-based coordinates
    x, y, z, xg, yg, zg = (P(o.array(n)) for n in ("x", "y", "z", "xg", "yg", "zg"))
    i = np.arange(2, nxg - 1)[:, None, None]
    j = np.arange(2, nyg)[None, :, None]
    k = np.arange(2, nzg - 1)[None, None, :]
    F = lambda a, di=0, dj=0, dk=0: a[1 + di:nxg - 2 + di, 1 + dj:nyg - 1 + dj, 1 + dk:nzg - 2 + dk]
    h = 0.5
    s11 = (F(U) - F(U, -1)) / (x[i] - x[i - 1])
    s22 = (F(V) - F(V, 0, -1)) / (y[j] - y[j - 1])
    s33 = (F(W) - F(W, 0, 0, -1)) / (z[k] - z[k - 1])
    e4 = lambda a, b: h * ((F(U, a - 1, b) - F(U, a - 1, b - 1)) / (yg[j + b] - yg[j + b - 1]) +
                           (F(V, a, b - 1) - F(V, a - 1, b - 1)) / (xg[i + a] - xg[i + a - 1]))
    e5 = lambda a, b: h * ((F(U, a - 1, 0, b) - F(U, a - 1, 0, b - 1)) / (zg[k + b] - zg[k + b - 1]) +
                           (F(W, a, 0, b - 1) - F(W, a - 1, 0, b - 1)) / (xg[i + a] - xg[i + a - 1]))
    e6 = lambda a, b: h * ((F(V, 0, a - 1, b) - F(V, 0, a - 1, b - 1)) / (zg[k + b] - zg[k + b - 1]) +
                           (F(W, 0, a, b - 1) - F(W, 0, a - 1, b - 1)) / (yg[j + a] - yg[j + a - 1]))
    s12 = 0.25 * (e4(0, 0) + e4(1, 0) + e4(0, 1) + e4(1, 1))
    s13 = 0.25 * (e5(0, 0) + e5(1, 0) + e5(0, 1) + e5(1, 1))
    s23 = 0.25 * (e6(0, 0) + e6(1, 0) + e6(0, 1) + e6(1, 1))
    # differences: dU_y(a, b) = U(i+a, j+b) - U(i+a, j+b-1) etc.
    dUx = lambda a=0, b=0, c=0: F(U, a, b, c) - F(U, a - 1, b, c)
    dUy = lambda a=0, b=0, c=0: F(U, a, b, c) - F(U, a, b - 1, c)
    dUz = lambda a=0, b=0, c=0: F(U, a, b, c) - F(U, a, b, c - 1)
    dVx = lambda a=0, b=0, c=0: F(V, a, b, c) - F(V, a - 1, b, c)
    dVy = lambda a=0, b=0, c=0: F(V, a, b, c) - F(V, a, b - 1, c)
    dVz = lambda a=0, b=0, c=0: F(V, a, b, c) - F(V, a, b, c - 1)
    dWx = lambda a=0, b=0, c=0: F(W, a, b, c) - F(W, a - 1, b, c)
    dWy = lambda a=0, b=0, c=0: F(W, a, b, c) - F(W, a, b - 1, c)
    dWz = lambda a=0, b=0, c=0: F(W, a, b, c) - F(W, a, b, c - 1)
    av = lambda p, q: h * (p + q)
    # U: faces i-1, i; y faces j, j+1 / z faces k, k+1
    uy = lambda f: av(av(f(-1, 0, 0), f(0, 0, 0)), av(f(-1, 1, 0), f(0, 1, 0)))
    uz = lambda f: av(av(f(-1, 0, 0), f(0, 0, 0)), av(f(-1, 0, 1), f(0, 0, 1)))
    # V: x faces i, i+1 with y rows j-1, j (y first) / z faces k, k+1 (y first)
    vx = lambda f: av(av(f(0, -1, 0), f(0, 0, 0)), av(f(1, -1, 0), f(1, 0, 0)))
    vz = lambda f: av(av(f(0, -1, 0), f(0, 0, 0)), av(f(0, -1, 1), f(0, 0, 1)))
    # W: x faces i, i+1 with z rows k-1, k (z first) / y faces j, j+1 (z first)
    wx = lambda f: av(av(f(0, 0, -1), f(0, 0, 0)), av(f(1, 0, -1), f(1, 0, 0)))
    wy = lambda f: av(av(f(0, 0, -1), f(0, 0, 0)), av(f(0, 1, -1), f(0, 1, 0)))
    sq = lambda d: (lambda a, b, c: d(a, b, c) ** 2)
    dyg = lambda b: yg[j + b] - yg[j + b - 1]
    dzg = lambda c: zg[k + c] - zg[k + c - 1]
    dxg = lambda a: xg[i + a] - xg[i + a - 1]
    den = dUx() ** 2 / (x[i] - x[i - 1]) ** 2
    den = den + uy(lambda a, b, c: dUy(a, b, c) ** 2 / dyg(b) ** 2)
    den = den + uz(lambda a, b, c: dUz(a, b, c) ** 2 / dzg(c) ** 2)
    den = den + dVy() ** 2 / (y[j] - y[j - 1]) ** 2
    den = den + vx(lambda a, b, c: dVx(a, b, c) ** 2 / dxg(a) ** 2)
    den = den + vz(lambda a, b, c: dVz(a, b, c) ** 2 / dzg(c) ** 2)
    den = den + dWz() ** 2 / (z[k] - z[k - 1]) ** 2
    den = den + wx(lambda a, b, c: dWx(a, b, c) ** 2 / dxg(a) ** 2)
    den = den + wy(lambda a, b, c: dWy(a, b, c) ** 2 / dyg(b) ** 2)
    num = dUx() ** 2 * s11
    num = num + uy(sq(dUy)) * s11
    num = num + uz(sq(dUz)) * s11
    num = num + dVy() ** 2 * s22
    num = num + vx(sq(dVx)) * s22
    num = num + vz(sq(dVz)) * s22
    num = num + dWz() ** 2 * s33
    num = num + wx(sq(dWx)) * s33
    num = num + wy(sq(dWy)) * s33
    num = num + 2.0 * (av(av(dVx(0, -1), dVx()), av(dVx(1, -1), dVx(1))) * dUx()) * s12
    num = num + 2.0 * (av(av(dUy(-1), dUy()), av(dUy(-1, 1), dUy(0, 1))) * dVy()) * s12
    num = num + 2.0 * av(av(dUz(-1), dUz()) * av(dVz(0, -1), dVz()), av(dUz(-1, 0, 1), dUz(0, 0, 1)) *
                         av(dVz(0, -1, 1), dVz(0, 0, 1))) * s12
    num = num + 2.0 * (av(av(dWx(0, 0, -1), dWx()), av(dWx(1, 0, -1), dWx(1))) * dUx()) * s13
    num = num + 2.0 * (av(av(dUz(-1), dUz()), av(dUz(-1, 0, 1), dUz(0, 0, 1))) * dWz()) * s13
    num = num + 2.0 * av(av(dUy(-1), dUy()) * av(dWy(0, 0, -1), dWy()), av(dUy(-1, 1), dUy(0, 1)) *
                         av(dWy(0, 1, -1), dWy(0, 1))) * s13
    num = num + 2.0 * (av(av(dWy(0, 0, -1), dWy()), av(dWy(0, 1, -1), dWy(0, 1))) * dVy()) * s23
    num = num + 2.0 * (av(av(dVz(0, -1), dVz()), av(dVz(0, -1, 1), dVz(0, 0, 1))) * dWz()) * s23
    num = num + 2.0 * av(av(dVx(0, -1), dVx()) * av(dWx(0, 0, -1), dWx()), av(dVx(1, -1), dVx(1)) *
                         av(dWx(1, 0, -1), dWx(1))) * s23
    with np.errstate(invalid="ignore", divide="ignore"):
        v = -0.3 * num / den
    return np.where(v > 0, v, 0.0), den


@pytest.mark.parametrize("check,dirichlet", [(True, 0), (False, 1), (False, 2)])
def test_amd_matches_point_formula(check, dirichlet):
    """The oracle's sgs_AMD (section operations of subgrid.f90:639-881 on
    NaN-filled temporaries) against the per-cell formula: the canonical cells
    agree to round-off and take nothing from an unset temporary; ghosts
    follow the periodic copies and the wall rule; avg_nu_t is the canonical
    plane mean; the model is Galilean invariant away from the walls."""
    from oracle import Oracle
    nx, ny, nz = 18, 17, 14
    case = channel_case(nx, ny, nz, stretch=1.5, les=3)
    case["prm"]["Dirichlet_nu_t"] = dirichlet
    o = Oracle(case["x"], case["y"], case["z"], case["prm"], check=check)
    o.set_fields(case["U"], case["V"], case["W"])
    o.apply_boundary_conditions()
    o.compute_eddy_viscosity()
    assert o.scalar("amd_nan_canonical") == 0
    f = o.fields()
    nt = o.array("nu_t")
    want, den = amd_point_formula(o, f["U"], f["V"], f["W"])
    assert (den > 0).all()
    can = nt[1:nx - 1, 1:ny, 1:nz - 1]
    assert abs(can - want).max() <= 1e-14 * abs(want).max()
    assert (want > 0).any() and (want == 0).any()
    nxg, nyg, nzg = nx + 1, ny + 1, nz + 1
    assert np.array_equal(nt[0], nt[nxg - 3]) and np.array_equal(nt[nxg - 2], nt[1]) and np.array_equal(nt[nxg - 1], nt[2])
    assert np.array_equal(nt[:, 1:-1, 0], nt[:, 1:-1, nzg - 3]) and np.array_equal(nt[:, 1:-1, nzg - 2], nt[:, 1:-1, 1])
    g = 2 * 0.38 * o.scalar("dPdx") ** 0.5 * (case["y"][1] - case["y"][0]) / 2 if dirichlet == 2 else 0.0
    sgn = 1.0 if dirichlet == 0 else -1.0
    assert abs(nt[:, 0, :] - (sgn * nt[:, 1, :] + g)).max() <= 1e-15
    avg = o.array("avg_nu_t").ravel()
    assert abs(avg[1:-1] - can.mean(axis=(0, 2))).max() <= 1e-15 * abs(can).max()
    o.set_fields(f["U"] + 0.7, f["V"], f["W"] - 0.3)
    o.apply_boundary_conditions()
    o.compute_eddy_viscosity()
    assert abs(o.array("nu_t")[:, 2:-2, :] - nt[:, 2:-2, :]).max() <= 1e-12 * abs(nt).max()


def test_monitor_reductions_match_numpy():
    """output_monitor (monitor.f90:28-52, 74-81) in the oracle against numpy
    on the same sections and normalisations."""
    nx, ny, nz = 18, 17, 14
    case = channel_case(nx, ny, nz)
    o = oracle_for(case)
    o.apply_boundary_conditions()
    o.compute_eddy_viscosity()
    m = o.output_monitor()
    f = o.fields()
    U, V, W, nt = f["U"], f["V"], f["W"], f["nu_t"]
    cells = (nx - 1) * (ny - 1) * (nz - 1)
    secs = [U[1:nx - 1, 1:ny, 1:nz], V[1:nx, 1:ny - 1, 1:nz], W[1:nx, 1:ny, 1:nz - 1], nt[1:nx, 1:ny, 1:nz]]
    want = [secs[0].sum() / cells, secs[1].sum() / cells, secs[2].sum() / cells, secs[0].max(), secs[1].max(),
            secs[2].max(), secs[3].sum() / ((nx + 1) * (ny + 1) * (nz + 1)), secs[3].max()]
    for q in range(8):
        assert abs(m[q] - want[q]) <= 1e-13 * max(1.0, abs(want[q])), (q, m[q], want[q])
    assert m[8] == o.check_divergence()[0]
