"""CPU tests of the library boundary: the C ABI exports every function the
header declares, and the input_parameters reader and snapshot format
(input_output.f90) round-trip.  No GPU calls."""
import os
import struct

import numpy as np

from conftest import ROOT

GOLDEN = os.path.join(ROOT, "tests", "golden")


def test_library_exports_every_declared_function():
    import channelflow as cf
    L = cf.load()
    names = cf.header_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_read_input_parameters():
    import channelflow as cf
    r = cf.read_input_parameters(os.path.join(GOLDEN, "input_parameters_re550"))
    p = r["params"]
    assert r["grid"] == (194, 129, 194)
    assert abs(p.CFL - 0.5) < 1e-15
    assert p.Retau_int == 0 and abs(p.nu - 9.97e-5) < 1e-20
    assert abs(p.dPdx - 3.01e-3) < 1e-18 and p.x_mass_cte == 1 and p.y_mass_cte == 0
    assert p.LES_model == 2 and p.iwall_model == 0
    assert (r["nsteps"], r["nsave"], r["nstats"], r["nmonitor"]) == (2000, 500, 10, 10)
    assert r["filein"] == "re550_start" and r["fileout"] == "re550"
    assert r["random_init"] == 0 and p.Dirichlet_nu_t == 0 and p.jref_eqwm == 6
    assert abs(p.freq_mult - 1.0) < 1e-15


def test_snapshot_roundtrip_big_endian(tmp_path):
    import channelflow as cf
    from channelflow import grids
    nx, ny, nz = 10, 9, 8
    x, y, z = grids.channel_grid(nx, ny, nz)
    U, V, W = grids.seeded_fields(x, y, z, seed=11)
    P = np.asfortranarray(np.random.default_rng(1).standard_normal((nx + 1, ny + 1, nz + 1)))
    path = str(tmp_path / "snap.100")
    cf.write_snapshot(path, x, y, z, U, V, W, P, P)
    raw = open(path, "rb").read()
    # mesh record: big-endian int32 count then big-endian doubles (input_output.f90:416)
    assert struct.unpack(">i", raw[:4])[0] == nx
    assert struct.unpack(">d", raw[4:12])[0] == x[0]
    # total length: 6 mesh records + 5 fields with 3-int headers
    n = 4 * 6 + 8 * (nx + ny + nz + (nx - 1) + (ny - 1) + (nz - 1))
    n += 5 * 12 + 8 * (U.size + V.size + W.size + 2 * P.size)
    assert len(raw) == n
    x2, y2, z2, U2, V2, W2 = cf.read_snapshot(path, nx, ny, nz)
    for a, b in ((x, x2), (y, y2), (z, z2), (U, U2), (V, V2), (W, W2)):
        assert np.array_equal(a, b)


def test_snapshot_rejects_wrong_size(tmp_path):
    import pytest
    import channelflow as cf
    from channelflow import grids
    x, y, z = grids.channel_grid(10, 9, 8)
    U, V, W = grids.seeded_fields(x, y, z)
    path = str(tmp_path / "snap")
    cf.write_snapshot(path, x, y, z, U, V, W)
    with pytest.raises(cf.CfError):
        cf.read_snapshot(path, 12, 9, 8)


def test_create_rejects_odd_nx_without_gpu_work():
    """cf_create validates sizes before touching the device (the reference's
    Stop 'Error: nx must be even', initialization.f90:54)."""
    import pytest
    import channelflow as cf
    from channelflow import grids
    x, y, z = grids.channel_grid(11, 9, 8)
    with pytest.raises(cf.CfError, match="nx must be even"):
        cf.Channel(x, y, z)


def test_statistics_text_file_known_answer(tmp_path):
    """output_statistics (input_output.f90:549-570): '(A,4F15.8,4I)' header
    and '(8F15.8)' records of seven values, written by hand from the Fortran
    edit rules: right-justified fields, eight decimals, a minus sign on
    negative values that round to zero but not on IEEE -0.0, asterisks when
    the value does not fit, I12 for the widthless integer descriptor."""
    import channelflow as cf
    ny = 3
    y = np.array([0.0, 1.0, 2.0])
    st = np.zeros(9 * ny + 8)
    prof = {0: [1.5, -1e-12, 2.25], 3: [0.125, -0.0, 999999.5], 4: [1234567.0, -99999.5, np.nan],
            5: [1e-9, 6e-9, -0.333333333333], 6: [0.0, 0.5, -0.5], 8: [7.0, 8.0, 9.0]}
    for q, v in prof.items():
        st[q * ny:(q + 1) * ny] = v
    st[9 * ny], st[9 * ny + 1] = 0.0638, 180.123456789  # utau, Retau
    p = tmp_path / "s.txt"
    cf.write_statistics(str(p), 0.125, 3.547e-4, 66, ny, 66, 200, y, st)
    got = p.read_text().split("\n")
    want = [
        "%" + "     0.12500000" + "   180.12345679" + "     0.06380000" + "     0.00035470"
        + "          66" + "           3" + "          66" + "         200",
        "     0.00000000" + "     1.50000000" + "     0.12500000" + "***************" + "     0.00000000"
        + "     0.00000000" + "     7.00000000",
        "     1.00000000" + "    -0.00000000" + "     0.00000000" + "-99999.50000000" + "     0.00000001"
        + "     0.50000000" + "     8.00000000",
        "     2.00000000" + "     2.25000000" + "999999.50000000" + "            NaN" + "    -0.33333333"
        + "    -0.50000000" + "     9.00000000",
        "",
    ]
    assert got == want
    assert cf.statistics_file_name("  run/out  ", 200, 1000) == "run/out.1200.stats.txt"
    assert cf.statistics_file_name("o", 123456789, 0) == "o.********.stats.txt"


def test_create_rejects_unsupported_models_without_gpu_work():
    """LES_model 1 (constant Smagorinsky) and an AMD wall rule other than
    0, 1, 2 are refused before any device work."""
    import pytest
    import channelflow as cf
    from channelflow import grids
    x, y, z = grids.channel_grid(10, 9, 8)
    with pytest.raises(cf.CfError, match="LES_model must be"):
        cf.Channel(x, y, z, LES_model=1)
    with pytest.raises(cf.CfError, match="Dirichlet_nu_t must be"):
        cf.Channel(x, y, z, LES_model=3, Dirichlet_nu_t=3)
