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
