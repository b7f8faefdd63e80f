"""A C caller of the ABI (tests/c_driver/rk3_mirror.c, compiled with gcc):
the reference's compute_time_step_RK3 (time_integration.f90:89-173) issued
call by call through the mirror entry points, in the reference's order and
with its mass-flow branches, against the graph-captured cf_time_step_rk3 on
the same snapshot.  FP64: U, V, W within 1e-13, nu_t within 1e-12, P within
1e-11 (the pseudo-pressure phi/(dt 8/15) carries the cancellation of
div u* = O(dt))."""
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, channel_case

SRC = os.path.join(ROOT, "tests", "c_driver", "rk3_mirror.c")
PKG = os.path.join(ROOT, "channel-flow_gb300")


def build_driver(out_dir):
    """gcc -std=c11 against include/channel_gpu.h and the in-tree library."""
    import channelflow as cf
    cf.load()  # builds the library when it is missing
    exe = os.path.join(str(out_dir), "rk3_mirror")
    cmd = ["gcc", "-O2", "-std=c11", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L", PKG, "-lchannel_gpu", f"-Wl,-rpath,{PKG}", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def test_c_driver_compiles_and_links(tmp_path):
    """The driver builds with gcc against the header and links every ABI call
    it makes against the library (no GPU needed)."""
    exe = build_driver(tmp_path)
    assert os.path.getsize(exe) > 0
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr


CASES = [
    # (faces, channel_case keywords, steps, x_mass_cte)
    ((34, 33, 34), dict(seed=2), 3, 1),
    ((18, 17, 18), dict(seed=3, stretch=0.0, wall=3, retau=2000.0, profile="plug", jref=3, ncv=30), 3, 1),
    ((26, 17, 22), dict(seed=4, les=3), 3, 1),
    ((18, 17, 18), dict(seed=5), 2, 0),
]


@pytest.mark.gpu
@pytest.mark.parametrize("dims,kw,steps,xmass", CASES)
def test_c_mirror_matches_fast_path(tmp_path, dims, kw, steps, xmass):
    import channelflow as cf
    exe = build_driver(tmp_path)
    case = channel_case(*dims, **kw)
    snap = str(tmp_path / "in.bin")
    cf.write_snapshot(snap, case["x"], case["y"], case["z"], case["U"], case["V"], case["W"])
    p = case["prm"]
    args = [exe, snap, *(str(d) for d in dims), repr(p["nu"]), repr(p["dPdx"]), str(p["LES_model"]),
            str(p["iwall_model"]), str(p["jref_eqwm"]), str(p["eqwm_ncv"]), str(xmass), "0", repr(case["dt"]),
            str(steps), str(cf.PREC_FP64)]
    r = subprocess.run(args, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    res = json.loads(r.stdout.strip().splitlines()[-1])
    print(dims, kw, res)
    for n in ("U", "V", "W"):
        assert res[n] <= 1e-13, (n, res[n])
    # nu_t: the fast path forms max(-C|S|/2, 0) inside the fused right-hand
    # side, the mirror materialises it first (different contraction)
    assert res["nu_t"] <= 1e-12, res["nu_t"]
    assert res["P"] <= 1e-11, res["P"]
    assert res["t"][0] == res["t"][1] and res["t"][0] > 0
    # dPdx = (Q0 - Q)/dt is a cancellation: compare the correction Q0 - Q
    # against the mass flow it corrects
    assert abs(res["dPdx"][0] - res["dPdx"][1]) * case["dt"] <= 1e-12 * abs(res["Qflow_x_0"])
    assert np.isfinite(list(res[n] for n in ("U", "V", "W", "P", "nu_t"))).all()
