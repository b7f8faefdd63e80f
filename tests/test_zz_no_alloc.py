"""cf_check_divergence_noalloc: the divergence check with static device scratch
and no device allocation, against cf_check_divergence (the context entry point)
on the same fields.  Collected last so that it also runs after every other
GPU test in the same process."""
import ctypes as C
import math
import re

import numpy as np
import pytest

from conftest import channel_case


def _bind():
    import channelflow as cf
    L = cf.load()
    f = L.cf_check_divergence_noalloc
    f.argtypes = [C.c_int, C.c_int, C.c_int] + [C.c_void_p] * 8
    f.restype = C.c_int
    L.cf_last_error.argtypes = [C.c_void_p]
    L.cf_last_error.restype = C.c_char_p
    return L, f


def test_noalloc_rejects_more_planes_than_the_scratch_holds():
    """Rejected on the host before any device work (no GPU needed)."""
    L, f = _bind()
    import channelflow as cf
    limit = int(re.search(r"CF_NOALLOC_MAX_PLANES = (\d+)", open(cf.lib.HEADER).read()).group(1))
    rc = f(8, 8, limit + 2, None, None, None, None, None, None, None, None)
    assert rc == 1
    msg = L.cf_last_error(None).decode()
    assert "exceed the static scratch" in msg and str(limit) in msg


@pytest.mark.gpu
def test_noalloc_divergence_matches_context_entry_point():
    import torch
    import channelflow as cf
    L, f = _bind()
    case = channel_case(34, 33, 38, seed=7)
    rng = np.random.default_rng(3)
    # raw fields: nonzero divergence everywhere, positive and negative
    for k in ("U", "V", "W"):
        case[k] = np.asfortranarray(rng.standard_normal(case[k].shape))
    ch = cf.Channel(case["x"], case["y"], case["z"], precision=cf.PREC_FP64, **case["prm"])
    ch.upload(case["U"], case["V"], case["W"])
    ref_div, ref_abs = ch.check_divergence()
    assert ref_div > 0 and ref_abs >= ref_div

    dev = torch.device("cuda:0")
    flat = {k: torch.from_numpy(np.ravel(case[k], order="F").copy()).to(dev) for k in ("U", "V", "W", "x", "y", "z")}
    out = torch.full((2,), math.nan, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    nx, ny, nz = len(case["x"]), len(case["y"]), len(case["z"])
    for call in range(2):  # two calls in a row: the second reuses the set-up scratch
        out.fill_(math.nan)
        rc = f(nx, ny, nz, *(flat[k].data_ptr() for k in ("U", "V", "W", "x", "y", "z")), out.data_ptr(),
               stream.cuda_stream)
        assert rc == 0, L.cf_last_error(None).decode()
        stream.synchronize()
        got = out.cpu().numpy()
        # same per-cell arithmetic and an exact max: equal up to 1e-14 relative
        assert abs(got[0] - ref_div) <= 1e-14 * ref_abs, (call, got, ref_div)
        assert abs(got[1] - ref_abs) <= 1e-14 * ref_abs, (call, got, ref_abs)
    ch.close()


@pytest.mark.gpu
def test_noalloc_and_context_report_a_nan_divergence():
    """A NaN in one interior cell makes both results of both divergence
    checks NaN (a blown-up field is not reported as a finite maximum)."""
    import torch
    import channelflow as cf
    L, f = _bind()
    case = channel_case(18, 17, 18, seed=9)
    case["U"][5, 6, 7] = math.nan
    ch = cf.Channel(case["x"], case["y"], case["z"], precision=cf.PREC_FP64, **case["prm"])
    ch.upload(case["U"], case["V"], case["W"])
    assert all(math.isnan(v) for v in ch.check_divergence())
    ch.close()
    dev = torch.device("cuda:0")
    flat = {k: torch.from_numpy(np.ravel(case[k], order="F").copy()).to(dev) for k in ("U", "V", "W", "x", "y", "z")}
    out = torch.zeros(2, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    nx, ny, nz = len(case["x"]), len(case["y"]), len(case["z"])
    rc = f(nx, ny, nz, *(flat[k].data_ptr() for k in ("U", "V", "W", "x", "y", "z")), out.data_ptr(),
           stream.cuda_stream)
    assert rc == 0, L.cf_last_error(None).decode()
    stream.synchronize()
    assert np.isnan(out.cpu().numpy()).all()
