#!/usr/bin/env python
"""Throughput of the RK3 step of the staggered finite-difference channel solver.

Workload (default): wall-resolved LES at Re_tau = 550 -- 2*pi x 2 x pi,
192 x 128 x 192 cells (input_parameters faces 194 129 194), tanh-stretched
wall-normal grid (stretch 1.5), dynamic Smagorinsky, no-slip walls, constant
mass flow, seeded perturbed laminar initial field made divergence-free by
one projection, CFL 0.5 (dt = 5e-3 by the reference's dt rule).  One "step"
is compute_dt + compute_time_step_RK3 + the mass-flow forcing
(time_integration.f90:89-227).  Metric: grid-point*steps/s with grid points =
the 192*128*192 unique cells.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 runs as replicas (one independent channel per rank, launched by
torch.distributed.run); rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "channel-flow_gb300")
sys.path.insert(0, PKG)

METRIC = "grid-pt·steps/s, mixed vs FP64 GPU at ≤1% stats error; HBM % of peak"
UNIT = "grid-pt·steps/s"

WORKLOADS = {
    "re550": dict(name="LES Re_tau=550, 192x128x192, DSM, no-slip, constant mass flow", nx=194, ny=129, nz=194,
                  retau=550.0, stretch=1.5, les=2, wall=0, jref=3, ncv=100, profile="laminar"),
    "re550_amd": dict(name="LES Re_tau=550, 192x128x192, AMD, no-slip, constant mass flow", nx=194, ny=129, nz=194,
                      retau=550.0, stretch=1.5, les=3, wall=0, jref=3, ncv=100, profile="laminar"),
    "re5200_wmlp": dict(name="WMLES Re_tau=5200, 512x128x512, DSM + learned wall stress (eqwm fallback, ncv 30), "
                             "uniform y, matched at 0.1 delta", nx=514, ny=129, nz=514, retau=5200.0, stretch=0.0, les=2,
                        wall=3, jref=8, ncv=30, profile="plug", mlp=True),
    "re5200_eqwm": dict(name="WMLES Re_tau=5200, 512x128x512, DSM + eqwm (ncv 30), uniform y, matched at 0.1 delta",
                        nx=514, ny=129, nz=514, retau=5200.0, stretch=0.0, les=2, wall=3, jref=8, ncv=30,
                        profile="plug"),
    "re180": dict(name="Re_tau=180, 64x64x64, DSM, no-slip, constant mass flow", nx=66, ny=65, nz=66, retau=180.0,
                  stretch=1.5, les=2, wall=0, jref=3, ncv=100, profile="laminar"),
    "re2000_eqwm": dict(name="WMLES Re_tau=2000, 256x96x256, DSM + eqwm (ncv 30), uniform y", nx=258, ny=97, nz=258,
                        retau=2000.0, stretch=0.0, les=2, wall=3, jref=6, ncv=30, profile="plug"),
}

# Algorithmic bytes per unique cell for one full step: one read or write of a
# full field per pass over the dependency-forced pass structure (DSM 4, RHS +
# update 10/13/13, div + forward FFT 4, tridiagonal 2, inverse FFT 2,
# projection 7, per substep; mass flow 2 and dt 3 per step): 98 accesses.
# Split path: 73 velocity-class accesses at 4 B, 11 u^n hi+lo at 8 B, 18
# spectrum/phi accesses at 8 B = 524 B; FP64 path: 98 x 8 = 784 B.
BYTES_PER_PT_STEP = {"split": 524.0, "fp64": 784.0}


def algorithmic_bytes(kernel: str, c, es: int) -> float | None:
    """Compulsory bytes of one launch of a kernel: every input element read once
    and every output element written once (es = bytes per state element)."""
    nC = c.nxp * c.nym * c.nzp  # unique cells
    cs = 2 * es                  # complex spectrum element
    nh = (c.nxp // 2 + 1) * c.nym * c.nzp
    tab = {
        # the dynamic Smagorinsky pass: read U, V, W, write |S| (4 field accesses per cell)
        "k_dsm_fused": 4 * nC * es,
        # the AMD pass: read U, V, W, write nu_t
        "k_amd": 4 * nC * es,
        # 3 velocity components in, |S| Sij (6), products (6), centre velocities (3), |S| out
        "k_dsm_a": (3 + 16) * nC * es,
        # 15 filtered quantities and Uf, Vf, Wf in (L, M and the plane sums formed in place)
        "k_dsm_b": (15 + 3) * nC * es,
        # one velocity component in and out
        "k_dsm_c_t": 2 * nC * es,
        "k_dsm_f": 2 * nC * es,
        # U, V, W, nu_t, Uo (+ lo), F1 in; out + F1 (substep 1 of 3 stores it)
        # one component: U, V, W, nu_t, Uo (+ its low word) and F1 in, the new
        # component out (F1 written in substep 1 instead of read)
        "k_rhs": 8 * nC * es,
        "k_fwd_x": 3 * nC * es + nh * cs,
        "k_fft_z": 2 * nh * cs,
        # FP32 LU replay: right-hand side in and out, multiplier and 1/d per (mode, row)
        "k_tri_split": 2 * nh * cs + 2 * nh * 4,
        # FP64 zgtsv replay (all modes in the FP64 path): data in/out, m, 1/d, du, dl, pivot flag
        "k_tri_mode": 2 * nh * cs + nh * 33,
        "k_inv_x": nh * cs + nC * es,
        # phi in, three velocity components in and out
        "k_project3": 7 * nC * es,
        # U, V, W in
        "k_dt_min": 3 * nC * es,
        "k_bc": None,
    }
    return tab.get(kernel)


def host_link(nbytes: int, dev: int) -> dict:
    """The host link's rate for the e2e bytes: plain pinned copies of nbytes
    each way (copy engine, CUDA events), and the per-step floor they set."""
    import torch
    h = torch.empty(nbytes // 8, dtype=torch.float64, pin_memory=True)
    d = torch.empty(nbytes // 8, dtype=torch.float64, device=f"cuda:{dev}")
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    for _ in range(2):
        d.copy_(h, non_blocking=True)
        h.copy_(d, non_blocking=True)
    torch.cuda.synchronize()
    reps = 3
    e0.record()
    for _ in range(reps):
        d.copy_(h, non_blocking=True)
    e1.record()
    for _ in range(reps):
        h.copy_(d, non_blocking=True)
    e2.record()
    e2.synchronize()
    up, down = e0.elapsed_time(e1) / reps, e1.elapsed_time(e2) / reps
    return {"link_h2d_gbs": nbytes / up / 1e6, "link_d2h_gbs": nbytes / down / 1e6,
            "link_floor_ms_per_step": up + down}


class _Nvml:
    """Reads the SM clock and the clock-event reasons of one GPU through
    libnvidia-ml (read-only queries)."""

    SM = 1  # NVML_CLOCK_SM
    BITS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown"}

    def __init__(self, index: int):
        import ctypes as C
        self.C = C
        self.lib = C.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit failed")
        self.h = C.c_void_p()
        if self.lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(index), C.byref(self.h)) != 0:
            raise RuntimeError("no NVML device %d" % index)
        self.reasons_fn = getattr(self.lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.lib.nvmlDeviceGetCurrentClocksThrottleReasons
        mx = C.c_uint()
        self.max_mhz = float(mx.value) if self.lib.nvmlDeviceGetMaxClockInfo(self.h, self.SM, C.byref(mx)) == 0 else None

    def sample(self):
        C = self.C
        clk, r = C.c_uint(), C.c_ulonglong()
        if self.lib.nvmlDeviceGetClockInfo(self.h, self.SM, C.byref(clk)) != 0:
            return None
        self.reasons_fn(self.h, C.byref(r))
        return float(clk.value), int(r.value)


class ClockSampler:
    """Samples the SM clock and throttle reasons while running: NVML polled
    about every millisecond from a thread (so that even a timed region of a
    few tens of milliseconds holds many samples), nvidia-smi at 200 ms when
    NVML cannot be loaded."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.nvml = None
        self.samples = []
        self.running = False

    def start(self):
        try:
            self.nvml = _Nvml(self.gpu)
            self.nvml.sample()
            self.running = True
            self.thread = threading.Thread(target=self._poll, daemon=True)
            self.thread.start()
            return
        except Exception:
            self.nvml = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _poll(self):
        while self.running:
            s = self.nvml.sample()
            if s is not None:
                self.samples.append(s)
            time.sleep(0.001)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.nvml is not None:
            self.running = False
            self.thread.join(timeout=5)
            sm = [c for c, _ in self.samples]
            reasons = sorted({n for _, r in self.samples for bit, n in _Nvml.BITS.items() if r & bit})
            return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": self.nvml.max_mhz,
                    "reasons": reasons, "samples": len(sm), "source": "nvml"}
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "source": "nvidia-smi"}


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


_NET = {}


def wall_net(wl, device):
    """The learned wall stress of a workload that uses it: trained once per
    process on 2^20 eqwm-labelled samples, half of them drawn from the
    solver's own wall-modelled runs across Re_tau 500-10000, with the
    project's own kernels."""
    key = (wl["ncv"], device)
    if key not in _NET:
        import torch
        from channelflow import wallmlp
        dev = torch.device("cuda", device)
        t0 = time.perf_counter()
        (u, h, nu, tau), n_solver = wallmlp.training_set_mixed(1 << 20, solver_fraction=0.5, seed=5200, device=dev,
                                                                ncv=wl["ncv"], stretch=1.10)
        t1 = time.perf_counter()
        net = wallmlp.WallMLP(seed=3, ncv=wl["ncv"], stretch=1.10)
        net.fit_normalisation(u, h, nu, tau)
        loss = net.train(u, h, nu, tau, epochs=8, batch=512, lr=3e-3, seed=0)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        ut, ht, nt, tt = wallmlp.training_set(1 << 16, seed=5201, device=dev, ncv=wl["ncv"], stretch=1.10,
                                              **wallmlp.OPERATING)
        err = (net.predict(ut, ht, nt) / tt - 1).abs()
        _NET[key] = (net, {"samples": int(u.numel()), "solver_samples": n_solver,
                           "harvest_and_label_seconds": t1 - t0, "train_seconds": t2 - t1,
                           "final_loss": float(loss[-1]), "heldout_max_rel_err": float(err.max()),
                           "heldout_mean_rel_err": float(err.mean())})
    return _NET[key]


def make_channel(wl, precision, device, seed, cfl=0.5):
    import channelflow as cf
    from channelflow import grids
    x, y, z = grids.channel_grid(wl["nx"], wl["ny"], wl["nz"], stretch=wl["stretch"])
    nu = grids.dean_nu(wl["retau"])
    U, V, W = grids.seeded_fields(x, y, z, seed=seed, profile=wl["profile"])
    prm = dict(nu=nu, CFL=cfl, dPdx=(wl["retau"] * nu) ** 2, LES_model=wl["les"], iwall_model=wl["wall"],
               x_mass_cte=1, jref_eqwm=wl["jref"], eqwm_ncv=wl["ncv"], precision=precision)
    ch = cf.Channel(x, y, z, device=device, **prm)
    if wl.get("mlp"):
        ch.set_wall_mlp(wall_net(wl, device)[0], check_every=100)
    ch.upload(U, V, W)
    ch.init_mass_flow()
    ch.apply_boundary_conditions()
    ch.set_scalars(dt=5e-3, rk_step=2)
    ch.compute_projection_step()
    ch.apply_boundary_conditions()
    return ch, (x, y, z, U, V, W, prm)


def cpu_baseline(wl, steps, threads, target_s=12.0):
    """The CPU oracle (C restatement of the reference CPU path, OpenMP) on the
    same workload: `steps` full RK3 steps after one untimed step; steps = 0
    takes as many as fill about `target_s` seconds at the untimed step's pace
    (at most 50)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import Oracle
    from channelflow import grids
    x, y, z = grids.channel_grid(wl["nx"], wl["ny"], wl["nz"], stretch=wl["stretch"])
    nu = grids.dean_nu(wl["retau"])
    U, V, W = grids.seeded_fields(x, y, z, seed=1, profile=wl["profile"])
    prm = dict(nu=nu, CFL=0.5, dPdx=(wl["retau"] * nu) ** 2, LES_model=wl["les"], iwall_model=wl["wall"],
               x_mass_cte=1, jref_eqwm=wl["jref"], eqwm_ncv=wl["ncv"])
    o = Oracle(x, y, z, prm, threads=threads)
    o.set_fields(U, V, W)
    o.init_mass_flow()
    o.apply_boundary_conditions()
    t0 = time.perf_counter()
    o.compute_dt(); o.time_step_rk3()
    if steps <= 0:
        steps = max(1, min(50, int(math.ceil(target_s / max(time.perf_counter() - t0, 1e-3)))))
    t0 = time.perf_counter()
    for _ in range(steps):
        o.compute_dt()
        o.time_step_rk3()
    dt = time.perf_counter() - t0
    o.close()
    nc = (wl["nx"] - 2) * (wl["ny"] - 1) * (wl["nz"] - 2)
    return nc * steps / dt, dt, steps


def long_run_stats(wl):
    """The committed result of the long-run split-vs-FP64 statistics
    comparison on developed turbulence for this workload (bench.py
    --stats-run with --stats-develop; about two minutes of FP64 steps, so it
    is not rerun by every bench invocation), or None."""
    try:
        tab = json.load(open(os.path.join(ROOT, "profiles", "stats_long_run.json")))
    except Exception:
        return None
    r = tab.get(wl["name"])
    if not r:
        return None
    keep = ("steps", "develop_steps", "retau", "error_split_vs_fp64 (max|a-b| / max|b|)",
            "error_fp64_perturbed_vs_fp64 (floor)", "command", "measured")
    return {k: r[k] for k in keep if k in r}


def channel_from_fields(wl, precision, device, fields, dPdx, cfl=0.5):
    """A channel of the workload's parameters started from given fields (a
    snapshot) with the given mean pressure gradient; its constant mass flow is
    the fields' own."""
    import channelflow as cf
    from channelflow import grids
    x, y, z, U, V, W = fields
    nu = grids.dean_nu(wl["retau"])
    prm = dict(nu=nu, CFL=cfl, dPdx=(wl["retau"] * nu) ** 2, LES_model=wl["les"], iwall_model=wl["wall"],
               x_mass_cte=1, jref_eqwm=wl["jref"], eqwm_ncv=wl["ncv"], precision=precision)
    ch = cf.Channel(x, y, z, device=device, **prm)
    ch.upload(U, V, W)
    ch.init_mass_flow()
    ch.apply_boundary_conditions()
    ch.set_scalars(dt=5e-3, rk_step=1, dPdx=dPdx)
    return ch


def profiles_of(mean, tail, ny):
    """Mean U+, u, v, w RMS and the uv Reynolds stress from time-averaged
    compute_statistics vectors (statistics.f90:43-118)."""
    import numpy as np
    U, V, W, U2, V2, W2, UV = (mean[q * ny:(q + 1) * ny] for q in range(7))
    utau = tail[0]
    return dict(Uplus=U / utau, urms=np.sqrt(np.maximum(U2 - U * U, 0.0)),
                vrms=np.sqrt(np.maximum(V2 - V * V, 0.0)), wrms=np.sqrt(np.maximum(W2 - W * W, 0.0)),
                uv=UV - U * V, utau=float(utau), retau=float(tail[1]))


def sample_run(ch, steps, every, ny):
    """Advances `steps` steps and time-averages compute_statistics sampled
    every `every` steps over the second half."""
    import numpy as np
    acc, tail, n = np.zeros(9 * ny), np.zeros(8), 0
    t0 = time.perf_counter()
    done = 0
    while done < steps:
        k = min(every, steps - done)
        ch.time_step_rk3(k)
        done += k
        if done > steps // 2:
            s = ch.statistics()
            acc += s[:9 * ny]
            tail += s[9 * ny:]
            n += 1
    out = profiles_of(acc / n, tail / n, ny)
    out.update(samples=n, seconds=time.perf_counter() - t0, finite=bool(np.isfinite(ch.download()["U"]).all()))
    return out


PROFILE_KEYS = ("Uplus", "urms", "vrms", "wrms", "uv")


def profile_errors(a, b):
    import numpy as np
    return {k: float(np.max(np.abs(a[k] - b[k])) / np.max(np.abs(b[k]))) for k in PROFILE_KEYS}


def stats_run(wl, steps, every, device, develop=0, perturb=6e-8, seed=1):
    """The long-run comparison of the split path against the FP64 path.

    develop > 0: the turbulent initial field (power-law mean plus large-scale
    modes) is advanced `develop` steps with the split path until the flow is
    turbulent (Re_tau is recorded along the way), written to and read back
    from a snapshot file in the reference's format, and three runs start from
    it: the FP64 path, the split path, and the FP64 path from the same field
    with every value perturbed by a relative `perturb` (the size of FP32
    rounding) -- the last one measures how far two FP64 runs that start a
    rounding error apart drift in the same window, the floor any precision
    change meets once the flow is chaotic.  develop = 0: both paths start from
    the seeded laminar field (no developed turbulence).
    Each run advances `steps` steps and time-averages compute_statistics
    (statistics.f90:43-159) sampled every `every` steps over the second half;
    mean U+, the u, v, w RMS and the uv Reynolds stress profiles are
    compared as max|a - b| / max|b|."""
    import tempfile
    import numpy as np
    import channelflow as cf
    ny = wl["ny"]
    line = {"workload": wl["name"], "steps": steps, "sample_every": every, "window": "second half"}
    if develop > 0:
        wl_t = dict(wl, profile="turbulent")
        ch, init = make_channel(wl_t, cf.PREC_SPLIT, device, seed=seed)
        hist = []
        t0 = time.perf_counter()
        done = 0
        while done < develop:
            k = min(1000, develop - done)
            ch.time_step_rk3(k)
            done += k
            s = ch.statistics()
            hist.append([done, round(float(s[9 * ny + 1]), 2)])
        dev_s = time.perf_counter() - t0
        f = ch.download()
        dPdx = ch.scalars()["dPdx"]
        ch.close()
        x, y, z = init[:3]
        with tempfile.TemporaryDirectory() as td:
            path = os.path.join(td, "developed.bin")
            cf.write_snapshot(path, x, y, z, f["U"], f["V"], f["W"], f["P"], f["nu_t"])
            fields = cf.read_snapshot(path, len(x), len(y), len(z))
        assert all(np.array_equal(fields[3 + q], f[k]) for q, k in enumerate("UVW"))
        line["develop"] = {"steps": develop, "precision": "split", "initial_field": "turbulent",
                           "retau_every_1000_steps": hist, "seconds": dev_s}
        runs = {}
        for name, prec in (("fp64", cf.PREC_FP64), ("split", cf.PREC_SPLIT), ("fp64_perturbed", cf.PREC_FP64)):
            flds = fields
            if name == "fp64_perturbed":
                rng = np.random.default_rng(seed + 100)
                flds = fields[:3] + tuple(np.asfortranarray(a * (1.0 + perturb * (2.0 * rng.random(a.shape) - 1.0)))
                                          for a in fields[3:])
            c = channel_from_fields(wl, prec, device, flds, dPdx)
            runs[name] = sample_run(c, steps, every, ny)
            c.close()
        b = runs["fp64"]
        line["error_split_vs_fp64 (max|a-b| / max|b|)"] = profile_errors(runs["split"], b)
        line["error_fp64_perturbed_vs_fp64 (floor)"] = profile_errors(runs["fp64_perturbed"], b)
        line["perturbation"] = perturb
    else:
        runs = {}
        for name, prec in (("fp64", cf.PREC_FP64), ("split", cf.PREC_SPLIT)):
            ch, init = make_channel(wl, prec, device, seed=seed)
            runs[name] = sample_run(ch, steps, every, ny)
            ch.close()
        line["error_split_vs_fp64 (max|a-b| / max|b|)"] = profile_errors(runs["split"], runs["fp64"])
    line["samples"] = runs["fp64"]["samples"]
    line["utau"] = {k: r["utau"] for k, r in runs.items()}
    line["retau"] = {k: r["retau"] for k, r in runs.items()}
    line["wall_seconds"] = {k: r["seconds"] for k, r in runs.items()}
    line["finite"] = all(r["finite"] for r in runs.values())
    line["profiles"] = {k: {q: [float(v) for v in r[q]] for q in PROFILE_KEYS} for k, r in runs.items()}
    print(json.dumps({"stats_run": line}))


ENSEMBLE = {"name": "ensemble of 16 channels: 6x(64x64x64), 6x(96x64x96), 4x(128x96x128), Re_tau from "
                    "{180, 395, 550}, DSM, no-slip, constant mass flow", "members": [(66, 65, 66)] * 6 +
            [(98, 65, 98)] * 6 + [(130, 97, 130)] * 4}


def ensemble_members(precision, device):
    """The 16 members: own seed, own Re_tau (seeded draw from 180, 395, 550),
    own perturbed laminar field and mass-flow target."""
    import numpy as np
    import channelflow as cf
    rng = np.random.default_rng(16)
    out = []
    for q, (nx, ny, nz) in enumerate(ENSEMBLE["members"]):
        retau = float(rng.choice([180.0, 395.0, 550.0]))
        wl = dict(nx=nx, ny=ny, nz=nz, retau=retau, stretch=1.5, les=2, wall=0, jref=3, ncv=100, profile="laminar")
        ch, _ = make_channel(wl, precision, device, seed=100 + q)
        out.append((ch, retau))
    return out


def run_ensemble(args, rank, world, local):
    """The ensemble workload: every member advanced by one ensemble step per
    step (one CUDA graph with a branch per member), against the same members
    stepped one after another on their own streams."""
    import numpy as np
    import torch
    import channelflow as cf
    dev = local
    torch.cuda.set_device(dev)
    mem = ensemble_members(cf.PREC_SPLIT, dev)
    chans = [m[0] for m in mem]
    nc = sum((c.nx - 2) * (c.ny - 1) * (c.nz - 2) for c in chans)
    tuned = None
    if args.autotune:
        # each grid shape picks its own chunking on its own warmed-up state
        tuned = []
        for c in chans:
            c.time_step_rk3(1)
            tuned.append(c.autotune(reps=2))
    ens = cf.Ensemble(chans, batched_tri=True)
    ens.step(args.warmup)
    ens_tuned = ens.autotune(steps=3) if args.autotune else None
    strm = torch.cuda.ExternalStream(ens.stream(), device=torch.device("cuda", dev))
    torch.cuda.synchronize()
    sampler = ClockSampler(dev)
    sampler.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(strm)
    ens.step(args.steps, sync=False)
    e1.record(strm)
    e1.synchronize()
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1)
    value = world * nc * args.steps / (ms / 1e3)
    # the same ensemble with every kernel in the members' branches (no
    # batched stencil launches), for comparison
    ens_b = cf.Ensemble(chans, batched_tri=False, batched_stencils=False)
    ens_b.step(args.warmup)
    strm_b = torch.cuda.ExternalStream(ens_b.stream(), device=torch.device("cuda", dev))
    torch.cuda.synchronize()
    e0.record(strm_b)
    ens_b.step(args.steps, sync=False)
    e1.record(strm_b)
    e1.synchronize()
    ms_b = e0.elapsed_time(e1)
    ens_b.close()
    # the same members stepped one after another (each its own graph)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for c in chans:
        c.time_step_rk3(args.steps, sync=True)
    seq = time.perf_counter() - t0
    # end to end: every member's fields up from and back to pinned host arrays each step
    pinned = []
    for c in chans:
        d = c.download()
        bufs = {}
        for k in ("U", "V", "W"):
            t = torch.empty(int(np.prod(c.shapes[k])), dtype=torch.float64, pin_memory=True)
            bufs[k] = t.numpy().reshape(c.shapes[k], order="F")
            bufs[k][...] = d[k]
        pinned.append(bufs)
    ke = max(2, min(args.steps, 5))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(ke):
        for c, b in zip(chans, pinned):
            c.upload(b["U"], b["V"], b["W"])
        ens.step(1, sync=False)
        for c, b in zip(chans, pinned):
            c.download_into(U=b["U"], V=b["V"], W=b["W"])
    torch.cuda.synchronize()
    te = time.perf_counter() - t0
    nbytes = sum(8 * sum(int(np.prod(c.shapes[k])) for k in ("U", "V", "W")) for c in chans)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        # one member of each grid through the CPU oracle, scaled by the member counts
        thr = os.cpu_count() or 1
        tot_s, tot_c, sample = 0.0, 0, []
        for nx, ny, nz, cnt in ((66, 65, 66, 6), (98, 65, 98, 6), (130, 97, 130, 4)):
            wl = dict(nx=nx, ny=ny, nz=nz, retau=395.0, stretch=1.5, les=2, wall=0, jref=3, ncv=100,
                      profile="laminar")
            v, sec, nst = cpu_baseline(wl, 0, thr, target_s=4.0)
            cells = (nx - 2) * (ny - 1) * (nz - 2)
            tot_s += cnt * cells / v
            tot_c += cnt * cells
            sample.append(f"{nst} steps of {nx}x{ny}x{nz} ({sec:.1f} s)")
        cpu = {"value": tot_c / tot_s, "unit": UNIT, "cores": thr, "kind": "port",
               "sample": "RK3 steps of one member of each grid: " + ", ".join(sample) +
                         " (C restatement of the reference CPU path, OpenMP), the ensemble's time as the "
                         "members' sum"}
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64 (split)", "data": "synthetic (16 seeded perturbed laminar fields)",
            "config": {"workload": ENSEMBLE["name"], "members": len(chans), "grid_points": nc,
                       "retau": [m[1] for m in mem], "precision": "split",
                       "graph": ("one CUDA graph per ensemble step: " +
                                 ("the tridiagonal systems of all members in one FP64 launch per substep; "
                                  if ens_tuned and "batched FP64" in ens_tuned["choice"] else
                                  "each member's tridiagonal solves in its branch; ") +
                                 ("every other kernel in a branch per member"
                                  if ens_tuned and ens_tuned["choice"].startswith("branches") else
                                  "the fused DSM passes and fused right-hand sides of all members as one launch "
                                  "each per substep, the other kernels in a branch per member") +
                                 " (chosen by cf_ensemble_autotune)"),
                       "autotune": None if tuned is None else sorted({(t["rhs_chunks"], t["dsm_chunk_len"])
                                                                     for t in tuned}),
                       "l2": "members' working set (~2.5 GB) larger than L2; no flush needed"},
            "ensemble_autotune": ens_tuned,
            "branches_only": {"value": world * nc * args.steps / (ms_b / 1e3), "ms_per_step": ms_b / args.steps,
                              "how": "the same ensemble graph with every kernel (tridiagonal solves included) "
                                     "in the members' branches"},
            "sequential_members": {"value": world * nc * args.steps / seq, "ms_per_step": 1e3 * seq / args.steps,
                                   "how": "each member's own graph, one member after another"},
            "ensemble_over_sequential": (world * nc * args.steps / seq and value / (world * nc * args.steps / seq)),
            "cpu_baseline": cpu,
            "e2e": dict({"value": world * nc * ke / te, "unit": UNIT, "h2d_bytes_per_step": nbytes,
                         "d2h_bytes_per_step": nbytes, "steps": ke,
                         "path": "cf_upload_fields x16 + cf_ensemble_step + cf_download_fields x16, pinned host buffers"},
                        **host_link(nbytes, dev)),
            "gpu_launches": ens.launches_per_step() * args.steps,
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    ens.close()
    for c in chans:
        c.close()


def run_reference(args, wl, rank, world):
    """Reference arm: the reference's CPU path (its C restatement; the Fortran
    reference needs ifort/MPI/FFTW, absent here) on all host threads."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    nc = (wl["nx"] - 2) * (wl["ny"] - 1) * (wl["nz"] - 2)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import Oracle
    from channelflow import grids
    x, y, z = grids.channel_grid(wl["nx"], wl["ny"], wl["nz"], stretch=wl["stretch"])
    nu = grids.dean_nu(wl["retau"])
    U, V, W = grids.seeded_fields(x, y, z, seed=1, profile=wl["profile"])
    prm = dict(nu=nu, CFL=0.5, dPdx=(wl["retau"] * nu) ** 2, LES_model=wl["les"], iwall_model=wl["wall"],
               x_mass_cte=1, jref_eqwm=wl["jref"], eqwm_ncv=wl["ncv"])
    o = Oracle(x, y, z, prm, threads=threads)
    o.set_fields(U, V, W)
    o.init_mass_flow()
    o.apply_boundary_conditions()
    for _ in range(args.warmup):
        o.compute_dt(); o.time_step_rk3()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.compute_dt(); o.time_step_rk3()
    el = time.perf_counter() - t0
    v = nc * args.steps / el
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": wl["name"], "faces": [wl["nx"], wl["ny"], wl["nz"]], "grid_points": nc},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full RK3 steps of the workload (C restatement of the reference "
                                   f"CPU path, OpenMP, {threads} threads)"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, wl, rank, world, local):
    import numpy as np
    import torch
    import channelflow as cf
    dev = local
    torch.cuda.set_device(dev)
    dist = world > 1
    if dist:
        import torch.distributed as td
        td.init_process_group("nccl", device_id=torch.device("cuda", dev))
    nc = (wl["nx"] - 2) * (wl["ny"] - 1) * (wl["nz"] - 2)

    def barrier():
        torch.cuda.synchronize()
        if dist:
            td.barrier()
        torch.cuda.synchronize()

    # ---- split path (headline) and FP64 path from the same initial field
    ch, init = make_channel(wl, cf.PREC_SPLIT, dev, seed=1 + rank)
    ch64, _ = make_channel(wl, cf.PREC_FP64, dev, seed=1 + rank)
    ncmp = max(args.warmup, 3)
    ch.time_step_rk3(ncmp)
    ch64.time_step_rk3(ncmp)
    tuned = ch.autotune(reps=3) if args.autotune else None
    s32, s64 = ch.statistics(), ch64.statistics()
    ny = wl["ny"]
    prof_err = {}
    for idx, nm in ((0, "U_mean"), (3, "U2_mean"), (4, "V2_mean"), (5, "W2_mean"), (6, "UV_mean")):
        a, b = s32[idx * ny:(idx + 1) * ny], s64[idx * ny:(idx + 1) * ny]
        prof_err[nm] = float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
    stream = torch.cuda.ExternalStream(ch.stream(), device=torch.device("cuda", dev))

    def timed(c, steps, strm):
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(strm)
        c.time_step_rk3(steps, sync=False)
        e1.record(strm)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        if dist:
            t = torch.tensor([ms], device="cuda")
            td.all_reduce(t, op=td.ReduceOp.MAX)
            ms = float(t.item())
        return ms

    sampler = ClockSampler(int(os.environ.get("CUDA_VISIBLE_DEVICES", str(dev)).split(",")[0])
                           if os.environ.get("CUDA_VISIBLE_DEVICES", "").replace(",", "").isdigit() else dev)
    sampler.start()
    ms = timed(ch, args.steps, stream)
    clocks = sampler.stop()
    value = world * nc * args.steps / (ms / 1e3)

    # FP64 path (fewer steps: the FP64 units of GB300 run at ~1/40 of FP32)
    k64 = max(2, min(args.steps, 6))
    stream64 = torch.cuda.ExternalStream(ch64.stream(), device=torch.device("cuda", dev))
    ms64 = timed(ch64, k64, stream64)
    v64 = world * nc * k64 / (ms64 / 1e3)

    # ---- per-kernel device time: two steps, each captured as one graph with
    # an event-record node after every kernel and launched like the timed
    # step graphs
    prof = ch.profile_steps(2, graph=True)
    tot = sum(v[0] for v in prof.values())
    top = sorted(prof.items(), key=lambda kv: -kv[1][0])
    dom, (dom_ms, dom_n) = top[0]
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    ab = algorithmic_bytes(dom, ch, 4)
    avg_s = dom_ms / dom_n / 1e3
    traffic, wavefronts = None, None
    try:
        tj = json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))
        traffic = tj.get(wl["name"], {}).get(dom)
        wavefronts = tj.get(wl["name"], {}).get(dom + ":smem_wavefronts")
    except Exception:
        pass
    roof = {"kernel": dom, "bound": "hbm", "unit": "GB/s", "peak": hbm_peak, "peak_source": peak_src,
            "achieved": (ab / avg_s / 1e9) if ab else None, "frac": (ab / avg_s / 1e9 / hbm_peak) if ab else None,
            "traffic": traffic, "avg_launch_ms": avg_s * 1e3, "launches_per_step": dom_n / 2,
            "share_of_step": dom_ms / tot if tot else None,
            "timing": "CUDA events captured as graph nodes around each launch of two graph-launched steps",
            "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum of one ncu launch of this kernel on "
                              "this workload (profiles/traffic.json)"}
    if wavefronts:
        # the bound the kernel actually meets: shared-memory wavefronts of one
        # launch (ncu) at one per clock per SM, at the clock sampled above
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        mhz = clocks.get("sm_mhz") or 2070.0
        floor_s = wavefronts / sms / (mhz * 1e6)
        roof["smem_bound"] = {"wavefronts_per_launch": wavefronts, "floor_ms": floor_s * 1e3,
                              "frac": floor_s / avg_s, "how": "ncu l1tex__data_pipe_lsu_wavefronts_mem_shared.sum "
                              "of one launch / (SMs x SM clock)"}

    # ---- end to end through the public API with host buffers
    shp = ch.shapes
    pinned = {}
    for k in ("U", "V", "W"):
        n = int(np.prod(shp[k]))
        t = torch.empty(n, dtype=torch.float64, pin_memory=True)
        pinned[k] = t.numpy().reshape(shp[k], order="F")
    d = ch.download()
    for k in ("U", "V", "W"):
        pinned[k][...] = d[k]
    ke = max(2, min(args.steps, 10))
    barrier()
    t0 = time.perf_counter()
    for _ in range(ke):
        ch.upload(pinned["U"], pinned["V"], pinned["W"])
        ch.time_step_rk3(1, sync=False)
        ch.download_into(U=pinned["U"], V=pinned["V"], W=pinned["W"])
    torch.cuda.synchronize()
    te = time.perf_counter() - t0
    if dist:
        t = torch.tensor([te], device="cuda")
        td.all_reduce(t, op=td.ReduceOp.MAX)
        te = float(t.item())
    nbytes = 8 * sum(int(np.prod(shp[k])) for k in ("U", "V", "W"))
    e2e = {"value": world * nc * ke / te, "unit": UNIT, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
           "steps": ke, "path": "cf_upload_fields + cf_time_step_rk3 + cf_download_fields, pinned host buffers"}
    e2e.update(host_link(nbytes, dev))

    # ---- CPU baseline (rank 0, N = 1 only)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        thr = os.cpu_count() or 1
        cv, csec, cst = cpu_baseline(wl, args.cpu_steps, thr)
        cpu = {"value": cv, "unit": UNIT, "cores": thr, "kind": "port",
               "sample": f"{cst} full RK3 steps of the same workload after 1 untimed step "
                         f"({csec:.1f} s; C restatement of the reference CPU path, OpenMP)"}

    launches = ch.launches_per_step() * args.steps
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64 (split: FP32 state/stencils/SGS, FP64 tridiagonal, mean mode, "
                                          "reductions)",
            "data": "synthetic (seeded perturbed laminar field, projected)",
            "config": {"workload": wl["name"], "faces": [wl["nx"], wl["ny"], wl["nz"]], "grid_points": nc,
                       "precision": "split", "dt_rule": "reference compute_dt (CFL 0.5 -> 5e-3 cap)",
                       "l2": "working set (~1 GB) larger than L2 (129 MB); no flush needed",
                       "replicas": world, "graph": "one CUDA graph per step",
                       "sgs_recompute": True, "autotune": tuned},
            "fp64": {"value": v64, "ms_per_step": ms64 / k64, "steps": k64},
            "split_over_fp64": value / v64,
            "short_horizon_err_vs_fp64": {"steps": ncmp, "what": "profile errors after a few steps from the same "
                                          "field; the long-run gate on developed turbulence is long_run_stats",
                                          **prof_err},
            "long_run_stats": long_run_stats(wl),
            "hbm_frac_step": value / world * BYTES_PER_PT_STEP["split"] / (hbm_peak * 1e9),
            "roofline": roof,
            "kernels_ms_per_step": {k: round(v[0] / 2, 4) for k, v in top[:10]},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": launches,
            "clocks": clocks,
        }
        if wl.get("mlp"):
            net_info = dict(wall_net(wl, dev)[1])
            net_info["checked_in_run"] = ch.wall_mlp_log()
            line["wall_mlp"] = net_info
        print(json.dumps(line), flush=True)
    ch.close()
    ch64.close()
    if dist:
        td.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="re550", choices=sorted(WORKLOADS) + ["ensemble16"])
    ap.add_argument("--cpu-steps", type=int, default=0,
                    help="steps of the CPU baseline (0: as many as fill about 12 s)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--profile-steps", type=int, default=0,
                    help="only run N steps of the split path after one warm-up step (for ncu)")
    ap.add_argument("--precision", default="split", choices=["split", "fp64"])
    ap.add_argument("--kernel-table", action="store_true",
                    help="with --profile-steps: also print per-kernel event times of two more steps")
    ap.add_argument("--autotune", type=int, default=1,
                    help="1: tune the z-chunk counts of the marching kernels on the warmed-up state (cf_autotune)")
    ap.add_argument("--stats-run", type=int, default=0,
                    help="only run the long-run statistics comparison of the split and FP64 paths over N steps")
    ap.add_argument("--stats-every", type=int, default=10)
    ap.add_argument("--stats-develop", type=int, default=0,
                    help="with --stats-run: first develop turbulence from the turbulent initial field for N split "
                         "steps, then compare FP64, split and a perturbed FP64 run from it")
    args = ap.parse_args()
    rank, world, local = dist_info()
    if args.workload == "ensemble16":
        if args.impl == "reference":
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the reference arm is timed on the "
                                  "single-channel workloads"}))
            return
        run_ensemble(args, rank, world, local)
        return
    wl = WORKLOADS[args.workload]
    if args.stats_run:
        stats_run(wl, args.stats_run, args.stats_every, local, develop=args.stats_develop)
        return
    if args.profile_steps:
        import channelflow as cf
        ch, _ = make_channel(wl, cf.PREC_SPLIT if args.precision == "split" else cf.PREC_FP64, local, seed=1)
        ch.time_step_rk3(1)
        ch.time_step_rk3(args.profile_steps)
        print(json.dumps({"profile_steps": args.profile_steps, "launches_per_step": ch.launches_per_step()}))
        if args.kernel_table:
            prof = ch.profile_steps(2, graph=True)
            tot = sum(v[0] for v in prof.values())
            for k, (ms, n) in sorted(prof.items(), key=lambda kv: -kv[1][0]):
                print(f"{k:16s} {n / 2:5.1f}/step {1e3 * ms / 2:9.1f} us/step {100 * ms / tot:5.1f}%"
                      f"  avg {1e3 * ms / n:8.1f} us")
            print(f"total {1e3 * tot / 2:.1f} us/step")
        ch.close()
        return
    if args.impl == "reference":
        run_reference(args, wl, rank, world)
    else:
        run_ours(args, wl, rank, world, local)


if __name__ == "__main__":
    main()
