"""Learned wall-stress model: Python side of the cf_mlp_* / cf_eqwm_solve_batch
entry points (device arrays are torch CUDA tensors; torch is used for device
memory only).

The network replaces the per-point ODE solve of the equilibrium wall model
(solve_u_eqwm, eqwm.f90:90-223) by a 3 -> 64 -> 64 -> 1 tanh map of
(log u_les, log matching height, log nu) to log tau_w, trained on labels the
batched eqwm solve produces."""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import grids
from .lib import CfError, load

NPARAM = 4481


def _bind():
    L = load()
    vp, dp, ip, fp = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_float)
    if getattr(L, "_wmlp_bound", False):
        return L
    L.cf_eqwm_solve_batch.argtypes = [C.c_int, vp, vp, vp, C.c_int, C.c_double, C.c_double, vp, vp, vp]
    L.cf_mlp_create.argtypes = [C.c_int, C.c_int, C.c_double, C.POINTER(vp)]
    L.cf_mlp_destroy.argtypes = [vp]
    L.cf_mlp_fit_normalisation.argtypes = [vp, C.c_int, vp, vp, vp, vp, vp]
    L.cf_mlp_train.argtypes = [vp, C.c_int, vp, vp, vp, vp, C.c_int, C.c_int, C.c_double, C.c_int, dp, vp]
    L.cf_mlp_gradient.argtypes = [vp, C.c_int, vp, vp, vp, vp, vp, dp, vp]
    L.cf_mlp_predict.argtypes = [vp, C.c_int, vp, vp, vp, vp, vp, C.c_int, vp]
    L.cf_mlp_get.argtypes = [vp, fp, dp, dp]
    L.cf_mlp_set.argtypes = [vp, fp, dp, dp]
    L.cf_set_wall_mlp.argtypes = [vp, vp, C.c_int]
    L.cf_get_wall_mlp_log.argtypes = [vp, dp]
    L.cf_mlp_wait_expired.argtypes = [vp, ip]
    L.cf_wall_model_inputs.argtypes = [vp, vp, C.c_long, C.POINTER(C.c_long), dp, dp]
    L.cf_mlp_set_train_tensor_cores.argtypes = [vp, C.c_int]
    L.cf_mlp_test_skip_mma.argtypes = [vp, C.c_int]
    L._wmlp_bound = True
    return L


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream(t):
    import torch
    return C.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)


def _check(L, rc, what):
    if rc != 0:
        raise CfError(f"{what} failed ({rc}): {L.cf_last_error(None).decode()}")


def eqwm_solve_batch(u, h, nu, ncv=30, stretch=1.10, tau_init=1e-3, iters=False):
    """eqwm wall stress per sample (device float64 tensors of one length)."""
    import torch
    L = _bind()
    n = u.numel()
    tau = torch.empty_like(u)
    it = torch.empty(n, dtype=torch.int32, device=u.device) if iters else None
    _check(L, L.cf_eqwm_solve_batch(n, _ptr(u), _ptr(h), _ptr(nu), ncv, stretch, tau_init, _ptr(tau), _ptr(it),
                                    _stream(u)), "cf_eqwm_solve_batch")
    return (tau, it) if iters else tau


# The operating range the network is checked on: channels at Re_tau 500-10000
# matched at 0.04-0.2 half-heights, instantaneous u_les within about +-25 % of
# the log law.  The training distribution (the defaults of training_inputs)
# extends it on every side, so that the operating range lies inside the
# training envelope rather than at its sparse edges.
OPERATING = dict(retau=(500.0, 10000.0), height=(0.04, 0.2), spread=0.25)


def training_inputs(n: int, seed: int = 0, retau=(250.0, 20000.0), height=(0.03, 0.3), spread=0.35):
    """Seeded inputs (u_les, h, nu) of wall-modelled channels (bulk velocity 1,
    half-height 1): Re_tau log-uniform in `retau`, nu from Dean's correlation,
    matching height log-uniform in `height`, u_les the log-law velocity at h
    times 1 + spread * N(0, 1) clipped to [0.3, 1.9]."""
    rng = np.random.Generator(np.random.Philox(seed))
    re = np.exp(rng.uniform(math.log(retau[0]), math.log(retau[1]), n))
    nu = np.array([grids.dean_nu(r) for r in re]) if n < 4096 else 2.0 / (re / 0.09) ** (1.0 / 0.88)
    utau = re * nu
    h = np.exp(rng.uniform(math.log(height[0]), math.log(height[1]), n))
    ulog = utau * (np.log(h * utau / nu) / 0.41 + 5.2)
    f = np.clip(1.0 + spread * rng.standard_normal(n), 0.3, 1.9)
    return ulog * f, h, nu


def training_set(n: int, seed: int = 0, device=None, ncv: int = 30, stretch: float = 1.10, **kw):
    """n inputs of training_inputs labelled by the batched eqwm solve, as
    device float64 tensors (u, h, nu, tau); samples whose solve did not
    converge within the reference's 100 passes are dropped."""
    import torch
    dev = device or torch.device("cuda", torch.cuda.current_device())
    u, h, nu = training_inputs(n, seed=seed, **kw)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    u, h, nu = T(u), T(h), T(nu)
    tau, it = eqwm_solve_batch(u, h, nu, ncv=ncv, stretch=stretch, iters=True)
    keep = (it < 100) & torch.isfinite(tau) & (tau > 0)
    return u[keep].contiguous(), h[keep].contiguous(), nu[keep].contiguous(), tau[keep].contiguous()


def wall_model_inputs(channel):
    """The inputs the equilibrium wall model of `channel` (iwall_model 3)
    hands to its eqwm solve for the current fields: (u_les, h, nu) with u_les
    a device float64 tensor of every wall point's matching-plane velocity
    (wallmodel.f90:597-621) and h, nu the matching height and viscosity."""
    import torch
    L = _bind()
    n, h, nu = C.c_long(), C.c_double(), C.c_double()
    _check(L, L.cf_wall_model_inputs(channel.h, None, 0, C.byref(n), C.byref(h), C.byref(nu)), "cf_wall_model_inputs")
    u = torch.empty(n.value, dtype=torch.float64, device=torch.device("cuda", channel.device))
    _check(L, L.cf_wall_model_inputs(channel.h, _ptr(u), n.value, C.byref(n), C.byref(h), C.byref(nu)),
           "cf_wall_model_inputs")
    return u, h.value, nu.value


# Wall-modelled channels that supply solver samples: the layout of the
# Re_tau 2000 configuration (2 pi x 2 x pi, uniform wall-normal grid, dynamic
# Smagorinsky, equilibrium wall model, plug initial field) on a 64 x 48 x 64
# grid, at friction Reynolds numbers spanning the operating range, matched at
# the 3rd, 4th and 5th cell centres (0.06, 0.10, 0.15 half-heights).
HARVEST_RUNS = ((500.0, 4), (1000.0, 3), (2000.0, 5), (4000.0, 4), (7000.0, 3), (10000.0, 5))


def harvest_inputs(n: int, device=None, runs=HARVEST_RUNS, faces=(66, 49, 66), warm=600, every=40, ncv: int = 30,
                   stretch: float = 1.10, seed: int = 1):
    """About n wall-model inputs (u_les, h, nu) drawn from the solver's own
    wall-modelled runs: each run of `runs` (Re_tau, jref) is advanced `warm`
    split-path steps from its seeded plug field, then its wall-model inputs
    are collected every `every` steps until it has supplied its share.
    Returns device float64 tensors (u, h, nu) and the steps run."""
    import torch
    from . import lib
    dev = device or torch.device("cuda", torch.cuda.current_device())
    x, y, z = grids.channel_grid(*faces, stretch=0.0)
    share = -(-n // len(runs))
    us, hs, nus, steps = [], [], [], 0
    for q, (retau, jref) in enumerate(runs):
        nu = grids.dean_nu(retau)
        U, V, W = grids.seeded_fields(x, y, z, seed=seed + q, profile="plug")
        ch = lib.Channel(x, y, z, device=dev.index or 0, precision=lib.PREC_SPLIT, nu=nu, CFL=0.5,
                         dPdx=(retau * nu) ** 2, LES_model=2, iwall_model=3, x_mass_cte=1, jref_eqwm=jref,
                         eqwm_ncv=ncv, eqwm_stretch=stretch)
        ch.upload(U, V, W)
        ch.init_mass_flow()
        ch.apply_boundary_conditions()
        ch.time_step_rk3(warm)
        steps += warm
        got = 0
        while got < share:
            ch.time_step_rk3(every)
            steps += every
            u, h, nuv = wall_model_inputs(ch)
            us.append(u)
            hs.append(torch.full_like(u, h))
            nus.append(torch.full_like(u, nuv))
            got += u.numel()
        ch.close()
    return torch.cat(us)[:n].contiguous(), torch.cat(hs)[:n].contiguous(), torch.cat(nus)[:n].contiguous(), steps


def training_set_mixed(n: int, solver_fraction: float = 0.5, seed: int = 0, device=None, ncv: int = 30,
                       stretch: float = 1.10, **kw):
    """n labelled samples: a solver_fraction share drawn from the solver's own
    wall-modelled runs (harvest_inputs), the rest from training_inputs (which
    covers the envelope around the operating range evenly), all labelled by
    the batched eqwm solve; unconverged solves are dropped.  Returns (u, h, nu,
    tau) and the number of solver samples kept."""
    import torch
    dev = device or torch.device("cuda", torch.cuda.current_device())
    ns = int(n * solver_fraction)
    hu, hh, hn, _ = harvest_inputs(ns, device=dev, ncv=ncv, stretch=stretch, seed=seed + 1)
    su, sh, sn = training_inputs(n - ns, seed=seed, **kw)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    src = torch.cat([torch.ones(hu.numel(), dtype=torch.bool, device=dev),
                     torch.zeros(n - ns, dtype=torch.bool, device=dev)])
    u, h, nu = torch.cat([hu, T(su)]), torch.cat([hh, T(sh)]), torch.cat([hn, T(sn)])
    tau, it = eqwm_solve_batch(u, h, nu, ncv=ncv, stretch=stretch, iters=True)
    keep = (it < 100) & torch.isfinite(tau) & (tau > 0)
    return ((u[keep].contiguous(), h[keep].contiguous(), nu[keep].contiguous(), tau[keep].contiguous()),
            int((keep & src).sum().item()))


class WallMLP:
    """A device-resident network (FP32 master weights, Adam state)."""

    def __init__(self, seed: int = 0, ncv: int = 30, stretch: float = 1.10):
        self.L = _bind()
        h = C.c_void_p()
        _check(self.L, self.L.cf_mlp_create(seed, ncv, stretch, C.byref(h)), "cf_mlp_create")
        self.h = h
        self.ncv, self.stretch = ncv, stretch

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.L.cf_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def fit_normalisation(self, u, h, nu, tau):
        _check(self.L, self.L.cf_mlp_fit_normalisation(self.h, u.numel(), _ptr(u), _ptr(h), _ptr(nu), _ptr(tau),
                                                        _stream(u)), "cf_mlp_fit_normalisation")

    def train(self, u, h, nu, tau, epochs=20, batch=4096, lr=3e-3, seed=0):
        loss = np.zeros(epochs)
        _check(self.L, self.L.cf_mlp_train(self.h, u.numel(), _ptr(u), _ptr(h), _ptr(nu), _ptr(tau), epochs, batch,
                                            lr, seed, loss.ctypes.data_as(C.POINTER(C.c_double)), _stream(u)),
               "cf_mlp_train")
        return loss

    def gradient(self, u, h, nu, tau):
        import torch
        g = torch.empty(NPARAM, dtype=torch.float64, device=u.device)
        loss = C.c_double()
        _check(self.L, self.L.cf_mlp_gradient(self.h, u.numel(), _ptr(u), _ptr(h), _ptr(nu), _ptr(tau), _ptr(g),
                                               C.byref(loss), _stream(u)), "cf_mlp_gradient")
        return g, loss.value

    def predict(self, u, h, nu, tensor_cores=True, inside=False):
        import torch
        tau = torch.empty_like(u)
        ins = torch.empty(u.numel(), dtype=torch.int32, device=u.device) if inside else None
        _check(self.L, self.L.cf_mlp_predict(self.h, u.numel(), _ptr(u), _ptr(h), _ptr(nu), _ptr(tau), _ptr(ins),
                                              1 if tensor_cores else 0, _stream(u)), "cf_mlp_predict")
        return (tau, ins) if inside else tau

    def train_tensor_cores(self, on: bool):
        """Gradients with layer 2's products on the tensor cores (default) or,
        on=False, on the FP32 pipes."""
        _check(self.L, self.L.cf_mlp_set_train_tensor_cores(self.h, 1 if on else 0), "cf_mlp_set_train_tensor_cores")

    def wait_expired(self) -> bool:
        """True when a tensor-core inference since the last call gave up
        waiting for its MMA (its unfinished samples were left to eqwm); clears
        the record."""
        e = C.c_int()
        _check(self.L, self.L.cf_mlp_wait_expired(self.h, C.byref(e)), "cf_mlp_wait_expired")
        return bool(e.value)

    def test_skip_mma(self, on: bool):
        """Test hook: the tensor-core inference issues no MMA, so its bounded
        waits run out."""
        _check(self.L, self.L.cf_mlp_test_skip_mma(self.h, 1 if on else 0), "cf_mlp_test_skip_mma")

    def get(self):
        p = np.zeros(NPARAM, dtype=np.float32)
        norm, env = np.zeros(8), np.zeros(6)
        _check(self.L, self.L.cf_mlp_get(self.h, p.ctypes.data_as(C.POINTER(C.c_float)),
                                          norm.ctypes.data_as(C.POINTER(C.c_double)),
                                          env.ctypes.data_as(C.POINTER(C.c_double))), "cf_mlp_get")
        return p, norm, env

    def set(self, params=None, norm=None, env=None):
        f = lambda a, t, ct: None if a is None else np.ascontiguousarray(a, dtype=t).ctypes.data_as(C.POINTER(ct))
        keep = [np.ascontiguousarray(a, dtype=t) if a is not None else None
                for a, t in ((params, np.float32), (norm, np.float64), (env, np.float64))]
        _check(self.L, self.L.cf_mlp_set(self.h, f(keep[0], np.float32, C.c_float), f(keep[1], np.float64, C.c_double),
                                          f(keep[2], np.float64, C.c_double)), "cf_mlp_set")
