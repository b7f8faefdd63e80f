"""ctypes binding of libchannel_gpu.so and a host mirror of the reference's
time-integration interface (time_integration.f90).

``Channel`` exposes the subroutines that ``compute_time_step_RK3`` calls under
their Fortran names (``compute_eddy_viscosity``, ``compute_rhs_u``, ...,
``compute_projection_step``) plus the device fast path ``time_step_rk3``.
Every call goes through the C ABI declared in include/channel_gpu.h; there is
no CPU fallback: a missing or unloadable library raises immediately.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import re

import numpy as np

from . import grids

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
ROOT = os.path.dirname(PKG)
LIB_PATH = os.path.join(PKG, "libchannel_gpu.so")
HEADER = os.path.join(ROOT, "include", "channel_gpu.h")

PREC_FP64, PREC_SPLIT = 0, 1
ENS_TUNE_CANDIDATES = 8  # CF_ENS_TUNE_CANDIDATES


class CfParams(C.Structure):
    _fields_ = [
        ("nu", C.c_double), ("CFL", C.c_double), ("dPdx", C.c_double), ("dPdz", C.c_double),
        ("Rossby_plus", C.c_double), ("freq_mult", C.c_double),
        ("Retau_int", C.c_int), ("x_mass_cte", C.c_int), ("y_mass_cte", C.c_int),
        ("LES_model", C.c_int), ("iwall_model", C.c_int), ("Dirichlet_nu_t", C.c_int), ("jref_eqwm", C.c_int),
        ("precision", C.c_int), ("eqwm_ncv", C.c_int), ("eqwm_stretch", C.c_double), ("sgs_recompute", C.c_int),
        ("dsm_unfused", C.c_int), ("cfl_corrected", C.c_int),
    ]


class CfError(RuntimeError):
    pass


_lib = None


def header_functions() -> list[str]:
    """Names of the functions declared in include/channel_gpu.h."""
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(cf_[a-z0-9_]+)\s*\(", src)))


def load(build_if_missing: bool = True):
    """Loads the library (building it in-tree when it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise CfError(f"{LIB_PATH} not built")
        import importlib.util
        spec = importlib.util.spec_from_file_location("build_lib", os.path.join(PKG, "build_lib.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    L = C.CDLL(LIB_PATH)
    vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int)
    L.cf_default_params.argtypes = [C.POINTER(CfParams)]
    L.cf_default_params.restype = None
    L.cf_create.argtypes = [C.c_int, C.c_int, C.c_int, dp, dp, dp, C.POINTER(CfParams), C.c_int, C.POINTER(vp)]
    L.cf_last_error.argtypes = [vp]
    L.cf_last_error.restype = C.c_char_p
    L.cf_destroy.argtypes = [vp]
    L.cf_upload_fields.argtypes = [vp, dp, dp, dp]
    L.cf_download_fields.argtypes = [vp, dp, dp, dp, dp, dp]
    L.cf_download_wall.argtypes = [vp, dp, dp, dp]
    L.cf_upload_wall.argtypes = [vp, dp, dp, dp]
    L.cf_set_scalars.argtypes = [vp, C.c_double, C.c_double, C.c_int, C.c_double, C.c_double]
    L.cf_get_scalars.argtypes = [vp, dp, dp, ip, dp, dp]
    L.cf_init_mass_flow.argtypes = [vp, dp]
    L.cf_compute_dt.argtypes = [vp, dp]
    for n in ["cf_compute_eddy_viscosity", "cf_compute_wall_model", "cf_apply_boundary_conditions",
              "cf_compute_projection_step", "cf_save_old_state", "cf_synchronize", "cf_launches_per_step",
              "cf_compute_pressure"]:
        getattr(L, n).argtypes = [vp]
    for n in ["cf_compute_rhs_u", "cf_compute_rhs_v", "cf_compute_rhs_w", "cf_rk_update", "cf_set_fixed_dt"]:
        getattr(L, n).argtypes = [vp, C.c_int]
    L.cf_set_fixed_dt.argtypes = [vp, C.c_double]
    for n in ["cf_compute_dPx_for_constant_mass_flow", "cf_compute_dPy_for_constant_mass_flow",
              "cf_compute_dPx_for_constant_Ucenterline"]:
        getattr(L, n).argtypes = [vp, dp]
    L.cf_check_divergence.argtypes = [vp, dp, dp]
    L.cf_apply_mass_flow_correction.argtypes = [vp, C.c_int, C.c_double]
    L.cf_download_rhs.argtypes = [vp, C.c_int, C.c_int, dp]
    L.cf_download_avg_nu_t.argtypes = [vp, dp]
    L.cf_get_eqwm_counters.argtypes = [vp, ip, ip]
    L.cf_copy_wait_expired.argtypes = [vp, ip]
    L.cf_test_skip_plane_copy.argtypes = [vp, C.c_int]
    L.cf_time_step_rk3.argtypes = [vp, C.c_int, C.c_int]
    L.cf_get_stream.argtypes = [vp]
    L.cf_get_stream.restype = vp
    L.cf_compute_statistics.argtypes = [vp, dp]
    L.cf_output_monitor.argtypes = [vp, dp]
    L.cf_profile_steps.argtypes = [vp, C.c_int, C.c_int, C.c_char_p, dp, ip, ip]
    L.cf_profile_graph_steps.argtypes = [vp, C.c_int, C.c_int, C.c_char_p, dp, ip, ip]
    L.cf_read_input_parameters.argtypes = [C.c_char_p, C.POINTER(CfParams), ip, C.c_char_p, C.c_char_p, ip, ip]
    L.cf_read_snapshot.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, dp, dp, dp, dp, dp, dp]
    L.cf_write_snapshot.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, dp, dp, dp, dp, dp, dp, dp, dp]
    L.cf_write_statistics.argtypes = [C.c_char_p, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, dp, dp]
    L.cf_statistics_file_name.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_char_p, C.c_int]
    _lib = L
    return L


def _dp(a):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(C.c_double))


def default_params(**kw) -> CfParams:
    p = CfParams()
    load().cf_default_params(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


class Channel:
    """One channel on one GPU, arrays in the reference's Fortran layout."""

    def __init__(self, x, y, z, params: CfParams | None = None, device: int = 0, **kw):
        self.L = load()
        self.x = np.ascontiguousarray(x, dtype=np.float64)
        self.y = np.ascontiguousarray(y, dtype=np.float64)
        self.z = np.ascontiguousarray(z, dtype=np.float64)
        self.nx, self.ny, self.nz = len(self.x), len(self.y), len(self.z)
        self.params = params if params is not None else default_params(**kw)
        h = C.c_void_p()
        rc = self.L.cf_create(self.nx, self.ny, self.nz, _dp(self.x), _dp(self.y), _dp(self.z),
                              C.byref(self.params), device, C.byref(h))
        if rc != 0:
            msg = self.L.cf_last_error(h if h.value else None).decode() or f"cf_create failed ({rc})"
            if h.value:
                self.L.cf_destroy(h)
            raise CfError(msg)
        self.h = h
        self.device = device
        self.shapes = grids.field_shapes(self.nx, self.ny, self.nz)
        # unique (periodic) cells: nxp x nym x nzp (initialization.f90:246-247)
        self.nxp, self.nym, self.nzp = self.nx - 2, self.ny - 1, self.nz - 2

    # ---------------------------------------------------------------- utils
    def _check(self, rc):
        if rc != 0:
            raise CfError(self.L.cf_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.L.cf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---------------------------------------------------------- transfers
    def upload(self, U, V, W):
        U = np.asfortranarray(U, dtype=np.float64)
        V = np.asfortranarray(V, dtype=np.float64)
        W = np.asfortranarray(W, dtype=np.float64)
        for n, a in (("U", U), ("V", V), ("W", W)):
            if a.shape != self.shapes[n]:
                raise ValueError(f"{n} has shape {a.shape}, expected {self.shapes[n]}")
        self._check(self.L.cf_upload_fields(self.h, _dp(U), _dp(V), _dp(W)))

    def download(self):
        out = {k: np.zeros(self.shapes[k], order="F") for k in ("U", "V", "W", "P", "nu_t")}
        self._check(self.L.cf_download_fields(self.h, *[_dp(out[k]) for k in ("U", "V", "W", "P", "nu_t")]))
        return out

    def download_into(self, U=None, V=None, W=None, P=None, nu_t=None):
        """Downloads into caller-owned Fortran-ordered float64 arrays (e.g.
        pinned host buffers); any may be None."""
        arrs = [U, V, W, P, nu_t]
        for a, k in zip(arrs, ("U", "V", "W", "P", "nu_t")):
            if a is not None and (a.shape != self.shapes[k] or a.dtype != np.float64 or not a.flags.f_contiguous):
                raise ValueError(f"{k}: need a Fortran-ordered float64 array of shape {self.shapes[k]}")
        self._check(self.L.cf_download_fields(self.h, *[_dp(a) for a in arrs]))

    def download_wall(self):
        nx, nz = self.nx, self.nz
        ax = np.zeros((nx, 2, nz + 1), order="F")
        az = np.zeros((nx + 1, 2, nz), order="F")
        tau = np.zeros((nx, 2, nz + 1), order="F")
        self._check(self.L.cf_download_wall(self.h, _dp(ax), _dp(az), _dp(tau)))
        return dict(alpha_x=ax, alpha_z=az, tau_eqwm_initial=tau)

    def download_rhs(self, comp: int, slot: int):
        shp = [self.shapes["U"], self.shapes["V"], self.shapes["W"]][comp]
        a = np.zeros(shp, order="F")
        self._check(self.L.cf_download_rhs(self.h, comp, slot, _dp(a)))
        return a

    def avg_nu_t(self):
        a = np.zeros(self.ny + 1)
        self._check(self.L.cf_download_avg_nu_t(self.h, _dp(a)))
        return a

    def set_scalars(self, t=0.0, dt=0.0, rk_step=1, dPdx=None, dPdy=0.0):
        if dPdx is None:
            dPdx = self.scalars()["dPdx"]
        self._check(self.L.cf_set_scalars(self.h, t, dt, rk_step, dPdx, dPdy))

    def scalars(self):
        t, dt, dpx, dpy = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        rk = C.c_int()
        self._check(self.L.cf_get_scalars(self.h, C.byref(t), C.byref(dt), C.byref(rk), C.byref(dpx), C.byref(dpy)))
        return dict(t=t.value, dt=dt.value, rk_step=rk.value, dPdx=dpx.value, dPdy=dpy.value)

    # ---------------------------------------------- reference subroutines
    def init_mass_flow(self):
        q = C.c_double()
        self._check(self.L.cf_init_mass_flow(self.h, C.byref(q)))
        return q.value

    def compute_dt(self):
        v = C.c_double()
        self._check(self.L.cf_compute_dt(self.h, C.byref(v)))
        return v.value

    def compute_eddy_viscosity(self):
        self._check(self.L.cf_compute_eddy_viscosity(self.h))

    def compute_wall_model(self):
        self._check(self.L.cf_compute_wall_model(self.h))

    def compute_rhs_u(self, slot):
        self._check(self.L.cf_compute_rhs_u(self.h, slot))

    def compute_rhs_v(self, slot):
        self._check(self.L.cf_compute_rhs_v(self.h, slot))

    def compute_rhs_w(self, slot):
        self._check(self.L.cf_compute_rhs_w(self.h, slot))

    def save_old_state(self):
        self._check(self.L.cf_save_old_state(self.h))

    def rk_update(self, substep):
        self._check(self.L.cf_rk_update(self.h, substep))

    def apply_boundary_conditions(self):
        self._check(self.L.cf_apply_boundary_conditions(self.h))

    def compute_projection_step(self):
        self._check(self.L.cf_compute_projection_step(self.h))

    def compute_pressure(self):
        """Actual pressure of the current fields into P (pressure.f90:21)."""
        self._check(self.L.cf_compute_pressure(self.h))

    def compute_dPx_for_constant_mass_flow(self):
        v = C.c_double()
        self._check(self.L.cf_compute_dPx_for_constant_mass_flow(self.h, C.byref(v)))
        return v.value

    def apply_mass_flow_correction(self, comp, value):
        self._check(self.L.cf_apply_mass_flow_correction(self.h, comp, value))

    def check_divergence(self):
        a, b = C.c_double(), C.c_double()
        self._check(self.L.cf_check_divergence(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def eqwm_counters(self):
        a, b = C.c_int(), C.c_int()
        self._check(self.L.cf_get_eqwm_counters(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def copy_wait_expired(self):
        """Blocks of the FP32 multi-pass filter kernel whose plane-copy wait
        expired since the last query (the count is cleared)."""
        a = C.c_int()
        self._check(self.L.cf_copy_wait_expired(self.h, C.byref(a)))
        return a.value

    def test_skip_plane_copy(self, on):
        """Test hook: leave out the first plane copy of every filter block."""
        self._check(self.L.cf_test_skip_plane_copy(self.h, 1 if on else 0))

    def statistics(self):
        out = np.zeros(9 * self.ny + 8)
        self._check(self.L.cf_compute_statistics(self.h, _dp(out)))
        return out

    def output_statistics(self, fileout: str, istep: int, nstep_init: int = 0, stats=None) -> str:
        """output_statistics (input_output.f90:549-570): writes
        fileout.<istep+nstep_init>.stats.txt from compute_statistics (or the
        given statistics vector) and returns the file name."""
        if stats is None:
            stats = self.statistics()
        path = statistics_file_name(fileout, istep, nstep_init)
        write_statistics(path, self.scalars()["t"], self.params.nu, self.nx, self.ny, self.nz, istep, self.y, stats)
        return path

    def monitor(self) -> dict:
        """The reductions of output_monitor (monitor.f90:28-52)."""
        out = np.zeros(9)
        self._check(self.L.cf_output_monitor(self.h, _dp(out)))
        keys = ["meanU", "meanV", "meanW", "maxU", "maxV", "maxW", "meanNut", "maxNut", "max_divergence"]
        return dict(zip(keys, out.tolist()))

    def output_monitor(self, istep: int, retau: float = float("nan"), qflow=(float("nan"), float("nan")),
                       elapsed: float = float("nan"), file=None) -> dict:
        """Prints the block of output_monitor (monitor.f90:20-150) for this
        step; Retau and the mass flows are the last statistics' values, as in
        the reference.  Returns the reductions."""
        import sys
        m = self.monitor()
        sc = self.scalars()
        p = self.params
        f = file or sys.stdout
        w = lambda label, v: print(f" {label}{v}", file=f)
        w("step number :", istep)
        w("time        :", sc["t"])
        w("time step   :", sc["dt"])
        print(" ", file=f)
        w("Retau:      :", retau)
        print(" ", file=f)
        w("Maximum U   :", m["maxU"])
        w("Maximum V   :", m["maxV"])
        w("Maximum W   :", m["maxW"])
        w("Mean U      :", m["meanU"])
        w("Mean V      :", m["meanV"])
        w("Mean W      :", m["meanW"])
        if p.LES_model > 0:
            print(" ", file=f)
            w("Maximum nu_t: ", m["maxNut"])
            w("Average nu_t: ", m["meanNut"])
        print(" ", file=f)
        w("Mean mass flow in x         :", qflow[0])
        w("Mean mass flow in y         :", qflow[1])
        w("Mean pressure gradient in x :", sc["dPdx"])
        w("Mean pressure gradient in y :", sc["dPdy"])
        w("Spanwise rotation Omega_z   :", p.Rossby_plus * math.sqrt(p.dPdx) / 2.0)  # input_output.f90:83-84
        print(" ", file=f)
        if p.iwall_model == 3:
            n_nan, n_iter = self.eqwm_counters()
            w("Wall model     : ", "Equilibrium wall model (Larsson)")
            w("      jref     : ", p.jref_eqwm)
            w("      NaN eqwm : ", n_nan)
            w("      Max iter : ", n_iter)
        else:
            w("No wall model", "")
        print(" ", file=f)
        w("Maximum divergence          :", m["max_divergence"])
        w("Elapsed time (s)            :", elapsed)
        w("------------------------------------------------------", "")
        return m

    def autotune(self, reps: int = 3) -> dict:
        """cf_autotune: times every admissible z-chunk count of the marching
        kernels on the current state and keeps the fastest."""
        self.L.cf_autotune.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double)]
        out = np.zeros(6)
        self._check(self.L.cf_autotune(self.h, reps, _dp(out)))
        return dict(rhs_chunks=int(out[0]), rhs_us=out[1], dsm_chunk_len=int(out[2]), dsm_us=out[3],
                    amd_chunks=int(out[4]), amd_us=out[5])

    def set_wall_mlp(self, net, check_every: int = 100):
        """Serves the wall stress of the equilibrium wall model from a trained
        channelflow.wallmlp.WallMLP (eqwm outside its envelope); every
        `check_every` wall-model calls eqwm also runs and the network's error
        is recorded (wall_mlp_log).  None detaches it."""
        from . import wallmlp
        wallmlp._bind()
        self._wall_net = net  # keeps the network alive while it serves
        self._check(self.L.cf_set_wall_mlp(self.h, None if net is None else net.h, check_every))

    def wall_mlp_log(self) -> dict:
        out = np.zeros(5)
        self._check(self.L.cf_get_wall_mlp_log(self.h, _dp(out)))
        return dict(calls=int(out[0]), max_rel_err=out[1], mean_rel_err=out[2], served=int(out[3]),
                    fallback=int(out[4]))

    # ------------------------------------------------------------ fast path
    def time_step_rk3(self, nsteps: int = 1, sync: bool = True):
        self._check(self.L.cf_time_step_rk3(self.h, nsteps, 1 if sync else 0))

    def set_fixed_dt(self, dt: float):
        self._check(self.L.cf_set_fixed_dt(self.h, dt))

    def synchronize(self):
        self._check(self.L.cf_synchronize(self.h))

    def stream(self) -> int:
        return self.L.cf_get_stream(self.h)

    def launches_per_step(self) -> int:
        return self.L.cf_launches_per_step(self.h)

    def profile_steps(self, nsteps: int = 1, graph: bool = False) -> dict:
        """Per-kernel device time (ms, summed) and launch counts over nsteps
        steps, from CUDA events on the context's stream: eager steps, or
        (graph=True) each step captured with the events as graph nodes and
        launched as one graph."""
        mx = 64
        names = C.create_string_buffer(48 * mx)
        ms = np.zeros(mx)
        cnt = (C.c_int * mx)()
        n = C.c_int()
        fn = self.L.cf_profile_graph_steps if graph else self.L.cf_profile_steps
        self._check(fn(self.h, nsteps, mx, names, _dp(ms), cnt, C.byref(n)))
        out = {}
        for k in range(n.value):
            nm = names.raw[48 * k:48 * (k + 1)].split(b"\0", 1)[0].decode()
            out[nm] = (float(ms[k]), int(cnt[k]))
        return out

    def compute_time_step_rk3_mirror(self):
        """The reference's compute_time_step_RK3 (time_integration.f90:89-173)
        driven call by call through the fine-grained ABI."""
        sc = self.scalars()
        to, dt = sc["t"], sc["dt"]
        rk_t = [8.0 / 15.0, 2.0 / 3.0, 1.0]
        self.save_old_state()
        p = self.params
        for s in (1, 2, 3):
            self.set_scalars(t=self.scalars()["t"], dt=dt, rk_step=s)
            self.compute_eddy_viscosity()
            if s == 1:
                self.compute_wall_model()
                self.compute_eddy_viscosity()
            self.compute_rhs_u(s)
            self.compute_rhs_v(s)
            self.compute_rhs_w(s)
            self.rk_update(s)
            self.set_scalars(t=to + rk_t[s - 1] * dt, dt=dt, rk_step=s)
            self.apply_boundary_conditions()
            self.compute_projection_step()
            self.apply_boundary_conditions()
        if p.x_mass_cte == 1:
            d = self.compute_dPx_for_constant_mass_flow()
            self.apply_mass_flow_correction(0, d)
            self.apply_boundary_conditions()


class Ensemble:
    """Independent channels advanced together: one CUDA graph per ensemble
    step with a branch per member (cf_ensemble_*), the tridiagonal systems of
    all members solved by one FP64 launch per substep (batched_tri), the fused
    dynamic Smagorinsky passes and fused right-hand sides of all members as
    one launch each per substep (batched_stencils).  The members stay usable
    as Channel objects between steps."""

    def __init__(self, members, batched_tri: bool = True, batched_stencils: bool = False):
        self.L = load()
        L = self.L
        vp = C.c_void_p
        L.cf_ensemble_set_batched_tri.argtypes = [vp, C.c_int]
        L.cf_ensemble_set_batched_stencils.argtypes = [vp, C.c_int]
        L.cf_ensemble_create.argtypes = [C.c_int, C.POINTER(vp), C.POINTER(vp)]
        L.cf_ensemble_destroy.argtypes = [vp]
        L.cf_ensemble_step.argtypes = [vp, C.c_int, C.c_int]
        L.cf_ensemble_stream.argtypes = [vp]
        L.cf_ensemble_stream.restype = vp
        L.cf_ensemble_launches_per_step.argtypes = [vp]
        self.members = list(members)
        arr = (vp * len(self.members))(*[m.h.value for m in self.members])
        h = vp()
        rc = L.cf_ensemble_create(len(self.members), arr, C.byref(h))
        if rc != 0:
            raise CfError(L.cf_last_error(None).decode() or f"cf_ensemble_create failed ({rc})")
        self.h = h
        L.cf_ensemble_set_batched_tri(h, 1 if batched_tri else 0)
        if L.cf_ensemble_set_batched_stencils(h, 1 if batched_stencils else 0) != 0:
            raise CfError(L.cf_last_error(None).decode())

    def autotune(self, steps: int = 3) -> dict:
        """cf_ensemble_autotune: times whole ensemble steps with every kernel
        in the members' branches and with the batched stencil launches (three
        z-chunk plans), each with the members' own tridiagonal solves and with
        one FP64 launch for all of them, and keeps the fastest; the ensemble
        advances ENS_TUNE_CANDIDATES * (steps + 1) steps."""
        self.L.cf_ensemble_autotune.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_int)]
        rep = np.zeros(ENS_TUNE_CANDIDATES)
        ch = C.c_int()
        rc = self.L.cf_ensemble_autotune(self.h, steps, _dp(rep), C.byref(ch))
        if rc != 0:
            raise CfError(self.L.cf_last_error(None).decode() or f"cf_ensemble_autotune failed ({rc})")
        modes = ["branches", "batched, member plans", "batched, one z chunk", "batched, two z chunks"]
        names = [f"{m}; {t}" for t in ("own tridiagonal solves", "batched FP64 tridiagonal") for m in modes]
        return dict(choice=names[ch.value], ms_per_step=dict(zip(names, rep.tolist())))

    def step(self, nsteps: int = 1, sync: bool = True):
        rc = self.L.cf_ensemble_step(self.h, nsteps, 1 if sync else 0)
        if rc != 0:
            raise CfError(self.L.cf_last_error(None).decode() or f"cf_ensemble_step failed ({rc})")

    def stream(self) -> int:
        return self.L.cf_ensemble_stream(self.h)

    def launches_per_step(self) -> int:
        return self.L.cf_ensemble_launches_per_step(self.h)

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.L.cf_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def read_input_parameters(path: str):
    """Parses an input_parameters file (input_output.f90:21-133)."""
    L = load()
    p = CfParams()
    grid = (C.c_int * 3)()
    fi, fo = C.create_string_buffer(200), C.create_string_buffer(200)
    ints, ints2 = (C.c_int * 4)(), (C.c_int * 2)()
    rc = L.cf_read_input_parameters(path.encode(), C.byref(p), grid, fi, fo, ints, ints2)
    if rc != 0:
        raise CfError(f"cannot parse {path} ({rc})")
    return dict(params=p, grid=tuple(grid), filein=fi.value.decode(), fileout=fo.value.decode(),
                nsteps=ints[0], nsave=ints[1], nstats=ints[2], nmonitor=ints[3], nstep_init=ints2[0],
                random_init=ints2[1])


def read_snapshot(path: str, nx: int, ny: int, nz: int):
    L = load()
    x, y, z = np.zeros(nx), np.zeros(ny), np.zeros(nz)
    s = grids.field_shapes(nx, ny, nz)
    U, V, W = (np.zeros(s[k], order="F") for k in ("U", "V", "W"))
    rc = L.cf_read_snapshot(path.encode(), nx, ny, nz, _dp(x), _dp(y), _dp(z), _dp(U), _dp(V), _dp(W))
    if rc != 0:
        raise CfError(f"cannot read snapshot {path} ({rc})")
    return x, y, z, U, V, W


def write_snapshot(path: str, x, y, z, U, V, W, P=None, nu_t=None):
    L = load()
    f = lambda a: None if a is None else np.asfortranarray(a, dtype=np.float64)
    x, y, z = (np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z))
    U, V, W, P, nu_t = f(U), f(V), f(W), f(P), f(nu_t)
    rc = L.cf_write_snapshot(path.encode(), len(x), len(y), len(z), _dp(x), _dp(y), _dp(z), _dp(U), _dp(V), _dp(W),
                             _dp(P), _dp(nu_t))
    if rc != 0:
        raise CfError(f"cannot write snapshot {path} ({rc})")


def statistics_file_name(fileout: str, istep: int, nstep_init: int = 0) -> str:
    """fileout.<istep+nstep_init>.stats.txt (input_output.f90:557-558)."""
    L = load()
    buf = C.create_string_buffer(512)
    rc = L.cf_statistics_file_name(fileout.encode(), istep, nstep_init, buf, len(buf))
    if rc != 0:
        raise CfError(f"statistics file name too long ({rc})")
    return buf.value.decode()


def write_statistics(path: str, t: float, nu: float, nx: int, ny: int, nz: int, istep: int, y, stats):
    """output_statistics (input_output.f90:549-570) from the cf_compute_statistics vector."""
    L = load()
    y = np.ascontiguousarray(y, dtype=np.float64)
    stats = np.ascontiguousarray(stats, dtype=np.float64)
    if y.size != ny or stats.size != 9 * ny + 8:
        raise CfError("y needs ny values and stats 9*ny+8")
    rc = L.cf_write_statistics(path.encode(), t, nu, nx, ny, nz, istep, _dp(y), _dp(stats))
    if rc != 0:
        raise CfError(f"cannot write statistics {path} ({rc})")
