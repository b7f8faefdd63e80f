"""ctypes binding of the CPU FP64 oracle (oracle/cf_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of ``bench.py``.  The product path never imports
this module.  Parity status of the oracle: unpinned (the Fortran reference
cannot be compiled here and ships no golden vectors).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


class Params(C.Structure):
    _fields_ = [
        ("nu", C.c_double), ("CFL", C.c_double), ("dPdx", C.c_double), ("dPdz", C.c_double),
        ("Rossby_plus", C.c_double), ("freq_mult", C.c_double),
        ("Retau_int", C.c_int), ("x_mass_cte", C.c_int), ("y_mass_cte", C.c_int),
        ("LES_model", C.c_int), ("iwall_model", C.c_int), ("Dirichlet_nu_t", C.c_int),
        ("jref_eqwm", C.c_int), ("eqwm_ncv", C.c_int), ("eqwm_stretch", C.c_double),
    ]


def build(check: bool = False) -> str:
    """Compile the oracle with its Makefile; returns the library path."""
    target = "libcf_oracle_check.so" if check else "libcf_oracle.so"
    subprocess.run(["make", "-s", "-C", HERE, target], check=True)
    return os.path.join(HERE, target)


_libs: dict = {}


def lib(check: bool = False):
    key = bool(check)
    if key not in _libs:
        path = os.path.join(HERE, "libcf_oracle_check.so" if check else "libcf_oracle.so")
        src = os.path.join(HERE, "cf_oracle.c")
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
            build(check)
        L = C.CDLL(path)
        vp = C.c_void_p
        dp = C.POINTER(C.c_double)
        L.cfo_create.restype = vp
        L.cfo_create.argtypes = [C.c_int, C.c_int, C.c_int, dp, dp, dp, C.POINTER(Params)]
        L.cfo_destroy.argtypes = [vp]
        L.cfo_set_fields.argtypes = [vp, dp, dp, dp]
        L.cfo_get_fields.argtypes = [vp, dp, dp, dp, dp, dp]
        L.cfo_array.restype = dp
        L.cfo_array.argtypes = [vp, C.c_char_p, C.POINTER(C.c_int)]
        L.cfo_scalar.restype = C.c_double
        L.cfo_scalar.argtypes = [vp, C.c_char_p]
        L.cfo_set_scalar.argtypes = [vp, C.c_char_p, C.c_double]
        for name in ["cfo_init_mass_flow", "cfo_compute_dt", "cfo_time_step_rk3", "cfo_compute_eddy_viscosity",
                     "cfo_compute_wall_model", "cfo_apply_boundary_conditions", "cfo_compute_projection_step",
                     "cfo_compute_pseudo_pressure_rhs", "cfo_solve_poisson_equation", "cfo_project_velocity",
                     "cfo_compute_pressure"]:
            getattr(L, name).argtypes = [vp]
        for name in ["cfo_compute_rhs_u", "cfo_compute_rhs_v", "cfo_compute_rhs_w", "cfo_rk_update"]:
            getattr(L, name).argtypes = [vp, C.c_int]
        L.cfo_check_divergence.restype = C.c_double
        L.cfo_check_divergence.argtypes = [vp, dp]
        for name in ["cfo_compute_dPx_for_constant_mass_flow", "cfo_compute_mean_mass_flow_U",
                     "cfo_compute_mean_mass_flow_V"]:
            getattr(L, name).restype = C.c_double
            getattr(L, name).argtypes = [vp]
        L.cfo_compute_statistics.argtypes = [vp, dp]
        L.cfo_output_monitor.argtypes = [vp, dp]
        L.cfo_solve_u_eqwm.restype = C.c_double
        L.cfo_solve_u_eqwm.argtypes = [C.c_double, C.c_double, C.c_double, C.c_int, C.c_double, C.c_double,
                                       C.POINTER(C.c_int)]
        L.cfo_fft.argtypes = [dp, C.c_int, C.c_int]
        L.cfo_zgtsv.restype = C.c_int
        L.cfo_zgtsv.argtypes = [C.c_int, dp, dp, dp, dp]
        L.cfo_set_threads.restype = C.c_int
        L.cfo_set_threads.argtypes = [C.c_int]
        _libs[key] = L
    return _libs[key]


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Oracle:
    """One channel held by the CPU oracle, arrays in the reference layout."""

    def __init__(self, x, y, z, params: dict, check: bool = False, threads: int = 0):
        self.L = lib(check)
        self.x = np.ascontiguousarray(x, dtype=np.float64)
        self.y = np.ascontiguousarray(y, dtype=np.float64)
        self.z = np.ascontiguousarray(z, dtype=np.float64)
        self.nx, self.ny, self.nz = len(self.x), len(self.y), len(self.z)
        p = Params()
        defaults = dict(nu=1e-3, CFL=-5e-3, dPdx=0.0, dPdz=0.0, Rossby_plus=0.0, freq_mult=0.0, Retau_int=0,
                        x_mass_cte=0, y_mass_cte=0, LES_model=0, iwall_model=0, Dirichlet_nu_t=0, jref_eqwm=3,
                        eqwm_ncv=100, eqwm_stretch=1.10)
        defaults.update(params)
        for k, v in defaults.items():
            setattr(p, k, v)
        self.params = p
        if threads:
            self.L.cfo_set_threads(threads)
        self.h = self.L.cfo_create(self.nx, self.ny, self.nz, _dp(self.x), _dp(self.y), _dp(self.z), C.byref(p))
        if not self.h:
            raise ValueError("oracle rejected the grid (nx, nz must be even, >= 6)")

    def close(self):
        if self.h:
            self.L.cfo_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # shapes (Fortran order)
    @property
    def shapes(self):
        nx, ny, nz = self.nx, self.ny, self.nz
        return dict(U=(nx, ny + 1, nz + 1), V=(nx + 1, ny, nz + 1), W=(nx + 1, ny + 1, nz), P=(nx + 1, ny + 1, nz + 1))

    def set_fields(self, U, V, W):
        U = np.asfortranarray(U, dtype=np.float64)
        V = np.asfortranarray(V, dtype=np.float64)
        W = np.asfortranarray(W, dtype=np.float64)
        s = self.shapes
        assert U.shape == s["U"] and V.shape == s["V"] and W.shape == s["W"]
        self.L.cfo_set_fields(self.h, _dp(U), _dp(V), _dp(W))

    def array(self, name: str) -> np.ndarray:
        dims = (C.c_int * 4)()
        ptr = self.L.cfo_array(self.h, name.encode(), dims)
        if not ptr:
            raise KeyError(name)
        shape = tuple(d for d in dims)
        n = int(np.prod(shape))
        a = np.ctypeslib.as_array(ptr, shape=(n,)).copy()
        shape = tuple(d for d in shape)
        while len(shape) > 1 and shape[-1] == 1:
            shape = shape[:-1]
        return a.reshape(shape, order="F")

    def fields(self):
        return {k: self.array(k) for k in ("U", "V", "W", "P", "nu_t")}

    def scalar(self, name):
        return self.L.cfo_scalar(self.h, name.encode())

    def set_scalar(self, name, v):
        self.L.cfo_set_scalar(self.h, name.encode(), float(v))

    def __getattr__(self, name):
        # oracle.compute_dt() -> cfo_compute_dt(h)
        if name.startswith("_") or name in ("L", "h"):
            raise AttributeError(name)
        fn = getattr(self.L, "cfo_" + name, None)
        if fn is None:
            raise AttributeError(name)
        return lambda *a: fn(self.h, *a)

    def check_divergence(self):
        m = C.c_double()
        s = self.L.cfo_check_divergence(self.h, C.byref(m))
        return s, m.value

    def output_monitor(self):
        out = np.zeros(9)
        self.L.cfo_output_monitor(self.h, _dp(out))
        return out

    def statistics(self):
        out = np.zeros(9 * self.ny + 8)
        self.L.cfo_compute_statistics(self.h, _dp(out))
        return out


def solve_u_eqwm(u, nu, h, ncv, stretch, tau_in):
    """eqwm.f90:90-223 for one point (the oracle's restatement): (tau_w, iterations)."""
    L = lib()
    it = C.c_int()
    t = L.cfo_solve_u_eqwm(float(u), float(nu), float(h), int(ncv), float(stretch), float(tau_in), C.byref(it))
    return t, it.value
