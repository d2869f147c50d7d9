"""ctypes binding of the CPU oracle (test infrastructure only)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import build as _build

_LIB = None


class OracleError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"oracle status {code}: {msg}")
        self.code = code


def lib() -> C.CDLL:
    global _LIB
    if _LIB is None:
        path = _build.build()
        L = C.CDLL(str(path))
        vp, dp = C.c_void_p, C.POINTER(C.c_double)
        L.zfvm_oracle_create.argtypes = [C.c_int, C.c_int64, dp, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_int, C.c_int, C.c_int] + [C.c_void_p] * 7 + [C.c_int] * 3 + \
                                        [dp, C.POINTER(C.c_void_p)]
        L.zfvm_oracle_destroy.argtypes = [vp]
        L.zfvm_oracle_set_threads.argtypes = [vp, C.c_int]
        L.zfvm_oracle_set_pinv.argtypes = [vp, C.c_int64, C.c_int, dp, C.c_int, C.c_int]
        L.zfvm_oracle_set_lsq_mode.argtypes = [vp, C.c_int]
        L.zfvm_oracle_rate_of_change.argtypes = [vp, dp, dp]
        L.zfvm_oracle_cfl_dt.argtypes = [vp, dp, dp]
        L.zfvm_oracle_reconstruct_eval.argtypes = [vp, dp, C.c_int64, C.c_void_p, dp, dp]
        L.zfvm_oracle_step.argtypes = [vp, dp, C.c_double]
        L.zfvm_oracle_run.argtypes = [vp, dp, C.c_int64, C.c_double, dp, C.POINTER(C.c_int64)]
        L.zfvm_oracle_rate_of_change_av.argtypes = [vp, dp, dp, dp, dp]
        L.zfvm_oracle_step_av.argtypes = [vp, dp, dp, C.c_double]
        L.zfvm_oracle_run_av.argtypes = [vp, dp, dp, C.c_int64, C.c_double, dp, C.POINTER(C.c_int64)]
        L.zfvm_oracle_tracer_flux.argtypes = [C.c_int, C.c_double, dp, dp, C.c_double, C.c_double, dp]
        L.zfvm_oracle_flux.argtypes = [C.c_int, C.c_double, dp, dp, dp]
        L.zfvm_oracle_euler_flux.argtypes = [C.c_double, dp, dp]
        L.zfvm_oracle_poly_eval.argtypes = [C.c_int, C.c_int, dp, dp, dp, C.c_double, dp, dp]
        L.zfvm_oracle_local_equilibrium.argtypes = [C.c_double, C.c_double, C.c_int, C.c_double, dp, C.c_int, dp, dp,
                                                    dp, dp]
        L.zfvm_oracle_equilibrium_average.argtypes = [C.c_double, C.c_int, C.c_double, dp, dp, dp, C.c_int, dp]
        L.zfvm_oracle_rk_ode_error.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double]
        L.zfvm_oracle_rk_ode_error.restype = C.c_double
        L.zfvm_oracle_eos_roundtrips.argtypes = [C.c_double, C.c_double, C.c_double, C.c_double, dp]
        L.zfvm_oracle_quasi_newton_problem.argtypes = [C.c_int, dp]
        L.zfvm_oracle_rule.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), dp, dp]
        L.zfvm_oracle_gravity.argtypes = [dp, C.c_int64, dp, dp, dp]
        L.zfvm_oracle_last_error.restype = C.c_char_p
        _LIB = L
    return _LIB


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _check(code):
    if code != 0:
        raise OracleError(code, lib().zfvm_oracle_last_error().decode())


# entries the oracle reads from a scheme vector (zfvm_oracle_create's table),
# a gravity table's radii and potentials following
SCHEME_VECTOR_MIN = 32


class Oracle:
    """The reference's time loop on the CPU for one mesh and scheme."""

    def __init__(self, raw, stencils: dict, scheme_vector: np.ndarray, quad=(3, 3, 2), threads: int = 1):
        L = lib()
        self._keep = []

        def arr(a, dtype):
            a = np.ascontiguousarray(a, dtype=dtype)
            self._keep.append(a)
            return a

        v = arr(raw.vertices, np.float64)
        vi = arr(raw.vertex_indices, np.int64)
        g = arr(raw.ghost, np.uint8) if raw.ghost is not None else None
        s = arr(raw.source, np.int64) if raw.source is not None else None
        st = {k: arr(x, x.dtype) for k, x in stencils.items()}
        self.scheme = arr(scheme_vector, np.float64)
        if self.scheme.shape[0] < SCHEME_VECTOR_MIN:
            raise ValueError(f"scheme vector of {self.scheme.shape[0]} entries; the oracle reads {SCHEME_VECTOR_MIN}")
        h = C.c_void_p()
        _check(L.zfvm_oracle_create(raw.n_dims, v.shape[0], _dp(v), vi.shape[0], vi.ctypes.data,
                                    g.ctypes.data if g is not None else None,
                                    s.ctypes.data if s is not None else None, quad[0], quad[1], quad[2],
                                    st["n_stencils"].ctypes.data, st["k_high"].ctypes.data,
                                    st["n_l2g"].ctypes.data, st["l2g"].ctypes.data, st["order"].ctypes.data,
                                    st["size"].ctypes.data, st["local"].ctypes.data, st["l2g"].shape[1],
                                    st["order"].shape[1], st["local"].shape[2], _dp(self.scheme), C.byref(h)))
        self._h = h
        self.n_cells = vi.shape[0]
        L.zfvm_oracle_set_threads(h, threads)

    def __del__(self):
        if getattr(self, "_h", None) is not None and _LIB is not None:
            _LIB.zfvm_oracle_destroy(self._h)
            self._h = None

    def set_threads(self, n: int) -> None:
        lib().zfvm_oracle_set_threads(self._h, n)

    def use_pinv(self, mesh) -> None:
        """Use the product's pseudo-inverses instead of the per-call LDLT solve."""
        st = mesh.stencils()
        for i in range(self.n_cells):
            for k in range(int(st["n_stencils"][i])):
                if st["order"][i, k] >= 2:
                    P = np.ascontiguousarray(mesh.pinv(i, k))
                    _check(lib().zfvm_oracle_set_pinv(self._h, i, k, _dp(P), P.shape[1], P.shape[0]))
        lib().zfvm_oracle_set_lsq_mode(self._h, 1)

    def rate_of_change(self, state: np.ndarray, avars: np.ndarray | None = None):
        """Tendency of the state; with advected variables (n x na) also theirs:
        (tendency, avars tendency)."""
        u = np.ascontiguousarray(state, dtype=np.float64)
        out = np.zeros_like(u)
        if avars is None:
            _check(lib().zfvm_oracle_rate_of_change(self._h, _dp(u), _dp(out)))
            return out
        q = np.ascontiguousarray(avars, dtype=np.float64)
        qout = np.zeros_like(q)
        _check(lib().zfvm_oracle_rate_of_change_av(self._h, _dp(u), _dp(q), _dp(out), _dp(qout)))
        return out, qout

    def reconstruct_eval(self, state: np.ndarray, cells, x) -> np.ndarray:
        """Reconstruction of cells[k] at x[k] (n x 3): n x 5 rows."""
        u = np.ascontiguousarray(state, dtype=np.float64)
        c = np.ascontiguousarray(cells, dtype=np.int64)
        xx = np.ascontiguousarray(x, dtype=np.float64).reshape(len(c), 3)
        out = np.zeros((len(c), 5))
        _check(lib().zfvm_oracle_reconstruct_eval(self._h, _dp(u), len(c), c.ctypes.data, _dp(xx), _dp(out)))
        return out

    def cfl_dt(self, state: np.ndarray) -> float:
        u = np.ascontiguousarray(state, dtype=np.float64)
        dt = C.c_double()
        _check(lib().zfvm_oracle_cfl_dt(self._h, _dp(u), C.byref(dt)))
        return dt.value

    def step(self, state: np.ndarray, dt: float, avars: np.ndarray | None = None):
        u = np.array(state, dtype=np.float64, copy=True)
        if avars is None:
            _check(lib().zfvm_oracle_step(self._h, _dp(u), dt))
            return u
        q = np.array(avars, dtype=np.float64, copy=True)
        _check(lib().zfvm_oracle_step_av(self._h, _dp(u), _dp(q), dt))
        return u, q

    def run(self, state: np.ndarray, n_steps: int = 0, t_end: float = 0.0, t0: float = 0.0,
            avars: np.ndarray | None = None):
        """(state, t, steps), or (state, avars, t, steps) with advected variables."""
        u = np.array(state, dtype=np.float64, copy=True)
        t = C.c_double(t0)
        s = C.c_int64()
        if avars is None:
            _check(lib().zfvm_oracle_run(self._h, _dp(u), n_steps, t_end, C.byref(t), C.byref(s)))
            return u, t.value, s.value
        q = np.array(avars, dtype=np.float64, copy=True)
        _check(lib().zfvm_oracle_run_av(self._h, _dp(u), _dp(q), n_steps, t_end, C.byref(t), C.byref(s)))
        return u, q, t.value, s.value


def flux(kind: int, gamma: float, uL, uR) -> np.ndarray:
    a, b, f = np.asarray(uL, float), np.asarray(uR, float), np.zeros(5)
    lib().zfvm_oracle_flux(kind, gamma, _dp(a), _dp(b), _dp(f))
    return f


def tracer_flux(kind: int, gamma: float, uL, uR, qL: float, qR: float) -> float:
    """Flux of an advected variable between face-frame states uL, uR."""
    a = np.ascontiguousarray(uL, dtype=np.float64)
    b = np.ascontiguousarray(uR, dtype=np.float64)
    f = C.c_double()
    _check(lib().zfvm_oracle_tracer_flux(kind, gamma, _dp(a), _dp(b), qL, qR, C.byref(f)))
    return f.value


def euler_flux(gamma: float, u) -> np.ndarray:
    a, f = np.asarray(u, float), np.zeros(5)
    lib().zfvm_oracle_euler_flux(gamma, _dp(a), _dp(f))
    return f


def poly_eval(n_dims, coeffs, moments, x_center, length, x) -> float:
    c, m = np.asarray(coeffs, float), np.asarray(moments, float)
    xc, xx, out = np.asarray(x_center, float), np.asarray(x, float), np.zeros(1)
    lib().zfvm_oracle_poly_eval(n_dims, len(c), _dp(c), _dp(m), _dp(xc), length, _dp(xx), _dp(out))
    return float(out[0])


def local_equilibrium(gamma, R, gravity_kind, g, tri, quad_deg, rhoE_bar, x):
    t, rb, xx = np.asarray(tri, float).ravel(), np.asarray(rhoE_bar, float), np.asarray(x, float)
    out, th = np.zeros(2), np.zeros(2)
    st = lib().zfvm_oracle_local_equilibrium(gamma, R, gravity_kind, g, _dp(t), quad_deg, _dp(rb), _dp(xx), _dp(out),
                                             _dp(th))
    return st, out, th


def equilibrium_average(gamma, gravity_kind, g, theta, x_ref, tri, quad_deg):
    th, xr, t, out = np.asarray(theta, float), np.asarray(x_ref, float), np.asarray(tri, float).ravel(), np.zeros(2)
    lib().zfvm_oracle_equilibrium_average(gamma, gravity_kind, g, _dp(th), _dp(xr), _dp(t), quad_deg, _dp(out))
    return out


def gravity(scheme_vector, x):
    """The oracle's potential and its gradient at points x (n x 3)."""
    sv = np.ascontiguousarray(scheme_vector, dtype=np.float64)
    xx = np.ascontiguousarray(np.atleast_2d(x), dtype=np.float64)
    n = xx.shape[0]
    phi, grad = np.zeros(n), np.zeros((n, 3))
    _check(lib().zfvm_oracle_gravity(_dp(sv), n, _dp(xx), _dp(phi), _dp(grad)))
    return phi, grad


def rk_ode_error(stages: int, ode: int, dt: float, t_final: float = 3.0) -> float:
    return lib().zfvm_oracle_rk_ode_error(stages, ode, dt, t_final)


def eos_roundtrips(gamma: float, R: float, rho: float, E: float) -> np.ndarray:
    """(rho, E) through (h, K) and back, and through (rho, p) and back: 2 x 2."""
    out = np.zeros(4)
    _check(lib().zfvm_oracle_eos_roundtrips(gamma, R, rho, E, _dp(out)))
    return out.reshape(2, 2)


def quasi_newton_problem(which: int):
    """The oracle's quasi_newton on a known problem: (solution, status)."""
    x = np.zeros(2)
    st = lib().zfvm_oracle_quasi_newton_problem(which, _dp(x))
    return (x[:1] if which == 0 else x), st


def rule(kind: str, deg: int):
    """The oracle's reference-element rule ("edge", "triangle", "tetrahedron"):
    (weights summing to 1, points: [-1, 1] coordinates or barycentric rows)."""
    k = {"edge": 0, "triangle": 1, "tetrahedron": 2}[kind]
    nc = 1 if k == 0 else k + 2
    n = C.c_int()
    w, x = np.zeros(16), np.zeros(16 * nc)
    _check(lib().zfvm_oracle_rule(k, deg, 16, C.byref(n), _dp(w), _dp(x)))
    m = n.value
    return w[:m].copy(), x[:m * nc].reshape(m, nc).copy()
