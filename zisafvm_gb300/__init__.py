"""GB300-native rate-of-change / SSP-RK solver for unstructured finite volumes.

Python host binding of ``libzfvm.so`` (C ABI in ``include/zfvm.h``).  The
objects mirror ZisaFVM's own: a mesh with its stencil families and LSQ
operators (``Grid`` + ``compute_stencil_families`` + ``LSQSolver``), and a solver
that exposes ``RateOfChange::compute``, ``RungeKutta::compute_step``,
``LocalCFL`` and the ``TimeLoop`` on the GPU.

There is no CPU fallback: importing works without a GPU (mesh set-up is host
code), but every solver call needs the CUDA library and a device, and raises
``ZfvmError`` otherwise.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

__all__ = [
    "ZfvmError", "RawMesh", "Mesh", "Solver", "Batch", "Scheme", "StencilSpec", "library_path", "load_library",
    "FLUX_HLLC", "FLUX_RUSANOV",
]

PKG = Path(__file__).resolve().parent
MAX_STENCILS = 5
MAX_L2G = 40
MAX_STENCIL_SIZE = 24

FLUX_HLLC, FLUX_RUSANOV = 0, 1
EQ_NONE, EQ_ISENTROPIC = 0, 1
GRAVITY_NONE, GRAVITY_CONSTANT_RADIAL, GRAVITY_HARMONIC_RADIAL = 0, 1, 2
# PolytropeGravityRadial, PolytropeGravityWithJumpRadial, PointMassGravityRadial, RadialGravity
GRAVITY_POLYTROPE_RADIAL, GRAVITY_POLYTROPE_JUMP_RADIAL, GRAVITY_POINT_MASS_RADIAL, GRAVITY_RADIAL_TABLE = 3, 4, 5, 6
FLUX_BC_NONE, FLUX_BC_CONSTANT, FLUX_BC_ISENTROPIC = 0, 1, 2
BC_NONE, BC_PERIODIC, BC_FROZEN = 0, 1, 2
FP64, MIXED = 0, 1
RC_CWENO_AO, RC_WENO_AO = 0, 1

STATUS = {0: "ok", 1: "EINVAL", 2: "ENOMEM", 3: "ENONPHYSICAL", 4: "ENEWTON", 5: "ETIMEDOUT", 6: "ECUDA",
          7: "ESETUP"}


class ZfvmError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class _MeshDesc(C.Structure):
    _fields_ = [("n_dims", C.c_int32), ("n_vertices", C.c_int64), ("n_cells", C.c_int64),
                ("vertices", C.POINTER(C.c_double)), ("vertex_indices", C.POINTER(C.c_int64)),
                ("ghost", C.POINTER(C.c_uint8)), ("source", C.POINTER(C.c_int64)),
                ("quad_edge", C.c_int32), ("quad_volume", C.c_int32), ("quad_moments", C.c_int32),
                ("n_stencils", C.c_int32), ("orders", C.c_int32 * MAX_STENCILS),
                ("biased", C.c_int32 * MAX_STENCILS), ("overfit", C.c_double * MAX_STENCILS)]


class _MeshInfo(C.Structure):
    _fields_ = [("n_dims", C.c_int32), ("n_cells", C.c_int64), ("n_interior_cells", C.c_int64),
                ("n_edges", C.c_int64), ("n_interior_edges", C.c_int64), ("n_cell_qp", C.c_int32),
                ("n_face_qp", C.c_int32), ("n_moments", C.c_int32), ("min_inradius", C.c_double),
                ("max_circum_radius", C.c_double), ("total_volume", C.c_double),
                ("setup_geometry_s", C.c_double), ("setup_stencils_s", C.c_double), ("setup_lsq_s", C.c_double)]


class _ServerDesc(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_int64), ("max_slots", C.c_int32), ("steps_per_round", C.c_int32)]


class _ServerStats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("submitted", "completed", "failed", "queued", "running", "bytes_in_use",
                                          "bytes_peak", "budget_bytes", "cell_stage_updates", "rounds")] + \
               [("busy_s", C.c_double), ("setup_s", C.c_double)]


class _SchemeDesc(C.Structure):
    _fields_ = [("flux", C.c_int32), ("gamma", C.c_double), ("specific_gas_constant", C.c_double),
                ("linear_weights", C.c_double * MAX_STENCILS), ("epsilon", C.c_double),
                ("exponent", C.c_double), ("rk_stages", C.c_int32), ("cfl_number", C.c_double),
                ("equilibrium", C.c_int32), ("gravity", C.c_int32), ("gravity_strength", C.c_double),
                ("flux_bc", C.c_int32), ("boundary", C.c_int32), ("precision", C.c_int32),
                ("steps_per_recompute", C.c_int32), ("recompute_threshold", C.c_double),
                ("reconstruction", C.c_int32), ("step_rejection_drho", C.c_double),
                ("step_rejection_max_exponent", C.c_int32), ("heating_rate", C.c_double),
                ("heating_r0", C.c_double), ("heating_r1", C.c_double), ("n_avars", C.c_int32),
                ("gravity_params", C.c_double * 5), ("gravity_table_r", C.POINTER(C.c_double)),
                ("gravity_table_phi", C.POINTER(C.c_double)), ("gravity_table_n", C.c_int64)]


_LIB = None


def library_path() -> Path:
    return PKG / "libzfvm.so"


def load_library() -> C.CDLL:
    """Load the in-tree native library; it must have been built (``_build.build()``)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not path.exists():
        raise ZfvmError(6, f"native library {path} is missing; run zisafvm_gb300._build.build()")
    lib = C.CDLL(str(path))
    vp, i32, i64, dp = C.c_void_p, C.c_int32, C.c_int64, C.POINTER(C.c_double)
    pp = C.POINTER(C.c_void_p)
    sig = {
        "zfvm_rawmesh_generate": [i32, C.POINTER(C.c_int64), dp, C.c_uint64, i32, pp],
        "zfvm_rawmesh_sizes": [vp, C.POINTER(i32), C.POINTER(i64), C.POINTER(i64), C.POINTER(i32)],
        "zfvm_rawmesh_copy": [vp, dp, C.POINTER(C.c_int64), C.POINTER(C.c_uint8), C.POINTER(C.c_int64)],
        "zfvm_rawmesh_destroy": [vp],
        "zfvm_mesh_create": [C.POINTER(_MeshDesc), pp],
        "zfvm_mesh_destroy": [vp],
        "zfvm_mesh_get_info": [vp, C.POINTER(_MeshInfo)],
        "zfvm_mesh_get_stencils": [vp] + [C.c_void_p] * 8,
        "zfvm_mesh_get_pinv": [vp, i64, i32, dp, C.POINTER(i32), C.POINTER(i32)],
        "zfvm_mesh_get_geometry": [vp, dp, dp, dp, C.POINTER(C.c_uint8)],
        "zfvm_mesh_get_connectivity": [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)],
        "zfvm_mesh_get_faces": [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64), dp, dp],
        "zfvm_initial_conditions": [vp, i32, dp, dp],
        "zfvm_solver_create": [vp, C.POINTER(_SchemeDesc), pp],
        "zfvm_solver_destroy": [vp],
        "zfvm_set_state": [vp, dp, C.c_double],
        "zfvm_get_state": [vp, dp, dp],
        "zfvm_rate_of_change": [vp, dp],
        "zfvm_rate_of_change_noalloc": [vp, dp],
        "zfvm_cfl_dt": [vp, dp],
        "zfvm_step": [vp, C.c_double],
        "zfvm_advance": [vp, i64, C.c_double, dp, C.POINTER(i64)],
        "zfvm_advance_timed": [vp, i64, C.POINTER(C.c_float)],
        "zfvm_launches_per_step": [vp, C.POINTER(i32)],
        "zfvm_kernel_times": [vp, i64, C.POINTER(C.c_float)],
        "zfvm_device_bytes": [vp, C.POINTER(i64)],
        "zfvm_batch_create": [i32, pp],
        "zfvm_batch_destroy": [vp],
        "zfvm_batch_add": [vp, vp, i64, C.c_double, C.POINTER(i32)],
        "zfvm_batch_remove": [vp, i32],
        "zfvm_batch_advance": [vp, i32, C.POINTER(i32)],
        "zfvm_batch_step_host": [vp, pp, pp, i32, C.POINTER(i32)],
        "zfvm_batch_advance_timed": [vp, i32, C.POINTER(C.c_float)],
        "zfvm_batch_autotune": [vp, i32, C.POINTER(C.c_float)],
        "zfvm_batch_kernel_times": [vp, i32, C.POINTER(C.c_float)],
        "zfvm_batch_launch_shapes": [vp, i32, C.POINTER(i32), C.POINTER(i32)],
        "zfvm_batch_slot_status": [vp, i32, dp, C.POINTER(i64), C.POINTER(i32), C.POINTER(i32)],
        "zfvm_batch_slots": [vp, C.POINTER(i32)],
        "zfvm_solver_footprint": [vp, vp, C.POINTER(i64)],
        "zfvm_reconstruct": [vp],
        "zfvm_step_rejections": [vp, C.POINTER(i64)],
        "zfvm_reconstruction_eval": [vp, i64, C.POINTER(i64), dp, dp],
        "zfvm_server_create": [vp, pp],
        "zfvm_server_destroy": [vp],
        "zfvm_server_submit": [vp, vp, vp, dp, C.c_double, i64, C.c_double, C.POINTER(i64)],
        "zfvm_server_poll": [vp, i64, C.POINTER(i32)],
        "zfvm_server_wait": [vp, i64, C.c_double, dp, dp, C.POINTER(i64), dp],
        "zfvm_server_get_stats": [vp, vp],
        "zfvm_step_host": [vp, dp, C.c_double, i64, C.c_double, C.c_double, dp, dp, C.POINTER(i64)],
        "zfvm_set_avars": [vp, dp],
        "zfvm_get_avars": [vp, dp],
        "zfvm_rate_of_change_all": [vp, dp, dp],
        "zfvm_snapshot_write": [C.c_char_p, i64, dp, i32, dp, i32, C.c_double, i64],
        "zfvm_snapshot_info": [C.c_char_p, C.POINTER(i64), C.POINTER(i32), C.POINTER(i32)],
        "zfvm_snapshot_read": [C.c_char_p, i64, dp, i32, dp, dp, C.POINTER(i64)],
        "zfvm_solver_write_snapshot": [vp, C.c_char_p, i64],
        "zfvm_solver_read_snapshot": [vp, C.c_char_p, C.POINTER(i64)],
        "zfvm_numerical_flux": [i32, C.c_double, i64, dp, dp, dp, dp],
        "zfvm_tracer_flux": [i32, i64, dp, dp, dp, dp, dp, dp],
        "zfvm_apply_boundary": [vp, dp, dp, dp, dp],
    }
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int
    lib.zfvm_last_error.restype = C.c_char_p
    lib.zfvm_last_error.argtypes = []
    _LIB = lib
    return lib


def _check(code: int) -> None:
    if code != 0:
        msg = load_library().zfvm_last_error().decode(errors="replace")
        raise ZfvmError(code, msg)


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _i64p(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int64))


def numerical_flux(kind: int, gamma: float, uL, uR):
    """HLLCBatten::flux (or Rusanov) of face states on the GPU: rows of
    (rho, normal momentum, tangential momenta, E) -> (fluxes n x 5, speeds n x 3)."""
    a = np.ascontiguousarray(np.atleast_2d(uL), dtype=np.float64)
    b = np.ascontiguousarray(np.atleast_2d(uR), dtype=np.float64)
    if a.shape != b.shape or a.shape[1] != 5:
        raise ValueError("uL, uR: n x 5 face states")
    f, sp = np.zeros_like(a), np.zeros((a.shape[0], 3))
    _check(load_library().zfvm_numerical_flux(kind, gamma, a.shape[0], _dp(a), _dp(b), _dp(f), _dp(sp)))
    return f, sp


def tracer_flux(kind: int, uL, uR, mqL, mqR, speeds):
    """HLLCBatten::tracer_flux (or Rusanov) on the GPU for n face points."""
    a = np.ascontiguousarray(np.atleast_2d(uL), dtype=np.float64)
    b = np.ascontiguousarray(np.atleast_2d(uR), dtype=np.float64)
    qa = np.ascontiguousarray(np.atleast_1d(mqL), dtype=np.float64)
    qb = np.ascontiguousarray(np.atleast_1d(mqR), dtype=np.float64)
    sp = np.ascontiguousarray(np.atleast_2d(speeds), dtype=np.float64)
    f = np.zeros(a.shape[0])
    _check(load_library().zfvm_tracer_flux(kind, a.shape[0], _dp(a), _dp(b), _dp(qa), _dp(qb), _dp(sp), _dp(f)))
    return f


@dataclass
class RawMesh:
    """Vertices and cell->vertex indices in the reference's mesh schema."""
    n_dims: int
    vertices: np.ndarray          # (n_vertices, 3) float64
    vertex_indices: np.ndarray    # (n_cells, n_dims + 1) int64
    ghost: np.ndarray | None = None     # (n_cells,) uint8
    source: np.ndarray | None = None    # (n_cells,) int64

    @property
    def n_cells(self) -> int:
        return int(self.vertex_indices.shape[0])

    @staticmethod
    def generate(kind: str, *, n: int, halo: int = 0, radius: float = 1.0, jitter: float = 0.2,
                 seed: int = 1, renumber: bool = True) -> "RawMesh":
        """Synthetic meshes: 'periodic_square' (n squares per side + halo),
        'disk' (n rings), 'cube' (n^3 cubes of six tetrahedra)."""
        lib = load_library()
        kinds = {"periodic_square": 0, "disk": 1, "cube": 2}
        ip = np.array([n, halo], dtype=np.int64)
        dp = np.array([jitter] if kind != "disk" else [radius, jitter], dtype=np.float64)
        h = C.c_void_p()
        _check(lib.zfvm_rawmesh_generate(kinds[kind], _i64p(ip), _dp(dp), seed, int(renumber), C.byref(h)))
        try:
            nd, nv, nc, hg = C.c_int32(), C.c_int64(), C.c_int64(), C.c_int32()
            _check(lib.zfvm_rawmesh_sizes(h, C.byref(nd), C.byref(nv), C.byref(nc), C.byref(hg)))
            v = np.zeros((nv.value, 3))
            vi = np.zeros((nc.value, nd.value + 1), dtype=np.int64)
            g = np.zeros(nc.value, dtype=np.uint8)
            s = np.zeros(nc.value, dtype=np.int64)
            _check(lib.zfvm_rawmesh_copy(h, _dp(v), _i64p(vi), g.ctypes.data_as(C.POINTER(C.c_uint8)),
                                         _i64p(s)))
        finally:
            lib.zfvm_rawmesh_destroy(h)
        return RawMesh(nd.value, v, vi, g if hg.value else None, s if hg.value else None)


@dataclass
class StencilSpec:
    """reconstruction.{orders, biases, overfit_factors} (hybrid_weno_params.cpp:164-182)."""
    orders: list
    biased: list
    overfit: list

    @staticmethod
    def cweno(order: int, n_dims: int) -> "StencilSpec":
        """make_hybrid_weno_params(order) with one one-sided stencil per face."""
        nb = n_dims + 1
        if order == 2:
            return StencilSpec([2] + [2] * nb, [0] + [1] * nb, [3.0] + [2.0] * nb)
        return StencilSpec([order] + [2] * nb, [0] + [1] * nb, [2.0] + [1.5] * nb)


class Mesh:
    """Geometry + stencil families + LSQ pseudo-inverses of a RawMesh (host only)."""

    def __init__(self, raw: RawMesh, stencils: StencilSpec, quad=(3, 3, 2)):
        lib = load_library()
        self.raw = raw
        self.stencils_spec = stencils
        self.quad = tuple(quad)
        d = _MeshDesc()
        self._v = np.ascontiguousarray(raw.vertices, dtype=np.float64)
        self._vi = np.ascontiguousarray(raw.vertex_indices, dtype=np.int64)
        d.n_dims, d.n_vertices, d.n_cells = raw.n_dims, self._v.shape[0], self._vi.shape[0]
        d.vertices, d.vertex_indices = _dp(self._v), _i64p(self._vi)
        if raw.ghost is not None:
            self._g = np.ascontiguousarray(raw.ghost, dtype=np.uint8)
            d.ghost = self._g.ctypes.data_as(C.POINTER(C.c_uint8))
        if raw.source is not None:
            self._s = np.ascontiguousarray(raw.source, dtype=np.int64)
            d.source = _i64p(self._s)
        d.quad_edge, d.quad_volume, d.quad_moments = quad
        ns = len(stencils.orders)
        d.n_stencils = ns
        for k in range(ns):
            d.orders[k], d.biased[k], d.overfit[k] = stencils.orders[k], stencils.biased[k], stencils.overfit[k]
        h = C.c_void_p()
        _check(lib.zfvm_mesh_create(C.byref(d), C.byref(h)))
        self._h = h
        info = _MeshInfo()
        _check(lib.zfvm_mesh_get_info(h, C.byref(info)))
        self.info = {f: getattr(info, f) for f, _ in _MeshInfo._fields_}

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _LIB is not None:
            _LIB.zfvm_mesh_destroy(h)
            self._h = None

    @property
    def n_cells(self) -> int:
        return int(self.info["n_cells"])

    def stencils(self) -> dict:
        """Stencil families as flat arrays (the oracle's input)."""
        n = self.n_cells
        out = {
            "n_stencils": np.zeros(n, np.int8), "k_high": np.zeros(n, np.int8), "n_l2g": np.zeros(n, np.int8),
            "l2g": np.zeros((n, MAX_L2G), np.int32), "order": np.zeros((n, MAX_STENCILS), np.int8),
            "size": np.zeros((n, MAX_STENCILS), np.int8), "bias": np.zeros((n, MAX_STENCILS), np.int8),
            "local": np.zeros((n, MAX_STENCILS, MAX_STENCIL_SIZE), np.int8),
        }
        keys = ["n_stencils", "k_high", "n_l2g", "l2g", "order", "size", "bias", "local"]
        _check(load_library().zfvm_mesh_get_stencils(self._h, *[out[k].ctypes.data for k in keys]))
        return out

    def pinv(self, cell: int, k: int) -> np.ndarray:
        rows, cols = C.c_int32(), C.c_int32()
        _check(load_library().zfvm_mesh_get_pinv(self._h, cell, k, None, C.byref(rows), C.byref(cols)))
        P = np.zeros((cols.value, rows.value))
        _check(load_library().zfvm_mesh_get_pinv(self._h, cell, k, _dp(P), C.byref(rows), C.byref(cols)))
        return P

    def geometry(self) -> dict:
        n = self.n_cells
        vol, rin, cen = np.zeros(n), np.zeros(n), np.zeros((n, 3))
        flags = np.zeros(n, np.uint8)
        _check(load_library().zfvm_mesh_get_geometry(self._h, _dp(vol), _dp(rin), _dp(cen),
                                                      flags.ctypes.data_as(C.POINTER(C.c_uint8))))
        return {"volumes": vol, "inradii": rin, "centers": cen, "flags": flags}

    def connectivity(self) -> dict:
        """Neighbour across every local face (-1: boundary) and the face's number,
        n_cells x (n_dims + 1) each."""
        n, nb = self.n_cells, int(self.info["n_dims"]) + 1
        nbr, edge = np.zeros((n, nb), np.int64), np.zeros((n, nb), np.int64)
        _check(load_library().zfvm_mesh_get_connectivity(self._h, _i64p(nbr), _i64p(edge)))
        return {"neighbours": nbr, "edge_indices": edge}

    def faces(self) -> dict:
        """Left / right cell (-1: boundary), unit normal out of the left cell and
        area of every face, interior faces first."""
        m = int(self.info["n_edges"])
        left, right = np.zeros(m, np.int64), np.zeros(m, np.int64)
        normals, areas = np.zeros((m, 3)), np.zeros(m)
        _check(load_library().zfvm_mesh_get_faces(self._h, _i64p(left), _i64p(right), _dp(normals), _dp(areas)))
        return {"left": left, "right": right, "normals": normals, "areas": areas}

    def initial_conditions(self, kind: str, **p) -> np.ndarray:
        """Cell averages (n_cells x 5) of 'vortex', 'polytrope' (phi = k r^2 / 2) or
        'polytrope_in' (any analytic radial potential) initial data."""
        if kind == "vortex":
            params = [p.get("gamma", 1.4), p.get("beta", 5.0), p.get("x0", 0.5), p.get("y0", 0.5),
                      p.get("length", 0.1), p.get("rho_inf", 1.0), p.get("u_inf", 1.0), p.get("v_inf", 1.0),
                      p.get("p_inf", 1.0)]
            k = 0
        elif kind == "polytrope":
            params = [p.get("gamma", 2.0), p.get("K", 1.0), p.get("rho_c", 1.0), p.get("k_phi", 1.0),
                      p.get("amplitude", 1e-4), p.get("width", 0.05), p.get("x0", 0.3), p.get("y0", 0.0)]
            k = 1
        elif kind == "polytrope_in":
            # isentropic polytrope in a radial potential: gravity=GRAVITY_*, strength, params
            gp = (list(p.get("gravity_params", [])) + [0.0] * 5)[:5]
            params = [p.get("gamma", 2.0), p.get("K", 1.0), p.get("rho_c", 1.0), p.get("amplitude", 1e-4),
                      p.get("width", 0.05), p.get("x0", 0.3), p.get("y0", 0.0), p["gravity"],
                      p.get("gravity_strength", 0.0), *gp]
            k = 2
        else:
            raise ValueError(kind)
        out = np.zeros((self.n_cells, 5))
        _check(load_library().zfvm_initial_conditions(self._h, k, _dp(np.array(params, dtype=np.float64)),
                                                      _dp(out)))
        return out


@dataclass
class Scheme:
    """The solver configuration, named after the reference's config keys."""
    flux: int = FLUX_HLLC
    gamma: float = 1.4
    specific_gas_constant: float = 1.0
    linear_weights: list = field(default_factory=lambda: [100.0, 1.0, 1.0, 1.0])
    epsilon: float = 1e-6
    exponent: float = 4.0
    rk_stages: int = 3
    cfl_number: float = 0.45
    equilibrium: int = EQ_NONE
    gravity: int = GRAVITY_NONE
    gravity_strength: float = 0.0
    flux_bc: int = FLUX_BC_NONE
    boundary: int = BC_NONE
    precision: int = FP64
    steps_per_recompute: int = 1
    recompute_threshold: float = 0.0
    reconstruction: int = 0  # RC_CWENO_AO or RC_WENO_AO
    step_rejection_drho: float = 0.0   # 0: RejectNothing
    step_rejection_max_exponent: int = 0
    heating_rate: float = 0.0  # heating.rate; 0: no heating
    heating_r0: float = 0.0
    heating_r1: float = 0.0
    n_avars: int = 0  # advected variables (mass-weighted tracers)
    # parameters of the gravity kind: (rhoC, K, G) polytrope; (r_crit, rhoC,
    # K_inner, K_outer, G) polytrope with a jump; (G, M, X) point mass
    gravity_params: list = field(default_factory=lambda: [0.0] * 5)
    # GRAVITY_RADIAL_TABLE: (radii, potentials), radii increasing
    gravity_table: tuple | None = None

    def desc(self) -> _SchemeDesc:
        d = _SchemeDesc()
        for f, _ in _SchemeDesc._fields_:
            if f == "linear_weights":
                for k, w in enumerate(self.linear_weights):
                    d.linear_weights[k] = w
            elif f == "gravity_params":
                for k, w in enumerate(self.gravity_params):
                    d.gravity_params[k] = w
            elif f in ("gravity_table_r", "gravity_table_phi", "gravity_table_n"):
                continue
            else:
                setattr(d, f, getattr(self, f))
        if self.gravity_table is not None:
            r = np.ascontiguousarray(self.gravity_table[0], dtype=np.float64)
            phi = np.ascontiguousarray(self.gravity_table[1], dtype=np.float64)
            if r.shape != phi.shape or r.ndim != 1:
                raise ValueError("gravity_table: radii and potentials of the same length")
            d._table = (r, phi)  # the arrays live as long as the descriptor
            d.gravity_table_r, d.gravity_table_phi, d.gravity_table_n = _dp(r), _dp(phi), len(r)
        return d

    def oracle_vector(self) -> np.ndarray:
        lw = list(self.linear_weights) + [0.0] * (5 - len(self.linear_weights))
        return np.array([self.flux, self.gamma, self.specific_gas_constant, *lw, self.epsilon, self.exponent,
                         self.rk_stages, self.cfl_number, self.equilibrium, self.gravity, self.gravity_strength,
                         self.flux_bc, self.boundary, self.steps_per_recompute, self.recompute_threshold,
                         self.reconstruction, self.step_rejection_drho, self.step_rejection_max_exponent,
                         self.heating_rate, self.heating_r0, self.heating_r1, self.n_avars,
                         *(list(self.gravity_params) + [0.0] * 5)[:5], *self._table_vector()],
                        dtype=np.float64)

    def _table_vector(self) -> list:
        if self.gravity_table is None:
            return [0.0]
        r, phi = (np.asarray(a, dtype=np.float64) for a in self.gravity_table)
        return [float(len(r)), *r.tolist(), *phi.tolist()]


class Solver:
    """Device-resident solver state; every method runs CUDA kernels."""

    def __init__(self, mesh: Mesh, scheme: Scheme):
        self.mesh, self.scheme = mesh, scheme
        lib = load_library()
        h = C.c_void_p()
        self._desc = scheme.desc()
        _check(lib.zfvm_solver_create(mesh._h, C.byref(self._desc), C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None) is not None and _LIB is not None:
            _LIB.zfvm_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def set_state(self, cvars: np.ndarray, t: float = 0.0) -> None:
        a = np.ascontiguousarray(cvars, dtype=np.float64)
        assert a.shape == (self.mesh.n_cells, 5)
        _check(load_library().zfvm_set_state(self._h, _dp(a), t))

    def get_state(self, out: np.ndarray | None = None) -> tuple[np.ndarray, float]:
        """Copy the state to the host (into `out` when given, e.g. pinned memory)."""
        a = out if out is not None else np.zeros((self.mesh.n_cells, 5))
        assert a.shape == (self.mesh.n_cells, 5) and a.dtype == np.float64 and a.flags.c_contiguous
        t = C.c_double()
        _check(load_library().zfvm_get_state(self._h, _dp(a), C.byref(t)))
        return a, t.value

    def step_host(self, cvars: np.ndarray, t: float = 0.0, n_steps: int = 1, t_end: float = 0.0,
                  fixed_dt: float = 0.0, out: np.ndarray | None = None) -> tuple[np.ndarray, float, int]:
        """Upload `cvars`, advance, download into `out` (e.g. pinned memory) in
        one call with one host synchronisation: (state, t, steps)."""
        a = np.ascontiguousarray(cvars, dtype=np.float64)
        assert a.shape == (self.mesh.n_cells, 5)
        o = out if out is not None else np.empty((self.mesh.n_cells, 5))
        assert o.shape == (self.mesh.n_cells, 5) and o.dtype == np.float64 and o.flags.c_contiguous
        tt, st = C.c_double(), C.c_int64()
        _check(load_library().zfvm_step_host(self._h, _dp(a), t, n_steps, t_end, fixed_dt, _dp(o), C.byref(tt),
                                             C.byref(st)))
        return o, tt.value, st.value

    def set_avars(self, avars: np.ndarray) -> None:
        """Advected variables (mass-weighted tracers), n_cells x n_avars."""
        a = np.ascontiguousarray(avars, dtype=np.float64).reshape(self.mesh.n_cells, self.scheme.n_avars)
        _check(load_library().zfvm_set_avars(self._h, _dp(a)))

    def get_avars(self) -> np.ndarray:
        a = np.zeros((self.mesh.n_cells, self.scheme.n_avars))
        _check(load_library().zfvm_get_avars(self._h, _dp(a)))
        return a

    def rate_of_change_all(self) -> tuple[np.ndarray, np.ndarray]:
        """Tendencies of the conserved and of the advected variables."""
        u = np.zeros((self.mesh.n_cells, 5))
        q = np.zeros((self.mesh.n_cells, self.scheme.n_avars))
        _check(load_library().zfvm_rate_of_change_all(self._h, _dp(u), _dp(q)))
        return u, q

    def write_snapshot(self, path, n_steps: int = 0) -> None:
        """Current state and time to a snapshot file (see `write_snapshot`)."""
        _check(load_library().zfvm_solver_write_snapshot(self._h, os.fsencode(path), n_steps))

    def read_snapshot(self, path) -> int:
        """Restart from a snapshot file: state and time; returns its step count."""
        n = C.c_int64()
        _check(load_library().zfvm_solver_read_snapshot(self._h, os.fsencode(path), C.byref(n)))
        return n.value

    def apply_boundary(self, cvars: np.ndarray, frozen: np.ndarray | None = None, avars=None,
                       frozen_avars=None):
        """BoundaryCondition::apply with this solver's ghost cells on host
        states: frozen ghosts from `frozen` (unchanged without), periodic
        images from their sources.  Returns new arrays."""
        u = np.array(cvars, dtype=np.float64, order="C", copy=True)
        fz = None if frozen is None else np.ascontiguousarray(frozen, dtype=np.float64)
        q = None if avars is None else np.array(avars, dtype=np.float64, order="C", copy=True)
        fq = None if frozen_avars is None else np.ascontiguousarray(frozen_avars, dtype=np.float64)
        _check(load_library().zfvm_apply_boundary(self._h, None if fz is None else _dp(fz),
                                                  None if fq is None else _dp(fq), _dp(u),
                                                  None if q is None else _dp(q)))
        return u if q is None else (u, q)

    def rate_of_change(self) -> np.ndarray:
        a = np.zeros((self.mesh.n_cells, 5))
        _check(load_library().zfvm_rate_of_change(self._h, _dp(a)))
        return a

    def step_rejections(self) -> int:
        n = C.c_int64()
        _check(load_library().zfvm_step_rejections(self._h, C.byref(n)))
        return n.value

    def reconstruct(self) -> None:
        """Reconstruct the current state (GlobalReconstruction::compute)."""
        _check(load_library().zfvm_reconstruct(self._h))

    def reconstruction_eval(self, cells, x) -> np.ndarray:
        """Reconstruction of cells[k] at the points x[k] (n x 3), as n x 5 rows."""
        c = np.ascontiguousarray(cells, dtype=np.int64)
        xx = np.ascontiguousarray(x, dtype=np.float64).reshape(len(c), 3)
        out = np.zeros((len(c), 5))
        _check(load_library().zfvm_reconstruction_eval(self._h, len(c), _i64p(c), _dp(xx), _dp(out)))
        return out

    def cfl_dt(self) -> float:
        dt = C.c_double()
        _check(load_library().zfvm_cfl_dt(self._h, C.byref(dt)))
        return dt.value

    def step(self, dt: float) -> None:
        _check(load_library().zfvm_step(self._h, dt))

    def advance(self, n_steps: int = 0, t_end: float = 0.0) -> tuple[float, int]:
        t, s = C.c_double(), C.c_int64()
        _check(load_library().zfvm_advance(self._h, n_steps, t_end, C.byref(t), C.byref(s)))
        return t.value, s.value

    def advance_timed(self, n_steps: int) -> float:
        ms = C.c_float()
        _check(load_library().zfvm_advance_timed(self._h, n_steps, C.byref(ms)))
        return float(ms.value)

    def kernel_times(self, n_steps: int) -> dict:
        """Average per-launch milliseconds of {reconstruct, face_flux, update}."""
        ms = (C.c_float * 3)()
        _check(load_library().zfvm_kernel_times(self._h, n_steps, ms))
        return {"reconstruct": ms[0], "face_flux": ms[1], "update": ms[2]}

    def launches_per_step(self) -> int:
        n = C.c_int32()
        _check(load_library().zfvm_launches_per_step(self._h, C.byref(n)))
        return n.value

    def device_bytes(self) -> int:
        n = C.c_int64()
        _check(load_library().zfvm_device_bytes(self._h, C.byref(n)))
        return n.value


class Batch:
    """Independent solves stepped together (one launch per phase per stage)."""

    def __init__(self, max_slots: int):
        h = C.c_void_p()
        _check(load_library().zfvm_batch_create(max_slots, C.byref(h)))
        self._h = h
        self._members = {}
        self._max_slots = max_slots

    def close(self):
        if getattr(self, "_h", None) is not None and _LIB is not None:
            _LIB.zfvm_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def add(self, solver: Solver, n_steps: int = 0, t_end: float = 0.0) -> int:
        slot = C.c_int32()
        _check(load_library().zfvm_batch_add(self._h, solver._h, n_steps, t_end, C.byref(slot)))
        self._members[slot.value] = solver
        return slot.value

    def remove(self, slot: int) -> Solver:
        _check(load_library().zfvm_batch_remove(self._h, slot))
        return self._members.pop(slot)

    def advance(self, max_steps: int) -> int:
        n = C.c_int32()
        _check(load_library().zfvm_batch_advance(self._h, max_steps, C.byref(n)))
        return n.value

    def advance_timed(self, n_steps: int) -> float:
        ms = C.c_float()
        _check(load_library().zfvm_batch_advance_timed(self._h, n_steps, C.byref(ms)))
        return float(ms.value)

    def step_host(self, states_in: dict | None, states_out: dict | None, max_steps: int = 1) -> int:
        """One host round trip for the whole batch (zfvm_batch_step_host): the
        slots in `states_in` ({slot: n_cells x 5 float64 array}) take those
        states, the batch advances up to max_steps steps, and the slots in
        `states_out` are read back into their arrays (which may be the input
        arrays; page-locked arrays make the copies asynchronous).  Returns the
        number of slots still running."""
        def table(states, writable):
            if states is None:
                return None
            arr = (C.c_void_p * self._max_slots)()
            for slot, a in states.items():
                if slot not in self._members:
                    raise ZfvmError(1, f"slot {slot} holds no solver")
                want = (self._members[slot].mesh.n_cells, 5)
                if a.dtype != np.float64 or not a.flags.c_contiguous or a.shape != want or (
                        writable and not a.flags.writeable):
                    raise ZfvmError(1, f"slot {slot}: need a C-contiguous float64 array of shape {want}")
                arr[slot] = a.ctypes.data
            return arr
        tin, tout = table(states_in, False), table(states_out, True)
        n = C.c_int32()
        _check(load_library().zfvm_batch_step_host(self._h, tin, tout, max_steps, C.byref(n)))
        return n.value

    def autotune(self, trial_steps: int = 4) -> float:
        ms = C.c_float()
        _check(load_library().zfvm_batch_autotune(self._h, trial_steps, C.byref(ms)))
        return float(ms.value)

    def kernel_times(self, n_steps: int) -> dict:
        ms = (C.c_float * 3)()
        _check(load_library().zfvm_batch_kernel_times(self._h, n_steps, ms))
        return {"reconstruct": ms[0], "face_flux": ms[1], "update": ms[2]}

    def tuned_shapes(self) -> list:
        """Launch shape of each kernel group: stencil shape id, threads per block
        (= tile size), grids of the three kernels (0: one block per tile), tuned."""
        buf = (C.c_int32 * (6 * 16))()
        n = C.c_int32()
        _check(load_library().zfvm_batch_launch_shapes(self._h, 16, buf, C.byref(n)))
        return [{"shape": buf[6 * k], "block": buf[6 * k + 1], "grid_recon": buf[6 * k + 2],
                 "grid_face": buf[6 * k + 3], "grid_update": buf[6 * k + 4], "tuned": bool(buf[6 * k + 5])}
                for k in range(min(n.value, 16))]

    def status(self, slot: int) -> dict:
        t, st, done, status = C.c_double(), C.c_int64(), C.c_int32(), C.c_int32()
        _check(load_library().zfvm_batch_slot_status(self._h, slot, C.byref(t), C.byref(st), C.byref(done),
                                                     C.byref(status)))
        return {"t": t.value, "steps": st.value, "done": bool(done.value), "status": status.value}


def write_snapshot(path, cvars: np.ndarray, t: float | None = None, n_steps: int | None = None,
                   avars: np.ndarray | None = None) -> None:
    """Write a snapshot file: the reference's datasets ("time", "n_steps", "rho",
    "mv1", "mv2", "mv3", "E", "n_avars", "mq<k>") in an uncompressed .npz.
    Without `t` the file has no clock (the steady-state file)."""
    u = np.ascontiguousarray(cvars, dtype=np.float64)
    assert u.ndim == 2 and u.shape[1] == 5
    q = None if avars is None else np.ascontiguousarray(avars, dtype=np.float64).reshape(u.shape[0], -1)
    na = 0 if q is None else q.shape[1]
    _check(load_library().zfvm_snapshot_write(os.fsencode(path), u.shape[0], _dp(u), na,
                                              None if q is None else _dp(q), int(t is not None),
                                              0.0 if t is None else float(t), int(n_steps or 0)))


def read_snapshot(path) -> dict:
    """Read a snapshot file: {"cvars", "avars", "time", "n_steps"} (the clock
    entries are None in a steady-state file)."""
    lib = load_library()
    n, na, hc = C.c_int64(), C.c_int32(), C.c_int32()
    _check(lib.zfvm_snapshot_info(os.fsencode(path), C.byref(n), C.byref(na), C.byref(hc)))
    u = np.zeros((n.value, 5))
    q = np.zeros((n.value, na.value))
    t, st = C.c_double(), C.c_int64()
    _check(lib.zfvm_snapshot_read(os.fsencode(path), n.value, _dp(u), na.value, _dp(q) if na.value else None,
                                  C.byref(t) if hc.value else None, C.byref(st) if hc.value else None))
    return {"cvars": u, "avars": q, "time": t.value if hc.value else None, "n_steps": st.value if hc.value else None}


def solver_footprint(mesh: "Mesh", scheme: "Scheme") -> int:
    """Device bytes a Solver of this mesh and scheme allocates (host-side count)."""
    desc = scheme.desc()
    n = C.c_int64()
    _check(load_library().zfvm_solver_footprint(mesh._h, C.byref(desc), C.byref(n)))
    return n.value


class Server:
    """Request loop with continuous batching (see zfvm_server_* in zfvm.h).

    submit() queues a solve and returns its id at once; wait() blocks until it
    is done and returns (final state, final time, steps, times in ms
    {queued, running, total}).  Meshes must stay alive until their requests
    have been waited for; this object keeps a reference for that."""

    QUEUED, RUNNING, DONE, FAILED = 0, 1, 2, 3

    def __init__(self, hbm_budget_bytes: int = 0, max_slots: int = 64, steps_per_round: int = 8):
        d = _ServerDesc(hbm_budget_bytes, max_slots, steps_per_round)
        h = C.c_void_p()
        _check(load_library().zfvm_server_create(C.byref(d), C.byref(h)))
        self._h = h
        self._meshes = {}

    def close(self):
        if getattr(self, "_h", None) is not None and _LIB is not None:
            _LIB.zfvm_server_destroy(self._h)
            self._h = None
            self._meshes.clear()

    def __del__(self):
        self.close()

    def submit(self, mesh: "Mesh", scheme: "Scheme", cvars: np.ndarray, t0: float = 0.0, n_steps: int = 0,
               t_end: float = 0.0) -> int:
        a = np.ascontiguousarray(cvars, dtype=np.float64)
        assert a.shape == (mesh.n_cells, 5)
        desc = scheme.desc()
        rid = C.c_int64()
        _check(load_library().zfvm_server_submit(self._h, mesh._h, C.byref(desc), _dp(a), t0, n_steps, t_end,
                                                 C.byref(rid)))
        self._meshes[rid.value] = mesh
        return rid.value

    def poll(self, rid: int) -> int:
        ph = C.c_int32()
        _check(load_library().zfvm_server_poll(self._h, rid, C.byref(ph)))
        return ph.value

    def wait(self, rid: int, timeout_s: float = -1.0):
        mesh = self._meshes[rid]
        out = np.empty((mesh.n_cells, 5))
        t, st = C.c_double(), C.c_int64()
        times = (C.c_double * 3)()
        try:
            _check(load_library().zfvm_server_wait(self._h, rid, timeout_s, _dp(out), C.byref(t), C.byref(st),
                                                   C.cast(times, C.POINTER(C.c_double))))
        except ZfvmError as e:
            if e.code != 5:  # a timeout keeps the request
                self._meshes.pop(rid, None)
            raise
        self._meshes.pop(rid, None)
        return out, t.value, st.value, {"queued": times[0], "running": times[1], "total": times[2]}

    def stats(self) -> dict:
        s = _ServerStats()
        _check(load_library().zfvm_server_get_stats(self._h, C.byref(s)))
        return {n: getattr(s, n) for n, _ in _ServerStats._fields_}
