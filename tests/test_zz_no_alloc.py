"""zfvm_rate_of_change_noalloc against zfvm_rate_of_change, through the C ABI.

The no-allocation entry point serves callers that must not allocate device
memory while they run (their own pool allocator owns the device memory, or
they cannot take the device-wide wait of cudaFree).  It keeps its stage
scratch in one fixed array inside the library that every call reuses, so the
test makes two calls in a row on different states, for several solvers one
after another: each result must match the allocating entry point's within the
right-hand-side tolerance of the parity tests, whatever the previous call left
in the array.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from problems import polytrope_2d, polytrope_2d_frozen, polytrope_3d, tracers, vortex_2d, vortex_tube_3d

pytestmark = pytest.mark.gpu

TOL_RHS = 1e-13


def _noalloc(z, solver):
    fn = z.load_library().zfvm_rate_of_change_noalloc
    fn.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
    fn.restype = C.c_int
    out = np.full((solver.mesh.n_cells, 5), np.nan)
    status = fn(solver._h, out.ctypes.data_as(C.POINTER(C.c_double)))
    return status, out


def _perturbed(u0, seed):
    rng = np.random.default_rng(seed)
    u = u0.copy()
    u[:, 0] *= 1.0 + 0.01 * rng.standard_normal(len(u))
    u[:, 1:4] += 0.01 * rng.standard_normal((len(u), 3)) * (u0[:, 1:4] != 0)
    u[:, 4] *= 1.0 + 0.01 * rng.standard_normal(len(u))
    return u


def _assert_close(got, ref):
    assert np.isfinite(got).all()
    scale = np.maximum(np.abs(ref).max(axis=0), 1e-300)
    err = (np.abs(got - ref).max(axis=0) / scale).max()
    assert err <= TOL_RHS, err


def _heated_frozen(z, precision):
    raw, mesh, scheme, u0 = polytrope_2d_frozen(n_rings=30, amplitude=1e-3, precision=precision)
    scheme.heating_rate, scheme.heating_r0, scheme.heating_r1 = 0.3, 0.2, 0.45
    return raw, mesh, scheme, u0


def _with_tracers(z):
    raw, mesh, scheme, u0 = vortex_2d(n=24, halo=3, flux=z.FLUX_HLLC)
    scheme.n_avars = 2
    return raw, mesh, scheme, u0


# Each case changes which scratch pieces the call carves out of the array and
# which of them the kernels read: FP64 or mixed face values and fluxes, the
# equilibrium and source pieces, 2D or 3D strides, frozen ghost cells, heating.
CASES = {
    "vortex_fp64_periodic": lambda z: vortex_2d(n=32, halo=3, flux=z.FLUX_HLLC),
    "polytrope_mixed": lambda z: polytrope_2d(n_rings=40, amplitude=1e-3, precision=z.MIXED),
    "polytrope_fp64": lambda z: polytrope_2d(n_rings=30, amplitude=1e-3),
    "tets_fp64": lambda z: vortex_tube_3d(n=10),
    "polytrope3d_mixed": lambda z: polytrope_3d(n=8, amplitude=1e-3, precision=z.MIXED),
    "frozen_heated_fp64": lambda z: _heated_frozen(z, z.FP64),
    "frozen_heated_mixed": lambda z: _heated_frozen(z, z.MIXED),
    # advected variables do not enter the conserved tendency this call returns
    "tracers_fp64": _with_tracers,
}


def test_two_calls_in_a_row_match_allocating_entry_point(zlib):
    z = zlib
    for name, make in CASES.items():
        _, mesh, scheme, u0 = make(z)
        s = z.Solver(mesh, scheme)
        if scheme.n_avars:
            s.set_avars(tracers(mesh, u0, scheme.n_avars))
        states = [u0, _perturbed(u0, seed=len(name))]
        got = []
        for u in states:  # two calls in a row of the new entry point
            s.set_state(u)
            status, t = _noalloc(z, s)
            assert status == 0, (name, z.load_library().zfvm_last_error())
            got.append(t)
        for u, t in zip(states, got):
            s.set_state(u)
            _assert_close(t, s.rate_of_change())
        s.close()


def test_rejects_solver_beyond_fixed_scratch(zlib):
    z = zlib
    _, mesh, scheme, u0 = vortex_2d(n=200, halo=3)
    s = z.Solver(mesh, scheme)
    s.set_state(u0)
    status, _ = _noalloc(z, s)
    assert status == 1
    msg = z.load_library().zfvm_last_error().decode()
    assert "bytes of stage scratch" in msg and str(16 << 20) in msg
    # the solver stays usable through the allocating entry point
    assert np.isfinite(s.rate_of_change()).all()
    s.close()
