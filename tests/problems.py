"""Problem set-ups shared by tests, smoke() and the benchmark.

Each returns (raw_mesh, mesh, scheme, initial_state).  The configurations are
the workloads of the benchmark suite (C1 periodic vortex, C2 well-balanced
polytrope, C3 tetrahedral vortex tube), optionally at smaller sizes.
"""
from __future__ import annotations

import zisafvm_gb300 as z


def vortex_2d(n: int = 160, halo: int = 3, flux: int = z.FLUX_RUSANOV, seed: int = 1):
    """C1: periodic unit square, n x n squares of two triangles, jitter 0.2 h,
    isentropic vortex (beta 5, core length 0.1) on rho = 1, u = (1, 1), p = 1,
    CWENO-AO order 3, SSP3, CFL 0.45."""
    raw = z.RawMesh.generate("periodic_square", n=n, halo=halo, jitter=0.2, seed=seed)
    mesh = z.Mesh(raw, z.StencilSpec.cweno(3, 2), quad=(3, 3, 2))
    scheme = z.Scheme(flux=flux, gamma=1.4, linear_weights=[100.0, 1.0, 1.0, 1.0], epsilon=1e-6, exponent=4.0,
                      rk_stages=3, cfl_number=0.45, boundary=z.BC_PERIODIC)
    u0 = mesh.initial_conditions("vortex", gamma=1.4, beta=5.0, x0=0.5, y0=0.5, length=0.1)
    return raw, mesh, scheme, u0


def polytrope_2d(n_rings: int = 178, amplitude: float = 1e-4, seed: int = 7, precision: int = z.FP64):
    """C2: disk of radius 1 (~2 pi n_rings^2 triangles), gamma = 2, K = 1,
    phi = r^2 / 2, polytrope rho = 1 - r^2 / 4 plus a Gaussian pressure bump of
    width 0.05 at r = 0.3; CWENO-AO order 3, HLLC, SSP3, CFL 0.45, isentropic
    well-balancing and equilibrium flux boundary."""
    raw = z.RawMesh.generate("disk", n=n_rings, radius=1.0, jitter=0.2, seed=seed)
    mesh = z.Mesh(raw, z.StencilSpec.cweno(3, 2), quad=(3, 3, 2))
    scheme = z.Scheme(flux=z.FLUX_HLLC, gamma=2.0, linear_weights=[100.0, 1.0, 1.0, 1.0], epsilon=1e-6,
                      exponent=4.0, rk_stages=3, cfl_number=0.45, equilibrium=z.EQ_ISENTROPIC,
                      gravity=z.GRAVITY_HARMONIC_RADIAL, gravity_strength=1.0, flux_bc=z.FLUX_BC_ISENTROPIC,
                      precision=precision)
    u0 = mesh.initial_conditions("polytrope", gamma=2.0, K=1.0, rho_c=1.0, k_phi=1.0, amplitude=amplitude,
                                 width=0.05, x0=0.3, y0=0.0)
    return raw, mesh, scheme, u0


def vortex_tube_3d(n: int = 70, order: int = 3, seed: int = 1):
    """C3: unit cube of n^3 x 6 jittered tetrahedra, vortex tube along z,
    HLLC, SSP3, CFL 0.3, constant flux boundary."""
    raw = z.RawMesh.generate("cube", n=n, jitter=0.1, seed=seed)
    quad = (2, 2, 2) if order == 3 else (2, 2, 1)
    mesh = z.Mesh(raw, z.StencilSpec.cweno(order, 3), quad=quad)
    scheme = z.Scheme(flux=z.FLUX_HLLC, gamma=1.4, linear_weights=[100.0, 1.0, 1.0, 1.0, 1.0], epsilon=1e-6,
                      exponent=4.0, rk_stages=3, cfl_number=0.3, flux_bc=z.FLUX_BC_CONSTANT)
    u0 = mesh.initial_conditions("vortex", gamma=1.4, beta=5.0, x0=0.5, y0=0.5, length=0.1, v_inf=1.0, u_inf=1.0)
    return raw, mesh, scheme, u0


def polytrope_2d_frozen(n_rings: int = 60, amplitude: float = 1e-4, seed: int = 11, precision: int = z.FP64,
                        r_frozen: float = 0.5):
    """The well-balanced polytrope with the reference's experiment boundary:
    cells with centres beyond r = 0.5 are frozen ghost cells
    (Polytrope::boundary_mask, experiments/polytrope.cpp:55-63, with FrozenBC)."""
    import numpy as np
    raw = z.RawMesh.generate("disk", n=n_rings, radius=1.0, jitter=0.2, seed=seed)
    c = raw.vertices[raw.vertex_indices].mean(axis=1)
    raw.ghost = (np.hypot(c[:, 0], c[:, 1]) > r_frozen).astype(np.uint8)
    raw.source = np.arange(raw.n_cells, dtype=np.int64)
    mesh = z.Mesh(raw, z.StencilSpec.cweno(3, 2), quad=(3, 3, 2))
    scheme = z.Scheme(flux=z.FLUX_HLLC, gamma=2.0, linear_weights=[100.0, 1.0, 1.0, 1.0], epsilon=1e-6,
                      exponent=4.0, rk_stages=3, cfl_number=0.45, equilibrium=z.EQ_ISENTROPIC,
                      gravity=z.GRAVITY_HARMONIC_RADIAL, gravity_strength=1.0, flux_bc=z.FLUX_BC_ISENTROPIC,
                      boundary=z.BC_FROZEN, precision=precision)
    u0 = mesh.initial_conditions("polytrope", gamma=2.0, K=1.0, rho_c=1.0, k_phi=1.0, amplitude=amplitude,
                                 width=0.05, x0=0.3, y0=0.0)
    return raw, mesh, scheme, u0


def polytrope_3d(n: int = 40, amplitude: float = 1e-4, seed: int = 3, precision: int = z.FP64, order: int = 3):
    """gamma = 2 isentropic polytrope on the unit cube of n^3 x 6 jittered
    tetrahedra, phi = r^2 / 2 about the origin (the cube is one octant of the
    star: rho = 1 - r^2 / 4 falls from 1 to 1/4 at the far corner), plus a
    Gaussian pressure tube along z of width 0.05 through (0.5, 0.4); CWENO-AO,
    HLLC, SSP3, CFL 0.3, isentropic well-balancing and flux boundary."""
    raw = z.RawMesh.generate("cube", n=n, jitter=0.1, seed=seed)
    quad = (2, 2, 2) if order == 3 else (2, 2, 1)
    mesh = z.Mesh(raw, z.StencilSpec.cweno(order, 3), quad=quad)
    scheme = z.Scheme(flux=z.FLUX_HLLC, gamma=2.0, linear_weights=[100.0, 1.0, 1.0, 1.0, 1.0], epsilon=1e-6,
                      exponent=4.0, rk_stages=3, cfl_number=0.3, equilibrium=z.EQ_ISENTROPIC,
                      gravity=z.GRAVITY_HARMONIC_RADIAL, gravity_strength=1.0, flux_bc=z.FLUX_BC_ISENTROPIC,
                      precision=precision)
    u0 = mesh.initial_conditions("polytrope", gamma=2.0, K=1.0, rho_c=1.0, k_phi=1.0, amplitude=amplitude,
                                 width=0.05, x0=0.5, y0=0.4)
    return raw, mesh, scheme, u0


def c4_instance_params(n_instances: int = 256, n_min: int = 5000, n_max: int = 200000, seed: int = 2024):
    """The ensemble's per-instance draws: disk rings (log-uniform cell count in
    [n_min, n_max]), perturbation amplitude (log-uniform in [1e-6, 1e-2]),
    centre radius U[0.1, 0.7] and angle, and the mesh seed."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_instances):
        n_cells = float(np.exp(rng.uniform(np.log(n_min), np.log(n_max))))
        rings = max(4, int(round(np.sqrt(n_cells / (2.0 * np.pi)))))
        amp = float(np.exp(rng.uniform(np.log(1e-6), np.log(1e-2))))
        r0, ang = float(rng.uniform(0.1, 0.7)), float(rng.uniform(0.0, 2.0 * np.pi))
        out.append(dict(rings=rings, amplitude=amp, r0=r0, angle=ang, mesh_seed=seed + 17 * k + 1))
    return out


def c4_instance(p: dict, precision: int = z.MIXED):
    """One ensemble instance: a seeded jittered disk, the gamma = 2, K = 1
    polytrope in phi = r^2 / 2 plus its Gaussian bump of width 0.05; CWENO-AO
    order 3, HLLC, SSP3, CFL 0.45, isentropic well-balancing."""
    import numpy as np
    raw = z.RawMesh.generate("disk", n=p["rings"], radius=1.0, jitter=0.2, seed=p["mesh_seed"])
    mesh = z.Mesh(raw, z.StencilSpec.cweno(3, 2), quad=(3, 3, 2))
    scheme = z.Scheme(flux=z.FLUX_HLLC, gamma=2.0, linear_weights=[100.0, 1.0, 1.0, 1.0], epsilon=1e-6,
                      exponent=4.0, rk_stages=3, cfl_number=0.45, equilibrium=z.EQ_ISENTROPIC,
                      gravity=z.GRAVITY_HARMONIC_RADIAL, gravity_strength=1.0,
                      flux_bc=z.FLUX_BC_ISENTROPIC, precision=precision)
    u0 = mesh.initial_conditions("polytrope", gamma=2.0, K=1.0, rho_c=1.0, k_phi=1.0, amplitude=p["amplitude"],
                                 width=0.05, x0=p["r0"] * np.cos(p["angle"]), y0=p["r0"] * np.sin(p["angle"]))
    return raw, mesh, scheme, u0


def ensemble_c4(n_instances: int = 256, n_min: int = 5000, n_max: int = 200000, seed: int = 2024,
                precision: int = z.MIXED):
    """C4: independent well-balanced polytrope solves on seeded jittered disk
    meshes with log-uniform sizes in [n_min, n_max] triangles, perturbation
    amplitudes log-uniform in [1e-6, 1e-2], centres at r ~ U[0.1, 0.7] and a
    random angle, width 0.05; CWENO-AO order 3, HLLC, SSP3."""
    return [c4_instance(p, precision) for p in c4_instance_params(n_instances, n_min, n_max, seed)]


def tracers(mesh, u0, n_avars: int = 2):
    """Mass-weighted tracers mq_k = rho q_k for n_avars mass fractions: a sharp
    tanh front across x = 0.45 (exercises the nonlinear weights), a smooth
    wave, then alternating copies."""
    import numpy as np
    c = mesh.geometry()["centers"]
    q = np.empty((u0.shape[0], n_avars))
    for k in range(n_avars):
        if k % 2 == 0:
            q[:, k] = 1.0 + 0.5 * np.tanh((c[:, 0] - 0.45) / 0.02)
        else:
            q[:, k] = 0.3 + 0.2 * np.sin(2 * np.pi * c[:, 1]) * np.cos(2 * np.pi * c[:, 0])
    return u0[:, :1] * q
