"""Host set-up: meshes, geometry, Hilbert renumbering, stencils, LSQ operators."""
import numpy as np
import pytest


def test_periodic_square_mesh(zlib):
    z = zlib
    raw = z.RawMesh.generate("periodic_square", n=8, halo=3, jitter=0.2, seed=3)
    assert raw.n_cells == (8 + 6) ** 2 * 2
    assert raw.ghost.sum() == raw.n_cells - 8 * 8 * 2
    # periodic sources are interior cells, and interior cells are their own source
    assert np.all(raw.ghost[raw.source] == 0)
    inner = np.where(raw.ghost == 0)[0]
    assert np.all(raw.source[inner] == inner)
    mesh = z.Mesh(raw, z.StencilSpec.cweno(3, 2))
    geo = mesh.geometry()
    assert np.all(geo["volumes"] > 0) and np.all(geo["inradii"] > 0)
    assert abs(mesh.info["total_volume"] - 1.0) < 1e-13
    # a ghost cell is an exact translate of its source: same area
    assert np.allclose(geo["volumes"], geo["volumes"][raw.source], rtol=1e-12)


def test_disk_mesh(zlib):
    z = zlib
    raw = z.RawMesh.generate("disk", n=12, radius=1.0, jitter=0.2, seed=5)
    mesh = z.Mesh(raw, z.StencilSpec.cweno(3, 2))
    geo = mesh.geometry()
    assert np.all(geo["volumes"] > 0)
    # inscribed polygon of the unit circle
    n_outer = max(6, round(2 * np.pi * 12))
    assert abs(mesh.info["total_volume"] - 0.5 * n_outer * np.sin(2 * np.pi / n_outer)) < 1e-12
    assert mesh.info["n_edges"] - mesh.info["n_interior_edges"] == n_outer


def test_delaunay(zlib):
    # the disk generator flips edges until no vertex lies inside a neighbour's circumcircle
    z = zlib
    raw = z.RawMesh.generate("disk", n=10, jitter=0.2, seed=2, renumber=False)
    V, T = raw.vertices, raw.vertex_indices
    edges = {}
    for t, tri in enumerate(T):
        for e in range(3):
            a, b = int(tri[e]), int(tri[(e + 1) % 3])
            edges.setdefault((min(a, b), max(a, b)), []).append((t, int(tri[(e + 2) % 3])))
    worst = 0.0
    for (a, b), ts in edges.items():
        if len(ts) != 2:
            continue
        (t0, c), (_, d) = ts
        A, B, Cc, D = V[a], V[b], V[c], V[d]
        m = np.array([[A[0] - D[0], A[1] - D[1], (A[0] - D[0]) ** 2 + (A[1] - D[1]) ** 2],
                      [B[0] - D[0], B[1] - D[1], (B[0] - D[0]) ** 2 + (B[1] - D[1]) ** 2],
                      [Cc[0] - D[0], Cc[1] - D[1], (Cc[0] - D[0]) ** 2 + (Cc[1] - D[1]) ** 2]])
        o = (B[0] - A[0]) * (Cc[1] - A[1]) - (B[1] - A[1]) * (Cc[0] - A[0])
        worst = max(worst, np.linalg.det(m) * np.sign(o))
    h = 0.1
    assert worst <= 1e-10 * h ** 4


def test_cube_mesh(zlib):
    z = zlib
    raw = z.RawMesh.generate("cube", n=4, jitter=0.1, seed=1)
    assert raw.n_cells == 6 * 64
    mesh = z.Mesh(raw, z.StencilSpec.cweno(2, 3), quad=(2, 2, 1))
    geo = mesh.geometry()
    assert np.all(geo["volumes"] > 0)
    assert abs(mesh.info["total_volume"] - 1.0) < 1e-13


def test_hilbert_renumbering_is_a_permutation_and_local(zlib):
    z = zlib
    a = z.RawMesh.generate("periodic_square", n=16, halo=0, jitter=0.0, seed=1, renumber=False)
    b = z.RawMesh.generate("periodic_square", n=16, halo=0, jitter=0.0, seed=1, renumber=True)
    ka = {tuple(sorted(r)) for r in a.vertex_indices.tolist()}
    kb = {tuple(sorted(r)) for r in b.vertex_indices.tolist()}
    assert ka == kb
    # consecutive cells along the curve are close
    c = b.vertices[b.vertex_indices].mean(axis=1)
    jumps = np.linalg.norm(np.diff(c, axis=0), axis=1)
    assert np.median(jumps) < 2.0 / 16


def test_stencil_families(zlib):
    z = zlib
    raw = z.RawMesh.generate("periodic_square", n=12, halo=3, jitter=0.2, seed=1)
    mesh = z.Mesh(raw, z.StencilSpec.cweno(3, 2))
    st = mesh.stencils()
    full = raw.ghost == 0
    # central stencil: 11 cells (required_stencil_size(2, 2.0, 2)), self first
    assert np.all(st["size"][full, 0] == 11) and np.all(st["order"][full, 0] == 3)
    assert np.all(st["l2g"][:, 0] == np.arange(raw.n_cells))
    # one-sided stencils: 4 cells, order 2; k_high is the central stencil
    assert np.all(st["size"][full, 1:4] == 4) and np.all(st["order"][full, 1:4] == 2)
    assert np.all(st["k_high"][full] == 0)


def test_pinv_is_a_left_inverse(zlib):
    z = zlib
    raw = z.RawMesh.generate("periodic_square", n=8, halo=3, jitter=0.2, seed=4)
    mesh = z.Mesh(raw, z.StencilSpec.cweno(3, 2))
    # P reproduces an exact polynomial's coefficients: check P A = I through the
    # LSQ of a random right-hand side in the column space
    rng = np.random.default_rng(0)
    for cell in np.where(raw.ghost == 0)[0][:20]:
        P = mesh.pinv(int(cell), 0)
        assert P.shape == (5, 10)
        # rank of P is full and its singular values are bounded
        s = np.linalg.svd(P, compute_uv=False)
        assert s.min() > 0 and s.max() / s.min() < 1e4
        b = rng.standard_normal(10)
        x = P @ b
        assert np.all(np.isfinite(x))


def test_rejects_bad_descriptions(zlib):
    z = zlib
    raw = z.RawMesh.generate("periodic_square", n=4, halo=0, jitter=0.0, seed=1)
    bad = z.RawMesh(raw.n_dims, raw.vertices, raw.vertex_indices.copy())
    bad.vertex_indices[0, 0] = 10 ** 9
    with pytest.raises(z.ZfvmError) as e:
        z.Mesh(bad, z.StencilSpec.cweno(3, 2))
    assert e.value.code == 1
    with pytest.raises(z.ZfvmError):
        z.Mesh(raw, z.StencilSpec([3, 2], [0, 1], [2.0, 1.5]), quad=(3, 3, 1))


def test_rejects_degenerate_cells(zlib):
    """Cells that repeat a vertex (whose faces would match each other) or have
    no volume, and non-finite coordinates, are refused with an error."""
    z = zlib
    raw = z.RawMesh.generate("periodic_square", n=4, halo=0, jitter=0.0, seed=1)
    rep = z.RawMesh(raw.n_dims, raw.vertices, raw.vertex_indices.copy())
    rep.vertex_indices[3, 2] = rep.vertex_indices[3, 0]
    with pytest.raises(z.ZfvmError, match="repeats a vertex"):
        z.Mesh(rep, z.StencilSpec.cweno(3, 2))
    flat = z.RawMesh(raw.n_dims, raw.vertices.copy(), raw.vertex_indices.copy())
    a, b, c = flat.vertex_indices[5]
    flat.vertices[c] = 0.5 * (flat.vertices[a] + flat.vertices[b])  # collinear: zero area
    with pytest.raises(z.ZfvmError, match="no volume"):
        z.Mesh(flat, z.StencilSpec.cweno(3, 2))
    nan = z.RawMesh(raw.n_dims, raw.vertices.copy(), raw.vertex_indices.copy())
    nan.vertices[2, 0] = np.nan
    with pytest.raises(z.ZfvmError, match="non-finite"):
        z.Mesh(nan, z.StencilSpec.cweno(3, 2))


_SETUP_DIGEST = r"""
import hashlib, sys
import numpy as np
import zisafvm_gb300 as z
h = hashlib.sha256()
cases = [("cube", dict(n=6, jitter=0.1, seed=2), 3, (2, 2, 2)),
         ("cube", dict(n=5, jitter=0.0, seed=1), 3, (2, 2, 2)),
         ("disk", dict(n=14, radius=1.0, jitter=0.2, seed=3), 3, (3, 3, 2)),
         ("periodic_square", dict(n=10, halo=3, jitter=0.0, seed=1), 3, (3, 3, 2))]
for kind, kw, order, quad in cases:
    raw = z.RawMesh.generate(kind, **kw)
    mesh = z.Mesh(raw, z.StencilSpec.cweno(order, raw.n_dims), quad=quad)
    info = mesh.info
    h.update(repr([info["n_cells"], info["n_edges"], info["n_interior_edges"]]).encode())
    for v in mesh.geometry().values():
        h.update(np.ascontiguousarray(v).tobytes())
    st = mesh.stencils()
    for k in sorted(st):
        h.update(st[k].tobytes())
    for i in range(mesh.n_cells):
        for s in range(int(st["n_stencils"][i])):
            if st["order"][i, s] >= 2:
                h.update(mesh.pinv(i, s).tobytes())
print(h.hexdigest())
"""


def test_setup_does_not_depend_on_the_thread_count(zlib):
    """The set-up runs its per-cell and per-face loops with OpenMP (face
    matching in hash buckets, edge numbers from prefix counts, stencils and
    pseudo-inverses per cell): geometry, neighbours, stencils and operators
    must be bit for bit the same on one thread and on several."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    digests = []
    for threads in ("1", "5"):
        env = dict(os.environ, OMP_NUM_THREADS=threads, PYTHONPATH=root)
        out = subprocess.run([sys.executable, "-c", _SETUP_DIGEST], env=env, cwd=root,
                             capture_output=True, text=True, timeout=300)
        assert out.returncode == 0, out.stderr
        digests.append(out.stdout.strip())
    assert len(digests[0]) == 64 and digests[0] == digests[1]


def test_small_and_empty_meshes(zlib):
    """Meshes too small for the requested stencils fall back to lower orders
    (deduce_max_order, stencil_family.cpp; order 1 when a one-sided region
    holds too few cells), the central stencil stays the highest-order one, and
    every stencil index is a cell of the mesh; an empty mesh is refused."""
    z = zlib
    cases = [("disk", dict(n=2, radius=1.0)), ("cube", dict(n=1)), ("periodic_square", dict(n=2, halo=1))]
    for kind, kw in cases:
        raw = z.RawMesh.generate(kind, jitter=0.0, seed=1, **kw)
        mesh = z.Mesh(raw, z.StencilSpec.cweno(3, raw.n_dims), quad=(3, 3, 2) if raw.n_dims == 2 else (2, 2, 2))
        st = mesh.stencils()
        n = raw.n_cells
        ns = int(st["n_stencils"].max())
        assert st["order"][:, :ns].min() >= 1 and np.all(st["k_high"] == 0)
        assert np.all(st["order"][:, 0] >= st["order"][:, 1:ns].max(axis=1))
        for i in range(n):
            l2g = st["l2g"][i, :st["n_l2g"][i]]
            assert l2g[0] == i and np.all((l2g >= 0) & (l2g < n)) and len(set(l2g)) == len(l2g)
            for k in range(int(st["n_stencils"][i])):
                if st["order"][i, k] >= 2:
                    P = mesh.pinv(i, k)
                    assert P.shape[1] == st["size"][i, k] - 1 and np.all(np.isfinite(P))
    # the six tetrahedra of one cube: too few cells for any linear fit
    raw = z.RawMesh.generate("cube", n=1, jitter=0.0, seed=1)
    st = z.Mesh(raw, z.StencilSpec.cweno(3, 3), quad=(2, 2, 2)).stencils()
    assert np.all(st["order"][:, :5] == 1)
    # one triangle: every stencil is the cell itself
    one = z.RawMesh(2, np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]]), np.array([[0, 1, 2]], np.int64))
    st = z.Mesh(one, z.StencilSpec.cweno(3, 2)).stencils()
    assert st["n_l2g"][0] == 1 and np.all(st["order"][0, :4] == 1)
    empty = z.RawMesh(2, np.zeros((0, 3)), np.zeros((0, 3), np.int64))
    with pytest.raises(z.ZfvmError, match="empty"):
        z.Mesh(empty, z.StencilSpec.cweno(3, 2))
