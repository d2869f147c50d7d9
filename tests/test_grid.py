"""The reference's grid tests, restated for the package's host set-up through the
mesh exports (zfvm_mesh_get_connectivity, zfvm_mesh_get_faces,
zfvm_mesh_get_geometry), on generated meshes (the reference's grid files are
missing):

- two triangles (test/zisa/unit_test/grid/grid.cpp:21-108): neighbours,
  interior-first face numbers, the interior normal and the areas;
- orientation of the normals: out of the left cell, towards the right cell's
  centre (grid.cpp:195-214);
- incidence: the two cells of an interior face are neighbours, and every cell
  meets as many interior faces as it has neighbours (grid.cpp:257-290);
- the interior-face count and the total volume of the unit square and cube,
  every cell with positive volume (grid.cpp:217-255).
"""
import numpy as np
import pytest

import zisafvm_gb300 as z


def test_two_triangles(zlib):
    raw = z.RawMesh(2, np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [1.0, 1.0, 0.0], [0.0, 1.0, 0.0]]),
                    np.array([[0, 1, 3], [1, 2, 3]], np.int64))
    mesh = z.Mesh(raw, z.StencilSpec.cweno(3, 2))
    con, faces = mesh.connectivity(), mesh.faces()
    assert con["neighbours"].tolist() == [[-1, 1, -1], [-1, -1, 0]]
    # the interior (diagonal) face first, then the boundary faces in cell order
    e = con["edge_indices"]
    assert e[0, 1] == 0 and e[1, 2] == 0
    assert (e[0, 0], e[0, 2], e[1, 0], e[1, 1]) == (1, 2, 3, 4)
    assert faces["normals"].shape == (5, 3)
    assert np.allclose(faces["normals"][0], [0.5 / np.sqrt(0.5), 0.5 / np.sqrt(0.5), 0.0], rtol=0, atol=1e-12)
    assert (faces["left"][0], faces["right"][0]) == (0, 1) and np.all(faces["right"][1:] == -1)
    assert np.allclose(mesh.geometry()["volumes"], 0.5, rtol=0, atol=1e-12)


def _meshes():
    yield z.Mesh(z.RawMesh.generate("periodic_square", n=12, halo=0, jitter=0.2, seed=1), z.StencilSpec.cweno(3, 2))
    yield z.Mesh(z.RawMesh.generate("disk", n=10, radius=1.0, jitter=0.2, seed=2), z.StencilSpec.cweno(3, 2))
    yield z.Mesh(z.RawMesh.generate("cube", n=4, jitter=0.1, seed=3), z.StencilSpec.cweno(2, 3), quad=(2, 2, 1))


def test_normals_point_from_left_to_right(zlib):
    for mesh in _meshes():
        f, c = mesh.faces(), mesh.geometry()["centers"]
        ni = int(mesh.info["n_interior_edges"])
        L, R, n = f["left"][:ni], f["right"][:ni], f["normals"][:ni]
        assert np.all(L < R)
        assert np.all(np.einsum("ed,ed->e", n, c[R] - c[L]) > 0.0)
        assert np.allclose(np.linalg.norm(f["normals"], axis=1), 1.0, rtol=0, atol=1e-14)
        # boundary faces come after the interior ones and belong to their left cell
        con = mesh.connectivity()
        for e in range(ni, len(f["left"])):
            assert f["right"][e] == -1 and e in con["edge_indices"][f["left"][e]]


def test_incidence(zlib):
    for mesh in _meshes():
        f, con = mesh.faces(), mesh.connectivity()
        ni = int(mesh.info["n_interior_edges"])
        for e in range(ni):
            assert f["right"][e] in con["neighbours"][f["left"][e]]
        count = np.bincount(np.concatenate([f["left"][:ni], f["right"][:ni]]), minlength=mesh.n_cells)
        assert np.array_equal(count, (con["neighbours"] >= 0).sum(axis=1))
        # every (cell, local face) names a face whose left or right cell is the cell
        rows = np.repeat(np.arange(mesh.n_cells), con["edge_indices"].shape[1])
        e = con["edge_indices"].ravel()
        assert np.all((f["left"][e] == rows) | (f["right"][e] == rows))


@pytest.mark.parametrize("kind", ["square", "cube"])
def test_volume(zlib, kind):
    if kind == "square":
        raw = z.RawMesh.generate("periodic_square", n=10, halo=0, jitter=0.0, seed=1)
        mesh = z.Mesh(raw, z.StencilSpec.cweno(3, 2))
    else:
        raw = z.RawMesh.generate("cube", n=4, jitter=0.1, seed=1)
        mesh = z.Mesh(raw, z.StencilSpec.cweno(2, 3), quad=(2, 2, 1))
    vol = mesh.geometry()["volumes"]
    assert np.all(vol > 0.0) and abs(vol.sum() - 1.0) <= 1e-12
    f = mesh.faces()
    assert int(mesh.info["n_interior_edges"]) == int((f["right"] >= 0).sum())
    if kind == "square":
        # n x n squares of two triangles: n^2 diagonals + 2 n (n - 1) grid edges inside
        assert int(mesh.info["n_interior_edges"]) == 10 * 10 + 2 * 10 * 9
