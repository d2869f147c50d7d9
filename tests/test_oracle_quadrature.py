"""The reference's quadrature tests, restated for the oracle's reference-element
rules (the same rules the product's set-up uses; the CUDA path matches the
oracle at 1e-12 only with identical quadrature):

- edge rules: degree -> number of Gauss-Legendre points, weights summing to 1,
  symmetric points and weights (test/zisa/unit_test/math/edge_rule.cpp:12-40);
- the four-point Gauss-Legendre nodes and weights against their closed forms
  within 2e-14 (math/gauss_legendre.cpp:39-63; the five-point rule is above
  the degrees this path uses);
- convergence of whole-domain quadrature of a smooth function under mesh
  refinement: rate above p + 1 - 0.3 for the rule of degree p, rates taken
  only where the error is above round-off (math/quadrature.cpp:17-74 for
  triangles, math/tetrahedral_rule.cpp:19-58 for tetrahedra).

The meshes are the package's generated unit square and unit cube (jittered);
the reference's grid files are missing.
"""
import numpy as np
import pytest

import zisafvm_gb300 as z


def test_edge_rule_basics(olib):
    for deg, n in [(0, 1), (1, 1), (2, 2), (3, 2), (4, 3), (5, 3), (6, 4), (7, 4)]:
        w, x = olib.rule("edge", deg)
        x = x[:, 0]
        assert len(w) == n and abs(w.sum() - 1.0) <= 1e-12
        assert np.all(np.abs(x + x[::-1]) <= 1e-12) and np.all(np.abs(w - w[::-1]) <= 1e-12)


def test_gauss_legendre_closed_forms(olib):
    s = 2.0 / 7.0 * np.sqrt(6.0 / 5.0)
    forms = {
        2: ([-1 / np.sqrt(3), 1 / np.sqrt(3)], [1.0, 1.0]),
        3: ([-np.sqrt(0.6), 0.0, np.sqrt(0.6)], [5 / 9, 8 / 9, 5 / 9]),
        4: ([-np.sqrt(3 / 7 + s), -np.sqrt(3 / 7 - s), np.sqrt(3 / 7 - s), np.sqrt(3 / 7 + s)],
            [(18 - np.sqrt(30)) / 36, (18 + np.sqrt(30)) / 36, (18 + np.sqrt(30)) / 36, (18 - np.sqrt(30)) / 36]),
    }
    for n, (points, weights) in forms.items():
        w, x = olib.rule("edge", 2 * n - 1)
        # the rules here are normalised to the unit length: weights / 2
        assert np.allclose(x[:, 0], points, rtol=0, atol=2e-14)
        assert np.allclose(2.0 * w, weights, rtol=2e-14, atol=0)


def _unit_square(n):
    """n x n squares of two triangles on [0, 1]^2, interior vertices moved by
    up to 0.2 h (the generator's periodic square moves its boundary too)."""
    raw = z.RawMesh.generate("periodic_square", n=n, halo=0, jitter=0.0, seed=3)
    v = raw.vertices.copy()
    inner = np.all((v[:, :2] > 1e-12) & (v[:, :2] < 1 - 1e-12), axis=1)
    v[inner, :2] += np.random.default_rng(n).uniform(-0.2 / n, 0.2 / n, size=(int(inner.sum()), 2))
    return z.RawMesh(2, v, raw.vertex_indices)


def _integral(raw, volumes, w, bary, f):
    X = np.einsum("qk,nkd->nqd", bary, raw.vertices[raw.vertex_indices])
    fx = f(X.reshape(-1, 3)).reshape(X.shape[:2])
    return float((volumes * (fx @ w)).sum())


def _rates(errors, res, atol):
    out = []
    for k in range(len(errors) - 1):
        if errors[k + 1] > atol:
            out.append(np.log(errors[k] / errors[k + 1]) / np.log(res[k] / res[k + 1]))
    return out


@pytest.mark.parametrize("deg", [1, 2, 3, 4, 5])
def test_triangle_rule_convergence(zlib, olib, deg):
    f = lambda X: np.sin(0.5 * np.pi * X[:, 0]) + np.sin(0.5 * np.pi * X[:, 1]) + np.sin(0.5 * np.pi * X[:, 2])
    w, bary = olib.rule("triangle", deg)
    errors, res = [], []
    for n in (4, 8, 16, 32):
        raw = _unit_square(n)
        mesh = z.Mesh(raw, z.StencilSpec.cweno(3, 2))
        errors.append(abs(_integral(raw, mesh.geometry()["volumes"], w, bary, f) - 2 * 2.0 / np.pi))
        res.append(mesh.info["max_circum_radius"])
    r = _rates(errors, res, 1e-14)
    print(f"triangle degree {deg}: errors {errors}, rates {np.round(r, 2)}")
    assert all(x > deg + 1 - 0.3 for x in r), r


@pytest.mark.parametrize("deg", [1, 2, 3])
def test_tetrahedron_rule_convergence(zlib, olib, deg):
    f = lambda X: np.sin(0.5 * np.pi * X[:, 0]) + np.cos(0.5 * np.pi * X[:, 1]) + np.sin(0.25 * np.pi * X[:, 2])
    exact = 2.0 / np.pi + 2.0 / np.pi + 4.0 / np.pi * (1.0 - np.cos(0.25 * np.pi))
    w, bary = olib.rule("tetrahedron", deg)
    errors, res = [], []
    for n in (3, 6, 12):
        raw = z.RawMesh.generate("cube", n=n, jitter=0.1, seed=3)
        mesh = z.Mesh(raw, z.StencilSpec.cweno(2, 3), quad=(2, 2, 1))
        errors.append(abs(_integral(raw, mesh.geometry()["volumes"], w, bary, f) - exact))
        res.append(mesh.info["max_circum_radius"])
    r = _rates(errors, res, 2e-12)
    print(f"tetrahedron degree {deg}: errors {errors}, rates {np.round(r, 2)}")
    assert all(x > deg + 1 - 0.3 for x in r), r
