"""Relative L1 / Linf differences of conserved variables (per variable)."""
import numpy as np


def rel_errors(a: np.ndarray, ref: np.ndarray, mask=None, cols=(0, 1, 2, 4)):
    if mask is not None:
        a, ref = a[mask], ref[mask]
    l1, linf = [], []
    for v in cols:
        d = np.abs(a[:, v] - ref[:, v])
        s1 = np.abs(ref[:, v]).sum()
        sinf = np.abs(ref[:, v]).max()
        l1.append(d.sum() / s1 if s1 > 0 else d.sum())
        linf.append(d.max() / sinf if sinf > 0 else d.max())
    return max(l1), max(linf)


def state_rel_l1(a: np.ndarray, ref: np.ndarray, mask=None, cols=(0, 1, 2, 3, 4)):
    """||a - ref||_1 / ||ref||_1 over all cells and conserved variables."""
    if mask is not None:
        a, ref = a[mask], ref[mask]
    c = list(cols)
    return float(np.abs(a[:, c] - ref[:, c]).sum() / np.abs(ref[:, c]).sum())


def perturbation_rel_l1(a: np.ndarray, ref: np.ndarray, base: np.ndarray, mask=None):
    """Relative L1 error of the perturbation a - base against ref - base."""
    if mask is not None:
        a, ref, base = a[mask], ref[mask], base[mask]
    return float(np.abs((a - base) - (ref - base)).sum() / np.abs(ref - base).sum())


def conserved_rel_errors(a: np.ndarray, ref: np.ndarray, mask=None):
    """Relative L1 and Linf norms of the error in the conserved variables,
    taken over the whole conserved state (every cell, every component):
    ||a - ref||_1 / ||ref||_1 and max|a - ref| / max|ref|."""
    if mask is not None:
        a, ref = a[mask], ref[mask]
    d = np.abs(a - ref)
    return float(d.sum() / np.abs(ref).sum()), float(d.max() / np.abs(ref).max())


def deviation_rel_max(a: np.ndarray, ref: np.ndarray, base: np.ndarray, mask=None):
    """max |(a - base) - (ref - base)| / max |ref - base|: the error measured
    against the size of the change from `base` (the perturbation of an
    equilibrium), the strictest scale a well-balanced run offers."""
    if mask is not None:
        a, ref, base = a[mask], ref[mask], base[mask]
    return float(np.abs(a - ref).max() / np.abs(ref - base).max())
