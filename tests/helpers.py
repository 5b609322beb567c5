"""Comparison helpers for Dyson solutions (rows [W, Z, x_0 .. x_{D-1}])."""
import numpy as np


def strong_diffs(ref, got, zmin=1e-6, etol=1e-7):
    """For every solution of `ref` with Z > zmin: relative energy error of the nearest
    solution in `got`, and the difference of the summed Z of the solutions within a
    relative window etol (eigenvector signs and splits inside exact degeneracies are
    arbitrary, so strength is compared per degenerate group)."""
    ref = np.asarray(ref).reshape(-1, ref.shape[-1]) if len(ref) else np.zeros((0, 2))
    got = np.asarray(got).reshape(-1, got.shape[-1]) if len(got) else np.zeros((0, 2))
    if not (np.isfinite(ref).all() and np.isfinite(got).all()):
        return np.inf, np.inf
    wE = wZ = 0.0
    for r in ref[ref[:, 1] > zmin]:
        if not len(got):
            return np.inf, np.inf
        k = np.argmin(np.abs(got[:, 0] - r[0]))
        wE = max(wE, abs(got[k, 0] - r[0]) / max(1.0, abs(r[0])))
        tol = etol * max(1.0, abs(r[0]))
        za = ref[np.abs(ref[:, 0] - r[0]) < tol, 1].sum()
        zb = got[np.abs(got[:, 0] - r[0]) < tol, 1].sum()
        wZ = max(wZ, abs(za - zb))
    return wE, wZ


def first_breakdown(rows, rel=1e-8):
    """Index of the first Lanczos row whose beta is below rel * max|alpha|."""
    b = np.where(rows[:, 1] < rel * np.abs(rows[:, 0]).max())[0]
    return int(b[0]) if len(b) else len(rows)


def koltun_energy(k):
    k = np.asarray(k).reshape(-1, 3)
    return float(((k[:, 0] + k[:, 1]) / 2.0).sum())
