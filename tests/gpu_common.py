"""Shared set-up for the -m gpu parity tests: build a case on the oracle and the library."""
import numpy as np

from oracle import oracle as O


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b.ravel())
    return np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0)


def is_bound_for(cbcpre):
    return [1, 1] + [0 if cbcpre[2 * d:2 * d + 2] == "PP" else 1 for d in (1, 2) for _ in (0, 1)]


def grid_for(n, l, cbc, gr):
    zper = cbc[4:6] == "PP"
    dzc, dzf, zc, zf = O.initgrid(1, n[2], 0.0 if zper else gr, l[2], zper)
    return dzc, dzf, 1.0 / dzc, 1.0 / dzf


def random_field(n, seed, zero_mean=False, dzf=None):
    rng = np.random.default_rng(seed)
    p = O.field(n)
    p[1:-1, 1:-1, 1:-1] = rng.standard_normal(n)
    if zero_mean:
        wts = dzf[1:-1][None, None, :] * np.ones(n)
        p[1:-1, 1:-1, 1:-1] -= (p[1:-1, 1:-1, 1:-1] * wts).sum() / wts.sum()
    return p


def singular(cbc, c_or_f="ccc"):
    """True when the discrete Poisson operator has the constant null mode (no Dirichlet side)."""
    return "D" not in cbc


def demean(f, dzf):
    """subtract the cell-volume-weighted mean (dz-weighted; x, y uniform) of an interior array"""
    w = np.asarray(dzf)[1:-1][None, None, :] * np.ones(f.shape)
    return f - (f * w).sum() / w.sum()


def gauge_rel_l2(got, want, dzf):
    """relative L2 after removing each field's mean: the comparison that is independent of the
    additive constant of a singular (all Neumann/periodic) Poisson problem"""
    return rel_l2(demean(got, dzf), demean(want, dzf))
