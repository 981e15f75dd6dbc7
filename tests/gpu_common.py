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


def solve_extended(n, dli, a, b, c, rhs):
    """Extended-precision (numpy longdouble) solution of the periodic-x, periodic-y,
    tridiagonal-z Poisson operator the solver inverts: second differences with the FP64
    coefficients dli^2 in x and y, and the FP64 a, b, c rows in z (Neumann folded into b).
    The constant mode is fixed the way the library pins it: transformed (0,0) column's last
    row = 0.  Dense DFT matrices: for small n1, n2 only."""
    L = np.longdouble
    n1, n2, n3 = n
    cx = L(dli[0]) ** 2
    cy = L(dli[1]) ** 2
    ii = np.arange(n1, dtype=L)
    jj = np.arange(n2, dtype=L)
    tp = L(2) * L(np.pi) if False else L("6.283185307179586476925286766559005768")
    Fx = np.exp(np.outer(ii, ii).astype(L) * (-tp / n1) * 1j).astype(np.clongdouble)
    Fy = np.exp(np.outer(jj, jj).astype(L) * (-tp / n2) * 1j).astype(np.clongdouble)
    lx = L(-2) * (L(1) - np.cos(ii * tp / n1)) * cx
    ly = L(-2) * (L(1) - np.cos(jj * tp / n2)) * cy
    r = rhs.astype(L)
    R = np.einsum("ki,ijz->kjz", Fx, r.astype(np.clongdouble))
    R = np.einsum("lj,kjz->klz", Fy, R)
    A, B, C = a.astype(L), b.astype(L), c.astype(L)
    X = np.zeros_like(R)
    for kx in range(n1):
        for ky in range(n2):
            lam = lx[kx] + ly[ky]
            y = np.zeros(n3, dtype=np.clongdouble)
            d = np.zeros(n3, dtype=L)
            z = L(1) / (B[0] + lam)
            d[0] = C[0] * z
            y[0] = R[kx, ky, 0] * z
            pinned = kx == 0 and ky == 0
            for k in range(1, n3):
                if pinned and k == n3 - 1:
                    d[k] = 0
                    y[k] = 0
                    continue
                z = L(1) / (B[k] + lam - A[k] * d[k - 1])
                d[k] = C[k] * z
                y[k] = (R[kx, ky, k] - A[k] * y[k - 1]) * z
            for k in range(n3 - 2, -1, -1):
                y[k] = y[k] - d[k] * y[k + 1]
            X[kx, ky] = y
    X = np.einsum("ik,klz->ilz", np.conj(Fx), X)
    X = np.einsum("jl,ilz->ijz", np.conj(Fy), X)
    return (X.real / (n1 * n2)).astype(np.float64), X.real / (n1 * n2)
