"""Finite-element sets (FESetQ4, FESetH8, FESetH20, FESetT4, FESetT10).

Mirror of src/FESetModule.jl for the element types of the assembly path: the
connectivity (nelem x nne, 1-based, as ``fes.conn``), and the basis functions
and their parametric gradients evaluated at a point (``bfun``/``bfundpar``,
src/FESetModule.jl:210-225).  Node orders are the reference's: H20 corners
then edges 1-2, 2-3, 3-4, 4-1, 5-6, 6-7, 7-8, 8-5, 1-5, 2-6, 3-7, 4-8; T10
corners then edges 1-2, 2-3, 3-1, 4-1, 4-2, 4-3.

The functions are written from the standard Lagrange/serendipity
definitions on reference-element node coordinates (not the reference's
expanded expressions); the tests check both against each other.
"""
from __future__ import annotations

import numpy as np

from . import _native as nat

# parametric node coordinates
_HEX8 = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                  [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], dtype=np.float64)
_HEX20_EDGES = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4),
                (0, 4), (1, 5), (2, 6), (3, 7)]
_HEX20 = np.vstack([_HEX8] + [0.5 * (_HEX8[a] + _HEX8[b])[None, :] for a, b in _HEX20_EDGES])
_QUAD4 = np.array([[-1, -1], [1, -1], [1, 1], [-1, 1]], dtype=np.float64)
_TET10_EDGES = [(0, 1), (1, 2), (2, 0), (3, 0), (3, 1), (3, 2)]


class AbstractFESet:
    nne = 0
    mdim = 0
    code = -1

    def __init__(self, conn):
        conn = np.ascontiguousarray(conn, dtype=np.int64)
        if conn.ndim != 2 or conn.shape[1] != self.nne:
            raise ValueError(f"{type(self).__name__}: connectivity must be nelem x {self.nne}")
        self.conn = conn
        self.label = np.zeros(conn.shape[0], dtype=np.int64)

    def count(self) -> int:
        return self.conn.shape[0]

    def __len__(self):
        return self.conn.shape[0]

    def nodesperelem(self) -> int:
        return self.nne

    def manifdim(self) -> int:
        return self.mdim

    def bfun(self, pc) -> np.ndarray:  # nne x 1
        raise NotImplementedError

    def bfundpar(self, pc) -> np.ndarray:  # nne x mdim
        raise NotImplementedError


class FESetQ4(AbstractFESet):
    nne, mdim, code = 4, 2, nat.Q4

    def bfun(self, pc):
        x, y = pc[0], pc[1]
        return (0.25 * (1 + _QUAD4[:, 0] * x) * (1 + _QUAD4[:, 1] * y)).reshape(4, 1)

    def bfundpar(self, pc):
        x, y = pc[0], pc[1]
        xi, yi = _QUAD4[:, 0], _QUAD4[:, 1]
        return np.stack([0.25 * xi * (1 + yi * y), 0.25 * yi * (1 + xi * x)], axis=1)


class FESetH8(AbstractFESet):
    nne, mdim, code = 8, 3, nat.H8

    def bfun(self, pc):
        f = [(1 + _HEX8[:, d] * pc[d]) for d in range(3)]
        return (f[0] * f[1] * f[2] / 8.0).reshape(8, 1)

    def bfundpar(self, pc):
        f = [(1 + _HEX8[:, d] * pc[d]) for d in range(3)]
        out = np.empty((8, 3))
        out[:, 0] = _HEX8[:, 0] * f[1] * f[2] / 8.0
        out[:, 1] = f[0] * _HEX8[:, 1] * f[2] / 8.0
        out[:, 2] = f[0] * f[1] * _HEX8[:, 2] / 8.0
        return out


class FESetH20(AbstractFESet):
    nne, mdim, code = 20, 3, nat.H20

    def bfun(self, pc):
        N = np.empty(20)
        for k in range(20):
            a = _HEX20[k]
            if k < 8:
                N[k] = 0.125 * np.prod(1 + a * pc) * (a @ pc - 2)
            else:
                z = int(np.flatnonzero(a == 0)[0])  # the edge direction
                o = [d for d in range(3) if d != z]
                N[k] = 0.25 * (1 - pc[z] ** 2) * (1 + a[o[0]] * pc[o[0]]) * (1 + a[o[1]] * pc[o[1]])
        return N.reshape(20, 1)

    def bfundpar(self, pc):
        G = np.empty((20, 3))
        for k in range(20):
            a = _HEX20[k]
            f = 1 + a * pc
            if k < 8:
                s = a @ pc - 2
                for d in range(3):
                    o = [e for e in range(3) if e != d]
                    G[k, d] = 0.125 * a[d] * f[o[0]] * f[o[1]] * (s + f[d])
            else:
                z = int(np.flatnonzero(a == 0)[0])
                o = [d for d in range(3) if d != z]
                G[k, z] = 0.25 * (-2 * pc[z]) * f[o[0]] * f[o[1]]
                G[k, o[0]] = 0.25 * (1 - pc[z] ** 2) * a[o[0]] * f[o[1]]
                G[k, o[1]] = 0.25 * (1 - pc[z] ** 2) * f[o[0]] * a[o[1]]
        return G


def _bary(pc):
    r, s, t = pc[0], pc[1], pc[2]
    lam = np.array([1 - r - s - t, r, s, t])
    dlam = np.array([[-1.0, -1.0, -1.0], [1.0, 0, 0], [0, 1.0, 0], [0, 0, 1.0]])
    return lam, dlam


class FESetT4(AbstractFESet):
    nne, mdim, code = 4, 3, nat.T4

    def bfun(self, pc):
        return _bary(pc)[0].reshape(4, 1)

    def bfundpar(self, pc):
        return _bary(pc)[1].copy()


class FESetT10(AbstractFESet):
    nne, mdim, code = 10, 3, nat.T10

    def bfun(self, pc):
        lam, _ = _bary(pc)
        N = np.empty(10)
        N[:4] = lam * (2 * lam - 1)
        for k, (a, b) in enumerate(_TET10_EDGES):
            N[4 + k] = 4 * lam[a] * lam[b]
        return N.reshape(10, 1)

    def bfundpar(self, pc):
        lam, dl = _bary(pc)
        G = np.empty((10, 3))
        for k in range(4):
            G[k] = (4 * lam[k] - 1) * dl[k]
        for k, (a, b) in enumerate(_TET10_EDGES):
            G[4 + k] = 4 * (dl[a] * lam[b] + lam[a] * dl[b])
        return G


FESETS = {nat.Q4: FESetQ4, nat.H8: FESetH8, nat.H20: FESetH20, nat.T4: FESetT4, nat.T10: FESetT10}
