"""Integration rules: GaussRule (src/IntegRuleModule.jl:193-398) and TetRule
(src/IntegRuleModule.jl:470-516).

The point coordinates and weights are the reference's tabulated values (the
same truncated decimals), so that a rule built here integrates exactly as the
reference's does; the tensor-product order is i (xi) outer, k (zeta) inner.
"""
from __future__ import annotations

import numpy as np

# 1-D Gauss-Legendre points/weights as tabulated by the reference
_GAUSS_1D = {
    1: ([0.0], [2.0]),
    2: ([-0.577350269189626, 0.577350269189626], [1.0, 1.0]),
    3: ([-0.774596669241483, 0.0, 0.774596669241483],
        [0.5555555555555556, 0.8888888888888889, 0.5555555555555556]),
    4: ([-0.86113631159405, -0.33998104358486, 0.33998104358486, 0.86113631159405],
        [0.34785484513745, 0.65214515486255, 0.65214515486255, 0.34785484513745]),
}


def _gauss_1d(order):
    """Points (ascending) and weights of the order-point Gauss-Legendre rule:
    the reference's tabulated decimals for orders 1-4, the double-precision
    values (numpy's Legendre roots) for orders 5-10, which agree with any
    15-digit table to within an ulp or two."""
    if order in _GAUSS_1D:
        return _GAUSS_1D[order]
    if 5 <= order <= 10:
        x, w = np.polynomial.legendre.leggauss(order)
        return list(x), list(w)
    raise ValueError(f"Gauss rule of order {order} not available")


class GaussRule:
    """Gauss rule on [-1, 1]^dim with `order` points per direction (orders 1
    to 10, as the reference tabulates, src/IntegRuleModule.jl:193-398)."""

    def __init__(self, dim: int = 1, order: int = 1):
        if not 1 <= dim <= 3:
            raise ValueError(f"Gauss rule of dimension {dim} not available")
        x, w = _gauss_1d(order)
        pts, wts = [], []
        if dim == 1:
            pts = [[a] for a in x]
            wts = list(w)
        elif dim == 2:
            for i in range(order):
                for j in range(order):
                    pts.append([x[i], x[j]])
                    wts.append(w[i] * w[j])
        else:
            for i in range(order):
                for j in range(order):
                    for k in range(order):
                        pts.append([x[i], x[j], x[k]])
                        wts.append(w[i] * w[j] * w[k])
        self.dim, self.order = dim, order
        self.param_coords = np.array(pts, dtype=np.float64)
        self.weights = np.array(wts, dtype=np.float64)
        self.npts = len(wts)


class TetRule:
    """Rules on the unit tetrahedron with 1, 4 or 5 points."""

    def __init__(self, npts: int = 1):
        if npts == 1:
            pc = [[0.25, 0.25, 0.25]]
            w = [1.0 / 6.0]
        elif npts == 4:
            a, b = 0.13819660, 0.58541020
            pc = [[a, a, a], [b, a, a], [a, b, a], [a, a, b]]
            w = [0.041666666666666666667] * 4
        elif npts == 5:
            a, b, c = 1.0 / 6.0, 0.25, 0.5
            pc = [[b, b, b], [c, a, a], [a, c, a], [a, a, c], [a, a, a]]
            w = [-0.8 / 6, 0.45 / 6, 0.45 / 6, 0.45 / 6, 0.45 / 6]
        else:
            raise ValueError("Unknown number of integration points")
        self.param_coords = np.array(pc, dtype=np.float64)
        self.weights = np.array(w, dtype=np.float64)
        self.npts = npts
