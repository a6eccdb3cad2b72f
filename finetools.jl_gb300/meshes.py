"""Block mesh generators with the reference's node and element numbering, and
the seeded synthetic meshes of the benchmark workloads.

Numbering rules restated from the reference generators:
  - H8blockx (src/MeshHexahedronModule.jl:59-111): nodes x fastest, then y,
    then z; cells loop i (x) outer, j (y), k (z) innermost;
  - T4blockx, orientation :a (src/MeshTetrahedronModule.jl:81-150): six
    tetrahedra per cell from a fixed local table, same cell order;
  - Q4blockx (src/MeshQuadrilateralModule.jl:171-214);
  - H8toH20 / T4toT10 (src/MeshHexahedronModule.jl:580-627,
    src/MeshTetrahedronModule.jl:158-211): mid-edge nodes numbered after the
    existing nodes in first-encounter order (element order x local edge
    order) and placed at the mean of the edge's end nodes.
All arrays are numpy; connectivity is 1-based int64 (nelem x nne).
"""
from __future__ import annotations

import numpy as np

from .fesets import FESetH8, FESetH20, FESetQ4, FESetT4, FESetT10


class FENodeSet:
    def __init__(self, xyz):
        self.xyz = np.ascontiguousarray(xyz, dtype=np.float64)

    def count(self) -> int:
        return self.xyz.shape[0]


def linearspace(start: float, stop: float, n: int) -> np.ndarray:
    """Julia's range(start, stop, length=n) (src/MeshUtilModule.jl:116-118):
    entry i is start + i*(stop-start)/(n-1) correctly rounded."""
    from fractions import Fraction
    if n == 1:
        return np.array([float(start)])
    a, b = Fraction(float(start)), Fraction(float(stop))
    return np.array([float(a + (b - a) * i / (n - 1)) for i in range(n)], dtype=np.float64)


def _grid_nodes(xs, ys, zs):
    X, Y, Z = np.meshgrid(xs, ys, zs, indexing="ij")
    # x fastest, then y, then z
    return np.stack([X.transpose(2, 1, 0).ravel(), Y.transpose(2, 1, 0).ravel(),
                     Z.transpose(2, 1, 0).ravel()], axis=1)


def _cell_corners(nL, nW, nH):
    i, j, k = np.meshgrid(np.arange(1, nL + 1), np.arange(1, nW + 1), np.arange(1, nH + 1),
                          indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()  # i outer, k inner
    b = (k - 1) * ((nL + 1) * (nW + 1)) + (j - 1) * (nL + 1) + i
    t = b + (nL + 1) * (nW + 1)
    return np.stack([b, b + 1, b + (nL + 1) + 1, b + (nL + 1),
                     t, t + 1, t + (nL + 1) + 1, t + (nL + 1)], axis=1).astype(np.int64)


def H8blockx(xs, ys, zs):
    xs, ys, zs = (np.asarray(v, dtype=np.float64) for v in (xs, ys, zs))
    return FENodeSet(_grid_nodes(xs, ys, zs)), FESetH8(_cell_corners(len(xs) - 1, len(ys) - 1,
                                                                     len(zs) - 1))


_T4A = np.array([[1, 8, 5, 6], [3, 4, 2, 7], [7, 2, 6, 8], [4, 7, 8, 2], [2, 1, 6, 8],
                 [4, 8, 1, 2]]) - 1


def T4blockx(xs, ys, zs):
    xs, ys, zs = (np.asarray(v, dtype=np.float64) for v in (xs, ys, zs))
    nn = _cell_corners(len(xs) - 1, len(ys) - 1, len(zs) - 1)
    conn = nn[:, _T4A].reshape(-1, 4)
    return FENodeSet(_grid_nodes(xs, ys, zs)), FESetT4(conn)


def Q4blockx(xs, ys):
    xs, ys = (np.asarray(v, dtype=np.float64) for v in (xs, ys))
    nL, nW = len(xs) - 1, len(ys) - 1
    X, Y = np.meshgrid(xs, ys, indexing="xy")  # rows y, columns x: x fastest
    xyz = np.stack([X.ravel(), Y.ravel()], axis=1)
    i, j = np.meshgrid(np.arange(1, nL + 1), np.arange(1, nW + 1), indexing="ij")
    i, j = i.ravel(), j.ravel()
    b = (j - 1) * (nL + 1) + i
    conn = np.stack([b, b + 1, b + (nL + 1) + 1, b + (nL + 1)], axis=1).astype(np.int64)
    return FENodeSet(xyz), FESetQ4(conn)


_H20_EDGES = np.array([[1, 2], [2, 3], [3, 4], [4, 1], [5, 6], [6, 7], [7, 8], [8, 5],
                       [1, 5], [2, 6], [3, 7], [4, 8]]) - 1
_T10_EDGES = np.array([[1, 2], [2, 3], [3, 1], [4, 1], [4, 2], [4, 3]]) - 1


def _quadratic(fens, conn, edges):
    xyz = fens.xyz
    n0 = xyz.shape[0]
    ends = conn[:, edges]                      # E x ne x 2, 1-based
    lo = np.minimum(ends[..., 0], ends[..., 1]).ravel()
    hi = np.maximum(ends[..., 0], ends[..., 1]).ravel()
    key = lo * (n0 + 1) + hi
    uniq, first, inv = np.unique(key, return_index=True, return_inverse=True)
    order = np.argsort(first, kind="stable")   # first-encounter order
    newnum = np.empty(len(uniq), dtype=np.int64)
    newnum[order] = n0 + 1 + np.arange(len(uniq))
    ulo, uhi = lo[first], hi[first]
    mid = np.empty((len(uniq), xyz.shape[1]))
    mid[newnum - n0 - 1] = (xyz[uhi - 1] + xyz[ulo - 1]) * 0.5
    econn = newnum[inv].reshape(conn.shape[0], len(edges))
    return FENodeSet(np.vstack([xyz, mid])), np.hstack([conn, econn])


def H8toH20(fens, fes):
    f, c = _quadratic(fens, fes.conn, _H20_EDGES)
    return f, FESetH20(c)


def T4toT10(fens, fes):
    f, c = _quadratic(fens, fes.conn, _T10_EDGES)
    return f, FESetT10(c)


def H8block(L, W, H, nL, nW, nH):
    return H8blockx(linearspace(0.0, L, nL + 1), linearspace(0.0, W, nW + 1),
                    linearspace(0.0, H, nH + 1))


def H20block(L, W, H, nL, nW, nH):
    return H8toH20(*H8block(L, W, H, nL, nW, nH))


def T4block(L, W, H, nL, nW, nH):
    return T4blockx(linearspace(0.0, L, nL + 1), linearspace(0.0, W, nW + 1),
                    linearspace(0.0, H, nH + 1))


def T10block(L, W, H, nL, nW, nH):
    return T4toT10(*T4block(L, W, H, nL, nW, nH))


def Q4block(L, W, nL, nW):
    return Q4blockx(linearspace(0.0, L, nL + 1), linearspace(0.0, W, nW + 1))


# ---------------------------------------------------------------------------
# seeded synthetic meshes of the benchmark workloads
def jitter_interior(xyz, n_cells, amplitude, seed, box=(1.0, 1.0, 1.0)):
    """Move nodes strictly inside the box by iid uniform(-a*h, a*h) per coordinate."""
    rng = np.random.default_rng(seed)
    out = xyz.copy()
    sd = xyz.shape[1]
    h = np.asarray(box[:sd], dtype=np.float64) / np.asarray(n_cells[:sd], dtype=np.float64)
    tol = 1e-12
    inside = np.all((xyz > tol) & (xyz < np.asarray(box[:sd]) - tol), axis=1)
    d = rng.uniform(-amplitude, amplitude, size=xyz.shape) * h
    out[inside] += d[inside]
    return out


def recompute_midpoints(fens, fes, nvert):
    """Place every mid-edge node back at the mean of its edge ends."""
    edges = _H20_EDGES if fes.nne == 20 else _T10_EDGES
    nv = 8 if fes.nne == 20 else 4
    xyz = fens.xyz
    ends = fes.conn[:, edges]           # E x ne x 2
    mids = fes.conn[:, nv:]             # E x ne
    lo = np.minimum(ends[..., 0], ends[..., 1])
    hi = np.maximum(ends[..., 0], ends[..., 1])
    xyz[mids.ravel() - 1] = (xyz[hi.ravel() - 1] + xyz[lo.ravel() - 1]) * 0.5
    return fens


def h8_diffusion_mesh(n=20, seed=1, amplitude=0.2):
    """H8 block on the unit cube, interior nodes jittered by +-amplitude*h."""
    fens, fes = H8block(1.0, 1.0, 1.0, n, n, n)
    fens.xyz = jitter_interior(fens.xyz, (n, n, n), amplitude, seed)
    return fens, fes


def t10_elastic_mesh(n=60, seed=2, amplitude=0.15):
    """T10 block (6 tets per cell) on the unit cube; vertices jittered by
    +-amplitude*h, mid-edge nodes recomputed as edge means (straight edges)."""
    fens, fes = T4block(1.0, 1.0, 1.0, n, n, n)
    fens.xyz = jitter_interior(fens.xyz, (n, n, n), amplitude, seed)
    nv = fens.xyz.shape[0]
    fens, fes = T4toT10(fens, fes)
    return recompute_midpoints(fens, fes, nv), fes


def h20_elastic_mesh(n=40, seed=3, amplitude=0.25, distort_fraction=0.01, ratio=0.05):
    """H20 block on the unit cube with jittered vertices; a seeded fraction of
    the elements gets one corner pulled toward the centroid until
    det J_min / det J_mean < ratio (det J > 0 kept at the 27 Gauss points)."""
    fens, fes = H8block(1.0, 1.0, 1.0, n, n, n)
    xyz = jitter_interior(fens.xyz, (n, n, n), amplitude, seed)
    rng = np.random.default_rng(seed + 100)
    E = fes.count()
    pick = rng.choice(E, size=max(1, int(round(distort_fraction * E))), replace=False)
    moved = np.zeros(xyz.shape[0], dtype=bool)
    h8 = FESetH8(fes.conn)
    from .rules import GaussRule
    rule = GaussRule(3, 3)
    dN = np.stack([h8.bfundpar(p) for p in rule.param_coords])  # q x 8 x 3
    flagged = []
    for e in np.sort(pick):
        conn = fes.conn[e] - 1
        # an interior corner not moved before keeps the neighbours valid
        cand = [c for c in conn if not moved[c]
                and np.all((xyz[c] > 1e-12) & (xyz[c] < 1 - 1e-12))]
        if not cand:
            continue
        c = cand[int(rng.integers(len(cand)))]
        X = xyz[conn].copy()
        ci = int(np.flatnonzero(conn == c)[0])
        cen = X.mean(axis=0)
        base = X[ci].copy()
        ok = False
        for t in np.linspace(0.05, 0.95, 91):
            X[ci] = base + t * (cen - base)
            dets = np.linalg.det(np.einsum("ks,qkm->qsm", X, dN))
            if np.all(dets > 0) and dets.min() / dets.mean() < ratio:
                ok = True
                break
        if ok and _neighbours_valid(xyz, fes.conn, c, X[ci], dN):
            xyz[c] = X[ci]
            moved[conn] = True  # later moves must not touch a flagged element
            flagged.append(e)
    fens.xyz = xyz
    nv = xyz.shape[0]
    fens, fes20 = H8toH20(fens, fes)
    fens = recompute_midpoints(fens, fes20, nv)
    return fens, fes20, np.array(flagged, dtype=np.int64)


def _neighbours_valid(xyz, conn, node, newpos, dN):
    els = np.flatnonzero(np.any(conn == node + 1, axis=1))
    for e in els:
        X = xyz[conn[e] - 1].copy()
        X[conn[e] - 1 == node] = newpos
        dets = np.linalg.det(np.einsum("ks,qkm->qsm", X, dN))
        if not np.all(dets > 0):
            return False
    return True


def nearest_block(etype: str, nelem: int, seed: int, amplitude: float = 0.15):
    """Unit block of about nelem elements of type etype ("H8", "H20", "T4",
    "T10" or "Q4"): the nx x ny (x nz) cell grid closest to the request (six
    tetrahedra per cell), vertices strictly inside jittered by +-amplitude*h,
    mid-edge nodes of quadratic elements recomputed as edge means."""
    if etype == "Q4":
        nx = max(1, int(round(np.sqrt(nelem))))
        ny = max(1, int(round(nelem / nx)))
        fens, fes = Q4block(1.0, 1.0, nx, ny)
        fens.xyz = jitter_interior(fens.xyz, (nx, ny), amplitude, seed, box=(1.0, 1.0))
        return fens, fes
    tets = etype in ("T4", "T10")
    cells = nelem / 6.0 if tets else float(nelem)
    nx = max(1, int(round(cells ** (1.0 / 3.0))))
    nz = max(1, int(round(cells / (nx * nx))))
    fens, fes = (T4block if tets else H8block)(1.0, 1.0, 1.0, nx, nx, nz)
    fens.xyz = jitter_interior(fens.xyz, (nx, nx, nz), amplitude, seed)
    if etype in ("H20", "T10"):
        nv = fens.xyz.shape[0]
        fens, fes = (T4toT10 if tets else H8toH20)(fens, fes)
        fens = recompute_midpoints(fens, fes, nv)
    elif etype not in ("H8", "T4"):
        raise ValueError(f"unknown element type {etype}")
    return fens, fes


def lame(E, nu):
    """Lame constants of an isotropic material."""
    E = np.asarray(E, dtype=np.float64)
    nu = np.asarray(nu, dtype=np.float64)
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    mu = E / (2 * (1 + nu))
    return lam, mu


def isotropic_D(E, nu):
    """6x6 Voigt (xx, yy, zz, xy, xz, yz) stiffness with engineering shear."""
    lam, mu = lame(E, nu)
    D = np.zeros((6, 6))
    D[:3, :3] = lam
    for i in range(3):
        D[i, i] = lam + 2 * mu
        D[3 + i, 3 + i] = mu
    return D
