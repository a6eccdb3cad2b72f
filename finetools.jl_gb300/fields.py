"""NodalField: nodal values, DOF numbers and DOF kinds.

Mirror of src/FieldModule.jl and src/NodalFieldModule.jl for what the
assembly path needs: ``values`` (nnodes x ndn), ``dofnums`` (nnodes x ndn,
1-based), ``kind`` (free / fixed), ``setebc``, ``numberdofs``
(free DOFs first, then fixed ones, node by node: src/FieldModule.jl:328-377),
``gathersysvec``.
"""
from __future__ import annotations

import numpy as np

DOF_KIND_FREE = 1
DOF_KIND_DATA = 2


class NodalField:
    def __init__(self, data):
        v = np.array(data, dtype=np.result_type(np.asarray(data).dtype, np.float64))
        if v.ndim == 1:
            v = v.reshape(-1, 1)
        self.values = v
        self.dofnums = np.zeros(v.shape, dtype=np.int64)
        self.kind = np.full(v.shape, DOF_KIND_FREE, dtype=np.int8)
        self.ranges = {}

    # --- sizes (src/FieldModule.jl:62-110)
    def ndofs(self) -> int:
        return self.values.shape[1]

    def nents(self) -> int:
        return self.values.shape[0]

    def nalldofs(self) -> int:
        return int(sum(len(r) for r in self.ranges.values()))

    def nfreedofs(self) -> int:
        return len(self.ranges.get(DOF_KIND_FREE, range(0)))


def setebc(field: NodalField, nodes, is_fixed=True, comps=None, val=0.0):
    """Mark components of nodes (1-based) as fixed with a prescribed value."""
    nodes = np.atleast_1d(np.asarray(nodes, dtype=np.int64)) - 1
    if comps is None:
        comps = np.ones(len(nodes), dtype=np.int64)
    comps = np.atleast_1d(np.asarray(comps, dtype=np.int64)) - 1
    if len(comps) == 1 and len(nodes) > 1:
        comps = np.full(len(nodes), comps[0])
    for n, c in zip(nodes, comps):
        field.kind[n, c] = DOF_KIND_DATA if is_fixed else DOF_KIND_FREE
        if is_fixed:
            field.values[n, c] = val
    return field


def numberdofs(field: NodalField, entperm=None, kinds=(DOF_KIND_FREE, DOF_KIND_DATA)):
    """Number the DOFs: each kind in turn, entities in `entperm` order
    (1-based permutation), components in order."""
    n, d = field.values.shape
    order = np.arange(n) if entperm is None else np.asarray(entperm, dtype=np.int64) - 1
    field.dofnums[:] = 0
    nxt = 1
    field.ranges = {}
    for k in kinds:
        start = nxt
        sel = field.kind[order] == k            # (n, d) in entity order
        cnt = int(sel.sum())
        num = np.zeros(sel.shape, dtype=np.int64)
        num[sel] = np.arange(nxt, nxt + cnt)    # row-major = node by node
        rows = order[np.any(sel, axis=1)]
        field.dofnums[order[:, None].repeat(d, 1)[sel], np.nonzero(sel)[1]] = num[sel]
        nxt += cnt
        field.ranges[k] = range(start, nxt)
        del rows
    return field


def gathersysvec(field: NodalField, kind=DOF_KIND_FREE):
    """Vector of the values of the DOFs of `kind` ('all' for every DOF)."""
    if kind == "all":
        n = field.nalldofs()
        mask = field.dofnums > 0
    else:
        r = field.ranges.get(kind, range(0))
        n = len(r)
        mask = field.kind == kind
    out = np.zeros(n, dtype=field.values.dtype)
    base = 1 if kind == "all" else (field.ranges[kind].start if n else 1)
    out[field.dofnums[mask] - base] = field.values[mask]
    return out
