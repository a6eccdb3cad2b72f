"""Serving loop: re-assembly requests on resident meshes (fegpu_server_* of
include/fegpu.h), continuously batched onto the GPU.

    server = AssemblyServer(lanes=2)
    mid, K = server.add_mesh("lin_elastic", femm, geom, u, IsotropicElementwise(E, nu))
    rid = server.submit_coef(mid, new_lame)          # (nelem, 2) lambda, mu
    rid2 = server.submit_coords(mid, new_xyz)         # (nnodes, 3)
    latency_ms = server.wait(rid)                     # K holds the request's matrix

Each request is evaluated as the mixed-precision batch path; a request's
matrix does not depend on which other requests shared its launch.
"""
from __future__ import annotations

import ctypes as C
import weakref

import numpy as np

from . import _native as nat
from .assembly import DeviceMatrix
from .batch import _FORMS
from .femm import DeforModelRed3D, FEMMBase, _coef, _prepare


def _destroy(L, h):
    try:
        L.fegpu_server_destroy(h)
    except Exception:
        pass


class AssemblyServer:
    """Resident meshes + a worker thread that batches re-assembly requests."""

    def __init__(self, lanes: int = 2, max_jobs: int = 64, device: int = 0):
        L = nat.load()
        out = C.c_void_p()
        nat.check(L.fegpu_server_create(nat.context(device), int(lanes), int(max_jobs),
                                        C.byref(out)))
        self.h = out.value
        self.device = device
        self.meshes = []        # (femm, geom, u, matrix) per mesh id
        self._fin = weakref.finalize(self, _destroy, L, self.h)

    def close(self):
        """Stop the worker and free the server (its meshes' matrices stay)."""
        self._fin()

    def add_mesh(self, form: str, femm: FEMMBase, geom, u, cf, m: int = 3,
                 model=DeforModelRed3D):
        """Register a resident mesh; returns (mesh id, its DeviceMatrix)."""
        if form not in _FORMS:
            raise ValueError(f"form must be one of {sorted(_FORMS)}")
        if form == "lin_elastic" and model is not DeforModelRed3D:
            raise NotImplementedError("only DeforModelRed3D is supported")
        L = nat.load()
        dm = _prepare(femm, geom, u)
        out = C.c_void_p()
        nat.check(L.fegpu_matrix_create(dm.h, C.byref(out)))
        dm.matrices[("server", id(self), len(dm.matrices))] = out.value
        keep = []
        coef = _coef(femm, geom, cf, keep)
        mid = C.c_int64()
        nat.check(L.fegpu_server_add_mesh(self.h, out.value, _FORMS[form], C.byref(coef), int(m),
                                          C.byref(mid)))
        M = DeviceMatrix(out.value, dm, drop_zeros=True)
        self.meshes.append((femm, geom, u, M))
        return mid.value, M

    def submit_coef(self, mesh: int, values) -> int:
        """New per-element (or per-point) coefficient values, laid out as the
        coefficient the mesh was added with (e.g. nelem x 2 Lame pairs)."""
        v = np.ascontiguousarray(values, dtype=np.float64)
        rid = C.c_int64()
        nat.check(nat.load().fegpu_server_submit(self.h, int(mesh), nat.REQUEST_COEF, v.ctypes.data,
                                                 v.size, C.byref(rid)))
        return rid.value

    def submit_coords(self, mesh: int, xyz) -> int:
        """New node coordinates (nnodes x sdim, as geom.values)."""
        x = np.asfortranarray(xyz, dtype=np.float64)
        rid = C.c_int64()
        nat.check(nat.load().fegpu_server_submit(self.h, int(mesh), nat.REQUEST_COORDS,
                                                 x.ctypes.data, x.size, C.byref(rid)))
        return rid.value

    def wait(self, request: int) -> float:
        """Block until the request completed; returns its latency in ms."""
        lat = C.c_double()
        nat.check(nat.load().fegpu_server_wait(self.h, int(request), C.byref(lat)))
        return lat.value

    def drain(self):
        nat.check(nat.load().fegpu_server_drain(self.h))

    def hold(self, on: bool = True):
        """Pause (True) or resume (False) new launches; requests accumulate."""
        nat.check(nat.load().fegpu_server_hold(self.h, int(bool(on))))

    def stats(self):
        b, j, p = C.c_int64(), C.c_int64(), C.c_int64()
        nat.check(nat.load().fegpu_server_stats(self.h, C.byref(b), C.byref(j), C.byref(p)))
        return {"batches": b.value, "jobs": j.value, "pending": p.value}

    def memory(self):
        f, t = C.c_int64(), C.c_int64()
        nat.check(nat.load().fegpu_server_memory(self.h, C.byref(f), C.byref(t)))
        return f.value, t.value
