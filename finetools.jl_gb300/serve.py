"""Serving loop: re-assembly requests on resident meshes (fegpu_server_* of
include/fegpu.h), continuously batched onto the GPU on concurrent lanes, in slices of bounded
work.

    server = AssemblyServer(lanes=2)
    mid, K = server.add_mesh("lin_elastic", femm, geom, u, IsotropicElementwise(E, nu))
    rid = server.submit_coef(mid, new_lame)          # (nelem, 2) lambda, mu
    rid2 = server.submit_coords(mid, new_xyz)         # (nnodes, 3)
    latency_ms = server.wait(rid)                     # K holds the request's matrix

Each request is evaluated as the mixed-precision batch path (or, with
precision="fp64" / "fp64_fast", by the single-call FP64 form, one request at a
time); a request's matrix does not depend on which other requests shared its
launches.  ``lanes`` is the number of CUDA streams launches run on; a request
runs in slices of at most ``slice_elements`` elements on one lane.  A mesh is admitted only
if the device memory it needs fits (and stays within memory_limit, if set).
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

    def __init__(self, lanes: int = 2, max_jobs: int = 64, device: int = 0,
                 precision: str = "mixed", slice_elements: int | None = None,
                 memory_limit: int | None = None):
        L = nat.load()
        out = C.c_void_p()
        nat.check(L.fegpu_server_create(nat.context(device), int(lanes), int(max_jobs),
                                        C.byref(out)))
        self.h = out.value
        self.device = device
        self.meshes = {}        # mesh id -> (femm, geom, u, matrix)
        self._fin = weakref.finalize(self, _destroy, L, self.h)
        codes = {"mixed": nat.MIXED, "fp64": nat.FP64, "fp64_fast": nat.FP64_FAST}
        if precision not in codes:
            raise ValueError("precision must be 'mixed', 'fp64' or 'fp64_fast'")
        if precision != "mixed":
            nat.check(L.fegpu_server_set_precision(self.h, codes[precision]))
        if slice_elements is not None:
            nat.check(L.fegpu_server_set_slice(self.h, int(slice_elements)))
        if memory_limit is not None:
            self.set_memory_limit(memory_limit)

    def set_memory_limit(self, nbytes: int):
        """Refuse meshes that would bring the served meshes' device memory
        above nbytes (0: no limit)."""
        nat.check(nat.load().fegpu_server_set_memory_limit(self.h, int(nbytes)))

    def mesh_bytes(self, mesh: int = -1) -> int:
        """Device bytes held by a served mesh (-1: by all of them)."""
        b = C.c_int64()
        nat.check(nat.load().fegpu_server_mesh_bytes(self.h, int(mesh), C.byref(b)))
        return b.value

    def remove_mesh(self, mesh: int):
        """Stop serving a mesh (no request of it waiting or in flight)."""
        nat.check(nat.load().fegpu_server_remove_mesh(self.h, int(mesh)))
        self.meshes.pop(mesh, None)

    def cancel(self, request: int):
        """Withdraw a request that is still waiting; its wait then raises."""
        nat.check(nat.load().fegpu_server_cancel(self.h, int(request)))

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
        self.meshes[mid.value] = (femm, geom, u, M)
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


def estimate_mesh_bytes(etype: int, nelem: int, nnodes: int, ndn: int) -> int:
    """Device bytes a mesh of this size needs to be created and served (an
    estimate from the element type's average node degree), for admission
    before anything is allocated."""
    b = C.c_int64()
    nat.check(nat.load().fegpu_estimate_mesh_bytes(int(etype), int(nelem), int(nnodes), int(ndn),
                                                   C.byref(b)))
    return b.value
