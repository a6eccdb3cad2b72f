"""Many assemblies in one persistent GPU launch (fegpu_batch_* of include/fegpu.h).

A reference caller that assembles many models -- a parameter sweep, a
multi-part structure, a queue of requests -- writes a loop of
``bilform_diffusion`` / ``bilform_lin_elastic`` / ``bilform_dot`` calls
(src/FEMMBaseModule.jl:1462-1545, 1774-1824, 1335-1376), one per FEMM.
``AssemblyBatch`` takes the same arguments per job and evaluates all of them
in one persistent kernel (replayed as a CUDA graph), each job in the
mixed-precision mode (FP32 element arithmetic, FP64 accumulation); every
matrix equals the single-call ``SysmatAssemblerGPU(precision="mixed")``
result.

    batch = AssemblyBatch()
    K1 = batch.add("lin_elastic", femm1, geom1, u1, DataCache(D))
    K2 = batch.add("diffusion", femm2, geom2, T2, DataCache(kappa))
    batch.tune("tiles.txt")    # optional: per element-type tile sizes, cached
    batch.run()                # K1, K2: DeviceMatrix handles, filled
"""
from __future__ import annotations

import ctypes as C
import weakref

from . import _native as nat
from .assembly import DeviceMatrix
from .femm import DeforModelRed3D, FEMMBase, _coef, _prepare

_FORMS = {"diffusion": nat.FORM_DIFFUSION, "lin_elastic": nat.FORM_LIN_ELASTIC,
          "dot": nat.FORM_DOT}


def _destroy(L, b):
    # the batch touches no matrix, dofmap or FEMM when it is destroyed, so the
    # order of finalizers (the FEMMs own the jobs' matrices) does not matter
    try:
        L.fegpu_batch_destroy(b)
    except Exception:
        pass


class AssemblyBatch:
    """A set of (form, FEMM, fields, coefficient) jobs run in one launch."""

    def __init__(self, device: int = 0):
        L = nat.load()
        out = C.c_void_p()
        nat.check(L.fegpu_batch_create(nat.context(device), C.byref(out)))
        self.h = out.value
        self.device = device
        self._femms = []      # the FEMMs own the dofmaps and matrices the jobs use
        self.matrices = []
        weakref.finalize(self, _destroy, L, self.h)

    def add(self, form: str, femm: FEMMBase, geom, u, cf, m: int = 3,
            model=DeforModelRed3D) -> DeviceMatrix:
        """Add one assembly; returns its (not yet filled) device matrix.
        ``form``: "diffusion", "lin_elastic" or "dot"; ``m``: the manifold
        dimension of the dot form's measure."""
        if form not in _FORMS:
            raise ValueError(f"form must be one of {sorted(_FORMS)}")
        if form == "lin_elastic" and model is not DeforModelRed3D:
            raise NotImplementedError("only DeforModelRed3D is supported")
        L = nat.load()
        dm = _prepare(femm, geom, u)
        out = C.c_void_p()
        nat.check(L.fegpu_matrix_create(dm.h, C.byref(out)))
        # owned by the dofmap (destroyed with the FEMM, after this batch's jobs)
        dm.matrices[("batch", id(self), len(dm.matrices))] = out.value
        keep = []
        coef = _coef(femm, geom, cf, keep)
        job = C.c_int64()
        nat.check(L.fegpu_batch_add(self.h, out.value, _FORMS[form], C.byref(coef), int(m),
                                    C.byref(job)))
        self._femms.append((femm, geom))
        M = DeviceMatrix(out.value, dm, drop_zeros=True)
        M.job = job.value
        self.matrices.append(M)
        return M

    def set_coef(self, job: int, cf):
        """New coefficient values for a job (same form and kind of data)."""
        femm, geom = self._femms[job]
        keep = []
        coef = _coef(femm, geom, cf, keep)
        nat.check(nat.load().fegpu_batch_set_coef(self.h, int(job), C.byref(coef)))

    def tune(self, cache_path: str | None = None):
        """Pick elements per tile for each job kind by timing (cached in cache_path)."""
        p = cache_path.encode() if cache_path else None
        nat.check(nat.load().fegpu_batch_tune(self.h, p))

    def tile(self, job: int) -> int:
        t = C.c_int()
        nat.check(nat.load().fegpu_batch_tile(self.h, int(job), C.byref(t)))
        return t.value

    def set_wait_limit(self, seconds: float):
        nat.check(nat.load().fegpu_batch_set_wait_limit(self.h, float(seconds)))

    def withhold(self, job: int):
        """Test of the failure path: withhold the completion of job's first
        element stage (job = -1: none), so the waits on it run out."""
        nat.check(nat.load().fegpu_batch_withhold(self.h, int(job)))

    def launch(self):
        nat.check(nat.load().fegpu_batch_launch(self.h))

    def wait(self):
        nat.check(nat.load().fegpu_batch_wait(self.h))

    def run(self):
        nat.check(nat.load().fegpu_batch_run(self.h))
        return self.matrices

    def stats(self):
        jobs, items = C.c_int64(), C.c_int64()
        nat.check(nat.load().fegpu_batch_stats(self.h, C.byref(jobs), C.byref(items)))
        return {"jobs": jobs.value, "items": items.value}
