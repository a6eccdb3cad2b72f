"""The build with device index checks (libfegpu_checked.so, -DFEGPU_DEVICE_CHECKS).

Its kernels check every node number they read and every CSR slot and vector
entry they write, skip an access out of range and record the first one in the
context's check word; the entry point then returns FEGPU_ERR_DEVICE.  Here
the checked library is built, loaded in a child process (FEGPU_DEVICE_CHECKS=1)
and run over the forms and precisions of the assembly path on valid inputs:
every call succeeds (no false alarm) and every matrix equals the regular
library's bit for bit (the checks change no arithmetic)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r'''
import ctypes as C, json, sys
import numpy as np
sys.path.insert(0, ROOT)
import __graft_entry__ as g
ft = g.load_package()
from importlib import import_module
nat = import_module(ft.__name__ + "._native")
on = C.c_int(-1)
nat.check(nat.load().fegpu_context_device_checks(nat.context(0), C.byref(on)))
out = {"checks": on.value}
def field(n, ndn):
    return ft.numberdofs(ft.NodalField(np.zeros((n, ndn))))
# reference-order FP64 elasticity (symmetric export), T10
fens, fes = ft.t10_elastic_mesh(n=4)
femm = ft.FEMMBase(ft.IntegDomain(fes, ft.TetRule(4)))
geom = ft.NodalField(fens.xyz); u = field(fens.count(), 3)
D = ft.isotropic_D(210e9, 0.3)
out["t10_fp64"] = ft.bilform_lin_elastic(femm, geom, u, ft.DeforModelRed3D, ft.DataCache(D)).data.tolist()
out["t10_fast"] = ft.bilform_lin_elastic(femm, ft.SysmatAssemblerGPU(precision="fp64_fast"), geom, u,
                                         ft.DeforModelRed3D, ft.DataCache(D)).data.tolist()
# mixed H20 with per-element Lame pairs
fens, fes, _ = ft.h20_elastic_mesh(n=3, distort_fraction=0.05)
femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(3, 3)))
rng = np.random.default_rng(3)
cf = ft.IsotropicElementwise(rng.lognormal(np.log(70e9), 0.5, fes.count()), rng.uniform(0.2, 0.35, fes.count()))
out["h20_mixed"] = ft.bilform_lin_elastic(femm, ft.SysmatAssemblerGPU(precision="mixed"),
                                          ft.NodalField(fens.xyz), field(fens.count(), 3),
                                          ft.DeforModelRed3D, cf).data.tolist()
# H8 diffusion (fast colour kernels) and a load vector
fens, fes = ft.h8_diffusion_mesh(n=4)
femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(3, 2)))
geom = ft.NodalField(fens.xyz); t = field(fens.count(), 1)
out["h8_fast"] = ft.bilform_diffusion(femm, ft.SysmatAssemblerGPU(precision="fp64_fast"), geom, t,
                                      ft.DataCache(1.5)).data.tolist()
out["h8_load"] = ft.distribloads(femm, geom, t, ft.ForceIntensity(2.0), 3).tolist()
# a batch (persistent kernel)
b = ft.AssemblyBatch()
M = b.add("diffusion", femm, geom, t, ft.DataCache(1.5))
b.run()
out["h8_batch"] = M.values().tolist()
json.dump(out, open(OUT, "w"))
'''


def _run(tmp_path, checked):
    path = str(tmp_path / ("checked.json" if checked else "regular.json"))
    env = dict(os.environ)
    env["FEGPU_DEVICE_CHECKS"] = "1" if checked else "0"
    code = CHILD.replace("ROOT", repr(ROOT)).replace("OUT", repr(path))
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    with open(path) as f:
        return json.load(f)


def test_checked_build_runs_clean_and_matches(tmp_path):
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "fegpu_build", os.path.join(ROOT, "finetools.jl_gb300", "build.py"))
    fegpu_build = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(fegpu_build)
    fegpu_build.build(device_checks=True)
    reg = _run(tmp_path, False)
    chk = _run(tmp_path, True)
    assert reg["checks"] == 0 and chk["checks"] == 1
    for key in reg:
        if key == "checks":
            continue
        a, b = np.array(reg[key]), np.array(chk[key])
        assert a.shape == b.shape and np.array_equal(a.view(np.int64), b.view(np.int64)), key
