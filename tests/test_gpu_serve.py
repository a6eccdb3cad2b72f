"""Serving loop (fegpu_server_*): re-assembly requests on resident meshes.

Bar: a request's matrix equals the single-call FEGPU_MIXED assembly with the
request's data bit for bit, whether the request ran alone or batched with
others; requests of one mesh complete in submission order; coordinate
updates move the mesh.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _fp32_pipe_single_calls(monkeypatch):
    """The persistent batch kernel forms element blocks on the FP32 pipe; the
    single-call references of these tests use the same tile (the single-call
    tensor-core blocks are checked against FP64 in test_gpu_parity)."""
    monkeypatch.setenv("FEGPU_MIXED_TC", "0")


def _field(ft, n, ndn):
    return ft.numberdofs(ft.NodalField(np.zeros((n, ndn))))


def _meshes(ft, seed=6):
    rng = np.random.default_rng(seed)
    out = []
    for i, (et, n) in enumerate([("H8", 3000), ("T10", 4000), ("H8", 800), ("T10", 1500),
                                 ("H20", 600), ("T4", 2000)]):
        fens, fes = ft.nearest_block(et, n, seed=100 + i)
        E = fes.count()
        rule = {"H8": ft.GaussRule(3, 2), "H20": ft.GaussRule(3, 3), "T4": ft.TetRule(1),
                "T10": ft.TetRule(4)}[et]
        femm = ft.FEMMBase(ft.IntegDomain(fes, rule))
        geom = ft.NodalField(fens.xyz)
        if i % 2 == 0:
            form, ndn = "diffusion", 1
            cf = ft.ElementwiseData(rng.lognormal(0.0, 1.0, E))
        else:
            form, ndn = "lin_elastic", 3
            cf = ft.IsotropicElementwise(rng.lognormal(np.log(70e9), 1.0, E), np.full(E, 0.3))
        out.append(dict(form=form, femm=femm, geom=geom, u=_field(ft, fens.count(), ndn), cf=cf,
                        fens=fens, E=E))
    return out


def _new_coef(ft, c, rng):
    if c["form"] == "diffusion":
        cf = ft.ElementwiseData(rng.lognormal(0.0, 1.0, c["E"]))
        return cf, cf.values
    cf = ft.IsotropicElementwise(rng.lognormal(np.log(70e9), 1.0, c["E"]), np.full(c["E"], 0.3))
    return cf, cf.lame


def _single_mixed(ft, c, cf, geom=None):
    asm = ft.SysmatAssemblerGPU(precision="mixed", result="device")
    g = geom if geom is not None else c["geom"]
    if c["form"] == "diffusion":
        return ft.bilform_diffusion(c["femm"], asm, g, c["u"], cf).values()
    return ft.bilform_lin_elastic(c["femm"], asm, g, c["u"], ft.DeforModelRed3D, cf).values()


def test_requests_in_the_mix_equal_single_calls(ft):
    cases = _meshes(ft)
    srv = ft.AssemblyServer(lanes=2, max_jobs=4)
    ids = [srv.add_mesh(c["form"], c["femm"], c["geom"], c["u"], c["cf"]) for c in cases]
    rng = np.random.default_rng(9)
    reqs, cfs = [], []
    srv.hold(True)                               # a burst, admitted at once
    for (mid, _), c in zip(ids, cases):
        cf, data = _new_coef(ft, c, rng)
        cfs.append(cf)
        reqs.append(srv.submit_coef(mid, data))
    srv.hold(False)
    lat = [srv.wait(r) for r in reqs]
    assert all(x > 0 for x in lat)
    st = srv.stats()
    # 6 requests, at most 4 per launch, 2 lanes: two launches of 4 + 2 jobs
    assert st["jobs"] == len(cases) and st["batches"] == 2
    mixed = [M.values() for _, M in ids]
    srv.close()
    for v, c, cf in zip(mixed, cases, cfs):
        assert np.array_equal(v, _single_mixed(ft, c, cf))
    # the same requests alone (one per launch)
    srv1 = ft.AssemblyServer(lanes=1, max_jobs=1)
    for (mid0, _), c, cf, v in zip(ids, cases, cfs, mixed):
        mid, M = srv1.add_mesh(c["form"], c["femm"], c["geom"], c["u"], c["cf"])
        data = cf.values if c["form"] == "diffusion" else cf.lame
        srv1.wait(srv1.submit_coef(mid, data))
        assert np.array_equal(M.values(), v)
    srv1.close()


def test_requests_of_one_mesh_complete_in_order(ft):
    c = _meshes(ft)[1]
    srv = ft.AssemblyServer(lanes=3, max_jobs=8)
    mid, M = srv.add_mesh(c["form"], c["femm"], c["geom"], c["u"], c["cf"])
    rng = np.random.default_rng(2)
    cfs, reqs = [], []
    for _ in range(4):
        cf, data = _new_coef(ft, c, rng)
        cfs.append(cf)
        reqs.append(srv.submit_coef(mid, data))
    srv.drain()
    lat = [srv.wait(r) for r in reqs]
    # submitted back to back and served one at a time: latencies grow
    assert all(b >= a for a, b in zip(lat, lat[1:]))
    got = M.values()
    srv.close()
    assert np.array_equal(got, _single_mixed(ft, c, cfs[-1]))


def test_coordinate_update(ft):
    c = _meshes(ft)[3]
    srv = ft.AssemblyServer(lanes=2)
    mid, M = srv.add_mesh(c["form"], c["femm"], c["geom"], c["u"], c["cf"])
    rng = np.random.default_rng(5)
    xyz = c["geom"].values.copy()
    inside = np.all((xyz > 1e-9) & (xyz < 1 - 1e-9), axis=1)
    xyz[inside] += rng.uniform(-0.002, 0.002, (inside.sum(), 3))
    srv.wait(srv.submit_coords(mid, xyz))
    got = M.values()
    srv.close()
    assert np.array_equal(got, _single_mixed(ft, c, c["cf"], geom=ft.NodalField(xyz)))


def test_server_rejects_bad_requests(ft):
    c = _meshes(ft)[0]
    srv = ft.AssemblyServer()
    mid, _ = srv.add_mesh(c["form"], c["femm"], c["geom"], c["u"], c["cf"])
    with pytest.raises(ft.FegpuError, match="Size mismatch"):
        srv.submit_coef(mid, np.ones(c["E"] + 1))
    with pytest.raises(ft.FegpuError, match="no such mesh"):
        srv.submit_coef(mid + 5, np.ones(c["E"]))
    mid2, _ = srv.add_mesh("diffusion", c["femm"], c["geom"], c["u"], ft.DataCache(1.0))
    with pytest.raises(ft.FegpuError, match="constant coefficient"):
        srv.submit_coef(mid2, np.ones(c["E"]))
    free, total = srv.memory()
    assert 0 < free <= total
    srv.close()


def test_large_request_in_slices_equals_single_call(ft):
    """A request cut into several slices (one element chunk per launch of its
    lane, its block ring carried from one launch to the next) gives the
    single-call matrix bit for bit, also with other requests sharing its
    launches."""
    cases = _meshes(ft)
    big = dict(cases[1])
    fens, fes = ft.nearest_block("T10", 60000, seed=77)
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.TetRule(4)))
    rng = np.random.default_rng(12)
    E = fes.count()
    big.update(femm=femm, geom=ft.NodalField(fens.xyz), u=_field(ft, fens.count(), 3), E=E,
               cf=ft.IsotropicElementwise(rng.lognormal(np.log(70e9), 1.0, E), np.full(E, 0.3)))
    srv = ft.AssemblyServer(lanes=2, max_jobs=8, slice_elements=1)  # one chunk per launch
    mid, M = srv.add_mesh(big["form"], big["femm"], big["geom"], big["u"], big["cf"])
    small = [srv.add_mesh(c["form"], c["femm"], c["geom"], c["u"], c["cf"]) for c in cases[2:4]]
    cf, data = _new_coef(ft, big, rng)
    scf = [_new_coef(ft, c, rng) for c in cases[2:4]]
    srv.hold(True)
    r = srv.submit_coef(mid, data)
    rs = [srv.submit_coef(sm, d) for (sm, _), (_, d) in zip(small, scf)]
    srv.hold(False)
    srv.wait(r)
    for x in rs:
        srv.wait(x)
    st = srv.stats()
    nchunks = st["jobs"] - len(rs)
    got = M.values()
    got_small = [Ms.values() for _, Ms in small]
    srv.close()
    assert nchunks > 2 and st["batches"] >= nchunks  # the big request took several launches
    assert np.array_equal(got, _single_mixed(ft, big, cf))
    for v, c, (cfs, _) in zip(got_small, cases[2:4], scf):
        assert np.array_equal(v, _single_mixed(ft, c, cfs))


def test_mesh_admitted_while_requests_stream(ft):
    """A mesh is added while requests on the others are in flight; its own
    requests then run beside theirs, and every result equals the single
    call."""
    cases = _meshes(ft)
    srv = ft.AssemblyServer(lanes=2, max_jobs=8, slice_elements=2000)
    ids = [srv.add_mesh(c["form"], c["femm"], c["geom"], c["u"], c["cf"]) for c in cases[:3]]
    rng = np.random.default_rng(4)
    reqs = []
    for _ in range(3):
        for (mid, _), c in zip(ids, cases[:3]):
            cf, data = _new_coef(ft, c, rng)
            reqs.append((srv.submit_coef(mid, data), c, cf, mid))
    late = cases[3]
    lid, LM = srv.add_mesh(late["form"], late["femm"], late["geom"], late["u"], late["cf"])
    lcf, ldata = _new_coef(ft, late, rng)
    lreq = srv.submit_coef(lid, ldata)
    last = {}
    for rid, c, cf, mid in reqs:
        srv.wait(rid)
        last[mid] = (c, cf)
    srv.wait(lreq)
    got = {mid: M.values() for mid, M in ids}
    lgot = LM.values()
    srv.close()
    for mid, (c, cf) in last.items():
        assert np.array_equal(got[mid], _single_mixed(ft, c, cf))
    assert np.array_equal(lgot, _single_mixed(ft, late, lcf))


def test_admission_refused_above_the_memory_limit(ft):
    """Out-of-memory on admission without exhausting the GPU: under a memory
    limit of 1.5 times one mesh's footprint, a second matrix of the same mesh
    does not fit and add_mesh returns FEGPU_ERR_MEMORY through the C ABI;
    after the first is removed the second is admitted and served."""
    c = _meshes(ft)[0]
    srv = ft.AssemblyServer()
    a, _ = srv.add_mesh(c["form"], c["femm"], c["geom"], c["u"], c["cf"])
    held = srv.mesh_bytes(a)
    assert held > 0 and srv.mesh_bytes() == held
    srv.set_memory_limit(held + held // 2)
    with pytest.raises(ft.FegpuError, match="not enough device memory"):
        srv.add_mesh(c["form"], c["femm"], c["geom"], c["u"], c["cf"])
    srv.remove_mesh(a)
    assert srv.mesh_bytes() == 0
    b, M = srv.add_mesh(c["form"], c["femm"], c["geom"], c["u"], c["cf"])
    rng = np.random.default_rng(3)
    cf, data = _new_coef(ft, c, rng)
    srv.wait(srv.submit_coef(b, data))
    got = M.values()
    with pytest.raises(ft.FegpuError, match="no such mesh"):
        srv.submit_coef(a, np.ones(c["E"]))
    srv.close()
    assert np.array_equal(got, _single_mixed(ft, c, cf))
    # the estimate for admission before creating a mesh is of the same order
    fe = c["femm"].integdomain.fes
    est = ft.estimate_mesh_bytes(fe.code, fe.count(), c["geom"].values.shape[0], 1)
    assert held // 4 <= est <= 8 * held


def test_cancelled_request(ft):
    """A request still waiting is withdrawn: its wait returns an error status
    through the C ABI; a running or finished one cannot be cancelled."""
    c = _meshes(ft)[0]
    srv = ft.AssemblyServer()
    mid, M = srv.add_mesh(c["form"], c["femm"], c["geom"], c["u"], c["cf"])
    rng = np.random.default_rng(8)
    cf1, d1 = _new_coef(ft, c, rng)
    cf2, d2 = _new_coef(ft, c, rng)
    srv.hold(True)
    r1 = srv.submit_coef(mid, d1)
    r2 = srv.submit_coef(mid, d2)
    srv.cancel(r2)
    srv.hold(False)
    srv.wait(r1)
    with pytest.raises(ft.FegpuError, match="cancelled"):
        srv.wait(r2)
    with pytest.raises(ft.FegpuError, match="no such request"):
        srv.cancel(r1)
    got = M.values()
    srv.close()
    assert np.array_equal(got, _single_mixed(ft, c, cf1))


@pytest.mark.parametrize("precision", ["fp64", "fp64_fast"])
def test_fp64_server(ft, precision):
    """An FP64 server runs each request through the single-call FP64 form, one
    at a time: results equal the single calls bit for bit."""
    cases = _meshes(ft)[:2]
    srv = ft.AssemblyServer(precision=precision)
    ids = [srv.add_mesh(c["form"], c["femm"], c["geom"], c["u"], c["cf"]) for c in cases]
    rng = np.random.default_rng(6)
    out = []
    for (mid, M), c in zip(ids, cases):
        cf, data = _new_coef(ft, c, rng)
        srv.wait(srv.submit_coef(mid, data))
        out.append((M.values(), c, cf))
    srv.close()
    for v, c, cf in out:
        asm = ft.SysmatAssemblerGPU(precision=precision, result="device")
        if c["form"] == "diffusion":
            ref = ft.bilform_diffusion(c["femm"], asm, c["geom"], c["u"], cf).values()
        else:
            ref = ft.bilform_lin_elastic(c["femm"], asm, c["geom"], c["u"], ft.DeforModelRed3D,
                                         cf).values()
        assert np.array_equal(v, ref)
