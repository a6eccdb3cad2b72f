#!/usr/bin/env python
"""Assembly throughput on one GB300: elements/s and HBM-roofline fraction.

Headline workload: FP64 linear-elasticity stiffness (bilform_lin_elastic,
DeforModelRed3D) of a seeded T10 block, 60 x 60 x 60 cells split into six
tetrahedra each (1,296,000 elements, 1,771,561 nodes, 3 DOFs per node,
451,604,169 nonzeros), 4-point tet rule, isotropic E = 210e9, nu = 0.3,
assembled by the drop-in default (FEGPU_FP64: the reference's operation
order, the matrix equal to the reference algorithm's bit for bit).  A step is
one full assembly into the device-resident CSR matrix.

Also measured (the `workloads` key): the same assembly with FEGPU_FP64_FAST
(fused multiply-adds) and in mixed precision, the H20 40^3 elasticity
stiffness with per-element (E, nu) in the three precisions, the H8 20^3
diffusion stiffness, the 256-mesh batch and the serving loop.  Mixed results
carry the error gate against FP64: max_ij |dK_ij| / max_k |K_ik| <= 1e-6 and
|dK x| / |K x| <= 1e-6.

  python bench.py [--steps K] [--warmup W] [--gpus N] [--impl reference]

Under torchrun every rank assembles its own replica (weak scaling, no
collective on the data path); rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

T10_N = 60          # cells per side of the headline mesh
H20_N = 40
H8_N = 20
CPU_SAMPLE_N = 24   # T10 cells per side of the timed CPU-baseline sample
REF_SAMPLE_N = 12   # per-worker T10 block of the all-core context figure
MIXED_GATE = 1e-6   # mixed vs FP64: row-scaled per nonzero and |dK x| / |K x|


# ---------------------------------------------------------------------------
def env_rank():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def max_over_ranks(torch, dist, value):
    """The largest of every rank's value (a time): the job is as slow as its
    slowest replica.  NCCL reduces a device tensor, gloo a host one."""
    if dist is None:
        return float(value)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank, world, seconds):
    """Whole-job throughput of weakly scaled replicas: every rank processed
    units_per_rank in (at most) `seconds`."""
    return world * units_per_rank / seconds


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 50 ms; entering
    waits (up to 3 s) for the first sample, so the region that follows is
    covered."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []
        self.skip = 0

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.perf_counter()
            while not self.lines and time.perf_counter() - t0 < 3.0:
                time.sleep(0.01)
            self.skip = len(self.lines)  # samples taken before the region
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines[self.skip:]:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p.get("hbm_gbs"), "measured"
    except (OSError, ValueError):
        return 6800.0, "fallback"


def traffic_record():
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def algorithmic_bytes(nelem, nne, nnodes, nnz, ndof, s_coef):
    """Pattern resident, values written once: connectivity (int32), FP64
    coordinates, coefficients, FP64 values written, int32 column indices read,
    int32 row pointers."""
    return nelem * nne * 4 + nnodes * 3 * 8 + nelem * s_coef + nnz * 8 + nnz * 4 + (ndof + 1) * 4


# ---------------------------------------------------------------------------
# CPU oracle baseline (the only place bench.py runs oracle/)
def _oracle_t10_sample(n, reps):
    import __graft_entry__ as entry
    ft = entry.load_package()
    O = entry.load_oracle()
    fens, fes = ft.t10_elastic_mesh(n=n)
    femm = ft.IntegDomain(fes, ft.TetRule(4))
    npts, Ns, dN, w, pc = femm.integrationdata()
    u = ft.numberdofs(ft.NodalField(np.zeros((fens.count(), 3))))
    D = ft.isotropic_D(210e9, 0.3)
    times, phases = [], []
    for _ in range(reps):
        t = time.perf_counter()
        _, _, ph = O.bilform(O.LIN_ELASTIC, O.T10, fes.conn, fens.xyz, u.dofnums, u.nalldofs(),
                             pc, w, D, phases=True)
        times.append(time.perf_counter() - t)
        phases.append(ph)
    return fes.count(), times, phases


_WORKER = {}


def _ref_worker_init(n):
    import __graft_entry__ as entry
    ft = entry.load_package()
    O = entry.load_oracle()
    fens, fes = ft.t10_elastic_mesh(n=n)
    dom = ft.IntegDomain(fes, ft.TetRule(4))
    npts, Ns, dN, w, pc = dom.integrationdata()
    u = ft.numberdofs(ft.NodalField(np.zeros((fens.count(), 3))))
    _WORKER.update(O=O, fes=fes, fens=fens, u=u, pc=pc, w=w, D=ft.isotropic_D(210e9, 0.3))


def _ref_worker_step(_):
    W = _WORKER
    O = W["O"]
    t = time.perf_counter()
    O.bilform(O.LIN_ELASTIC, O.T10, W["fes"].conn, W["fens"].xyz, W["u"].dofnums,
              W["u"].nalldofs(), W["pc"], W["w"], W["D"])
    return W["fes"].count(), time.perf_counter() - t


def _ref_full_assembly(n, out_q):
    """One serial assembly of the T10 n^3 configuration by the C restatement
    (child process, so its peak RSS is its own): elements, seconds, phases."""
    import resource
    import __graft_entry__ as entry
    ft = entry.load_package()
    O = entry.load_oracle()
    fens, fes = ft.t10_elastic_mesh(n=n)
    dom = ft.IntegDomain(fes, ft.TetRule(4))
    npts, Ns, dN, w, pc = dom.integrationdata()
    u = ft.numberdofs(ft.NodalField(np.zeros((fens.count(), 3))))
    D = ft.isotropic_D(210e9, 0.3)
    rss0 = resource.getrusage(resource.RUSAGE_SELF).ru_maxrss
    t = time.perf_counter()
    K, dropped, ph = O.bilform(O.LIN_ELASTIC, O.T10, fes.conn, fens.xyz, u.dofnums,
                               u.nalldofs(), pc, w, D, phases=True, tables=(Ns, dN))
    dt = time.perf_counter() - t
    rss = resource.getrusage(resource.RUSAGE_SELF).ru_maxrss
    out_q.put({"elements": fes.count(), "seconds": dt, "nnz": int(K.nnz),
               "zeros_dropped": int(dropped),
               "phases_s": {"element_loop": float(ph[0]), "sparse": float(ph[1]),
                            "symmetric_completion": float(ph[2])},
               "peak_rss_gb": rss / 1e6, "rss_before_gb": rss0 / 1e6})


def run_reference(args):
    """The reference algorithm on the headline configuration itself: the
    serial C restatement of bilform_lin_elastic + makematrix! (one core, as
    the reference runs) assembles the T10 60^3 block once -- the sample of
    this arm is one full assembly of the workload, phases timed apart, peak
    RSS recorded.  A full assembly takes about a minute, so the arm times one
    (the restatement has no JIT or cache to warm); the all-core throughput
    of one smaller block per core is reported beside it as context."""
    rank, world, _ = env_rank()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    p = ctx.Process(target=_ref_full_assembly, args=(args.t10_n, q))
    p.start()
    full = q.get()
    p.join()
    value = full["elements"] / full["seconds"]
    # context: every core assembling its own T10 12^3 block, a few steps
    with ctx.Pool(cores, initializer=_ref_worker_init, initargs=(REF_SAMPLE_N,)) as pool:
        pool.map(_ref_worker_step, range(cores))
        t0 = time.perf_counter()
        elems = 0
        for _ in range(3):
            elems += sum(e for e, _ in pool.map(_ref_worker_step, range(cores)))
        allcore = elems / (time.perf_counter() - t0)
    sample = (f"one full serial assembly of the T10 {args.t10_n}^3 configuration "
              f"({full['elements']} elements): bilform_lin_elastic + makematrix! in the C "
              "restatement (-O2 -ffp-contract=off), 1 core")
    out = {
        "impl": "reference", "metric": "elements/s", "value": value, "unit": "elements/s",
        "n_gpus": args.gpus, "steps": 1, "warmup": 0, "requested_steps": args.steps,
        "requested_warmup": args.warmup, "ms_per_step": 1e3 * full["seconds"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": f"synthetic: seeded T10 {args.t10_n}^3 block, interior vertices jittered +-0.15h",
        "config": {"workload": f"T10 {args.t10_n}^3 linear elasticity (bilform_lin_elastic), FP64",
                   "elements": full["elements"], "nnz": full["nnz"],
                   "same_config": True},
        "cpu_baseline": {"value": value, "unit": "elements/s", "cores": 1, "kind": "port",
                         "sample": sample, "host_cores": cores,
                         "phases_s": full["phases_s"], "peak_rss_gb": full["peak_rss_gb"],
                         "zeros_dropped": full["zeros_dropped"]},
        "all_cores_context": {"value": allcore, "unit": "elements/s", "cores": cores,
                              "sample": f"{cores} processes, each assembling a T10 "
                                        f"{REF_SAMPLE_N}^3 block per step, 3 steps"},
        "e2e": {"value": value, "unit": "elements/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


# ---------------------------------------------------------------------------
class Lib:
    """Thin access to the C ABI for timing."""

    def __init__(self, ft, device):
        from importlib import import_module
        self.nat = import_module(ft.__name__ + "._native")
        self.L = self.nat.load()
        self.ctx = self.nat.context(device)
        s = C.c_void_p()
        self.nat.check(self.L.fegpu_context_stream(self.ctx, C.byref(s)))
        self.stream = s.value
        self.nat.check(self.L.fegpu_context_timing(self.ctx, 1))

    def stats(self, reset=True):
        ms = C.c_double()
        n = C.c_int64()
        self.nat.check(self.L.fegpu_context_kernel_stats(self.ctx, C.byref(ms), C.byref(n),
                                                         int(reset)))
        return ms.value, n.value


def pinned(torch, shape, dtype):
    t = torch.empty(int(np.prod(shape)), dtype=dtype, pin_memory=True)
    return t.numpy().reshape(shape)


def mixed_errors(K64, K32, seed=3):
    """Error of a mixed-precision matrix against the FP64 one (same CSR
    pattern): max |dK| / max |K|; max |dK_ij| / max_k |K_ik| (row scale); max
    over nonzeros of |dK_ij| / |K_ij| raw (entries formed by cancellation,
    near zero in FP64, make it large) and with a floor of 1e-12 max_k |K_ik|
    in the row; |dK x| / |K x|."""
    v64, v32 = K64.values(), K32.values()
    d = np.abs(v32 - v64)
    a = np.abs(v64)
    rowptr, _ = K64.dm.pattern()
    rowptr = rowptr - 1
    counts = np.diff(rowptr)
    rowmax = np.zeros(len(counts))
    nz = counts > 0
    rowmax[nz] = np.maximum.reduceat(a, rowptr[:-1][nz])
    floor = np.repeat(1e-12 * rowmax, counts)
    raw = d[a > 0] / a[a > 0]
    x = np.random.default_rng(seed).uniform(-1, 1, K64.shape[0])
    y64, y32 = K64.spmv(x), K32.spmv(x)
    rowscale = np.repeat(np.where(rowmax > 0, rowmax, 1.0), counts)
    row = float((d / rowscale).max())
    kx = float(np.linalg.norm(y32 - y64) / np.linalg.norm(y64))
    return {"max_abs_over_max": float(d.max() / a.max()),
            "max_abs_over_row_max": row,
            "max_rel_nonzero_raw": float(raw.max()) if raw.size else 0.0,
            "max_rel_nonzero_floor_1e-12_rowmax": float((d / np.maximum(a, floor)).max()),
            "rel_Kx": kx,
            "gate": f"max_ij |dK_ij| / max_k |K_ik| <= {MIXED_GATE:g} and "
                    f"|dK x| / |K x| <= {MIXED_GATE:g}",
            "gate_ok": bool(row <= MIXED_GATE and kx <= MIXED_GATE)}


def time_steps(torch, stream, fn, steps, warmup, flush=None, dist=None):
    """Device time of `steps` calls of fn on the library stream (CUDA events),
    barrier + synchronize on both sides; max over ranks."""
    for _ in range(warmup):
        fn()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    if flush is None:
        ev[0].record(stream)
        for _ in range(steps):
            fn()
        ev[1].record(stream)
        torch.cuda.synchronize()
        ms = ev[0].elapsed_time(ev[1])
    else:  # per-step events with an L2 flush in between
        ms = 0.0
        for _ in range(steps):
            flush()
            torch.cuda.synchronize()
            ev[0].record(stream)
            fn()
            ev[1].record(stream)
            torch.cuda.synchronize()
            ms += ev[0].elapsed_time(ev[1])
    return max_over_ranks(torch, dist, ms)


def fp64_peak_tflops(torch):
    """Measured FP64 GEMM throughput (torch.matmul, float64, 8192^3)."""
    a = torch.randn(8192, 8192, dtype=torch.float64, device="cuda")
    b = torch.randn(8192, 8192, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ev[0].record()
    torch.matmul(a, b)
    ev[1].record()
    torch.cuda.synchronize()
    ms = ev[0].elapsed_time(ev[1])
    del a, b
    return 2 * 8192 ** 3 / (ms * 1e-3) / 1e12


def exact_integer_ops_per_element(nne, npts):
    """Sums of the reference-order isotropic elasticity blocks that run on the
    integer units, per element: per point, the nine sums over the points of an
    off-diagonal node-pair block (six of a diagonal one) and the first sum of
    each diagonal entry's three products (three)."""
    return npts * ((nne * (nne - 1) // 2) * (9 + 3) + nne * (6 + 3))


def exact_ops_per_element(nne, npts, nnz_per_element, ndn=3):
    """FP64 instructions per element of the reference-order path (isotropic
    D; every one a separately rounded multiply or add): per point J (2 nne 9),
    det J + inverse + 1/det (~60), gradients (nne 3 5), Jac w, the DB
    columns (nne 9 2); per point and node-pair block B' DB in the reference's
    order (42 per off-diagonal block, 30 per diagonal one); in the gather one
    add per element-matrix entry and one per stored value (S + S')."""
    per_qp = 2 * nne * 9 + 60 + nne * 3 * 5 + 1 + nne * 9 * 2
    per_qp += (nne * (nne - 1) // 2) * 42 + nne * 30
    return npts * per_qp + (nne * ndn) ** 2 + nnz_per_element


def elastic_flops_per_element(nne, npts):
    """FP64 operations per element of the elasticity kernel as written: per point
    J (2 nne 9), det + inverse (~60), gradients (nne 3 5), weighting (3 nne);
    per node-pair block the Gram sums (18 npts), the Lame map (33) and the
    scatter adds (9 per block written)."""
    per_qp = 2 * nne * 9 + 60 + nne * 3 * 5 + 3 * nne
    nblk = nne * (nne + 1) // 2
    return npts * per_qp + nblk * (18 * npts + 33) + 9 * nne * nne


def run_ours(args):
    import torch
    rank, world, local = env_rank()
    dist = None
    if world > 1:
        import torch.distributed as tdist
        tdist.init_process_group("nccl")
        dist = tdist
    torch.cuda.set_device(local)
    import __graft_entry__ as entry
    ft = entry.load_package()
    lib = Lib(ft, local)
    stream = torch.cuda.ExternalStream(lib.stream, device=local)
    if args.only in ("h20", "h8", "batch", "serve"):
        fn = {"h20": bench_h20, "h8": bench_h8, "batch": bench_batch,
              "serve": bench_serve}[args.only]
        res = fn(ft, torch, lib, stream, args, local, dist)
        if rank == 0:
            print(json.dumps({"only": args.only, "workload": res}), flush=True)
        return

    # ---------------- headline: T10 60^3, FP64
    t0 = time.perf_counter()
    fens, fes = ft.t10_elastic_mesh(n=args.t10_n)
    mesh_s = time.perf_counter() - t0
    geom = ft.NodalField(fens.xyz)
    u = ft.numberdofs(ft.NodalField(np.zeros((fens.count(), 3))))
    D = ft.isotropic_D(210e9, 0.3)
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.TetRule(4)), device=local)
    asm = ft.SysmatAssemblerGPU(result="device", device=local)
    t0 = time.perf_counter()
    femm.set_geometry(geom)
    dm = femm.dofmap(u)
    K = ft.bilform_lin_elastic(femm, asm, geom, u, ft.DeforModelRed3D, ft.DataCache(D))
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    ncol = femm.colors()[1]
    cD = np.ascontiguousarray(D.ravel())
    coef = lib.nat.Coef(lib.nat.COEF_CONST, 36, cD.ctypes.data)

    def step():
        lib.nat.check(lib.L.fegpu_bilform_lin_elastic(K.h, C.byref(coef), lib.nat.FP64))

    lib.stats(reset=True)
    with ClockSampler(local) as clk:
        ms = time_steps(torch, stream, step, args.steps, args.warmup, dist=dist)
    kms, launches = lib.stats(reset=True)
    # the warm-up steps are in the counters too
    nsteps_counted = args.steps + args.warmup
    kernel_ms_step = kms / nsteps_counted
    launches_timed = launches // nsteps_counted * args.steps
    E, N, nnz, ndof = fes.count(), fens.count(), dm.nnz, dm.ndof
    ms_step = ms / args.steps
    value = job_throughput(E, world, ms_step * 1e-3)
    B = algorithmic_bytes(E, 10, N, nnz, ndof, 0)
    peak, peak_src = measured_peaks()
    achieved = B / (kernel_ms_step * 1e-3) / 1e9
    traffic = traffic_record().get("t10_exact", {}).get("bytes_per_assembly")
    fp64_peak = fp64_peak_tflops(torch)
    ops = exact_ops_per_element(10, 4, nnz / E) * E
    int_ops = exact_integer_ops_per_element(10, 4) * E

    # ---------------- end to end through the C ABI with host buffers
    # Each step uploads the coordinates from pinned host memory, assembles and
    # copies all CSR values back to pinned host memory.  Two matrices of the
    # same dofmap are used in turn, so step k's device-to-host copy (on the
    # export stream) overlaps step k+1's upload and assembly; every step's
    # copies finish inside the timed region.  The same loop run strictly one
    # step after the other is reported beside it ("sequential").
    xyz_h = pinned(torch, (3, N), torch.float64)  # column-major nnodes x 3
    xyz_h[:] = fens.xyz.T
    vals_h = [pinned(torch, (nnz,), torch.float64) for _ in range(2)]
    k2 = C.c_void_p()
    lib.nat.check(lib.L.fegpu_matrix_create(dm.h, C.byref(k2)))
    mats = [K.h, k2.value]

    def e2e_step(i, pipelined):
        Kh = mats[i & 1] if pipelined else K.h
        lib.nat.check(lib.L.fegpu_femm_set_geometry(femm._h, 3, xyz_h.ctypes.data))
        lib.nat.check(lib.L.fegpu_bilform_lin_elastic(Kh, C.byref(coef), lib.nat.FP64))
        if pipelined:
            lib.nat.check(lib.L.fegpu_matrix_copy_values_async(Kh, vals_h[i & 1].ctypes.data))
        else:
            lib.nat.check(lib.L.fegpu_matrix_copy_values(Kh, vals_h[0].ctypes.data))

    def e2e_run(pipelined):
        for i in range(args.warmup):
            e2e_step(i, pipelined)
        for Kh in mats:
            lib.nat.check(lib.L.fegpu_matrix_wait_export(Kh))
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        t0 = time.perf_counter()
        for i in range(args.steps):
            e2e_step(i, pipelined)
        for Kh in mats:
            lib.nat.check(lib.L.fegpu_matrix_wait_export(Kh))
        torch.cuda.synchronize()
        e2e_s = max_over_ranks(torch, dist, time.perf_counter() - t0)
        return job_throughput(E * args.steps, world, e2e_s)

    e2e_seq = e2e_run(False)
    e2e_value = e2e_run(True)
    # every host buffer written by the pipelined loop holds the assembled
    # values (a strided sample against the device copy)
    ref = K.values()[::97]
    written = {i & 1 for i in range(args.warmup)} | {i & 1 for i in range(args.steps)}
    e2e_check = all(bool(np.array_equal(vals_h[i][::97], ref)) for i in sorted(written))
    lib.nat.check(lib.L.fegpu_matrix_destroy(k2.value))
    lib.stats(reset=True)

    workloads = {}
    if not args.headline_only and args.only is None:
        # the same T10 assembly with FEGPU_FP64_FAST (fused multiply-adds,
        # Gram-sum element blocks, colour-ordered sums) and in mixed precision
        # (FP32 element blocks, row gather with float-float sums rounded once
        # to FP64), and their errors against the reference-order matrix
        Kf = ft.bilform_lin_elastic(femm, ft.SysmatAssemblerGPU(precision="fp64_fast",
                                                                result="device", device=local),
                                    geom, u, ft.DeforModelRed3D, ft.DataCache(D))

        def fstep():
            lib.nat.check(lib.L.fegpu_bilform_lin_elastic(Kf.h, C.byref(coef),
                                                          lib.nat.FP64_FAST))

        lib.stats(reset=True)
        msf = time_steps(torch, stream, fstep, args.steps, args.warmup, dist=dist)
        kmsf, _ = lib.stats(reset=True)
        ef = mixed_errors(K, Kf)
        vf, vx = Kf.values(), K.values()
        workloads["t10_60_elasticity_fp64_fast"] = {
            "ms_per_step": msf / args.steps,
            "elements_per_s": job_throughput(E, world, msf / args.steps * 1e-3),
            "kernel_ms": kmsf / (args.steps + args.warmup),
            "hbm_frac": B / (msf / args.steps * 1e-3) / 1e9 / peak,
            "speedup_over_reference_order": ms_step / (msf / args.steps),
            "vs_reference_order": {k: ef[k] for k in ("max_abs_over_max", "max_abs_over_row_max",
                                                      "rel_Kx")},
            "exact_zeros": {"reference_order": int((vx == 0).sum()),
                            "fp64_fast": int((vf == 0).sum())}}
        del Kf, vf, vx
        K32 = ft.bilform_lin_elastic(femm, ft.SysmatAssemblerGPU(precision="mixed",
                                                                 result="device", device=local),
                                     geom, u, ft.DeforModelRed3D, ft.DataCache(D))

        def mstep():
            lib.nat.check(lib.L.fegpu_bilform_lin_elastic(K32.h, C.byref(coef), lib.nat.MIXED))

        lib.stats(reset=True)
        ms32 = time_steps(torch, stream, mstep, args.steps, args.warmup, dist=dist)
        kms32, _ = lib.stats(reset=True)
        workloads["t10_60_elasticity_mixed"] = {
            "ms_per_step": ms32 / args.steps,
            "elements_per_s": job_throughput(E, world, ms32 / args.steps * 1e-3),
            "kernel_ms": kms32 / (args.steps + args.warmup),
            "hbm_frac": B / (ms32 / args.steps * 1e-3) / 1e9 / peak,
            "speedup_over_fp64": ms_step / (ms32 / args.steps),
            "speedup_over_fp64_fast": (msf / args.steps) / (ms32 / args.steps),
            "mixed_vs_fp64": mixed_errors(K, K32)}
        del K32
    del K, asm
    femm = None
    torch.cuda.empty_cache()

    if not args.headline_only and args.only is None:
        workloads["h20_40_elasticity"] = bench_h20(ft, torch, lib, stream, args, local, dist)
        workloads["h8_20_diffusion"] = bench_h8(ft, torch, lib, stream, args, local, dist)
        workloads["batch_256_mixed_types"] = bench_batch(ft, torch, lib, stream, args, local,
                                                         dist)
        workloads["serve_32_resident_meshes"] = bench_serve(ft, torch, lib, stream, args, local,
                                                            dist)

    cpu = None
    if rank == 0 and not args.no_cpu:
        ne, times, phases = _oracle_t10_sample(CPU_SAMPLE_N, 3)
        best = int(np.argmin(times))
        ph = phases[best]
        cpu = {"value": ne / times[best], "unit": "elements/s", "cores": 1, "kind": "port",
               "sample": f"T10 {CPU_SAMPLE_N}^3 block ({ne} elements), bilform_lin_elastic + "
                         "makematrix! in the serial C restatement, best of 3",
               # the reference's phases: element loop with COO appends
               # (assemble!), sparse() of the triples, S + S' completion
               "phases_s": {"element_loop": float(ph[0]), "sparse": float(ph[1]),
                            "symmetric_completion": float(ph[2])},
               "host_cores": os.cpu_count()}
    if rank != 0:
        return
    out = {
        "metric": "elements/s", "value": value, "unit": "elements/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": f"synthetic: seeded T10 {args.t10_n}^3 block, interior vertices jittered +-0.15h",
        "config": {"workload": f"T10 {args.t10_n}^3 linear elasticity (bilform_lin_elastic), FP64",
                   "path": "FEGPU_FP64: the reference's operation order (bitwise equal to the "
                           "reference algorithm's matrix)",
                   "elements": E, "nodes": N, "dofs": ndof, "nnz": nnz, "colours": ncol,
                   "l2": "working set larger than L2 (CSR values alone 3.6 GB); no flush",
                   "parallelism": f"replicas x{world}"},
        "nnz_per_s": world * nnz / (ms_step * 1e-3),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)",
                     "algorithmic_bytes_per_assembly": B,
                     "kernel": "k_blocks_exact<T10, ELAST_ISO> (element blocks) with "
                               "k_gather_exact<10, 3, S+S'> (row gather), one pair per chunk of "
                               "elements; timed together",
                     "kernel_ms_per_assembly": kernel_ms_step,
                     "note": "bound by the FP64 pipe, not HBM: see fp64_pipe"},
        "fp64_pipe": {"achieved_instructions_per_s": (ops - int_ops) / (kernel_ms_step * 1e-3),
                      "peak_instructions_per_s": fp64_peak * 1e12 / 2,
                      "frac": (ops - int_ops) / (kernel_ms_step * 1e-3) / (fp64_peak * 1e12 / 2),
                      "peak_source": "measured: torch.matmul float64 8192^3 (TFLOP/s / 2 = "
                                     "FP64 FMA instructions per second)",
                      "dgemm_tflops": fp64_peak,
                      "instructions_per_assembly": ops - int_ops,
                      "reference_operations_per_assembly": ops,
                      "reference_operations_per_s": ops / (kernel_ms_step * 1e-3),
                      "integer_unit_sums_per_assembly": int_ops,
                      "note": "the reference's order: every operation a separately rounded "
                              "FP64 multiply or add; the element blocks' sums over the points "
                              "and the first sum of each diagonal entry run on the integer "
                              "units (bit-identical IEEE additions), the rest (instructions) "
                              "on the FP64 pipe"},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "elements/s", "h2d_bytes_per_step": N * 3 * 8,
                "d2h_bytes_per_step": nnz * 8,
                "path": "fegpu_femm_set_geometry (pinned host coordinates) + "
                        "fegpu_bilform_lin_elastic + fegpu_matrix_copy_values_async (pinned "
                        "host), two matrices in turn: step k's copy to the host overlaps step "
                        "k+1's upload and assembly",
                "sequential": {"value": e2e_seq, "unit": "elements/s",
                               "path": "the same calls with fegpu_matrix_copy_values, one step "
                                       "after the other"},
                "values_check": e2e_check},
        "gpu_launches": launches_timed,
        "clocks": clk.summary(),
        "setup_s": {"mesh": mesh_s, "pattern_colouring_first_assembly": setup_s},
        "workloads": workloads,
    }
    print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def bench_h20(ft, torch, lib, stream, args, local, dist):
    fens, fes, flagged = ft.h20_elastic_mesh(n=args.h20_n)
    rng = np.random.default_rng(4)
    E = rng.lognormal(np.log(70e9), 0.5, fes.count())
    nu = rng.uniform(0.2, 0.35, fes.count())
    cf = ft.IsotropicElementwise(E, nu)
    geom = ft.NodalField(fens.xyz)
    u = ft.numberdofs(ft.NodalField(np.zeros((fens.count(), 3))))
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(3, 3)), device=local)
    res = {"elements": fes.count(), "distorted_elements": int(len(flagged))}
    mats = {}
    for prec in ("fp64", "fp64_fast", "mixed"):
        asm = ft.SysmatAssemblerGPU(precision=prec, result="device", device=local)
        K = ft.bilform_lin_elastic(femm, asm, geom, u, ft.DeforModelRed3D, cf)
        lame = np.ascontiguousarray(cf.lame)
        coef = lib.nat.Coef(lib.nat.COEF_ISO_LAME, 2, lame.ctypes.data)
        code = {"fp64": lib.nat.FP64, "fp64_fast": lib.nat.FP64_FAST,
                "mixed": lib.nat.MIXED}[prec]

        def step(K=K, coef=coef, code=code):
            lib.nat.check(lib.L.fegpu_bilform_lin_elastic(K.h, C.byref(coef), code))

        lib.stats(reset=True)
        ms = time_steps(torch, stream, step, args.steps, args.warmup, dist=dist)
        kms, _ = lib.stats(reset=True)
        ms_step = ms / args.steps
        dm = K.dm
        B = algorithmic_bytes(fes.count(), 20, fens.count(), dm.nnz, dm.ndof, 16)
        peak, _ = measured_peaks()
        kstep = kms / (args.steps + args.warmup)
        res[prec] = {"elements_per_s": fes.count() / (ms_step * 1e-3), "ms_per_step": ms_step,
                     "kernel_ms": kstep,
                     "hbm_frac": B / (ms_step * 1e-3) / 1e9 / peak,
                     "hbm_frac_of_kernel_time": B / (kstep * 1e-3) / 1e9 / peak,
                     "algorithmic_bytes": B}
        mats[prec] = K
    # the same mixed assembly as a one-job persistent launch (element tiles of
    # chunk c+1 overlap the gather of chunk c)
    b = ft.AssemblyBatch(device=local)
    Mb = b.add("lin_elastic", femm, geom, u, cf)

    def bstep():
        lib.nat.check(lib.L.fegpu_batch_launch(b.h))

    lib.stats(reset=True)
    ms = time_steps(torch, stream, bstep, args.steps, args.warmup, dist=dist)
    b.wait()
    lib.stats(reset=True)
    ms_step = ms / args.steps
    B = algorithmic_bytes(fes.count(), 20, fens.count(), Mb.dm.nnz, Mb.dm.ndof, 16)
    res["mixed_persistent"] = {"elements_per_s": fes.count() / (ms_step * 1e-3),
                               "ms_per_step": ms_step,
                               "hbm_frac": B / (ms_step * 1e-3) / 1e9 / measured_peaks()[0],
                               "work_items": b.stats()["items"]}
    v32 = mats["mixed"].values()
    res["mixed_persistent"]["identical_to_mixed"] = bool(np.array_equal(Mb.values(), v32))
    del b, Mb
    res["mixed_vs_fp64"] = mixed_errors(mats["fp64"], mats["mixed"])
    res["speedup_mixed_over_fp64"] = res["mixed"]["elements_per_s"] / res["fp64"]["elements_per_s"]
    res["speedup_mixed_over_fp64_fast"] = (res["mixed"]["elements_per_s"] /
                                           res["fp64_fast"]["elements_per_s"])
    return res


BATCH_TYPES = ("H8", "H20", "T4", "T10", "Q4")


def batch_cases(ft, count, seed=5, emin=1e3, emax=2e5, device=0):
    """The mixed-type batch: `count` meshes with log-uniform element counts on
    [emin, emax], types uniform over H8/H20/T4/T10/Q4 (Q4: surface mass by the
    dot form, thickness 0.01), each non-Q4 mesh diffusion or elasticity at
    random, seeded per-element coefficients."""
    rng = np.random.default_rng(seed)
    rules = {"H8": lambda: ft.GaussRule(3, 2), "H20": lambda: ft.GaussRule(3, 3),
             "T4": lambda: ft.TetRule(1), "T10": lambda: ft.TetRule(4),
             "Q4": lambda: ft.GaussRule(2, 2)}
    cases = []
    for _ in range(count):
        n = int(round(np.exp(rng.uniform(np.log(emin), np.log(emax)))))
        et = BATCH_TYPES[int(rng.integers(len(BATCH_TYPES)))]
        fens, fes = ft.nearest_block(et, n, seed=int(rng.integers(1 << 31)))
        E = fes.count()
        if et == "Q4":
            form, ndn = "dot", 3
            femm = ft.FEMMBase(ft.IntegDomain(fes, rules[et](), 0.01), device=device)
            cf = ft.ElementwiseData(rng.lognormal(np.log(7.8e3), 0.3, E))
        else:
            femm = ft.FEMMBase(ft.IntegDomain(fes, rules[et]()), device=device)
            if rng.random() < 0.5:
                form, ndn = "diffusion", 1
                cf = ft.ElementwiseData(rng.lognormal(0.0, 0.5, E))
            else:
                form, ndn = "lin_elastic", 3
                cf = ft.IsotropicElementwise(rng.lognormal(np.log(70e9), 0.5, E),
                                             rng.uniform(0.2, 0.35, E))
        geom = ft.NodalField(fens.xyz)
        u = ft.numberdofs(ft.NodalField(np.zeros((fens.count(), ndn))))
        cases.append({"type": et, "form": form, "femm": femm, "geom": geom, "u": u, "cf": cf,
                      "elements": E, "nodes": fens.count()})
    return cases


def _single_call(ft, c, asm):
    if c["form"] == "diffusion":
        return ft.bilform_diffusion(c["femm"], asm, c["geom"], c["u"], c["cf"])
    if c["form"] == "lin_elastic":
        return ft.bilform_lin_elastic(c["femm"], asm, c["geom"], c["u"], ft.DeforModelRed3D,
                                      c["cf"])
    return ft.bilform_dot(c["femm"], asm, c["geom"], c["u"], c["cf"], m=3)


def bench_batch(ft, torch, lib, stream, args, local, dist):
    t0 = time.perf_counter()
    cases = batch_cases(ft, args.batch_meshes, device=local)
    mesh_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    b = ft.AssemblyBatch(device=local)
    mats = [b.add(c["form"], c["femm"], c["geom"], c["u"], c["cf"], m=3) for c in cases]
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    b.tune()
    tune_s = time.perf_counter() - t0
    st = b.stats()

    def step():
        lib.nat.check(lib.L.fegpu_batch_launch(b.h))

    lib.stats(reset=True)
    ms = time_steps(torch, stream, step, args.steps, args.warmup, dist=dist)
    b.wait()
    _, launches = lib.stats(reset=True)
    ms_step = ms / args.steps
    E = sum(c["elements"] for c in cases)
    nnz = sum(M.dm.nnz for M in mats)
    B = 0
    for c, M in zip(cases, mats):
        nne = c["femm"].integdomain.fes.conn.shape[1]
        s_coef = 16 if c["form"] == "lin_elastic" else 8
        B += algorithmic_bytes(c["elements"], nne, c["nodes"], M.dm.nnz, M.dm.ndof, s_coef)
    peak, _ = measured_peaks()
    res = {"meshes": len(cases), "elements": E, "nnz": nnz, "work_items": st["items"],
           "types": {t: sum(1 for c in cases if c["type"] == t) for t in BATCH_TYPES},
           "forms": {f: sum(1 for c in cases if c["form"] == f)
                     for f in ("diffusion", "lin_elastic", "dot")},
           "ms_per_step": ms_step, "elements_per_s": E / (ms_step * 1e-3),
           "nnz_per_s": nnz / (ms_step * 1e-3), "algorithmic_bytes": B,
           "hbm_frac": B / (ms_step * 1e-3) / 1e9 / peak,
           "gpu_launches_per_step": launches / (args.steps + args.warmup),
           "setup_s": {"meshes": mesh_s, "patterns_and_jobs": setup_s, "autotune": tune_s},
           "tiles": {t: sorted({b.tile(j) for j, c in enumerate(cases) if c["type"] == t})
                     for t in BATCH_TYPES}}
    # the same jobs one call at a time (mixed, then FP64), and the accuracy
    seq = {}
    refs = {}
    for prec in ("mixed", "fp64"):
        asm = ft.SysmatAssemblerGPU(precision=prec, result="device", device=local)
        Ks = [_single_call(ft, c, asm) for c in cases]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for c in cases:
            _single_call(ft, c, asm)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        seq[prec] = {"elements_per_s": E / dt, "ms": 1e3 * dt}
        refs[prec] = Ks
    res["one_call_per_mesh"] = seq
    res["speedup_over_one_call_per_mesh_mixed"] = seq["mixed"]["ms"] / ms_step
    rng = np.random.default_rng(3)
    worst_kx, worst_entry, identical = 0.0, 0.0, True
    small = [j for j, M in enumerate(mats) if M.dm.nnz <= 30_000_000]  # host copies stay small
    sample = set(rng.choice(small, size=min(8, len(small)), replace=False).tolist()) if small \
        else set()
    for j, (M, K64, K32) in enumerate(zip(mats, refs["fp64"], refs["mixed"])):
        x = rng.uniform(-1, 1, M.shape[0])
        y, y64 = M.spmv(x), K64.spmv(x)
        worst_kx = max(worst_kx, float(np.linalg.norm(y - y64) / np.linalg.norm(y64)))
        if j in sample:
            v, v64 = M.values(), K64.values()
            worst_entry = max(worst_entry, float(np.abs(v - v64).max() / np.abs(v64).max()))
            if cases[j]["form"] != "dot":
                identical &= bool(np.array_equal(v, K32.values()))
    res["vs_fp64"] = {"max_rel_Kx": worst_kx, "max_abs_over_max_sampled": worst_entry,
                      "sampled_meshes": len(sample)}
    res["identical_to_one_call_mixed_sampled"] = identical
    del refs, mats, b, cases
    import gc
    gc.collect()
    torch.cuda.empty_cache()
    return res


def serve_cases(ft, count, seed=6, emin=1e4, emax=2e6, device=0):
    """Resident meshes of the serving workload: `count` H8 or T10 blocks with
    log-uniform element counts on [emin, emax]; H8 meshes carry diffusion with a
    per-element conductivity, T10 meshes elasticity with per-element (E, nu)."""
    rng = np.random.default_rng(seed)
    cases = []
    for _ in range(count):
        n = int(round(np.exp(rng.uniform(np.log(emin), np.log(emax)))))
        et = "H8" if rng.random() < 0.5 else "T10"
        fens, fes = ft.nearest_block(et, n, seed=int(rng.integers(1 << 31)))
        E = fes.count()
        if et == "H8":
            form, ndn = "diffusion", 1
            femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(3, 2)), device=device)
            cf = ft.ElementwiseData(rng.lognormal(0.0, 1.0, E))
        else:
            form, ndn = "lin_elastic", 3
            femm = ft.FEMMBase(ft.IntegDomain(fes, ft.TetRule(4)), device=device)
            cf = ft.IsotropicElementwise(rng.lognormal(np.log(70e9), 1.0, E), np.full(E, 0.3))
        cases.append({"type": et, "form": form, "femm": femm, "geom": ft.NodalField(fens.xyz),
                      "u": ft.numberdofs(ft.NodalField(np.zeros((fens.count(), ndn)))),
                      "cf": cf, "elements": E, "nodes": fens.count(), "xyz": fens.xyz,
                      "h": 1.0 / round((E / (6.0 if et == "T10" else 1.0)) ** (1.0 / 3.0))})
    return cases


def _request_payloads(cases, rng):
    """Two coefficient vectors (lognormal, sigma 1) and two coordinate sets
    (interior nodes moved by +-0.05 h) per mesh, made once."""
    out = []
    for c in cases:
        E = c["elements"]
        if c["form"] == "diffusion":
            coefs = [rng.lognormal(0.0, 1.0, E) for _ in range(2)]
        else:
            coefs = []
            for _ in range(2):
                lam, mu = ftlame(rng.lognormal(np.log(70e9), 1.0, E), 0.3)
                coefs.append(np.ascontiguousarray(np.stack([lam, mu], axis=1)))
        xyz = c["xyz"]
        inside = np.all((xyz > 1e-9) & (xyz < 1 - 1e-9), axis=1)
        coords = []
        for _ in range(2):
            x = xyz.copy()
            x[inside] += rng.uniform(-0.05, 0.05, (int(inside.sum()), 3)) * c["h"]
            coords.append(np.asfortranarray(x))
        out.append({"coef": coefs, "coords": coords})
    return out


def ftlame(E, nu):
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    mu = E / (2 * (1 + nu))
    return lam, mu


def _percentiles(lat):
    a = np.sort(np.asarray(lat))
    return float(np.percentile(a, 50)), float(np.percentile(a, 99))


def _serve_stream(srv, rng, rate, nreq, submit, live, elems, admit_at=None, admit=None):
    """A Poisson stream of nreq requests at `rate` per second over the meshes
    in `live`; after admit_at requests admit() starts on a thread of its own
    (a second client adding meshes while this one submits: it appends each
    admitted mesh to `live`); returns the latencies (ms), the mesh of each
    request and the elements/s over the stream."""
    import threading
    arr = np.cumsum(rng.exponential(1.0 / rate, nreq))
    t_start = time.perf_counter()
    reqs, keys, work, th = [], [], 0.0, None
    for i, a in enumerate(arr):
        if admit is not None and i == admit_at:
            th = threading.Thread(target=admit)
            th.start()
        dt = t_start + a - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        k = live[int(rng.integers(0, len(live)))]
        reqs.append(submit(k, int(rng.integers(0, 2)), int(rng.integers(0, 2))))
        keys.append(k)
        work += elems[k]
    lat = [srv.wait(r) for r in reqs]
    eps = work / (time.perf_counter() - t_start)
    if th is not None:
        th.join()
    return lat, keys, eps


def _latency_stats(lat, keys, alone):
    """p50/p99 of the latencies, and of the slowdowns (latency over the
    request's mesh served alone on an idle server); `floor` is the p99/p50
    the same requests would show with no queueing at all (their alone
    latencies), which bounds p99/p50 of the raw latencies from below when
    request sizes differ by orders of magnitude."""
    p50, p99 = _percentiles(lat)
    sd = [x / alone[k] for x, k in zip(lat, keys)]
    s50, s99 = _percentiles(sd)
    f50, f99 = _percentiles([alone[k] for k in keys])
    by_size = {}
    for name, lo, hi in (("alone_lt_1ms", 0.0, 1.0), ("alone_1_to_5ms", 1.0, 5.0),
                         ("alone_ge_5ms", 5.0, np.inf)):
        sel = [x for x, k in zip(lat, keys) if lo <= alone[k] < hi]
        if sel:
            c50, c99 = _percentiles(sel)
            by_size[name] = {"requests": len(sel), "p50_ms": c50, "p99_ms": c99,
                             "p99_over_p50": c99 / c50}
    return {"p50_ms": p50, "p99_ms": p99, "p99_over_p50": p99 / p50,
            "floor_p99_over_p50": f99 / f50,
            "slowdown_p50": s50, "slowdown_p99": s99, "slowdown_p99_over_p50": s99 / s50,
            "by_size": by_size}


def bench_serve(ft, torch, lib, stream, args, local, dist):
    """32 resident meshes served on concurrent lanes in slices of bounded
    work; the last 8 meshes are admitted (by a second client thread) while the
    first stream runs; Poisson streams at 0.3 - 1.1 of the
    measured capacity; the FP64 comparison is a stream through an FP64 server."""
    import gc
    t0 = time.perf_counter()
    cases = serve_cases(ft, args.serve_meshes, device=local)
    mesh_s = time.perf_counter() - t0
    rng = np.random.default_rng(7)
    payloads = _request_payloads(cases, rng)
    srv = ft.AssemblyServer(lanes=args.serve_lanes, max_jobs=64, device=local,
                            slice_elements=args.serve_slice)
    ids = {}
    refused = []

    def admit(k):
        """Admission by the library's memory estimate, then add_mesh (which
        checks the memory serving the mesh still needs)."""
        c = cases[k]
        fe = c["femm"].integdomain.fes
        need = ft.estimate_mesh_bytes(fe.code, c["elements"], c["nodes"],
                                      1 if c["form"] == "diffusion" else 3)
        free, _ = srv.memory()
        if free - (1 << 30) < need:
            refused.append(k)
            return False
        try:
            ids[k] = srv.add_mesh(c["form"], c["femm"], c["geom"], c["u"], c["cf"])
        except ft.FegpuError:
            refused.append(k)
            return False
        return True

    n_initial = max(1, (3 * len(cases)) // 4)
    t0 = time.perf_counter()
    for k in range(n_initial):
        admit(k)
    setup_s = time.perf_counter() - t0
    elems = np.array([c["elements"] for c in cases], dtype=np.float64)

    def submit(k, kind, v):
        mid = ids[k][0]
        p = payloads[k]
        return srv.submit_coef(mid, p["coef"][v]) if kind == 0 else \
            srv.submit_coords(mid, p["coords"][v])

    def capacity():
        live = sorted(ids)
        for rep in range(2):
            srv.hold(True)
            reqs = [submit(k, 0, rep % 2) for k in live]
            t0 = time.perf_counter()
            srv.hold(False)
            for r in reqs:
                srv.wait(r)
            burst_s = time.perf_counter() - t0
        return elems[live].sum() / burst_s, elems[live].mean()

    cap0, mean0 = capacity()
    res = {"meshes_initial": len(ids), "lanes": args.serve_lanes,
           "slice_elements": args.serve_slice, "setup_s": {"meshes": mesh_s, "register": setup_s},
           "capacity_elements_per_s_initial": cap0, "sweep": []}
    nreq = args.serve_requests
    late = list(range(n_initial, len(cases)))
    admitted_mid = []

    def admit_late():
        for k in late:
            if admit(k):
                admitted_mid.append(k)
                live.append(k)  # the stream's next requests may pick it

    def alone():
        """Latency of one request per mesh on an idle server (best of two)."""
        out = {}
        for k in sorted(ids):
            out[k] = min(srv.wait(submit(k, 0, rep % 2)) for rep in range(2))
        return out

    for i, frac in enumerate((0.3, 0.6, 0.9, 1.1)):
        cap, mean_e = (cap0, mean0) if i == 0 else capacity()
        rate = frac * cap / mean_e
        live = sorted(ids)
        lat, keys, eps = _serve_stream(srv, rng, rate, nreq, submit, live, elems,
                                       admit_at=nreq // 2 if i == 0 else None,
                                       admit=admit_late if i == 0 else None)
        if i == 0:
            res["capacity_elements_per_s"] = capacity()[0]  # all meshes admitted
            alone_ms = alone()
            res["alone_ms"] = {"min": min(alone_ms.values()), "max": max(alone_ms.values())}
        row = {"load": frac, "rate_per_s": rate, "requests": nreq, "meshes": len(live)}
        row.update(_latency_stats(lat, keys, alone_ms))
        row["elements_per_s"] = float(eps)
        res["sweep"].append(row)
    res["admitted_mid_stream"] = len(admitted_mid)
    res["refused"] = len(refused)
    res["meshes"] = len(ids)
    res["elements"] = int(elems[sorted(ids)].sum())
    res["types"] = {t: sum(1 for k in ids if cases[k]["type"] == t) for t in ("H8", "T10")}
    res["server"] = srv.stats()
    res["held_bytes"] = srv.mesh_bytes()
    srv.close()
    # FP64: the same kind of stream through an FP64 server (FEGPU_FP64_FAST:
    # the single-call FP64 form, one request at a time, in the same loop)
    fsrv = ft.AssemblyServer(lanes=1, device=local, precision="fp64_fast")
    fids = {k: fsrv.add_mesh(cases[k]["form"], cases[k]["femm"], cases[k]["geom"], cases[k]["u"],
                             cases[k]["cf"]) for k in sorted(ids)}

    def fsubmit(k, kind, v):
        mid = fids[k][0]
        p = payloads[k]
        return fsrv.submit_coef(mid, p["coef"][v]) if kind == 0 else \
            fsrv.submit_coords(mid, p["coords"][v])

    live = sorted(fids)
    fsrv.hold(True)
    reqs = [fsubmit(k, 0, 0) for k in live]
    t0 = time.perf_counter()
    fsrv.hold(False)
    for r in reqs:
        fsrv.wait(r)
    fp64_capacity = elems[live].sum() / (time.perf_counter() - t0)
    rate = 0.6 * fp64_capacity / elems[live].mean()
    falone = {k: min(fsrv.wait(fsubmit(k, 0, rep % 2)) for rep in range(2)) for k in live}
    lat, keys, eps = _serve_stream(fsrv, rng, rate, max(32, nreq // 2), fsubmit, live, elems)
    res["fp64_fast_server"] = {"capacity_elements_per_s": fp64_capacity, "load": 0.6}
    res["fp64_fast_server"].update(_latency_stats(lat, keys, falone))
    res["fp64_fast_server"]["elements_per_s"] = float(eps)
    res["capacity_mixed_over_fp64_fast"] = res["capacity_elements_per_s"] / fp64_capacity
    fsrv.close()
    del fids, ids, cases, srv, fsrv
    gc.collect()
    torch.cuda.empty_cache()
    return res


def bench_h8(ft, torch, lib, stream, args, local, dist):
    fens, fes = ft.h8_diffusion_mesh(n=H8_N)
    geom = ft.NodalField(fens.xyz)
    u = ft.numberdofs(ft.NodalField(np.zeros((fens.count(), 1))))
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(3, 2)), device=local)
    asm = ft.SysmatAssemblerGPU(result="device", device=local)
    K = ft.bilform_diffusion(femm, asm, geom, u, ft.DataCache(1.0))
    c1 = np.array([1.0])
    coef = lib.nat.Coef(lib.nat.COEF_CONST, 1, c1.ctypes.data)
    scratch = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    def flush():
        scratch.zero_()

    def step():
        lib.nat.check(lib.L.fegpu_bilform_diffusion(K.h, C.byref(coef), lib.nat.FP64))

    ms = time_steps(torch, stream, step, args.steps, args.warmup, flush=flush, dist=dist)
    lib.stats(reset=True)
    ms_step = ms / args.steps
    out = {"elements": fes.count(), "nnz": K.dm.nnz, "ms_per_step": ms_step,
           "elements_per_s": fes.count() / (ms_step * 1e-3),
           "path": "FEGPU_FP64 (reference order)",
           "l2": "flushed between steps (256 MB write)"}
    Kf = ft.bilform_diffusion(femm, ft.SysmatAssemblerGPU(precision="fp64_fast",
                                                          result="device", device=local),
                              geom, u, ft.DataCache(1.0))

    def fstep():
        lib.nat.check(lib.L.fegpu_bilform_diffusion(Kf.h, C.byref(coef), lib.nat.FP64_FAST))

    ms = time_steps(torch, stream, fstep, args.steps, args.warmup, flush=flush, dist=dist)
    lib.stats(reset=True)
    out["fp64_fast"] = {"ms_per_step": ms / args.steps,
                        "elements_per_s": fes.count() / (ms / args.steps * 1e-3)}
    K32 = ft.bilform_diffusion(femm, ft.SysmatAssemblerGPU(precision="mixed", result="device",
                                                           device=local),
                               geom, u, ft.DataCache(1.0))

    def mstep():
        lib.nat.check(lib.L.fegpu_bilform_diffusion(K32.h, C.byref(coef), lib.nat.MIXED))

    ms = time_steps(torch, stream, mstep, args.steps, args.warmup, flush=flush, dist=dist)
    lib.stats(reset=True)
    out["mixed"] = {"ms_per_step": ms / args.steps,
                    "elements_per_s": fes.count() / (ms / args.steps * 1e-3)}
    out["mixed_vs_fp64"] = mixed_errors(K, K32)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--headline-only", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--only", choices=["t10", "h20", "h8", "batch", "serve"], default=None,
                    help="run one workload only (profiling); prints its numbers")
    ap.add_argument("--h20-n", type=int, default=H20_N)
    ap.add_argument("--batch-meshes", type=int, default=256,
                    help="meshes of the mixed-type batch workload")
    ap.add_argument("--serve-meshes", type=int, default=32,
                    help="resident meshes of the serving workload")
    ap.add_argument("--serve-requests", type=int, default=200,
                    help="requests per load level of the serving sweep")
    ap.add_argument("--serve-lanes", type=int, default=2)
    ap.add_argument("--serve-slice", type=int, default=16384,
                    help="elements of one request per launch of its lane")
    ap.add_argument("--t10-n", type=int, default=T10_N,
                    help="cells per side of the headline T10 block (60 = the benchmark size)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
