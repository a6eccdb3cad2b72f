"""Host-side check of the persistent kernel's work queue.

tests/queue_check.cpp builds queues with the library's own queue builder
(finetools.jl_gb300/csrc/batch_queue.cpp) for random job sets and runs them in
a discrete-event simulation of persistent CTAs; it checks that every item
completes (no dependency wait can block forever), that no element tile
overwrites a ring slot still read by a gather, that no gather starts before
the element blocks it reads, and that items cover every element and node
exactly once.  No GPU is involved.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = "/usr/local/cuda"


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_queue_schedule_properties(tmp_path):
    exe = str(tmp_path / "queue_check")
    cmd = ["g++", "-O1", "-std=c++17",
           "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "finetools.jl_gb300", "csrc"),
           "-I", os.path.join(CUDA, "include"),
           os.path.join(ROOT, "tests", "queue_check.cpp"),
           os.path.join(ROOT, "finetools.jl_gb300", "csrc", "batch_queue.cpp"),
           "-L", os.path.join(CUDA, "lib64"), "-Wl,-rpath," + os.path.join(CUDA, "lib64"),
           "-lcudart", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr
