"""The N > 1 path of bench.py on CPU (the GPU runs replicas, one per rank): with two
gloo ranks the job's time is the slowest rank's, the value counts every rank's cells,
and the reference arm prints on rank 0 alone."""
import contextlib
import io
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        elapsed = bench.max_over_ranks(1.5 + rank, dist, "cpu")
        q.put((rank, elapsed, bench.replica_value(1000.0, 10, world, elapsed)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_time_the_slowest_rank():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        got = sorted(q.get(timeout=120) for _ in procs)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert [p.exitcode for p in procs] == [0, 0]
    assert [g[1] for g in got] == [2.5, 2.5]
    assert all(g[2] == 1000.0 * 10 * 2 / 2.5 for g in got)


def test_one_rank_needs_no_process_group():
    import bench
    assert bench.max_over_ranks(3.0, None, "cpu") == 3.0
    assert bench.replica_value(10.0, 4, 1, 2.0) == 20.0


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    import argparse
    import bench
    monkeypatch.setenv("RANK", "1")
    out = io.StringIO()
    with contextlib.redirect_stdout(out):
        bench.run_reference(argparse.Namespace(size=(8, 8, 8), workload="convection", steps=1, warmup=1, gpus=2))
    assert out.getvalue() == ""


@pytest.mark.parametrize("name", ["convection", "convection_dynamic", "turbulence2d", "stretched_amd", "seamount"])
def test_workloads_build_descriptors(name):
    # every bench workload builds its grid, physics and inputs and translates into a
    # descriptor (no device work)
    import numpy as np
    import bench
    from oceananigans_gb300 import _lib as L
    from oceananigans_gb300.api import model_descriptor
    size = (32, 32, 1) if name == "turbulence2d" else (32, 32, 16)
    grid, physics, init = bench.workload(name, size, np.float32)
    d, tracers = model_descriptor(grid, **physics)
    assert set(init) <= {"u", "v", "w"} | set(tracers)
    if name == "convection_dynamic":
        assert d.closure == L.GBO_CLOSURE_DYNAMIC_SMAGORINSKY and d.closure_averaging == L.GBO_AVERAGING_XY
        assert bench.algorithmic_bytes("k_closure", size, 4, closure="dynamic") == 3.5 * 32 * 32 * 16 * 4
