"""Benchmark: NonhydrostaticModel RK3 cell-updates/s on one GB300 (replicas for N > 1).

Workload: 3-D free convection, 256×256×128 RectilinearGrid over x, y ∈ [0, 512] m,
z ∈ [-256, 0] m, (Periodic, Periodic, Bounded); BuoyancyTracer b = N² z + 1e-8
noise (N² = 1e-5 s⁻²), velocities 1e-3 U[-1, 1] (seeded), surface buoyancy flux
1e-8 m² s⁻³, WENO5, SmagorinskyLilly, FPlane(f = 1e-4), FFT/DCT pressure solver,
Δt = 2 s, FP32.  A "step" is one full RK3 time step (three substeps with their
pressure projections) of the whole grid.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "oceananigans.jl_gb300"))

SIZE = (256, 256, 128)
DT = 2.0
METRIC = "cell_updates_per_s"
UNIT = "cell-updates/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--size", type=int, nargs=3, default=list(SIZE))
    p.add_argument("--dtype", default="f32", choices=["f32", "f64"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--e2e-steps", type=int, default=5)
    return p.parse_args()


def workload(size, float_type):
    import oceananigans_gb300 as og
    Nx, Ny, Nz = size
    grid = og.RectilinearGrid(size=size, x=(0, 512.0), y=(0, 512.0), z=(-256.0, 0.0),
                              topology=("Periodic", "Periodic", "Bounded"), float_type=float_type)
    physics = dict(advection=og.WENO(), closure=og.SmagorinskyLilly(), buoyancy=og.BuoyancyTracer(),
                   coriolis=og.FPlane(1e-4), tracers=("b",),
                   boundary_conditions={"b": og.FieldBoundaryConditions(top=og.FluxBoundaryCondition(1e-8))})
    rng = np.random.default_rng(2024)
    _, _, zc = grid.nodes()
    init = {"u": 1e-3 * rng.uniform(-1, 1, (Nx, Ny, Nz)),
            "v": 1e-3 * rng.uniform(-1, 1, (Nx, Ny, Nz)),
            "w": 1e-3 * rng.uniform(-1, 1, (Nx, Ny, Nz + 1)),
            "b": 1e-5 * zc[None, None, :] + 1e-8 * rng.standard_normal((Nx, Ny, Nz))}
    return grid, physics, init


def config_dict(size, dtype, n):
    return {"workload": "free_convection_%dx%dx%d_weno5_smagorinsky_lilly_fft" % tuple(size),
            "grid": list(size), "dt_s": DT, "float": dtype, "parallelism": "replicas%d" % n,
            "l2_policy": "inputs larger than L2 (state + work arrays ≈ 20 fields × %.0f MB)" %
                         (np.prod(size) * (4 if dtype == "f32" else 8) / 1e6)}


# ---------------------------------------------------------------------------
# CPU baseline: the FP64 C++/OpenMP oracle (a restatement of the reference; the
# Julia reference cannot run on this machine)
# ---------------------------------------------------------------------------
def cpu_sample(steps_budget_s=20.0, size=None):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from oceananigans_gb300.api import model_descriptor
    oracle.build()
    nthreads = os.cpu_count() or 1
    oracle.set_threads(nthreads)
    # bounded sample: the same per-cell work on a 128×128×128 sub-grid of the workload
    size = size or (128, 128, 128)
    grid, physics, init = workload(size, np.float64)
    grid.x, grid.y = (0, 512.0 * size[0] / SIZE[0]), (0, 512.0 * size[1] / SIZE[1])
    d = grid.descriptor()
    g = oracle.GridDesc()
    for f, _ in oracle.GridDesc._fields_:
        setattr(g, f, getattr(d, f))
    md, tracers = model_descriptor(grid, **physics)
    m = oracle.ModelDesc()
    for f, _ in oracle.ModelDesc._fields_:
        setattr(m, f, getattr(md, f))
    ref = oracle.OracleModel(g, m, tracers=tracers)
    ref.set(**init)
    ref.finalize_set(True)
    ref.time_step(DT, 1)  # warm-up
    t0 = time.perf_counter()
    n = 0
    while True:
        ref.time_step(DT, 1)
        n += 1
        if time.perf_counter() - t0 > steps_budget_s or n >= 5:
            break
    el = time.perf_counter() - t0
    cells = int(np.prod(size))
    return {"value": cells * n / el, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": "%d RK3 steps of the workload's physics on a %dx%dx%d sub-grid (FP64 oracle, %d threads, %.1f s)" %
                      (n, size[0], size[1], size[2], nthreads, el)}


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 5 + i and r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) of one launch from an ncu
# capture of this workload; the capture, its command and the algorithmic bytes of the
# same launch are in the named profile.
PROFILED_TRAFFIC = {
    ("k_momentum", (256, 256, 128), "f32"): {
        "traffic": 426.7e6,
        "traffic_launch": "one RK3 stage-1 launch (algorithmic bytes of that launch 469.8e6; stages 2-3 also read G-)",
        "traffic_profile": "profiles/k_momentum_fused_free_convection_256x256x128_f32.md",
        "issue_active_frac": 0.578,
        "dram_throughput_frac": 0.053,
    },
}


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def algorithmic_bytes(group, size, s, closure=True, ntr=1):
    """Algorithmic bytes per launch (compulsory reads + writes of whole fields)."""
    N = float(np.prod(size))
    per = {
        # fused momentum + tracer 0: u,v,w,c (+νₑ, pHY′) read, U*, c*, Gⁿ written;
        # G⁻ read on 2 of 3 stages
        "k_momentum": (3 + ntr + (1 if closure else 0) + 1) + (3 + ntr) * 2 + (3 + ntr) * 2.0 / 3,
        "k_tracer": (3 + 1 + (1 if closure else 0)) + 2 + 2.0 / 3,
        "k_closure": 4 + 1,
        "k_hydrostatic": 2,
        "k_source": 4,
        "k_dct_z": 2,
        "k_rfft_x": 2 * (1 + 2.0 / size[0]),
        "k_fft_y": 2 * (1 + 2.0 / size[0]),
        "k_correct": 8,
        "k_copy": 2,
        "k_nan_check": 1,
    }
    return per.get(group, 0) * N * s


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    size = tuple(args.size)
    samples = []
    cpu = None
    for _ in range(max(1, args.warmup)):
        pass
    t_all = time.perf_counter()
    for _ in range(args.steps):
        cpu = cpu_sample(steps_budget_s=max(2.0, 60.0 / max(1, args.steps)))
        samples.append(cpu["value"])
    value = statistics.median(samples)
    cpu["value"] = value
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * np.prod(size) / value,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)", "config": config_dict(size, "f64", args.gpus),
            "cpu_baseline": cpu, "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "reference arm = FP64 CPU restatement of the reference's algorithm (Julia is not installed); "
                    "wall %.1f s" % (time.perf_counter() - t_all)}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import oceananigans_gb300 as og
    from oceananigans_gb300 import _lib as L
    lib = og.load()
    size = tuple(args.size)
    ft = np.float32 if args.dtype == "f32" else np.float64
    s = 4 if ft == np.float32 else 8
    grid, physics, init = workload(size, ft)
    model = og.NonhydrostaticModel(grid, **physics)
    og.set_(model, **init)
    sp = ctypes.c_void_p()
    lib.gbo_model_stream(model._h, ctypes.byref(sp))
    stream = torch.cuda.ExternalStream(sp.value)

    og.time_step_(model, DT, args.warmup)

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = lib.gbo_kernel_launches(model._h)
    barrier()
    with ClockSampler(local) as clk:
        e0.record(stream)
        og.time_step_(model, DT, args.steps)
        e1.record(stream)
        barrier()
    elapsed = e0.elapsed_time(e1) / 1e3
    launches = lib.gbo_kernel_launches(model._h) - launches0
    if dist is not None:
        t = torch.tensor([elapsed], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t.item())
    cells = float(np.prod(size))
    value = cells * args.steps * world / elapsed

    # per-kernel durations from an instrumented pass on the same stream
    ng = lib.gbo_kernel_group_count()
    ms = (ctypes.c_double * ng)()
    nt = 2
    L.check(lib.gbo_kernel_timings(model._h, DT, nt, ms, ng), model._h)
    names = [lib.gbo_kernel_group_name(g).decode() for g in range(ng)]
    per_step_launches = {"k_momentum": 3, "k_tracer": 3, "k_closure": 3, "k_hydrostatic": 3, "k_source": 3,
                         "k_dct_z": 6, "k_rfft_x": 6, "k_fft_y": 3, "k_correct": 3, "k_copy": 3}
    kernels = {}
    for g, n in enumerate(names):
        if ms[g] > 0:
            kernels[n] = {"ms_per_launch": ms[g], "launches_per_step": per_step_launches.get(n, 0),
                          "ms_per_step": ms[g] * per_step_launches.get(n, 0)}
    tot = sum(k["ms_per_step"] for k in kernels.values()) or 1.0
    for k in kernels.values():
        k["share"] = k["ms_per_step"] / tot
    top = max(kernels, key=lambda n: kernels[n]["ms_per_step"])
    peak, peak_kind = measured_peak()
    ab = algorithmic_bytes(top, size, s)
    achieved = ab / (kernels[top]["ms_per_launch"] / 1e3) / 1e9
    roofline = {"kernel": top, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind, "traffic": None,
                "algorithmic_bytes_per_launch": ab}
    prof = PROFILED_TRAFFIC.get((top, tuple(size), args.dtype))
    if prof:
        roofline.update(prof)
    for n, k in kernels.items():
        b = algorithmic_bytes(n, size, s)
        k["achieved_gbs"] = b / (k["ms_per_launch"] / 1e3) / 1e9 if b else None

    # end to end through the C ABI with host buffers: upload the state, step, download
    e2e = None
    fields = ["u", "v", "w", "b"] if args.e2e_steps > 0 else []
    host = {}
    for n in fields:
        shp = model.field_shape(n)
        t = torch.empty(int(np.prod(shp)), dtype=torch.float32 if ft == np.float32 else torch.float64, pin_memory=True)
        host[n] = t
    code = L.GBO_FLOAT32 if ft == np.float32 else L.GBO_FLOAT64
    for n in fields:
        L.check(lib.gbo_get_field(model._h, model._fid(n), host[n].data_ptr(), code, host[n].numel()), model._h)
    h2d = sum(h.numel() * h.element_size() for h in host.values())
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps if fields else 0):
        for n in fields:
            L.check(lib.gbo_set_field(model._h, model._fid(n), host[n].data_ptr(), code, host[n].numel()), model._h)
        L.check(lib.gbo_time_step(model._h, DT, 1), model._h)
        for n in fields:
            L.check(lib.gbo_get_field(model._h, model._fid(n), host[n].data_ptr(), code, host[n].numel()), model._h)
    barrier()
    e2e_el = time.perf_counter() - t0
    if dist is not None:
        t = torch.tensor([e2e_el], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_el = float(t.item())
    if fields:
        e2e = {"value": cells * args.e2e_steps * world / e2e_el, "unit": UNIT,
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": h2d,
               "path": "gbo_set_field x4 (pinned host) + gbo_time_step(1) + gbo_get_field x4"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_sample()
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": args.dtype, "data": "synthetic (seeded numpy PCG64)",
                "config": config_dict(size, args.dtype, world), "clocks": clk.summary(), "e2e": e2e,
                "gpu_launches": int(launches), "roofline": roofline, "cpu_baseline": cpu, "kernels": kernels}
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
