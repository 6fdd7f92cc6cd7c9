"""Benchmark: NonhydrostaticModel RK3 cell-updates/s on one GB300 (replicas for N > 1).

Default workload (the headline): 3-D free convection, 256×256×128 RectilinearGrid
over x, y ∈ [0, 512] m, z ∈ [-256, 0] m, (Periodic, Periodic, Bounded);
BuoyancyTracer b = N² z + 1e-8 noise (N² = 1e-5 s⁻²), velocities 1e-3 U[-1, 1]
(seeded), surface buoyancy flux 1e-8 m² s⁻³, WENO5, SmagorinskyLilly,
FPlane(f = 1e-4), FFT/DCT pressure solver, Δt = 2 s, FP32.  A "step" is one full
RK3 time step (three substeps with their pressure projections) of the whole grid.

Other workloads (--workload), each with seeded synthetic inputs of the stated
shapes and distributions:
  convection_dynamic  the headline workload with DynamicSmagorinsky(averaging=(1, 2))
  convection_lagrangian  the headline workload with DynamicSmagorinsky() (LagrangianAveraging)
  turbulence2d    128×128 (Periodic, Periodic, Flat), u, v ~ U[-1, 1] projected,
                  WENO5, FP64, Δt = 0.01
  stretched_amd   512×512×256 with faces z_k = -256(1 - tanh(2(1 - k/256))/tanh 2),
                  AnisotropicMinimumDissipation, FourierTridiagonalPoissonSolver
                  (FP64 Thomas sweep), FP32 state, Δt = 1 s
  seamount        256×256×128 ImmersedBoundaryGrid(GridFittedBottom) over
                  x, y ∈ [-5, 5] km, z ∈ [-2, 0] km, h = -2000 + 1200 exp(-r²/(2·800²)),
                  N² = 1e-6, u = 0.1 + 1e-3 noise, FFT-preconditioned CG to a 1e-8
                  relative residual (FP64 dot products), FP32 state; also reports the
                  Poisson-solve time of held-out right-hand sides

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                       [--workload NAME] [--size NX NY NZ] [--dtype f32|f64]
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

METRIC = "cell_updates_per_s"
UNIT = "cell-updates/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="convection", choices=sorted(WORKLOADS))
    p.add_argument("--size", type=int, nargs=3, default=None)
    p.add_argument("--dtype", default=None, choices=["f32", "f64"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-other-workloads", action="store_true",
                   help="skip the records of the other benchmark configurations in the headline line")
    p.add_argument("--timed-only", action="store_true",
                   help="the timed steps and the per-kernel pass only (no e2e, CPU baseline, yardstick or "
                        "secondary records): the run a profiler captures")
    p.add_argument("--e2e-steps", type=int, default=5)
    a = p.parse_args()
    if a.timed_only:
        a.no_cpu_baseline, a.no_other_workloads, a.e2e_steps = True, True, 0
    w = WORKLOADS[a.workload]
    a.size = tuple(a.size) if a.size else w["size"]
    a.dtype = a.dtype or w["dtype"]
    return a


PPB = ("Periodic", "Periodic", "Bounded")


def _noise_init(size, zc, N2, bnoise, U=0.0, seed=2024):
    """u = U + 1e-3 U[-1, 1], v, w = 1e-3 U[-1, 1], b = N² z + bnoise N(0, 1) (seeded)."""
    Nx, Ny, Nz = size
    rng = np.random.default_rng(seed)
    return {"u": U + 1e-3 * rng.uniform(-1, 1, (Nx, Ny, Nz)),
            "v": 1e-3 * rng.uniform(-1, 1, (Nx, Ny, Nz)),
            "w": 1e-3 * rng.uniform(-1, 1, (Nx, Ny, Nz + 1)),
            "b": N2 * zc[None, None, :] + bnoise * rng.standard_normal((Nx, Ny, Nz))}


# Each workload is described once in plain numbers: grid keywords, the oracle's model
# description (oracle.model_desc keywords) and the seeded initial fields.  The library's
# model objects are built from the same numbers by the functions after these.
def _convection_spec(size, float_type):
    Nx, Ny, Nz = size
    gkw = dict(size=size, x=(0, 512.0 * Nx / 256), y=(0, 512.0 * Ny / 256), z=(-256.0, 0.0), topology=PPB,
               float_type=float_type)
    ophys = dict(closure="SmagorinskyLilly", buoyancy=True, coriolis=1e-4, tracers=("b",), flux_top={"b": 1e-8})
    zc = -256.0 + (np.arange(Nz) + 0.5) * 256.0 / Nz
    return gkw, ophys, _noise_init(size, zc, 1e-5, 1e-8)


def _convection_dynamic_spec(size, float_type):
    gkw, ophys, init = _convection_spec(size, float_type)
    return gkw, dict(ophys, closure=("DynamicSmagorinsky", {"averaging": (1, 2)})), init


def _convection_lagrangian_spec(size, float_type):
    gkw, ophys, init = _convection_spec(size, float_type)
    return gkw, dict(ophys, closure="DynamicSmagorinsky"), init


def _turbulence2d_spec(size, float_type):
    Nx, Ny = size[0], size[1]
    gkw = dict(size=(Nx, Ny), x=(0, 2 * np.pi), y=(0, 2 * np.pi), topology=("Periodic", "Periodic", "Flat"),
               float_type=float_type)
    rng = np.random.default_rng(2024)
    return gkw, {}, {"u": rng.uniform(-1, 1, (Nx, Ny, 1)), "v": rng.uniform(-1, 1, (Nx, Ny, 1))}


def _stretched_amd_spec(size, float_type):
    Nx, Ny, Nz = size
    # faces -256 (1 - tanh(2 (1 - k/Nz)) / tanh 2), k = 0..Nz, in increasing order (finest at the surface)
    zf = np.sort([-256.0 * (1 - np.tanh(2 * (1 - k / Nz)) / np.tanh(2)) for k in range(Nz + 1)])
    gkw = dict(size=size, x=(0, 512.0 * Nx / 256), y=(0, 512.0 * Ny / 256), z=zf, topology=PPB, float_type=float_type)
    ophys = dict(closure="AnisotropicMinimumDissipation", buoyancy=True, coriolis=1e-4, tracers=("b",),
                 flux_top={"b": 1e-8}, pressure_solver="FourierTridiagonalPoissonSolver")
    return gkw, ophys, _noise_init(size, 0.5 * (zf[1:] + zf[:-1]), 1e-5, 1e-8)


def _seamount_bottom(x, y):
    return -2000.0 + 1200.0 * np.exp(-(x * x + y * y) / (2 * 800.0 ** 2))


def _seamount_spec(size, float_type):
    Nz = size[2]
    gkw = dict(size=size, x=(-5000.0, 5000.0), y=(-5000.0, 5000.0), z=(-2000.0, 0.0), topology=PPB,
               float_type=float_type)
    ophys = dict(buoyancy=True, tracers=("b",),
                 pressure_solver=("ConjugateGradientPoissonSolver", {"reltol": 1e-8, "abstol": 1e-30}))
    zc = -2000.0 + (np.arange(Nz) + 0.5) * 2000.0 / Nz
    return dict(gkw, bottom_height=_seamount_bottom), ophys, _noise_init(size, zc, 1e-6, 1e-9, U=0.1)


def _convection(size, float_type):
    import oceananigans_gb300 as og
    gkw, _, init = _convection_spec(size, float_type)
    physics = dict(advection=og.WENO(), closure=og.SmagorinskyLilly(), buoyancy=og.BuoyancyTracer(),
                   coriolis=og.FPlane(1e-4), tracers=("b",),
                   boundary_conditions={"b": og.FieldBoundaryConditions(top=og.FluxBoundaryCondition(1e-8))})
    return og.RectilinearGrid(**gkw), physics, init


def _convection_lagrangian(size, float_type):
    """The convection workload with DynamicSmagorinsky() (LagrangianAveraging) as the closure."""
    import oceananigans_gb300 as og
    grid, physics, init = _convection(size, float_type)
    physics["closure"] = og.DynamicSmagorinsky()
    return grid, physics, init


def _convection_dynamic(size, float_type):
    """The convection workload with DynamicSmagorinsky(averaging=(1, 2)) as the closure."""
    import oceananigans_gb300 as og
    grid, physics, init = _convection(size, float_type)
    physics["closure"] = og.DynamicSmagorinsky(averaging=(1, 2))
    return grid, physics, init


def _turbulence2d(size, float_type):
    import oceananigans_gb300 as og
    gkw, _, init = _turbulence2d_spec(size, float_type)
    return og.RectilinearGrid(**gkw), dict(advection=og.WENO()), init


def _stretched_amd(size, float_type):
    import oceananigans_gb300 as og
    gkw, _, init = _stretched_amd_spec(size, float_type)
    physics = dict(advection=og.WENO(), closure=og.AnisotropicMinimumDissipation(), buoyancy=og.BuoyancyTracer(),
                   coriolis=og.FPlane(1e-4), tracers=("b",),
                   boundary_conditions={"b": og.FieldBoundaryConditions(top=og.FluxBoundaryCondition(1e-8))},
                   pressure_solver=og.FourierTridiagonalPoissonSolver())
    return og.RectilinearGrid(**gkw), physics, init


def _seamount(size, float_type):
    import oceananigans_gb300 as og
    gkw, _, init = _seamount_spec(size, float_type)
    gkw = dict(gkw)
    bottom = gkw.pop("bottom_height")
    grid = og.ImmersedBoundaryGrid(og.RectilinearGrid(**gkw), og.GridFittedBottom(bottom))
    physics = dict(advection=og.WENO(), buoyancy=og.BuoyancyTracer(), tracers=("b",),
                   pressure_solver=og.ConjugateGradientPoissonSolver(reltol=1e-8, abstol=1e-30))
    return grid, physics, init


def ensemble_specs(n=64, float_type=np.float32, seed=2025):
    """Members of the ensemble workload: Nx = Ny from {64, 96, 128}, Nz from {32, 48, 64},
    N² log-uniform on [1e-6, 1e-4] s⁻², surface flux uniform on [1e-9, 1e-7] m² s⁻³."""
    import oceananigans_gb300 as og
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(n):
        Nh = int(rng.choice([64, 96, 128]))
        Nz = int(rng.choice([32, 48, 64]))
        N2 = float(10 ** rng.uniform(-6, -4))
        flux = float(rng.uniform(1e-9, 1e-7))
        grid = og.RectilinearGrid(size=(Nh, Nh, Nz), x=(0, 2.0 * Nh), y=(0, 2.0 * Nh), z=(-2.0 * Nz, 0.0),
                                  topology=("Periodic", "Periodic", "Bounded"), float_type=float_type)
        physics = dict(advection=og.WENO(), closure=og.SmagorinskyLilly(), buoyancy=og.BuoyancyTracer(),
                       tracers=("b",),
                       boundary_conditions={"b": og.FieldBoundaryConditions(top=og.FluxBoundaryCondition(flux))})
        _, _, zc = grid.nodes()
        init = {"u": 1e-3 * rng.uniform(-1, 1, (Nh, Nh, Nz)), "v": 1e-3 * rng.uniform(-1, 1, (Nh, Nh, Nz)),
                "w": 1e-3 * rng.uniform(-1, 1, (Nh, Nh, Nz + 1)),
                "b": N2 * zc[None, None, :] + 1e-8 * rng.standard_normal((Nh, Nh, Nz))}
        specs.append((grid, physics, init))
    return specs


WORKLOADS = {
    "convection": dict(build=_convection, spec=_convection_spec, size=(256, 256, 128), dtype="f32", dt=2.0, cpu_size=(128, 128, 128),
                       name="free_convection_%dx%dx%d_weno5_smagorinsky_lilly_fft"),
    "convection_dynamic": dict(build=_convection_dynamic, spec=_convection_dynamic_spec, size=(256, 256, 128), dtype="f32", dt=2.0,
                               cpu_size=(64, 64, 128), name="free_convection_%dx%dx%d_weno5_dynamic_smagorinsky_xy_fft"),
    "convection_lagrangian": dict(build=_convection_lagrangian, spec=_convection_lagrangian_spec, size=(256, 256, 128),
                                  dtype="f32", dt=2.0, cpu_size=(64, 64, 128),
                                  name="free_convection_%dx%dx%d_weno5_dynamic_smagorinsky_lagrangian_fft"),
    "turbulence2d": dict(build=_turbulence2d, spec=_turbulence2d_spec, size=(128, 128, 1), dtype="f64", dt=0.01, cpu_size=(128, 128, 1),
                         name="turbulence2d_%dx%dx%d_weno5_fft"),
    "stretched_amd": dict(build=_stretched_amd, spec=_stretched_amd_spec, size=(512, 512, 256), dtype="f32", dt=1.0, cpu_size=(64, 64, 256),
                          name="stretched_convection_%dx%dx%d_weno5_amd_fourier_tridiagonal"),
    "ensemble": dict(build=None, spec=None, size=(0, 0, 0), dtype="f32", dt=1.0, cpu_size=(128, 128, 128),
                     name="ensemble_64_members_convection_smagorinsky_fft"),
    "seamount": dict(build=_seamount, spec=_seamount_spec, size=(256, 256, 128), dtype="f32", dt=20.0, cpu_size=(64, 64, 128),
                     name="seamount_ibg_%dx%dx%d_weno5_fft_pcg"),
}


def workload(name, size, float_type):
    return WORKLOADS[name]["build"](size, float_type)


def workload_cells(args):
    if args.workload == "ensemble":
        return float(sum(np.prod(g.size()) for g, _, _ in ensemble_specs()))
    return float(np.prod(args.size))


def config_dict(args, n):
    w = WORKLOADS[args.workload]
    if args.workload == "ensemble":
        return {"workload": w["name"], "members": 64, "dt_s": w["dt"], "float": args.dtype,
                "parallelism": "replicas%d" % n}
    size = args.size
    s = 4 if args.dtype == "f32" else 8
    return {"workload": w["name"] % tuple(size), "grid": list(size), "dt_s": w["dt"], "float": args.dtype,
            "parallelism": "replicas%d" % n,
            "l2_policy": "inputs larger than L2 (state + work arrays ≈ 20 fields × %.0f MB)" % (np.prod(size) * s / 1e6)
            if np.prod(size) * s * 20 > 129e6 else "state fits in L2 (small 2-D case; no flush between steps)"}


# ---------------------------------------------------------------------------
# CPU baseline: the FP64 C++/OpenMP oracle (a restatement of the reference; the
# Julia reference cannot run on this machine)
# ---------------------------------------------------------------------------
def cpu_sample(name, steps_budget_s=20.0):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    nthreads = os.cpu_count() or 1
    oracle.set_threads(nthreads)
    # bounded sample: the same per-cell work (same spacings and physics) on a smaller grid
    w = WORKLOADS[name]
    size = w["cpu_size"]
    dt = w["dt"]
    # the ensemble's members carry the convection physics; the oracle is configured from
    # its own description of the workload (reference defaults), not through the library
    spec = WORKLOADS["convection" if name == "ensemble" else name]["spec"]
    gkw, ophys, init = spec(size, np.float64)
    ref = oracle.model(gkw, **ophys)
    ref.set(**init)
    ref.finalize_set(True)
    ref.time_step(dt, 1)  # warm-up
    t0 = time.perf_counter()
    n = 0
    while True:
        ref.time_step(dt, 1)
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
# capture of this workload, keyed by (workload, kernel group, grid, float type); the
# capture, its command and the algorithmic bytes of the same launch are in the named profile.
PROFILED_TRAFFIC = {
    ("convection", "k_momentum", (256, 256, 128), "f32"): {
        "traffic": 448.0e6,
        "traffic_launch": "one RK3 stage-1 launch (algorithmic bytes of that launch 469.8e6; stages 2-3 also read G-)",
        "traffic_profile": "profiles/k_momentum_fused_free_convection_256x256x128_f32.md",
        "issue_active_frac": 0.680,
        "fma_pipe_inst_frac": 0.250,
        "alu_pipe_inst_frac": 0.299,
        "dram_throughput_frac": 0.089,
    },
}


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def algorithmic_bytes(group, size, s, ntr=1, closure="smagorinsky", has_phy=True, fused=True):
    """Algorithmic bytes per launch: compulsory reads + writes of whole fields, G⁻ read
    on 2 of the 3 RK3 stages."""
    N = float(np.prod(size))
    nu = 1 if closure else 0
    kap = 1 if closure == "amd" else 0
    spec = 2 * (1 + 2.0 / size[0])  # half spectrum in and out (complex, Nx/2+1 of Nx)
    if fused:  # momentum + tracer 0 in one march
        mom = (3 + 1 + nu + kap + (1 if has_phy else 0)) + (3 + 1) * 2 + (3 + 1) * 2.0 / 3
    else:      # per-point momentum kernel; tracers separately
        mom = (3 + nu + (1 if has_phy else 0)) + 3 * 2 + 3 * 2.0 / 3
    per = {
        "k_momentum": mom,
        "k_tracer": (3 + 1 + nu) + 2 + 2.0 / 3,
        # DynamicSmagorinsky: Σ and Σ̄ (5), LM and MM (5), the coefficient (0) and νₑ (4),
        # averaged over its four launches
        "k_closure": 3.5 if closure == "dynamic" else 4 + 1 + kap,
        "k_hydrostatic": 2,
        "k_source": 4,
        "k_dct_z": 2,
        "k_rfft_x": spec,
        "k_fft_y": spec,
        "k_thomas_z": spec,
        "k_correct": 8,
        "k_copy": 2,
        "k_nan_check": 1,
    }
    return per.get(group, 0) * N * s


def max_over_ranks(x, dist, device):
    """x of the slowest rank: the job's time is the largest over all ranks (x itself
    on one rank, dist None)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(cells, steps, world, elapsed):
    """Whole-job cell-updates/s: every rank advances its own replica of `cells` cells
    `steps` times, and the job takes the slowest rank's `elapsed` seconds."""
    return cells * steps * world / elapsed


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    size = tuple(args.size)
    samples = []
    cpu = None
    # each sample takes one untimed warm-up step of its own (cpu_sample)
    t_all = time.perf_counter()
    for _ in range(args.steps):
        cpu = cpu_sample(args.workload, steps_budget_s=max(2.0, 60.0 / max(1, args.steps)))
        samples.append(cpu["value"])
    value = statistics.median(samples)
    cpu["value"] = value
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * workload_cells(args) / value,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)", "config": config_dict(args, args.gpus),
            "cpu_baseline": cpu, "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "reference arm = FP64 CPU restatement of the reference's algorithm (Julia is not installed); "
                    "wall %.1f s" % (time.perf_counter() - t_all)}
    print(json.dumps(line), flush=True)


def held_out_solves(model, grid, torch, stream, ft, n=50):
    """Time CG Poisson solves (to the model's tolerance) of held-out right-hand sides:
    V·div of the model's current velocity plus seeded perturbations, masked to the
    active cells with zero active mean, as the pressure correction builds them."""
    u, v, w = model.get("u"), model.get("v"), model.get("w")
    Nx, Ny, Nz = u.shape
    dx, dy = grid.Lx / Nx, grid.Ly / Ny
    _, _, zc = grid.nodes()
    dz = grid.Lz / Nz
    imm = zc[None, None, :] <= grid.bottom_height[:, :, None]
    rng = np.random.default_rng(7)
    tdt = torch.float32 if ft == np.float32 else torch.float64
    phi = torch.zeros(Nx * Ny * Nz, dtype=tdt, device="cuda")
    rhs = []
    for _ in range(n):
        du = u + 1e-3 * rng.standard_normal(u.shape)
        dv = v + 1e-3 * rng.standard_normal(v.shape)
        dw = w + 1e-3 * rng.standard_normal(w.shape)
        dw[:, :, 0] = dw[:, :, -1] = 0
        div = (np.roll(du, -1, 0) - du) / dx + (np.roll(dv, -1, 1) - dv) / dy + (dw[:, :, 1:] - dw[:, :, :-1]) / dz
        b = div * (dx * dy * dz)
        b[imm] = 0
        b[~imm] -= b[~imm].mean()
        rhs.append(torch.tensor(b.ravel(order="F"), dtype=tdt, device="cuda"))
    times, iters = [], []
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for r in rhs:
        phi.zero_()
        torch.cuda.synchronize()
        e0.record(stream)
        model.poisson_solve_device(phi.data_ptr(), r.data_ptr())
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
        iters.append(model.solver_iterations)
    return {"solves": n, "ms_mean": float(np.mean(times)), "ms_median": float(np.median(times)),
            "iterations_mean": float(np.mean(iters)), "ms_per_iteration": float(np.sum(times) / max(1, np.sum(iters))),
            "preconditioner": "fft", "reltol": 1e-8,
            "path": "gbo_poisson_solve_device from a zero initial guess (host reads the stop flag each iteration)"}


def torch_fft_poisson(torch, rhs, Lx, Ly, Lz):
    """∇²ϕ = rhs on a regular (Periodic, Periodic, Bounded) grid with torch.fft (cuFFT):
    DCT-II in z by Makhoul's reordering and one complex FFT, real FFT in x and FFT in y,
    division by the eigenvalues (zero mean), and the inverse transforms -- the transform
    chain of the reference's GPU solver, which calls cuFFT (fft_based_poisson_solver.jl:94-136,
    ext/OceananigansCUDAExt.jl:118-129).  rhs: (Nz, Ny, Nx) tensor, x fastest.  Used only
    as a timing yardstick beside the library's hand-written passes."""
    Nz, Ny, Nx = rhs.shape
    dev, rdt = rhs.device, rhs.dtype
    k = torch.arange(Nz, device=dev, dtype=rdt)
    w = torch.polar(torch.ones_like(k), -torch.pi * k / (2 * Nz)).reshape(Nz, 1, 1)
    v = torch.cat([rhs[0::2], rhs[1::2].flip(0)], 0)
    X = (w * torch.fft.fft(v, dim=0)).real                       # DCT-II along z
    F = torch.fft.rfft2(X, dim=(1, 2))                           # FFT in y, real FFT in x
    lx = (2 * torch.sin(torch.pi * torch.arange(Nx // 2 + 1, device=dev, dtype=rdt) / Nx) / (Lx / Nx)) ** 2
    ly = (2 * torch.sin(torch.pi * torch.arange(Ny, device=dev, dtype=rdt) / Ny) / (Ly / Ny)) ** 2
    lz = (2 * torch.sin(torch.pi * k / (2 * Nz)) / (Lz / Nz)) ** 2
    lam = -(lz.reshape(Nz, 1, 1) + ly.reshape(1, Ny, 1) + lx.reshape(1, 1, -1))
    lam[0, 0, 0] = 1
    F = F / lam
    F[0, 0, 0] = 0
    X = torch.fft.irfft2(F, s=(Ny, Nx), dim=(1, 2))
    # inverse DCT-II: V_k = e^{iπk/2N} (X_k - i X_{N-k}), X_N = 0, v = ifft(V), then un-reorder
    Xr = torch.cat([torch.zeros_like(X[:1]), X[1:].flip(0)], 0)
    V = torch.conj(w) * torch.complex(X, -Xr)
    vv = torch.fft.ifft(V, dim=0).real
    out = torch.empty_like(rhs)
    h = (Nz + 1) // 2
    out[0::2] = vv[:h]
    out[1::2] = vv[h:].flip(0)
    return out


def cufft_yardstick(model, grid, torch, stream, ft, reps=20):
    """The library's FFT Poisson solve (gbo_poisson_solve_device) and the torch.fft (cuFFT)
    solve of the same right-hand side: time per solve (CUDA events, each on its own stream)
    and their relative difference (the yardstick must solve the same problem)."""
    Nx, Ny, Nz = grid.Nx, grid.Ny, grid.Nz
    tdt = torch.float32 if ft == np.float32 else torch.float64
    rng = np.random.default_rng(9)
    b = rng.standard_normal((Nx, Ny, Nz))
    b -= b.mean()
    rhs = torch.tensor(b.ravel(order="F"), dtype=tdt, device="cuda")
    phi = torch.empty_like(rhs)
    rhs3 = rhs.reshape(Nz, Ny, Nx)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    times = {}
    for name in ("gbo", "cufft"):
        for _ in range(3):
            if name == "gbo":
                model.poisson_solve_device(phi.data_ptr(), rhs.data_ptr())
            else:
                ref = torch_fft_poisson(torch, rhs3, grid.Lx, grid.Ly, grid.Lz)
        torch.cuda.synchronize()
        st = stream if name == "gbo" else torch.cuda.current_stream()
        e0.record(st)
        for _ in range(reps):
            if name == "gbo":
                model.poisson_solve_device(phi.data_ptr(), rhs.data_ptr())
            else:
                ref = torch_fft_poisson(torch, rhs3, grid.Lx, grid.Ly, grid.Lz)
        e1.record(st)
        torch.cuda.synchronize()
        times[name] = e0.elapsed_time(e1) / reps
    ref = ref.reshape(-1)
    diff = float(torch.linalg.vector_norm((phi - ref).double()) / torch.linalg.vector_norm(ref.double()))
    return {"gbo_ms": times["gbo"], "cufft_reference_ms": times["cufft"], "speedup": times["cufft"] / times["gbo"],
            "rel_l2_difference": diff, "grid": [Nx, Ny, Nz], "solves": reps,
            "cufft_path": "torch.fft (cuFFT): Makhoul DCT-II in z + rfft2 in x, y, eigenvalue divide, inverse",
            "gbo_path": "gbo_poisson_solve_device (k_dct_z, k_rfft_x, k_fft_y hand-written passes)"}


def seamount_poisson_record(torch, og, L, n=20):
    """Poisson-solve ms to a 1e-8 relative residual on the seamount benchmark grid
    (256x256x128 ImmersedBoundaryGrid, FP32 state, FP64 dot products): FFT-preconditioned
    CG and the learned flexible PCG on the same held-out right-hand sides, after two
    spin-up steps."""
    lib = og.load()
    size = WORKLOADS["seamount"]["size"]
    grid, physics, init = workload("seamount", size, np.float32)
    model = og.NonhydrostaticModel(grid, **physics)
    og.set_(model, **init)
    og.time_step_(model, WORKLOADS["seamount"]["dt"], 2)
    sp = ctypes.c_void_p()
    lib.gbo_model_stream(model._h, ctypes.byref(sp))
    stream = torch.cuda.ExternalStream(sp.value)
    rec = {"grid": list(size), "fft_pcg": held_out_solves(model, grid, torch, stream, np.float32, n=n)}
    wpath = os.path.join(os.path.dirname(og.__file__), "weights", "seamount_%dx%dx%d.npy" % tuple(size))
    if os.path.exists(wpath):
        model.set_learned_preconditioner(wpath)
        try:
            rec["learned_pcg"] = held_out_solves(model, grid, torch, stream, np.float32, n=n)
            rec["learned_pcg"]["preconditioner"] = "fft + learned correction (flexible CG), %s" % os.path.basename(wpath)
        except L.NotConvergedError as e:
            rec["learned_pcg"] = {"not_converged": str(e)}
        model.set_learned_preconditioner(None)
        if "ms_mean" in rec["learned_pcg"]:
            rec["learned_over_fft_time"] = rec["learned_pcg"]["ms_mean"] / rec["fft_pcg"]["ms_mean"]
    return rec


def kernel_table(lib, L, model, dt, size, s, nt=2, **ab_kw):
    """Per-kernel-group ms per launch, launches per step and achieved GB/s from the
    instrumented pass (CUDA events around every launch on the model's stream)."""
    ng = lib.gbo_kernel_group_count()
    ms = (ctypes.c_double * ng)()
    cnt = (ctypes.c_int64 * ng)()
    L.check(lib.gbo_kernel_timings(model._h, dt, nt, ms, ng), model._h)
    L.check(lib.gbo_kernel_timing_counts(model._h, cnt, ng), model._h)
    out = {}
    for g in range(ng):
        n = lib.gbo_kernel_group_name(g).decode()
        if ms[g] > 0 and n != "k_nan_check":
            b = algorithmic_bytes(n, size, s, **ab_kw)
            out[n] = {"ms_per_launch": ms[g], "launches_per_step": cnt[g] / nt, "ms_per_step": ms[g] * cnt[g] / nt,
                      "achieved_gbs": b / (ms[g] / 1e3) / 1e9 if b else None}
    tot = sum(k["ms_per_step"] for k in out.values()) or 1.0
    for k in out.values():
        k["share"] = k["ms_per_step"] / tot
    return out


def workload_record(name, torch, og, L, lib, steps, warmup=2):
    """One benchmark configuration timed on this GPU: cell-updates/s from CUDA events on
    the model's stream around `steps` graph-replayed steps, and its top kernel groups."""
    w = WORKLOADS[name]
    size = w["size"]
    ft = np.float32 if w["dtype"] == "f32" else np.float64
    s = 4 if ft == np.float32 else 8
    grid, physics, init = workload(name, size, ft)
    model = og.NonhydrostaticModel(grid, **physics)
    og.set_(model, **init)
    sp = ctypes.c_void_p()
    lib.gbo_model_stream(model._h, ctypes.byref(sp))
    stream = torch.cuda.ExternalStream(sp.value)
    og.time_step_(model, w["dt"], warmup)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    og.time_step_(model, w["dt"], steps)
    e1.record(stream)
    torch.cuda.synchronize()
    el = e0.elapsed_time(e1) / 1e3
    cells = float(np.prod(size))
    cl = physics.get("closure")
    closure = None if cl is None else ("amd" if isinstance(cl, og.AnisotropicMinimumDissipation) else "smagorinsky")
    ntr = len(physics.get("tracers", ()))
    kern = kernel_table(lib, L, model, w["dt"], size, s, ntr=ntr, closure=closure,
                        has_phy=ntr > 0 and grid.topology[2] == "Bounded", fused=grid.bottom_height is None)
    top = sorted(kern, key=lambda n: -kern[n]["ms_per_step"])[:4]
    rec = {"workload": w["name"] % tuple(size), "float": w["dtype"], "dt_s": w["dt"], "steps": steps,
           "value": cells * steps / el, "unit": UNIT, "ms_per_step": 1e3 * el / steps,
           "top_kernels": {n: kern[n] for n in top}}
    if isinstance(physics.get("pressure_solver"), og.ConjugateGradientPoissonSolver):
        rec["cg_iterations_last_solve"] = model.solver_iterations
    del model
    torch.cuda.synchronize()
    return rec


def ensemble_record(torch, og, L, lib, steps=10):
    """The 64-member ensemble (one graph launch per step) against the same members
    stepped one after another: cell-updates/s of each."""
    dt = WORKLOADS["ensemble"]["dt"]
    specs = ensemble_specs(64, np.float32)
    ens = og.Ensemble([(g, p) for g, p, _ in specs])
    for mm, (_, _, init) in zip(ens.members, specs):
        og.set_(mm, **init)
    cells = float(sum(np.prod(g.size()) for g, _, _ in specs))
    sp = ctypes.c_void_p()
    lib.gbo_ensemble_stream(ens._h, ctypes.byref(sp))
    stream = torch.cuda.ExternalStream(sp.value)
    ens.time_step(dt, 2)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    ens.time_step(dt, steps)
    e1.record(stream)
    torch.cuda.synchronize()
    batched = cells * steps / (e0.elapsed_time(e1) / 1e3)
    del ens
    singles = []
    for g, p, init in specs:
        m = og.NonhydrostaticModel(g, **p)
        og.set_(m, **init)
        og.time_step_(m, dt, 1)
        singles.append(m)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for m in singles:
        og.time_step_(m, dt, steps)
    torch.cuda.synchronize()
    seq = cells * steps / (time.perf_counter() - t0)
    return {"workload": WORKLOADS["ensemble"]["name"], "members": len(specs), "cells": int(cells), "float": "f32",
            "steps": steps, "value": batched, "unit": UNIT, "ms_per_step": 1e3 * cells / batched,
            "sequential_value": seq, "speedup_of_batched": batched / seq}


def run_ensemble(args, torch, og, L, lib, local):
    """64 uneven members advanced by one graph launch per step, against the same
    members stepped one after another (each with its own step graph)."""
    ft = np.float32 if args.dtype == "f32" else np.float64
    dt = WORKLOADS["ensemble"]["dt"]
    specs = ensemble_specs(64, ft)
    ens = og.Ensemble([(g, p) for g, p, _ in specs])
    for mm, (_, _, init) in zip(ens.members, specs):
        og.set_(mm, **init)
    cells = float(sum(np.prod(g.size()) for g, _, _ in specs))
    sp = ctypes.c_void_p()
    lib.gbo_ensemble_stream(ens._h, ctypes.byref(sp))
    stream = torch.cuda.ExternalStream(sp.value)
    ens.time_step(dt, args.warmup)
    launches0 = sum(lib.gbo_kernel_launches(mm._h) for mm in ens.members)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        e0.record(stream)
        ens.time_step(dt, args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
    elapsed = e0.elapsed_time(e1) / 1e3
    launches = sum(lib.gbo_kernel_launches(mm._h) for mm in ens.members) - launches0
    value = cells * args.steps / elapsed
    # the same members one after another (separate models, each its own graph per step)
    singles = []
    for g, p, init in specs:
        s = og.NonhydrostaticModel(g, **p)
        og.set_(s, **init)
        og.time_step_(s, dt, 1)
        singles.append(s)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in singles:
        og.time_step_(s, dt, args.steps)
    torch.cuda.synchronize()
    seq = cells * args.steps / (time.perf_counter() - t0)
    del singles
    # per-kernel timings and the roofline on the largest member
    big = max(range(len(specs)), key=lambda i: np.prod(specs[i][0].size()))
    g, p, _ = specs[big]
    mm = ens.members[big]
    ng = lib.gbo_kernel_group_count()
    ms = (ctypes.c_double * ng)()
    cnt = (ctypes.c_int64 * ng)()
    L.check(lib.gbo_kernel_timings(mm._h, dt, 2, ms, ng), mm._h)
    L.check(lib.gbo_kernel_timing_counts(mm._h, cnt, ng), mm._h)
    s_ = 4 if ft == np.float32 else 8
    kernels = {}
    for gi in range(ng):
        n = lib.gbo_kernel_group_name(gi).decode()
        if ms[gi] > 0 and n != "k_nan_check":
            b = algorithmic_bytes(n, g.size(), s_)
            kernels[n] = {"ms_per_launch": ms[gi], "launches_per_step": cnt[gi] / 2, "ms_per_step": ms[gi] * cnt[gi] / 2,
                          "achieved_gbs": b / (ms[gi] / 1e3) / 1e9 if b else None}
    top = max(kernels, key=lambda n: kernels[n]["ms_per_step"])
    peak, peak_kind = measured_peak()
    ab = algorithmic_bytes(top, g.size(), s_)
    achieved = ab / (kernels[top]["ms_per_launch"] / 1e3) / 1e9
    roofline = {"kernel": top, "member_grid": list(g.size()), "bound": "hbm", "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind, "traffic": None,
                "algorithmic_bytes_per_launch": ab}
    # end to end: upload every member's prognostic fields, one ensemble step, download
    code = L.GBO_FLOAT32 if ft == np.float32 else L.GBO_FLOAT64
    host = []
    for mm in ens.members:
        for n in ("u", "v", "w", "b"):
            t = torch.empty(int(np.prod(mm.field_shape(n))), dtype=torch.float32 if ft == np.float32 else torch.float64,
                            pin_memory=True)
            L.check(lib.gbo_get_field(mm._h, mm._fid(n), t.data_ptr(), code, t.numel()), mm._h)
            host.append((mm, n, t))
    nbytes = sum(t.numel() * t.element_size() for _, _, t in host)
    e2e = None
    if args.e2e_steps > 0:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            for mm, n, t in host:
                L.check(lib.gbo_set_field(mm._h, mm._fid(n), t.data_ptr(), code, t.numel()), mm._h)
            ens.time_step(dt, 1)
            for mm, n, t in host:
                L.check(lib.gbo_get_field(mm._h, mm._fid(n), t.data_ptr(), code, t.numel()), mm._h)
        e2e = {"value": cells * args.e2e_steps / (time.perf_counter() - t0), "unit": UNIT,
               "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
               "path": "gbo_set_field + gbo_ensemble_time_step(1) + gbo_get_field for all 64 members"}
    cpu = None
    if not args.no_cpu_baseline:
        cpu = cpu_sample("convection", steps_budget_s=20.0)
        cpu["sample"] = "ensemble members share the convection physics; " + cpu["sample"]
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": args.dtype, "data": "synthetic (seeded numpy PCG64)",
            "config": {"workload": WORKLOADS["ensemble"]["name"], "members": len(specs), "cells": int(cells),
                       "dt_s": dt, "float": args.dtype, "parallelism": "replicas1",
                       "l2_policy": "inputs larger than L2 (%.0f MB of state)" % (cells * 20 * s_ / 1e6)},
            "clocks": clk.summary(), "e2e": e2e, "gpu_launches": int(launches), "roofline": roofline,
            "cpu_baseline": cpu, "kernels": kernels,
            "sequential": {"value": seq, "unit": UNIT, "speedup_of_batched": value / seq,
                           "path": "the same 64 models stepped one after another"}}
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
    if args.workload == "ensemble":
        if rank == 0:
            run_ensemble(args, torch, og, L, lib, local)
        return
    size = tuple(args.size)
    ft = np.float32 if args.dtype == "f32" else np.float64
    s = 4 if ft == np.float32 else 8
    DT = WORKLOADS[args.workload]["dt"]
    grid, physics, init = workload(args.workload, size, ft)
    model = og.NonhydrostaticModel(grid, **physics)
    og.set_(model, **init)
    sp = ctypes.c_void_p()
    lib.gbo_model_stream(model._h, ctypes.byref(sp))
    stream = torch.cuda.ExternalStream(sp.value)
    closure = {type(None): None}.get(type(physics.get("closure")), None)
    cl = physics.get("closure")
    closure = None if cl is None else ("amd" if isinstance(cl, og.AnisotropicMinimumDissipation) else
                                       "dynamic" if isinstance(cl, og.DynamicSmagorinsky) else "smagorinsky")
    ntr = len(physics.get("tracers", ()))
    has_phy = ntr > 0 and grid.topology[2] == "Bounded" and physics.get("buoyancy") is not None
    fused = grid.bottom_height is None
    ab_kw = dict(ntr=ntr, closure=closure, has_phy=has_phy, fused=fused)

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
    elapsed = max_over_ranks(e0.elapsed_time(e1) / 1e3, dist, "cuda")
    launches = lib.gbo_kernel_launches(model._h) - launches0
    cells = float(np.prod(size))
    value = replica_value(cells, args.steps, world, elapsed)

    # per-kernel durations from an instrumented pass on the same stream: every launch
    # bracketed by CUDA events, launched one by one
    ng = lib.gbo_kernel_group_count()
    ms = (ctypes.c_double * ng)()
    cnt = (ctypes.c_int64 * ng)()
    nt = 2
    L.check(lib.gbo_kernel_timings(model._h, DT, nt, ms, ng), model._h)
    L.check(lib.gbo_kernel_timing_counts(model._h, cnt, ng), model._h)
    names = [lib.gbo_kernel_group_name(g).decode() for g in range(ng)]
    kernels = {}
    for g, n in enumerate(names):
        if ms[g] > 0 and n != "k_nan_check":
            per_step = cnt[g] / nt
            kernels[n] = {"ms_per_launch": ms[g], "launches_per_step": per_step, "ms_per_step": ms[g] * per_step}
    tot = sum(k["ms_per_step"] for k in kernels.values()) or 1.0
    for k in kernels.values():
        k["share"] = k["ms_per_step"] / tot
    top = max(kernels, key=lambda n: kernels[n]["ms_per_step"])
    peak, peak_kind = measured_peak()
    ab = algorithmic_bytes(top, size, s, **ab_kw)
    achieved = ab / (kernels[top]["ms_per_launch"] / 1e3) / 1e9
    roofline = {"kernel": top, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind, "traffic": None,
                "algorithmic_bytes_per_launch": ab}
    prof = PROFILED_TRAFFIC.get((args.workload, top, tuple(size), args.dtype))
    if prof:
        roofline.update(prof)
    for n, k in kernels.items():
        b = algorithmic_bytes(n, size, s, **ab_kw)
        k["achieved_gbs"] = b / (k["ms_per_launch"] / 1e3) / 1e9 if b else None

    # end to end through the C ABI with host buffers: upload the state, step, download
    e2e = None
    prognostic = ["u", "v"] + (["w"] if grid.topology[2] != "Flat" else []) + list(physics.get("tracers", ()))
    fields = prognostic if args.e2e_steps > 0 else []
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
    e2e_el = max_over_ranks(time.perf_counter() - t0, dist, "cuda")
    if fields:
        e2e = {"value": replica_value(cells, args.e2e_steps, world, e2e_el), "unit": UNIT,
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": h2d,
               "path": "gbo_set_field x%d (pinned host) + gbo_time_step(1) + gbo_get_field x%d" % (len(fields), len(fields))}

    poisson = None
    if isinstance(physics.get("pressure_solver"), og.ConjugateGradientPoissonSolver):
        poisson = held_out_solves(model, grid, torch, stream, ft, n=50)
        # the learned correction of the preconditioner, trained for this grid, on the same
        # right-hand sides (flexible CG)
        wpath = os.path.join(os.path.dirname(og.__file__), "weights", "seamount_%dx%dx%d.npy" % tuple(size))
        if os.path.exists(wpath):
            model.set_learned_preconditioner(wpath)
            try:
                learned = held_out_solves(model, grid, torch, stream, ft, n=50)
            except L.NotConvergedError as e:
                learned = {"not_converged": str(e)}
            model.set_learned_preconditioner(None)
            learned["preconditioner"] = "fft + learned correction (flexible CG), %s" % os.path.basename(wpath)
            poisson = {"fft_pcg": poisson, "learned_pcg": learned}

    # the rest of the metric on the headline run: the cuFFT yardstick of the FFT solve on this
    # grid, and the seamount grid's Poisson-solve times (FFT-PCG and learned PCG to 1e-8)
    yard = None
    if (rank == 0 and not args.timed_only and physics.get("pressure_solver") is None and grid.bottom_height is None
            and grid.z_faces is None and grid.topology[2] == "Bounded"):
        yard = cufft_yardstick(model, grid, torch, stream, ft)
    others = None
    if (rank == 0 and not args.timed_only and args.workload == "convection"
            and tuple(size) == WORKLOADS["convection"]["size"]):
        poisson = seamount_poisson_record(torch, og, L)
        # the other benchmark configurations, each timed on this GPU in the same run
        if not args.no_other_workloads:
            others = {"turbulence2d": workload_record("turbulence2d", torch, og, L, lib, steps=400),
                      "stretched_amd": workload_record("stretched_amd", torch, og, L, lib, steps=10),
                      "seamount": workload_record("seamount", torch, og, L, lib, steps=5),
                      "convection_lagrangian": workload_record("convection_lagrangian", torch, og, L, lib, steps=5),
                      "ensemble": ensemble_record(torch, og, L, lib)}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_sample(args.workload)
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": args.dtype, "data": "synthetic (seeded numpy PCG64)",
                "config": config_dict(args, world), "clocks": clk.summary(), "e2e": e2e,
                "gpu_launches": int(launches), "roofline": roofline, "cpu_baseline": cpu, "kernels": kernels}
        if poisson:
            line["poisson_solve"] = poisson
        if yard:
            line["fft_poisson_vs_cufft"] = yard
        if others:
            line["other_workloads"] = others
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
