"""Launch-shape autotuner: measures, per size class, the tiles of the spectral Poisson
passes (z DCT columns, x real-FFT lines, y FFT columns) and the levels each block of the
fused tendency kernel marches, and writes the fastest of each into the table compiled
into the library (csrc/gbo_launch_table.h):

    python -m oceananigans_gb300.autotune                 # measure and print
    python -m oceananigans_gb300.autotune --write PATH    # also write the table header
    python -m oceananigans_gb300.autotune --from-log LOG --write PATH   # table from a recorded sweep

The pass tiles change speed only (bitwise equal results) and the levels per block
change rounding only (tests/test_gpu_launch_shape.py).  Each parameter drives one kernel
group, so each is chosen independently: one parameter is swept while the others keep
their default, and each kernel group is timed with CUDA events around every launch
(gbo_kernel_timings), the best of two passes per candidate.  The size classes are those
of the benchmark workloads, including every member size of the ensemble workload.
"""
import argparse
import ctypes
import json
import os
import re

import numpy as np

# levels need not divide Nz or be a power of two: a value whose blocks fill the resident
# slots of the GPU evenly can beat its power-of-two neighbours
CANDIDATES = {"dct_columns": (4, 8, 16, 32, 64), "x_lines": (1, 2, 4, 8, 16, 32),
              "y_columns": (2, 4, 8, 16, 32), "levels": (1, 2, 4, 8, 12, 16, 19, 24, 32)}
GROUP = {"dct_columns": "k_dct_z", "x_lines": "k_rfft_x", "y_columns": "k_fft_y", "levels": "k_momentum"}

# (Nx, Ny, Nz, float type, grid): "rect" Periodic-Periodic-Bounded with the FFT solver,
# "ibg" the seamount's immersed grid with the CG solver (FFT preconditioner),
# "stretched" tanh-stretched z with the Fourier-tridiagonal solver, "flat" a 2-D grid
CLASSES = [(256, 256, 128, np.float32, "rect"), (256, 256, 128, np.float64, "rect"),
           (256, 256, 128, np.float32, "ibg"), (512, 512, 256, np.float32, "stretched"),
           (128, 128, 1, np.float64, "flat")] + \
          [(n, n, nz, np.float32, "rect") for n in (64, 96, 128) for nz in (32, 48, 64)]


def build_model(nx, ny, nz, float_type, kind, seed=0):
    import oceananigans_gb300 as og
    rng = np.random.default_rng(seed)
    if kind == "flat":
        grid = og.RectilinearGrid(size=(nx, ny), x=(0.0, 2 * np.pi), y=(0.0, 2 * np.pi),
                                  topology=("Periodic", "Periodic", "Flat"), float_type=float_type)
        m = og.NonhydrostaticModel(grid, advection=og.WENO())
        og.set_(m, u=rng.uniform(-1, 1, (nx, ny, 1)), v=rng.uniform(-1, 1, (nx, ny, 1)))
        return m, 1e-3
    kw = dict(size=(nx, ny, nz), x=(0.0, 512.0), y=(0.0, 512.0), topology=("Periodic", "Periodic", "Bounded"),
              float_type=float_type)
    solver = {}
    if kind == "stretched":
        k = np.arange(nz + 1)
        kw["z"] = np.sort(-256.0 * (1 - np.tanh(2 * (1 - k / nz)) / np.tanh(2)))
        solver = {"pressure_solver": og.FourierTridiagonalPoissonSolver()}
    else:
        kw["z"] = (-256.0, 0.0)
    grid = og.RectilinearGrid(**kw)
    if kind == "ibg":
        grid = og.ImmersedBoundaryGrid(grid, og.GridFittedBottom(
            lambda x, y: -256.0 + 150.0 * np.exp(-((x - 256.0) ** 2 + (y - 256.0) ** 2) / (2 * 80.0 ** 2))))
        solver = {"pressure_solver": og.ConjugateGradientPoissonSolver(reltol=1e-7)}
    # the seamount workload has no closure (the fused kernel's immersed instance); the others SmagorinskyLilly
    closure = {} if kind == "ibg" else {"closure": og.SmagorinskyLilly()}
    m = og.NonhydrostaticModel(grid, advection=og.WENO(), buoyancy=og.BuoyancyTracer(), tracers=("b",), **closure,
                               **solver)
    zc = np.linspace(-256.0, 0.0, nz)
    og.set_(m, u=1e-3 * rng.uniform(-1, 1, (nx, ny, nz)), v=1e-3 * rng.uniform(-1, 1, (nx, ny, nz)),
            w=1e-3 * rng.uniform(-1, 1, (nx, ny, nz + 1)), b=1e-5 * zc[None, None, :] + np.zeros((nx, ny, nz)))
    return m, 1.0


def group_times(model, dt, steps=2):
    from . import _lib as L
    lib = L.load()
    ng = lib.gbo_kernel_group_count()
    ms = (ctypes.c_double * ng)()
    L.check(lib.gbo_kernel_timings(model._h, dt, steps, ms, ng), model._h)
    return {lib.gbo_kernel_group_name(g).decode(): ms[g] for g in range(ng)}


def tune_class(nx, ny, nz, float_type, kind, log=print):
    model, dt = build_model(nx, ny, nz, float_type, kind)
    base = model.launch_shape
    group_times(model, dt, 1)  # warm-up
    best = dict(base)
    report = {}
    for param, cands in CANDIDATES.items():
        if param == "dct_columns" and kind in ("flat", "stretched"):
            continue  # no z DCT pass
        if param == "levels" and kind == "flat":
            continue
        times = {}
        for c in cands:
            try:
                model.set_launch_shape(**{**base, param: c})
            except ValueError:
                continue
            t = min(group_times(model, dt)[GROUP[param]] for _ in range(2))
            if t > 0:
                times[c] = t
        model.set_launch_shape(**base)
        if times:
            report[param] = {str(k): round(v * 1e3, 2) for k, v in times.items()}  # µs
    entry = {"size": [nx, ny, nz], "fp64": float_type == np.float64, "ibg": kind == "ibg", "kind": kind,
             "default": base, "us_per_launch": report}
    entry["tuned"] = choose(entry)
    log(json.dumps(entry))
    del model
    return entry


# a candidate replaces the default only when it is faster by more than this fraction
# (timing noise must not move the shape)
MARGIN = 0.02


def choose(entry):
    best = dict(entry["default"])
    for param, times in entry["us_per_launch"].items():
        t = {int(k): v for k, v in times.items()}
        d = best[param]
        c = min(t, key=t.get)
        if d not in t or t[c] < (1 - MARGIN) * t[d]:
            best[param] = c
    return best


TABLE_RE = re.compile(r"// BEGIN TABLE\n.*// END TABLE\n", re.S)


def table_text(entries):
    rows = ["// BEGIN TABLE\n", "static const LaunchShapeEntry kLaunchTable[] = {\n"]
    for e in entries:
        nx, ny, nz = e["size"]
        t = e["tuned"]
        rows.append("    {%d, %d, %d, %d, %d, %d, %d, %d, %d},  // %s\n" % (
            nx, ny, nz, int(e["fp64"]), int(e["ibg"]), t["dct_columns"], t["x_lines"], t["y_columns"], t["levels"],
            e["kind"]))
    rows += ["    {0, 0, 0, 0, 0, 0, 0, 0, 0},  // end\n", "};\n", "// END TABLE\n"]
    return "".join(rows)


def write_table(entries, path, template):
    with open(template) as f:
        text = f.read()
    text = TABLE_RE.sub(lambda _: table_text(entries), text)
    with open(path, "w") as f:
        f.write(text)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--write", help="write the table header (csrc/gbo_launch_table.h with the new entries) here")
    ap.add_argument("--from-log", help="take the measurements from the JSON lines of an earlier run instead")
    args = ap.parse_args(argv)
    if args.from_log:
        with open(args.from_log) as f:
            entries = [json.loads(line) for line in f if line.startswith("{")]
        for e in entries:
            e["tuned"] = choose(e)
    else:
        entries = [tune_class(*c) for c in CLASSES]
    if args.write:
        here = os.path.dirname(os.path.abspath(__file__))
        write_table(entries, args.write, os.path.join(here, "..", "csrc", "gbo_launch_table.h"))


if __name__ == "__main__":
    main()
