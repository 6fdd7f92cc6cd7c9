"""FP32 against FP64 on the GPU for the benchmark configurations: relative L2 per
field after 1, 10, 50 and 100 steps, the floor set by FP32 initial fields (FP64 run
from the FP32-rounded initial state), and the worst of the 64 ensemble members.
Writes the JSON report to the path in PRECISION_REPORT (default precision_report.json
in the working directory).  Usage: python tests/precision_report.py
[conv] [conv_fp32init] [stretched] [seamount] [ensemble]  (all by default).
A GPU script, not a pytest module; the bars it reports are asserted by
tests/test_gpu_parity.py, test_gpu_precision.py and test_gpu_horizons.py."""
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oceananigans.jl_gb300"), os.path.join(ROOT, "tests"), os.path.join(ROOT, "oracle")]
import oceananigans_gb300 as og  # noqa: E402
import cases  # noqa: E402

out = {}


def pair(label, c32, c64, dt, steps, names=("u", "v", "w", "b")):
    t0 = time.time()
    m32, m64 = c32.start_gpu(), c64.start_gpu()
    res = {}
    done = 0
    for s in [x for x in (1, 10, 50, 100, 200, 500) if x <= steps]:
        og.time_step_(m32, dt, s - done)
        og.time_step_(m64, dt, s - done)
        done = s
        res[s] = {n: cases.rel_l2(m32.get(n), m64.get(n)) for n in names}
    out[label] = res
    print(label, "%.1f s" % (time.time() - t0), json.dumps(res[steps]), flush=True)
    return m32, m64


which = sys.argv[1:] or ["conv", "conv_fp32init", "stretched", "ensemble", "seamount"]
if "conv" in which:
    m32, m64 = pair("convection 256x256x128", cases.convection_3d((256, 256, 128), float_type=np.float32, seed=5),
                    cases.convection_3d((256, 256, 128), seed=5), 2.0, 100, ("u", "v", "w", "b", "p", "pHY", "nu"))
    print("profile b", m32.reference_profile("b")[:3], flush=True)
if "conv_fp32init" in which:
    # the floor of FP32 initial fields: FP64 run from the FP32-rounded initial state
    c64 = cases.convection_3d((256, 256, 128), seed=5)
    c64r = cases.convection_3d((256, 256, 128), seed=5)
    c64r.init = {k: v.astype(np.float32).astype(np.float64) for k, v in c64r.init.items()}
    pair("convection fp64 from fp32-rounded init", c64r, c64, 2.0, 100)
if "stretched" in which:
    pair("stretched amd 128x128x64", cases.convection_3d((128, 128, 64), closure="amd", stretched=True, float_type=np.float32),
         cases.convection_3d((128, 128, 64), closure="amd", stretched=True), 1.0, 100)
    pair("stretched amd 512x512x256", cases.convection_3d((512, 512, 256), closure="amd", stretched=True, float_type=np.float32),
         cases.convection_3d((512, 512, 256), closure="amd", stretched=True), 1.0, 100)
if "seamount" in which:
    pair("seamount 64x64x32 cg", cases.seamount((64, 64, 32), float_type=np.float32, solver="cg", reltol=1e-7, abstol=1e-30),
         cases.seamount((64, 64, 32), solver="cg", reltol=1e-12, abstol=1e-300), 20.0, 100)
if "ensemble" in which:
    import bench
    t0 = time.time()
    s32 = bench.ensemble_specs(64, np.float32)
    s64 = bench.ensemble_specs(64, np.float64)
    e32 = og.Ensemble([(g, p) for g, p, _ in s32])
    e64 = og.Ensemble([(g, p) for g, p, _ in s64])
    for e, s in ((e32, s32), (e64, s64)):
        for m, (_, _, init) in zip(e.members, s):
            og.set_(m, **init)
    e32.time_step(1.0, 100)
    e64.time_step(1.0, 100)
    errs = []
    for i, (a, b) in enumerate(zip(e32.members, e64.members)):
        errs.append({n: cases.rel_l2(a.get(n), b.get(n)) for n in ("u", "v", "w", "b")} | {"size": list(s32[i][0].size())})
    worst = {n: max(e[n] for e in errs) for n in ("u", "v", "w", "b")}
    out["ensemble"] = {"members": errs, "worst": worst}
    print("ensemble 64 members 100 steps %.1f s" % (time.time() - t0), json.dumps(worst), flush=True)
path = os.environ.get("PRECISION_REPORT", "precision_report.json")
if os.path.dirname(path):
    os.makedirs(os.path.dirname(path), exist_ok=True)
with open(path, "w") as f:
    json.dump(out, f, indent=1, default=str)
