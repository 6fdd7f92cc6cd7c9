"""Train and evaluate the learned correction of the CG preconditioner on the seamount
workload (256×256×128 ImmersedBoundaryGrid(GridFittedBottom), WENO5, BuoyancyTracer,
ConjugateGradientPoissonSolver(reltol=1e-8) in FP32):

    python -m oceananigans_gb300.train_preconditioner --out weights.npy

1. spin-up with the FFT-preconditioned CG, recording a pair (b = V∇²x, x = pNHS) per
   step (exact pairs of the model's own operator) and the residuals of a few
   FFT-preconditioned CG iterations on each b with their errors (learned.collect_pairs);
2. fit the U-Net on the GPU with the library's own kernels (learned.train: tcgen05
   convolutions, tensor-core weight gradients, Adam); after every epoch the flexible PCG
   with the current weights solves the right-hand sides of a few validation steps, and
   the weights with the fewest CG iterations there (the initial, nearly-zero correction
   included) are saved (numpy .npy, FP32): the training loss is not what CG needs, so
   the stopping rule measures CG itself;
3. held-out comparison: the right-hand sides of later steps solved from a zero initial
   guess with FFT-PCG and with the learned flexible PCG, timed with CUDA events on the
   model's stream.  Prints one JSON line.
"""
import argparse
import ctypes
import json
import time

import numpy as np


def seamount(size, float_type=np.float32, seed=2024):
    import oceananigans_gb300 as og
    Nx, Ny, Nz = size
    under = og.RectilinearGrid(size=size, x=(-5000.0, 5000.0), y=(-5000.0, 5000.0), z=(-2000.0, 0.0),
                               topology=("Periodic", "Periodic", "Bounded"), float_type=float_type)
    grid = og.ImmersedBoundaryGrid(under, og.GridFittedBottom(
        lambda x, y: -2000.0 + 1200.0 * np.exp(-(x * x + y * y) / (2 * 800.0 ** 2))))
    model = og.NonhydrostaticModel(grid, advection=og.WENO(), buoyancy=og.BuoyancyTracer(), tracers=("b",),
                                   pressure_solver=og.ConjugateGradientPoissonSolver(reltol=1e-8, abstol=1e-30))
    rng = np.random.default_rng(seed)
    _, _, zc = under.nodes()
    og.set_(model, u=0.1 + 1e-3 * rng.uniform(-1, 1, (Nx, Ny, Nz)), v=1e-3 * rng.uniform(-1, 1, (Nx, Ny, Nz)),
            w=1e-3 * rng.uniform(-1, 1, (Nx, Ny, Nz + 1)),
            b=1e-6 * zc[None, None, :] + 1e-9 * rng.standard_normal((Nx, Ny, Nz)))
    return model


def timed_solves(model, rhs, torch):
    """Solve every right-hand side from zero: mean ms, mean iterations, failures."""
    from . import _lib as L
    lib = L.load()
    st = ctypes.c_void_p()
    L.check(lib.gbo_model_stream(model._h, ctypes.byref(st)), model._h)
    stream = torch.cuda.ExternalStream(st.value)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    phi = torch.zeros_like(rhs[0])
    ms, its, failed = [], [], 0
    for r in rhs:
        phi.zero_()
        torch.cuda.synchronize()
        e0.record(stream)
        try:
            model.poisson_solve_device(phi.data_ptr(), r.data_ptr())
        except L.NotConvergedError:
            failed += 1
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
        its.append(model.solver_iterations)
    return {"ms_mean": float(np.mean(ms)), "iterations_mean": float(np.mean(its)), "not_converged": failed}


def main(argv=None):
    import torch
    from . import learned
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--size", type=int, nargs=3, default=(256, 256, 128))
    ap.add_argument("--dt", type=float, default=20.0)
    ap.add_argument("--pairs", type=int, default=60)
    ap.add_argument("--heldout", type=int, default=40)
    ap.add_argument("--validation", type=int, default=6, help="steps whose systems choose the epoch")
    ap.add_argument("--keep-trained", action="store_true",
                    help="choose among the trained epochs only (not the initial weights)")
    ap.add_argument("--epochs", type=int, default=6)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--cg-iterations", type=int, default=4)
    ap.add_argument("--every", type=int, default=1, help="record the pressure system of every n-th spin-up step")
    ap.add_argument("--data-float64", action="store_true",
                    help="collect the samples from an FP64 model (the plain FP64 CG); evaluate on the FP32 model")
    args = ap.parse_args(argv)
    log = lambda s: print(s, flush=True)  # noqa: E731
    model = seamount(tuple(args.size))
    data_model = seamount(tuple(args.size), np.float64) if args.data_float64 else model
    t0 = time.time()
    b, z, x, active = learned.collect_pairs(data_model, args.dt, args.pairs, every=args.every,
                                            cg_iterations=args.cg_iterations)
    log("collected %d triples (%s CG) in %.1f s" % (b.shape[0], "FP64" if args.data_float64 else "FP32", time.time() - t0))
    if args.data_float64:
        del data_model
        from .api import time_step_  # noqa: PLC0415
        time_step_(model, args.dt, args.pairs)  # the FP32 model to the same time (the same number of steps)
    vb, _, _, _ = learned.collect_pairs(model, args.dt, args.validation)
    val = [vb[i].contiguous() for i in range(vb.shape[0])]
    best = {}

    def score(label, weights):
        model.set_learned_preconditioner(weights)
        r = timed_solves(model, val, torch)
        model.set_learned_preconditioner(None)
        key = (r["not_converged"], r["iterations_mean"], r["ms_mean"])
        log("%s: validation CG iterations %.2f, %.2f ms" % (label, r["iterations_mean"], r["ms_mean"]))
        if not best or key < best["key"]:
            best.update(key=key, weights=weights, label=label)

    if not args.keep_trained:
        score("initial weights", learned.initial_weights(0))
    t0 = time.time()
    learned.train(b, z, x, active, epochs=args.epochs, lr=args.lr, log=log,
                  on_epoch=lambda ep, loss, w: score("epoch %d" % ep, w))
    log("trained on the GPU in %.1f s; kept %s" % (time.time() - t0, best["label"]))
    w = best["weights"]
    np.save(args.out, w)
    n_triples = int(b.shape[0])
    del b, z, x
    hb, _, _, _ = learned.collect_pairs(model, args.dt, args.heldout)
    rhs = [hb[i].contiguous() for i in range(hb.shape[0])]
    fft = timed_solves(model, rhs, torch)
    model.set_learned_preconditioner(w)
    lrn = timed_solves(model, rhs, torch)
    print(json.dumps({"heldout_solves": len(rhs), "reltol": 1e-8, "size": list(args.size),
                      "spinup_steps": args.pairs, "every": args.every, "training_triples": n_triples,
                      "epochs": args.epochs,
                      "data": "FP64 CG" if args.data_float64 else "FP32 CG", "trained_on": "GPU (gbo_learned_trainer)",
                      "kept": best["label"], "validation_steps": args.validation,
                      "fft_pcg": fft, "learned_pcg": lrn,
                      "time_ratio_learned_over_fft": lrn["ms_mean"] / fft["ms_mean"]}), flush=True)


if __name__ == "__main__":
    main()
