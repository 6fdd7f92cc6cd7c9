"""In-tree build of libgb300ocean.so for sm_103a (nvcc, one -gencode)."""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(HERE)
CSRC = os.path.join(PKG_ROOT, "csrc")
BUILD = os.path.join(PKG_ROOT, "_build")
LIB = os.path.join(BUILD, "libgb300ocean.so")
SOURCES = ["gbo_model.cu", "gbo_fused_f32_tracer.cu", "gbo_fused_f32_momentum.cu", "gbo_fused_f64_tracer.cu",
           "gbo_fused_f64_momentum.cu", "gbo_fft.cu", "gbo_static_poisson.cu", "gbo_learned.cu", "gbo_dynamic_f32.cu",
           "gbo_dynamic_f64.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# extra nvcc options, e.g. GBO_NVCC_EXTRA="-DGBO_FUSED_MIN_BLOCKS=4" for a tuning build
EXTRA = os.environ.get("GBO_NVCC_EXTRA", "").split()


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(PKG_ROOT, "..", "include", "gbo.h")]
    if not force and not _stale(LIB, deps):
        return LIB
    nvcc = os.environ.get("NVCC", "nvcc")
    objs = []
    procs = []
    for src in SOURCES:
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", *EXTRA, "-c",
               os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd))
        procs.append((subprocess.Popen(cmd), cmd))
        objs.append(obj)
    for p, cmd in procs:
        if p.wait() != 0:
            raise RuntimeError("nvcc failed: %s" % " ".join(cmd))
    cmd = [nvcc, *ARCH, "-shared", "-o", LIB + ".tmp", *objs]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
