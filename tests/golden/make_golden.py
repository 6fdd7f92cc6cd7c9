"""Extract known-answer values from the reference's docstrings into reference_doctests.json.

Run in the build container (it reads the reference source tree, which is not
available on the GPU machine); the JSON it writes is committed.  Sources:
  src/Advection/reconstruction_coefficients.jl   (calc_reconstruction_stencil jldoctest,
                                                  uniform_reconstruction_coefficients examples)
  src/Solvers/index_permutations.jl              (permute_index / unpermute_index sequences)
  src/TimeSteppers/runge_kutta_3.jl              (RK3 constants)
  src/Advection/weno_interpolants.jl             (C★ and smoothness coefficients)
"""
import json
import os
import re
import sys

if len(sys.argv) != 2:
    sys.exit("usage: python tests/golden/make_golden.py <path of the Oceananigans.jl source tree>")
REF = sys.argv[1]


def read(rel):
    with open(os.path.join(REF, rel)) as f:
        return f.read()


out = {}
rc = read("src/Advection/reconstruction_coefficients.jl")
# jldoctest of calc_reconstruction_stencil: Float32 symmetric buffer 2 and left buffer 3
m = re.search(r"calc_reconstruction_stencil\(Float32, 2, :symmetric, :x\)\n:\((.*?)\)\n", rc)
out["centered4_f32"] = [float(v.rstrip("f0").replace("f0", "")) if False else float(v.replace("f0", "e0"))
                        for v in re.findall(r"(-?[0-9.]+f0) \*", m.group(1))]
m = re.search(r"calc_reconstruction_stencil\(Float32, 3, :left, :x\)\n:\((.*?)\)\n", rc)
out["upwind5_left_f32_by_offset"] = [float(v.replace("f0", "e0")) for v in re.findall(r"(-?[0-9.]+f0) \*", m.group(1))]
m = re.search(r"calc_reconstruction_stencil\(Float64, 1, :symmetric, :y\)\n:\((.*?)\)\n", rc)
out["centered2_f64"] = [float(v) for v in re.findall(r"(-?[0-9.]+) \*", m.group(1))]

ip = read("src/Solvers/index_permutations.jl")
seqs = re.findall(r"\[1, 2, 3, 4, 5, 6, 7, 8(?:, 9)?\] -> \[([0-9, ]+)\]", ip)
out["permute_index_8"] = [int(v) for v in seqs[0].split(",")]
out["permute_index_9"] = [int(v) for v in seqs[1].split(",")]
out["unpermute_index_8"] = [int(v) for v in seqs[2].split(",")]
out["unpermute_index_9"] = [int(v) for v in seqs[3].split(",")]

rk = read("src/TimeSteppers/runge_kutta_3.jl")
out["rk3"] = {k: [int(a), int(b)] for k, a, b in re.findall(r"(γ¹|γ²|γ³|ζ²|ζ³) = (-?\d+) // (\d+)", rk)}

wi = read("src/Advection/weno_interpolants.jl")
cst = re.findall(r"C★\(::WENO\{3, \$FT\}, ::Val\{(\d)\}\) = \$\(FT\((\d+)//(\d+)\)\)", wi)
out["cstar_weno5"] = [[int(a), int(b)] for _, a, b in cst]
sm = re.findall(r"smoothness_coefficients\(::Val\{\$FT\}, ::Val\{3\}, ::Val\{(\d)\}\) = \$\(FT\.\(\(([^)]*)\)\)\)", wi)
out["smoothness_weno5"] = [[int(x) for x in body.split(",")] for _, body in sm]
out["epsilon_literal"] = re.search(r"const ϵ = (\S+)", wi).group(1)

path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_doctests.json")
with open(path, "w") as f:
    json.dump(out, f, indent=1)
print(json.dumps(out, indent=1))
