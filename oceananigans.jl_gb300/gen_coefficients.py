"""Generate the reconstruction constants used by the CUDA kernels (and the CPU oracle).

The coefficients are the uniform-grid finite-volume reconstruction weights of
Shu (1998, "Essentially non-oscillatory and weighted essentially non-oscillatory
schemes for hyperbolic conservation laws", eq. 2.21), evaluated exactly with
rational arithmetic and rounded to the working precision.  Following
Oceananigans' ``stencil_coefficients`` (src/Advection/reconstruction_coefficients.jl:58-77)
the last coefficient of every stencil is *not* rounded independently but set to
``1 - sum(others)`` evaluated in the working precision, so that the weights sum
to one exactly in that precision.  That rule shifts the last weight by an ulp or
two and is reproduced here bit for bit.

Run ``python gen_coefficients.py`` to rewrite ``csrc/gbo_coeffs.h``; the test
suite checks that the committed header matches this script.
"""
from fractions import Fraction
import os
import numpy as np


def shu_coefficients(k, r):
    """Exact weights c_{r,j}, j=0..k-1, reconstructing at x_{i+1/2} from cells i-r..i-r+k-1."""
    out = []
    for j in range(k):
        c = Fraction(0)
        for m in range(j + 1, k + 1):
            num = Fraction(0)
            for l in range(k + 1):
                if l == m:
                    continue
                prod = Fraction(1)
                for q in range(k + 1):
                    if q == m or q == l:
                        continue
                    prod *= (r - q + 1)
                num += prod
            den = Fraction(1)
            for l in range(k + 1):
                if l == m:
                    continue
                den *= (m - l)
            c += num / den
        out.append(c)
    return out


def round_to(frac, dtype):
    """Correctly rounded conversion of an exact rational to float32/float64."""
    if dtype == np.float64:
        return np.float64(float(frac))
    x = np.float32(float(frac))
    best, err = x, abs(Fraction(float(x)) - frac)
    for cand in (np.nextafter(x, np.float32(np.inf)), np.nextafter(x, np.float32(-np.inf))):
        e = abs(Fraction(float(cand)) - frac)
        if e < err:
            best, err = cand, e
    return best


def weights(k, r, dtype):
    """Weights in ascending cell order with the last set to 1 - (left-to-right sum of the others)."""
    exact = shu_coefficients(k, r)
    head = [round_to(c, dtype) for c in exact[:-1]]
    s = dtype(0) if len(head) == 0 else head[0]
    for h in head[1:]:
        s = dtype(s + h)
    last = dtype(dtype(1) - s)
    return head + [last]


def uniform_reconstruction_coefficients(dtype, shift, buffer):
    """Restatement of Oceananigans' uniform_reconstruction_coefficients (reconstruction_coefficients.jl:100-102)."""
    if shift == "symmetric":
        return tuple(weights(2 * buffer, buffer - 1, dtype))
    if buffer == 1:
        return (dtype(1),)
    if shift == "left":
        return tuple(weights(2 * buffer - 1, buffer - 2, dtype))
    return tuple(weights(2 * buffer - 1, buffer - 1, dtype))


def symmetric_stencil(dtype, buffer):
    """Weights of Centered(order=2*buffer) keyed by offset -buffer..buffer-1 (calc_reconstruction_stencil, :symmetric)."""
    coeff = uniform_reconstruction_coefficients(dtype, "symmetric", buffer)
    order = 2 * buffer
    return [coeff[order - idx - 1] for idx in range(order)]  # idx 0 <-> offset -buffer


def weno_coeff_p(buffer, dtype):
    """coeff_p(WENO{buffer}, stencil s) for s=0..buffer-1 (weno_interpolants.jl:101-110)."""
    return [weights(buffer, s, dtype) for s in range(buffer)]


C_STAR = {2: [Fraction(2, 3), Fraction(1, 3)],
          3: [Fraction(3, 10), Fraction(3, 5), Fraction(1, 10)]}
SMOOTHNESS = {2: [[1, -2, 1], [1, -2, 1]],
              3: [[10, -31, 11, 25, -19, 4], [4, -13, 5, 13, -13, 4], [4, -19, 11, 25, -31, 10]]}


def fmt(x, dtype):
    if dtype == np.float32:
        return "%.9ef" % float(x)
    return "%.17e" % float(x)


def header_text():
    lines = []
    w = lines.append
    w("// Generated by gen_coefficients.py -- do not edit by hand.")
    w("// Uniform finite-volume reconstruction weights (Shu 1998, eq. 2.21) rounded to the")
    w("// working precision with the last weight of each stencil = 1 - sum(others) in that")
    w("// precision, as Oceananigans' stencil_coefficients does")
    w("// (src/Advection/reconstruction_coefficients.jl:58-77).")
    w("#pragma once")
    w("")
    w("template <typename FT> struct GboCoeffs;")
    for dtype, name in ((np.float64, "double"), (np.float32, "float")):
        w("")
        w("template <> struct GboCoeffs<%s> {" % name)
        for buf in (3, 2):
            cp = weno_coeff_p(buf, dtype)
            for s in range(buf):
                vals = ", ".join(fmt(v, dtype) for v in cp[s])
                w("  // WENO{%d} (order %d) stencil %d" % (buf, 2 * buf - 1, s))
                w("  static constexpr %s weno%d_p%d[%d] = {%s};" % (name, buf, s, buf, vals))
            cs = ", ".join(fmt(round_to(c, dtype), dtype) for c in C_STAR[buf])
            w("  static constexpr %s weno%d_cstar[%d] = {%s};" % (name, buf, buf, cs))
        sym4 = symmetric_stencil(dtype, 2)
        w("  // Centered(order=4) weights for offsets -2, -1, 0, +1 relative to the face")
        w("  static constexpr %s c4[4] = {%s};" % (name, ", ".join(fmt(v, dtype) for v in sym4)))
        sym2 = symmetric_stencil(dtype, 1)
        w("  // Centered(order=2) weights for offsets -1, 0")
        w("  static constexpr %s c2[2] = {%s};" % (name, ", ".join(fmt(v, dtype) for v in sym2)))
        # epsilon is the Float32 literal 1f-8 promoted to the working precision
        eps32 = np.float32(1e-8)
        w("  // WENO regulariser: the single-precision literal 1e-8 promoted (weno_interpolants.jl:71)")
        w("  static constexpr %s eps = %s;" % (name, fmt(dtype(eps32), dtype)))
        for k, (g, z) in enumerate(((Fraction(8, 15), None), (Fraction(5, 12), Fraction(-17, 60)),
                                    (Fraction(3, 4), Fraction(-5, 12)))):
            w("  static constexpr %s rk3_gamma%d = %s;" % (name, k + 1, fmt(round_to(g, dtype), dtype)))
            zz = fmt(round_to(z, dtype), dtype) if z is not None else fmt(0.0, dtype)
            w("  static constexpr %s rk3_zeta%d = %s;" % (name, k + 1, zz))
        w("};")
    w("")
    w("// Smoothness-indicator coefficients (weno_interpolants.jl:169-174), exact integers")
    for buf in (3, 2):
        for s in range(buf):
            vals = ", ".join(str(v) for v in SMOOTHNESS[buf][s])
            w("#define GBO_WENO%d_BETA%d {%s}" % (buf, s, vals))
    w("")
    return "\n".join(lines)


if __name__ == "__main__":
    here = os.path.dirname(os.path.abspath(__file__))
    path = os.path.join(here, "csrc", "gbo_coeffs.h")
    with open(path, "w") as f:
        f.write(header_text())
    print("wrote", path)
