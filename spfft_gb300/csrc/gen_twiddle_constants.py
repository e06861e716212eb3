"""Generates twiddle_constants.hpp: cos(2*pi*m/R) and sin(2*pi*m/R) for the register DFT sizes R,
computed with mpmath at 40 significant digits and printed with 25 (more than a double holds), so
the compiler rounds each literal once to the nearest float or double.

Run from this directory:  python gen_twiddle_constants.py > twiddle_constants.hpp
"""
import mpmath as mp

mp.mp.dps = 40
SIZES = [6, 9, 10, 12, 15, 16, 18, 20, 24, 25, 27, 30, 32]

print("// Generated by gen_twiddle_constants.py -- do not edit.")
print("// cos / sin of 2*pi*m/R for the composite register DFT sizes, as compile-time constants.")
print("#pragma once")
print("")
print("namespace spfft {")
print("namespace gb300 {")
print("")
for name, fn in (("tw_cos", mp.cos), ("tw_sin", mp.sin)):
    print(f"__host__ __device__ constexpr double {name}(int r, int m) {{")
    print("  // m is reduced modulo r by the caller")
    print("  switch (r * 64 + m) {")
    for r in SIZES:
        for m in range(r):
            v = fn(2 * mp.pi * m / r)
            if abs(v) < mp.mpf(10) ** -35:
                v = mp.mpf(0)
            print(f"    case {r * 64 + m}: return {mp.nstr(v, 25, strip_zeros=False)};")
    print("    default: return 0.0;")
    print("  }")
    print("}")
    print("")
print("}  // namespace gb300")
print("}  // namespace spfft")
