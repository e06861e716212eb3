"""Generates twiddle_constants.hpp: cos(2*pi*m/R) and sin(2*pi*m/R) for the register DFT sizes R,
computed with mpmath at 40 significant digits and printed with 25 (more than a double holds), so
the compiler rounds each literal once to the nearest float or double. For double-float arithmetic
the same constants are also emitted as float pairs (hi = nearest float, lo = nearest float of the
remainder), so no binary64 arithmetic is needed to form them on the device.

Run from this directory:  python gen_twiddle_constants.py > twiddle_constants.hpp
"""
import struct

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
def f32(x):
    return struct.unpack("f", struct.pack("f", float(x)))[0]


def split(v):
    hi = f32(v)
    rem = v - mp.mpf(hi)
    lo = 0.0 if abs(rem) < mp.mpf(10) ** -30 else f32(rem)  # exact constants (0, 1/2, 1) have no tail
    return hi, lo


for name, fn in (("tw_cos_pair", mp.cos), ("tw_sin_pair", mp.sin)):
    for part in (0, 1):
        fname = f"{name}_{'hi' if part == 0 else 'lo'}"
        print(f"__host__ __device__ constexpr float {fname}(int r, int m) {{")
        print("  switch (r * 64 + m) {")
        for r in SIZES:
            for m in range(r):
                v = fn(2 * mp.pi * m / r)
                if abs(v) < mp.mpf(10) ** -35:
                    v = mp.mpf(0)
                val = split(v)[part]
                print(f"    case {r * 64 + m}: return {float.hex(val)}f;" if val != 0 else f"    case {r * 64 + m}: return 0.0f;")
        print("    default: return 0.0f;")
        print("  }")
        print("}")
        print("")
print("}  // namespace gb300")
print("}  // namespace spfft")
