"""Generates tests/golden/primitives.json: known-answer vectors for the bit-level
primitives of the lighting back end, computed by an independent restatement in
Python/numpy of the reference's shader text:

  shader/rand.hlsl:9-46 (jenkins_hash, lcg_xorshift, lcg_uint_to_float),
  shader/rand.hlsl:82-112 (un-seeded XXHash32 variant),
  shader/restir/reservoir.hlsl:56-71 (ReservoirSimple 32-bit pack, with its quirk),
  shader/enc.inc.hlsl:18-63 (octahedral normals), gbuffer.hlsl:20-32, 79-103,
  f32tof16 (round to nearest even, numpy.float16),
  B10G11R11_UFLOAT (round to nearest even, computed with exact rationals).

The reference ships no tests or fixtures of its own (there is nothing to pin the
CPU oracle against but the shader text), so these vectors are the oracle's pin.
Run: python tests/golden/make_golden.py
"""
import json
import os
from fractions import Fraction

import numpy as np

M32 = 0xFFFFFFFF
f32 = np.float32


def jenkins_hash(x):
    x = (x + (x << 10)) & M32
    x ^= x >> 6
    x = (x + (x << 3)) & M32
    x ^= x >> 11
    x = (x + (x << 15)) & M32
    return x


def xorshift(x):
    x ^= (x << 13) & M32
    x ^= x >> 17
    x ^= (x << 5) & M32
    return x


def lcg_uint_to_float(x):
    return float(np.array([0x3F800000 | (x >> 9)], np.uint32).view(np.float32)[0] - f32(1.0))


def rotl(h, r):
    return ((h << r) | (h >> (32 - r))) & M32


def xxh_init(p):
    return (p + 374761393) & M32


def xxh_add(h, p):
    h = (h + p * 3266489917) & M32
    return (668265263 * rotl(h, 17)) & M32


def xxh_eval(h):
    h = (668265263 * rotl(h, 17)) & M32
    h = (2246822519 * (h ^ (h >> 15))) & M32
    h = (3266489917 * (h ^ (h >> 13))) & M32
    return h ^ (h >> 16)


def f2u(f):
    return int(np.array([f], np.float32).view(np.uint32)[0])


def u2f(u):
    return np.array([u], np.uint32).view(np.float32)[0]


def rsv_encode(M, W):
    return (min(M, 0xFF) | ((f2u(W) << 1) & 0xFFFFFF00)) & M32


def rsv_decode(u):
    return u & 0xFF, float(u2f((u >> 1) & 0x7FFFFFE0))


def to_ufloat(x, mb):
    """Exact RNE conversion of a binary32 value to an unsigned 5-bit-exponent float."""
    x = np.float32(x)
    if np.isnan(x) or x <= 0 or np.signbit(x):
        return 0
    maxc = (30 << mb) | ((1 << mb) - 1)
    if np.isinf(x):
        return maxc
    v = Fraction(float(x))
    best = None
    # enumerate candidate codes around the value (exponent e, mantissa m)
    for e in range(0, 31):
        for m in range(0, 1 << mb):
            val = Fraction(m, 1 << mb) * Fraction(2) ** (-14) if e == 0 else \
                (1 + Fraction(m, 1 << mb)) * Fraction(2) ** (e - 15)
            code = (e << mb) | m
            d = abs(val - v)
            if best is None or d < best[0] or (d == best[0] and (code & 1) == 0):
                best = (d, code)
    return best[1]


def normal_encode_oct(n):
    n = np.asarray(n, np.float32)
    s = f32(f32(abs(n[0]) + abs(n[1])) + abs(n[2]))
    n = np.array([n[0] / s, n[1] / s, n[2] / s], np.float32)
    if not n[2] >= 0:
        x, y = n[0], n[1]
        n = np.array([f32(f32(1) - abs(y)) * (f32(1) if x >= 0 else f32(-1)),
                      f32(f32(1) - abs(x)) * (f32(1) if y >= 0 else f32(-1)), n[2]], np.float32)
    return np.array([f32(n[0] * f32(0.5)) + f32(0.5), f32(n[1] * f32(0.5)) + f32(0.5)], np.float32)


def normal_decode_oct(f):
    f = np.asarray(f, np.float32)
    f = np.array([f32(f[0] * f32(2)) - f32(1), f32(f[1] * f32(2)) - f32(1)], np.float32)
    n = np.array([f[0], f[1], f32(f32(f32(1) - abs(f[0])) - abs(f[1]))], np.float32)
    t = f32(min(max(-n[2], f32(0)), f32(1)))
    n[0] = f32(n[0] + (-t if n[0] >= 0 else t))
    n[1] = f32(n[1] + (-t if n[1] >= 0 else t))
    d = f32(f32(f32(n[0] * n[0]) + f32(n[1] * n[1])) + f32(n[2] * n[2]))
    inv = f32(f32(1) / np.sqrt(d, dtype=np.float32))
    return np.array([n[0] * inv, n[1] * inv, n[2] * inv], np.float32)


def trunc_u(x):
    return int(np.float32(x)) if x > 0 else 0


def oct_u16(n):
    e = normal_encode_oct(n)
    return trunc_u(f32(e[0] * f32(255))) | (trunc_u(f32(e[1] * f32(255))) << 8)


def oct_u32(n):
    e = normal_encode_oct(n)
    return trunc_u(f32(e[0] * f32(65535))) | (trunc_u(f32(e[1] * f32(65535))) << 16)


def main():
    rng = np.random.default_rng(2024)
    out = {}
    xs = [0, 1, 2, 3, 0xFFFFFFFF, 0x80000000, 12345, 0xDEADBEEF] + [int(v) for v in rng.integers(0, 2**32, 56)]
    out["jenkins_hash"] = [[x, jenkins_hash(x)] for x in xs]
    out["lcg_xorshift"] = [[x, xorshift(x)] for x in xs]
    out["lcg_uint_to_float_bits"] = [[x, f2u(lcg_uint_to_float(x))] for x in xs]
    out["frame_rand_chain"] = []
    for fi in (0, 1, 2, 7, 100, 4096):
        s, chain = fi, []
        for _ in range(8):
            s = jenkins_hash(s)
            chain.append(s)
        out["frame_rand_chain"].append([fi, chain])
    out["xxh32_one"] = [[x, xxh_eval(xxh_init(x))] for x in xs]
    out["xxh32_three"] = [[x, xxh_eval(xxh_add(xxh_add(xxh_init(x), x ^ 0x9E3779B9), 7))] for x in xs]
    Ws = [0.0, 1.0, 0.5, 3.14159, 1e-3, 123.456, 7.0e4, 1e-30] + [float(v) for v in rng.uniform(0, 50, 24)]
    Ms = [0, 1, 2, 63, 64, 65, 127, 128, 191, 192, 255, 256, 300]
    enc = []
    for M in Ms:
        for W in Ws[:12]:
            u = rsv_encode(M, W)
            dm, dw = rsv_decode(u)
            enc.append([M, f2u(np.float32(W)), u, dm, f2u(np.float32(dw))])
    out["reservoir_32b"] = enc
    hv = [0.0, -0.0, 1.0, -1.0, 0.1, 65504.0, 65519.0, 65520.0, 1e6, 6.1e-5, 6.0e-5, 5.96e-8, 2.98e-8, 3.0e-8,
          1.0e-8, np.inf, -np.inf, 0.333333, 2049.0, 2051.0] + [float(v) for v in rng.normal(0, 100, 40)]
    out["f32tof16"] = [[f2u(np.float32(v)), int(np.array([v], np.float32).astype(np.float16).view(np.uint16)[0])]
                       for v in hv]
    uv = [0.0, -1.0, 1.0, 0.5, 1e-5, 6.2e-5, 3e-6, 65024.0, 65025.0, 70000.0, 1e9, 3.0e-7, 0.123456, 7.77,
          1234.5, 4.9e-7] + [float(v) for v in np.exp(rng.uniform(-12, 11, 24))]
    out["ufloat11"] = [[f2u(np.float32(v)), to_ufloat(v, 6)] for v in uv]
    out["ufloat10"] = [[f2u(np.float32(v)), to_ufloat(v, 5)] for v in uv]
    nv = [[0, 0, 1], [0, 0, -1], [1, 0, 0], [0, -1, 0], [0.3, -0.4, 0.866], [-0.5, -0.5, -0.707]]
    nv += [list(v / np.linalg.norm(v)) for v in rng.normal(size=(30, 3))]
    octs = []
    for n in nv:
        n32 = [f2u(np.float32(c)) for c in n]
        u16 = oct_u16(n)
        d16 = normal_decode_oct(np.array([(u16 & 0xFF) / np.float32(255), ((u16 >> 8) & 0xFF) / np.float32(255)],
                                         np.float32))
        octs.append([n32, u16, oct_u32(n), [f2u(c) for c in d16]])
    out["oct"] = octs
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "primitives.json")
    with open(path, "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print("wrote", path)


if __name__ == "__main__":
    main()
