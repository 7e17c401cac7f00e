"""Numerics of the generated 3D table entries (csrc/cui_gen.cuh), restated in numpy.

The device generator forms exp(-j k~ D) / D in FP32 with two steps in FP32 pairs:
the squared distance as a pair sum of squares given in FP64, refined by one
Newton step, and the phase kr*D with its product error kept by an FMA and the
reduction modulo 2 pi done in two parts (Cody and Waite).  This test repeats
those operations on float32 arrays -- an FMA as the float32 rounding of the
exact float64 product plus the addend -- over random entries of the 3d
workload's geometry (128^3 grid at 0.1 mm from 5 mm depth, 32 x 32 array at
0.3 mm, 2.5-5.5 MHz, absorbing medium) and bounds, against FP64:

- the reduced phase: 3e-7 rad (its own FP32 rounding);
- the entry, with exact sine and cosine: 6e-7 relative (the reciprocal square root's error included).

The GPU tests compare the device entries, through the operator, against the
stored FP64-built table (2e-6) and the FP64 oracle (1e-5).
"""

import numpy as np

F32 = np.float32
TWO_PI = 6.283185307179586476925
HI = F32(TWO_PI)
LO = F32(TWO_PI - np.float64(HI))
INV = F32(1.0 / TWO_PI)


def _fma(a, b, c):
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(F32)


def _split(v):
    hi = v.astype(F32)
    return hi, (v - hi.astype(np.float64)).astype(F32)


def _pair_add(ah, al, bh, bl):
    s = ah + bh
    bb = s - ah
    e = ((ah - (s - bb)) + (bh - bb)) + (al + bl)
    hi = s + e
    return hi, e - (hi - s)


def test_generator_phase_and_entry_accuracy():
    rng = np.random.default_rng(0)
    n = 200_000
    dx, nox = 1e-4, 128 + 31 * 3
    ox = rng.integers(0, nox, n)
    oy = rng.integers(0, nox, n)
    z = rng.integers(0, 128, n)
    X = (ox - 0.5 * (nox - 1)) * dx
    Y = (oy - 0.5 * (nox - 1)) * dx
    Z = 5e-3 + (z + 0.5) * dx
    kr = 2 * np.pi * rng.uniform(2.5e6, 5.5e6, n) / 1500.0
    ki = -rng.uniform(0.0, 40.0, n)
    D = np.sqrt(X * X + Y * Y + Z * Z)
    ref = np.exp(-1j * (kr + 1j * ki) * D) / D

    xh, xl = _split(X * X)
    yh, yl = _split(Y * Y)
    zh, zl = _split(Z * Z)
    yzh, yzl = _pair_add(yh, yl, zh, zl)
    d2h, d2l = _pair_add(xh, xl, yzh, yzl)
    # the device takes d = d2 * rsqrt(d2) with the hardware's approximate reciprocal square root:
    # modelled as the exact one off by up to 2e-7 relative (the Newton step removes it from D; 1/D keeps it)
    inv = ((1.0 / np.sqrt(d2h.astype(np.float64))) * (1.0 + rng.uniform(-2e-7, 2e-7, n))).astype(F32)
    d = d2h * inv
    dl = F32(0.5) * (_fma(-d, d, d2h) + d2l) * inv
    krh, krl = _split(kr)
    p = krh * d
    pe = _fma(krh, d, -p)
    small = _fma(krh, dl, _fma(krl, d, pe))
    nrev = np.rint(p * INV).astype(F32)
    ph = _fma(-nrev, np.full(n, LO, F32), _fma(-nrev, np.full(n, HI, F32), p)) + small

    exact = kr * D - nrev.astype(np.float64) * TWO_PI
    assert np.max(np.abs(ph.astype(np.float64) - exact)) <= 3e-7
    m = np.exp(ki.astype(F32).astype(np.float64) * (d + dl).astype(np.float64)) * inv.astype(np.float64)
    val = m * (np.cos(ph.astype(np.float64)) - 1j * np.sin(ph.astype(np.float64)))
    rel = np.abs(val - ref) / np.abs(ref)
    assert np.max(rel) <= 6e-7
