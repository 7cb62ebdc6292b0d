"""CPU check of the polynomial sin/cos the FP32 direct kernel evaluates on the FP32 pipe
for some q-vector pairs (sincos2_poly in sassena_gb300/csrc/phase_sum.cu): Taylor series
of sin and cos of the half angle h = pi f (through h^11 and h^12) and the double-angle
formulas (sin 2h = 2 sin h cos h, cos 2h = cos^2 h - sin^2 h), evaluated here in float32
with the kernel's operation order, against float64
sin/cos over the whole reduced range f in [-1/2, 1/2] revolutions."""
import numpy as np


def poly_sincos_f32(f):
    f = np.asarray(f, np.float32)
    c = lambda v: np.float32(v)  # noqa: E731
    h = f * c(np.pi)
    h2 = h * h
    ps = c(-1 / 39916800) * h2 + c(1 / 362880)
    for k in (-1 / 5040, 1 / 120, -1 / 6, 1.0):
        ps = ps * h2 + c(k)
    sh = ps * h
    pc = c(1 / 479001600) * h2 + c(-1 / 3628800)
    for k in (1 / 40320, -1 / 720, 1 / 24, -0.5, 1.0):
        pc = pc * h2 + c(k)
    ch = pc
    return np.float32(2) * (sh * ch), ch * ch + (sh * c(-1)) * sh


def test_poly_sincos_accuracy():
    f = np.linspace(-0.5, 0.5, 200001, dtype=np.float64).astype(np.float32)
    s, co = poly_sincos_f32(f)
    x = 2 * np.pi * f.astype(np.float64)
    es = np.abs(s.astype(np.float64) - np.sin(x)).max()
    ec = np.abs(co.astype(np.float64) - np.cos(x)).max()
    # float32 rounding of the half angle dominates; below the SFU approximation's 2^-21
    assert es < 2.0 ** -21 and ec < 2.0 ** -21, (es, ec)
    # exact values at the quarter turns
    s4, c4 = poly_sincos_f32(np.array([0.0, 0.25, -0.25, 0.5], np.float32))
    assert abs(s4[0]) == 0 and abs(c4[0] - 1) < 1e-7
    assert abs(s4[1] - 1) < 3e-7 and abs(c4[1]) < 3e-7
    assert abs(c4[3] + 1) < 3e-7
