"""The FP16 interpolation table's scale rule (DAS precision 1), read from the
kernel source: half_table_shift in csrc/bf_das_hercules.cuh (the exponent bias
and the target exponent) and the cubic segment coefficients of interp_table in
csrc/bf_das_hercules.cu (tangents, a2 and a3 as the kernel writes them). With m
the largest channel-data component and k the shift, every rotated cubic
coefficient times 2^k and every partial sum of its Horner evaluation at
f in [0, 1) stays below 17 sqrt(2) 2048 < 49300, so FP16 (largest finite 65504)
never overflows. A change to either piece of device code that breaks the bound
fails here."""
import os
import re

import numpy as np

from conftest import ROOT

CSRC = os.path.join(ROOT, "ogl_beamforming_cuda_gb300", "csrc")


def _body(path, start, end="\n}\n"):
    text = open(os.path.join(CSRC, path)).read()
    i = text.index(start)
    return text[i:text.index(end, i)]


def shift_rule():
    """(bias, target) of `e = ((bits >> 23) & 0xff) - bias; return target - e`."""
    body = _body("bf_das_hercules.cuh", "int half_table_shift(unsigned m_bits)")
    bias = int(re.search(r"\(m_bits >> 23\) & 0xffu\)\s*-\s*(\d+);", body).group(1))
    target = int(re.search(r"return\s+(\d+)\s*-\s*e;", body).group(1))
    lo = re.search(r"m >= (0x1p-?\d+)f", body).group(1)
    hi = re.search(r"m <= (0x1p-?\d+)f", body).group(1)
    return bias, target, float.fromhex(lo), float.fromhex(hi)


def shift(m):
    bias, target, lo, hi = shift_rule()
    if not (lo <= m <= hi):
        return 0
    bits = int(np.float32(m).view(np.uint32))
    return target - (((bits >> 23) & 0xFF) - bias)


def coefficient_forms():
    """The x-component expressions of t1, t2, d, a2 and a3 in interp_table<cubic>."""
    body = _body("bf_das_hercules.cu", "interp_table(const float2", "\n}\n\n")
    t1 = re.search(r"const float t1x = ([^,]+),", body).group(1)
    t2 = re.search(r"const float t2x = ([^,]+),", body).group(1)
    d = re.search(r"const float dx = ([^,]+),", body).group(1)
    a2 = re.search(r"float2 a2 = make_float2\(([^,]+),", body).group(1)
    a3 = re.search(r"float2 a3 = make_float2\(([^,]+),", body).group(1)
    py = lambda e: re.sub(r"(\d+\.\d+)f", r"\1", e).replace(".x", "")  # noqa: E731
    return {k: py(v) for k, v in dict(t1=t1, t2=t2, d=d, a2=a2, a3=a3).items()}


def segments(s0, s1, s2, s3):
    """Power-basis coefficients of the cubic segment between s1 and s2, by the
    kernel's own expressions (applied to complex samples)."""
    f = coefficient_forms()
    env = dict(s0=s0, s1=s1, s2=s2, s3=s3)
    env["t1x"], env["t2x"], env["dx"] = eval(f["t1"], {}, env), eval(f["t2"], {}, env), eval(f["d"], {}, env)
    return s1, env["t1x"], eval(f["a2"], {}, env), eval(f["a3"], {}, env)


def test_source_forms_are_found():
    bias, target, lo, hi = shift_rule()
    assert (bias, target) == (126, 11) and lo == 2.0 ** -100 and hi == 2.0 ** 100
    s = segments(0.0, 1.0, 2.0, 3.0)          # a straight line: a0 = 1, a1 = 1, a2 = a3 = 0
    assert np.allclose(s, (1.0, 1.0, 0.0, 0.0))


def test_scale_keeps_fp16_in_range():
    rng = np.random.default_rng(5)
    for m in (1.0, 3.7e-3, 1234.5, 8.4e6, 2.0 ** 60, 2.0 ** -60):
        k = shift(m)
        n = 200000
        # components up to m, including the extremes and alternating signs
        s = rng.uniform(-m, m, (4, n)) + 1j * rng.uniform(-m, m, (4, n))
        s[:, :4] = np.array([[m, -m, m, -m]]).T * (1 + 1j)
        a = segments(*s)
        rot = np.exp(1j * rng.uniform(-np.pi, np.pi, n))
        a = [c * rot * 2.0 ** k for c in a]
        f = rng.uniform(0, 1, n)
        parts = [a[3], a[3] * f + a[2], (a[3] * f + a[2]) * f + a[1], ((a[3] * f + a[2]) * f + a[1]) * f + a[0]]
        for v in list(a) + parts:
            assert np.max(np.abs(v.real)) < 49300 and np.max(np.abs(v.imag)) < 49300, (m, k)
        # and the largest sample lands in [1024, 2048) after scaling
        assert 1024 <= m * 2.0 ** k < 2048


def test_degenerate_magnitudes_keep_scale_one():
    for m in (0.0, 1e-35, 2.0 ** 101, np.inf, np.nan):
        assert shift(m) == 0
