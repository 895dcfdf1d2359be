"""The FP16 interpolation table's scale rule (DAS precision 1,
csrc/bf_das_hercules.cuh half_table_shift and csrc/bf_das_hercules.cu
interp_table<..., H>): with m the largest channel-data component and k = 11 - e,
m = f 2^e, f in [1/2, 1), every rotated cubic coefficient times 2^k and every
partial sum of its Horner evaluation at f in [0, 1) stays below 17 sqrt(2) 2048
< 49300, so FP16 (largest finite 65504) never overflows."""
import numpy as np


def shift(m):
    if not (2.0 ** -100 <= m <= 2.0 ** 100):
        return 0
    e = int(np.frexp(np.float32(m))[1])          # m = f 2^e, f in [1/2, 1)
    return 11 - e


def segments(s0, s1, s2, s3):
    """The table's power-basis coefficients of the cubic Hermite segment between
    s1 and s2 (tangents (s2 - s0)/2 and (s3 - s1)/2)."""
    t1, t2, d = 0.5 * (s2 - s0), 0.5 * (s3 - s1), s2 - s1
    return s1, t1, 3 * d - 2 * t1 - t2, t1 + t2 - 2 * d


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
