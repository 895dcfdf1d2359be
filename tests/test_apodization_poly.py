"""The DAS apodization polynomials of csrc/bf_das_hercules.cuh, read from the
source and evaluated in float32 Horner form as the kernel does, against
cos^2(sqrt(w)) on [0, (pi/2)^2] (das.glsl's cos^2 of the clamped aperture
argument): degree 5 within 6.4e-7 (FP32 path), degree 3 within 9.6e-4 and below
1.2e-7 at the aperture edge (DAS precision 1)."""
import os
import re

import numpy as np

from conftest import ROOT

SRC = os.path.join(ROOT, "ogl_beamforming_cuda_gb300", "csrc", "bf_das_hercules.cuh")


def coefficients(name):
    text = open(SRC).read()
    body = text[text.index(f"float {name}(float w)"):]
    body = body[:body.index("}")]
    return [np.float32(v) for v in re.findall(r"(-?\d+\.\d+(?:e[-+]?\d+)?)f", body)]


def horner(cs, w):
    c = np.float32(cs[0])
    for k in cs[1:]:
        c = np.float32(np.float32(c * w) + k)       # fmaf: one rounding; the bound has margin for two
    return c


def check(name, bound, edge=None):
    cs = coefficients(name)
    assert cs[-1] == np.float32(1.0)
    w = np.linspace(0.0, (np.pi / 2) ** 2, 200001).astype(np.float32)
    got = horner(cs, w).astype(np.float64)
    err = np.abs(got - np.cos(np.sqrt(w.astype(np.float64))) ** 2)
    assert err.max() <= bound, (name, err.max())
    if edge is not None:
        assert abs(float(horner(cs, np.float32((np.pi / 2) ** 2)))) <= edge
    return err.max()


def test_degree5_fp32_path():
    assert len(coefficients("apod_cos2_p5")) == 6
    check("apod_cos2_p5", 7e-7)


def test_degree3_precision_path():
    assert len(coefficients("apod_cos2_p3")) == 4
    check("apod_cos2_p3", 1e-3, edge=5e-7)
