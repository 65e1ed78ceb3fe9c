"""Restatement of AMDAT's Wave_Vectors bookkeeping: TEST INFRASTRUCTURE ONLY.

Wave_Vectors(System*, plane="xyz", max_length_scale) (src/wave_vectors.cpp:77-171):
  wavegrid_spacing = float(2*pi / min_size)      (min_size = min box length,
                                                  or max_length_scale if > 0)
  delta_wavenumber = float(wavegrid_spacing / 2)
  approx_wavenumber[m] = spacing + delta * m     (FP32), m = 0..98
  shell m = the vectors of file qvector.(m+2), each n * spacing in FP32.
show_mean_wavenumber / show_stdev_wavenumber / show_mean_wavevector
(src/wave_vectors.cpp:527-566) are restated with the same FP32 arithmetic.
"""
from __future__ import annotations

import math

import numpy as np

PI = 3.14159265358979323846  # src/wave_vectors.cpp:16


def f32(x):
    return np.float32(x)


def spacing(min_size: float) -> np.float32:
    return f32(2.0 * PI / float(f32(min_size)))


def approx_wavenumbers(sp: np.float32, n: int = 99):
    delta = f32(float(sp) / 2.0)
    return [f32(sp + f32(delta * f32(m))) for m in range(n)]


def shell_vectors(n_int: np.ndarray, sp: np.float32) -> np.ndarray:
    return (n_int.astype(np.float32) * sp).astype(np.float32)


def _length(v):
    x, y, z = (f32(c) for c in v)
    return f32(np.sqrt(f32(f32(f32(x * x) + f32(y * y)) + f32(z * z))))


def mean_wavenumber(vecs: np.ndarray) -> np.float32:
    m = f32(0)
    for v in vecs:
        m = f32(m + _length(v))
    return f32(m / f32(len(vecs)))


def stdev_wavenumber(vecs: np.ndarray) -> np.float32:
    mean = mean_wavenumber(vecs)
    var = f32(0)
    for v in vecs:
        var = f32(float(var) + math.pow(float(f32(_length(v) - mean)), 2.0))
    var = f32(var / f32(len(vecs)))
    return f32(math.pow(float(var), 0.5))


def mean_wavevector(vecs: np.ndarray):
    s = [f32(0), f32(0), f32(0)]
    for v in vecs:
        for c in range(3):
            s[c] = f32(s[c] + f32(v[c]))
    n = f32(len(vecs))
    return [f32(c / n) for c in s]
