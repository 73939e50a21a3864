"""The analytic pins of the CPU oracle (tests/test_oracle_pins.py) held by the CUDA
library directly: the PPM remap is the identity on coinciding grids and reproduces cell
means of a profile linear in pressure in the column interior; a resting atmosphere
stays at rest through a whole remap interval, in the FP64 and the mixed form; limiters
8 and 9 keep an advected cosine bell non-negative and below its maximum; hyperviscosity
dissipates and keeps the layer masses."""
import numpy as np
import pytest

import hxtest as H
from test_oracle_pins import _columns, _remap_case, bell_extremes, hyperviscosity_effect, resting_deviation

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("alg", [1, 2])
def test_gpu_remap_identity_and_linear_profiles(gpu_path, alg):
    rng, ps, tgt = _columns()
    v = 20.0 * rng.standard_normal(tgt.shape[:2] + (2, 4, 4))
    T = 250.0 + 30.0 * rng.standard_normal(tgt.shape)
    v1, T1, _ = _remap_case(gpu_path, alg, tgt, v, T)
    assert np.abs(v1 - v).max() <= 1e-12 * np.abs(v).max()
    assert np.abs(T1 - T).max() <= 1e-12 * np.abs(T).max()
    rng, ps, tgt = _columns(seed=6)
    k = np.arange(72)[None, :, None, None]
    src = tgt * (1.0 + 0.15 * np.sin(0.7 * k + rng.uniform(0, 6.3, (tgt.shape[0], 1, 4, 4))))
    src *= tgt.sum(axis=1, keepdims=True) / src.sum(axis=1, keepdims=True)
    hv = H.hvc()
    ptop = hv.hyai[0] * hv.ps0

    def means(dp, a, b):
        pi = ptop + np.concatenate([np.zeros_like(dp[:, :1]), np.cumsum(dp, axis=1)], axis=1)
        return a + b * 0.5 * (pi[:, :-1] + pi[:, 1:])

    v = np.zeros(src.shape[:2] + (2, 4, 4))
    v[:, :, 1] = means(src, 3.0, 2.0e-4)
    T = means(src, 200.0, 1.0e-3)
    _, T1, _ = _remap_case(gpu_path, alg, src, v, T)
    want = means(tgt, 200.0, 1.0e-3)
    assert np.abs(T1[:, 3:69] - want[:, 3:69]).max() <= 1e-12 * np.abs(want).max()


@pytest.mark.parametrize("precision", [0, 1])
def test_gpu_resting_atmosphere(gpu_path, precision):
    """The mixed form's limiter works on FP32 mixing ratios, formed once for the bounds and
    once for the values: where the two roundings differ by an ulp it redistributes, which
    moves Q by FP32 round-off (2.6e-10 on Q = 2e-3 seen); the rest is FP64 round-off."""
    d = resting_deviation(gpu_path, precision)
    assert d["v"] < 1e-9, d
    assert d["T"] < 1e-11 and d["dp"] < 1e-12 and d["ps"] < 1e-12, d
    assert d["Q"] < (1e-13 if precision == 0 else 2e-9), d


@pytest.mark.parametrize("limiter", [8, 9])
def test_gpu_limiters_keep_a_cosine_bell_bounded(gpu_path, limiter):
    lo, hi, top = bell_extremes(gpu_path, limiter)
    assert lo >= -1e-20, lo
    assert hi <= top * (1 + 1e-12), hi


def test_gpu_hyperviscosity_dissipates_and_conserves_layer_mass(gpu_path):
    h = hyperviscosity_effect(gpu_path)
    assert (h["var"][1] < h["var"][0]).all() and (h["ke"][1] < h["ke"][0]).all()
    assert h["ddp"] > 1e-9
    assert h["mass"] < 1e-14, h["mass"]
