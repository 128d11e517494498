"""The bilateral pre-filter of the tracking input (project-defined: the reference has no
bilateral filter; the tracked TSDF benchmark configuration asks for one: 5x5, sigma_space 4 px,
sigma_range 0.03 m, invalid pixels ignored). The oracle is checked against a float64 numpy
statement of the same definition, and its float exponential against numpy's."""
import numpy as np
import pytest


def _np_bilateral(depth, radius=2, ss=4.0, sr=0.03):
    d = depth.astype(np.float64)
    h, w = d.shape
    out = np.zeros_like(d)
    for y in range(h):
        for x in range(w):
            c = d[y, x]
            if not c > 0:
                continue
            num = den = 0.0
            for dy in range(-radius, radius + 1):
                for dx in range(-radius, radius + 1):
                    yy, xx = y + dy, x + dx
                    if 0 <= yy < h and 0 <= xx < w and d[yy, xx] > 0:
                        wgt = np.exp(-(dx * dx + dy * dy) / (2 * ss * ss)) * np.exp(-(d[yy, xx] - c) ** 2 / (2 * sr * sr))
                        num += wgt * d[yy, xx]
                        den += wgt
            out[y, x] = num / den
    return out


def test_exp_cw_accuracy(oracle):
    xs = np.concatenate([-np.logspace(-8, np.log10(87.0), 2000), [0.0, -0.5, -1.0, -86.9, -87.5, -100.0]])
    for x in xs:
        got = float(oracle.exp_cw(np.float32(x)))
        want = float(np.exp(np.float64(np.float32(x))))
        if x < -87.0:
            assert got == 0.0
        else:
            assert abs(got - want) <= 2e-7 * want


def test_filter_matches_float64_definition(oracle):
    rng = np.random.default_rng(5)
    depth = (1.0 + 0.01 * rng.standard_normal((24, 31))).astype(np.float32)
    depth[:, 15:] += 0.5                       # an edge the range weight must keep
    depth[rng.random(depth.shape) < 0.1] = 0   # holes
    depth[3, 4] = np.nan
    got = oracle.bilateral_filter(depth)
    want = _np_bilateral(np.nan_to_num(depth, nan=0.0))
    assert np.all(got[~(depth > 0)] == 0)
    ok = depth > 0
    assert np.max(np.abs(got[ok] - want[ok]) / want[ok]) < 1e-6
    # edge preserving: the two sides do not mix
    assert np.all(np.abs(got[:, 13][ok[:, 13]] - 1.0) < 0.05)
    assert np.all(np.abs(got[:, 16][ok[:, 16]] - 1.5) < 0.05)


def test_constant_image_is_kept(oracle):
    depth = np.full((12, 17), 2.5, np.float32)
    assert np.allclose(oracle.bilateral_filter(depth), 2.5, rtol=1e-6, atol=0)


def test_noise_is_reduced(oracle):
    from supereight2_gb300 import synthetic as syn
    spec, scene, poses, frames = syn.dataset("tsdf320", 1)
    clean = syn.render_depth(scene, spec, poses[0], 0, noise=False)
    noisy = frames[0]
    filt = oracle.bilateral_filter(noisy)
    m = (noisy > 0) & (clean > 0) & (filt > 0)
    assert np.mean(np.abs(filt[m] - clean[m])) < 0.8 * np.mean(np.abs(noisy[m] - clean[m]))
