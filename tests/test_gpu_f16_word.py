"""The FP16 storage word (SE_GPU_STORAGE_F16): a tsdf round trip through a map's voxels equals
the format's definition, FP16's sign and 5-bit exponent (bias 15) with an 18-bit significand,
rounded to nearest with ties to even: every value of at least 2^-14 in magnitude exactly, the
smaller ones (the format's subnormals, units of 2^-32) within one unit; the integer weight
0..255 exactly (clamped at 255)."""
import numpy as np
import pytest

from tests.test_gpu_map import _key

pytestmark = pytest.mark.gpu


def _reference(t):
    """The format's value of float32 t, in float64."""
    m = np.abs(t.astype(np.float64))
    out = np.zeros_like(m)
    big = m >= 2.0 ** -14
    e = np.floor(np.log2(np.where(big, m, 1.0)))
    ulp = 2.0 ** (e - 18)
    out[big] = np.round(m[big] / ulp[big]) * ulp[big]          # np.round: ties to even
    out[~big] = np.round(m[~big] * 2.0 ** 32) * 2.0 ** -32
    return np.copysign(out, t.astype(np.float64))


def test_f16_word_round_trip(gpu):
    rng = np.random.default_rng(7)
    n_blocks = 64
    vals = np.concatenate([
        rng.uniform(-1.0, 1.0, 8192),
        rng.uniform(-1e-3, 1e-3, 4096),
        rng.uniform(-2.0 ** -13, 2.0 ** -13, 4096),     # around the subnormal boundary
        np.array([1.0, -1.0, 0.0, -0.0, 2.0 ** -14, -2.0 ** -14, 2.0 ** -15, 2.0 ** -32, 2.0 ** -33]),
    ]).astype(np.float32)
    # exact ties of the 18-bit significand: 19 significant bits with the last one set
    k = rng.integers(2 ** 18, 2 ** 19, 2048)
    ties = (k * 2 + 1).astype(np.float64) * 2.0 ** -21
    vals = np.concatenate([vals, ties.astype(np.float32), -ties.astype(np.float32)])
    vals = np.resize(vals, n_blocks * 512).astype(np.float32)
    weights = np.resize(np.arange(0, 300, dtype=np.float32), n_blocks * 512)
    m = gpu.Map(10.24, 0.02, storage="f16", max_blocks=4096)
    keys = np.array([_key(8 * (i % 8), 8 * (i // 8), 0) for i in range(n_blocks)], np.uint64)
    m.upload_blocks(keys, vals.reshape(n_blocks, 512), weights.reshape(n_blocks, 512))
    gk, _, gt, gw, _ = m.download_blocks()
    order = np.argsort(gk)
    ref_order = np.argsort(keys)
    got_t = gt[order].reshape(-1).astype(np.float64)
    got_w = gw[order].reshape(-1)
    want_t = _reference(vals.reshape(n_blocks, 512)[ref_order].reshape(-1))
    want_w = np.minimum(weights.reshape(n_blocks, 512)[ref_order].reshape(-1), 255.0)
    big = np.abs(vals.reshape(n_blocks, 512)[ref_order].reshape(-1)) >= 2.0 ** -14
    assert np.array_equal(got_t[big], want_t[big])
    assert np.max(np.abs(got_t[~big] - want_t[~big])) <= 2.0 ** -32
    assert np.array_equal(got_w, want_w)
