"""preprocessor::downsample_depth (src/map/preprocessor.cpp:19-84) in the oracle against a plain
numpy statement: the median (upper middle for even counts) of the region's depths >= 1e-5, 0 and
the region's first pixel when none is valid; the map holds the chosen input pixel."""
import numpy as np
import pytest


def _np_downsample(depth, r):
    h, w = depth.shape
    out = np.zeros((h // r, w // r), np.float32)
    mp = np.zeros(out.shape, np.int64)
    for yo in range(h // r):
        for xo in range(w // r):
            vals = []
            for yr in range(r):
                for xr in range(r):
                    x, y = xo * r + xr, yo * r + yr
                    if depth[y, x] >= np.float32(1e-5):
                        vals.append((depth[y, x], x + y * w))
            if not vals:
                mp[yo, xo] = xo * r + yo * r * w
                continue
            vals.sort(key=lambda t: t[0])  # stable: equal depths keep their scan order
            out[yo, xo], mp[yo, xo] = vals[len(vals) // 2]
    return out, mp


@pytest.mark.parametrize("ratio", [1, 2, 3, 4])
def test_downsample_matches_definition(oracle, ratio):
    rng = np.random.default_rng(ratio)
    depth = rng.uniform(0.3, 5.0, (24, 36)).astype(np.float32)
    depth[rng.random(depth.shape) < 0.3] = 0.0
    depth[:ratio, :ratio] = 0.0                      # an all-invalid region
    depth[6:6 + ratio, 6:6 + ratio] = 2.0            # ties
    depth[0, 30] = np.nan
    out, mp = oracle.downsample_depth(depth, ratio)
    want, wmp = _np_downsample(depth, ratio)
    assert np.array_equal(out, want) and np.array_equal(mp, wmp)
    assert out[0, 0] == 0.0 and mp[0, 0] == 0


def test_downsampled_sensor():
    import supereight2_gb300 as se  # host-side only: no library call
    s = se.PinholeCamera(640, 480, 525.0, 525.0, 319.5, 239.5, 0.4, 6.0).downsampled(2)
    assert (s.width, s.height) == (320, 240)
    assert s.fx == np.float32(262.5) and s.cx == np.float32(159.5) and s.cy == np.float32(119.5)
