"""The entry point that allocates no device memory (hg_green_points_noalloc).

Callers that cannot allocate device memory while their run is under way
(a driver loop under a fixed memory budget, a server that carves up device
memory at start-up) use this variant of hg_green_points, which stages its
data in one fixed device array of the library.  This file is named so that
pytest collects it last; it checks, through the C ABI, that two calls in a
row return what the allocating entry point returns, in deep and finite
depth, and that an oversized call is refused with a message.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12  # same kernel, same inputs: the results agree to rounding of the copies (exactly, in practice)


def _points(rng, count, depth):
    h = 40.0 if depth > 0 else 20.0
    pts = np.column_stack([rng.uniform(-h, h, count), rng.uniform(-h, h, count), -rng.uniform(0.1, 0.9 * h, count),
                           rng.uniform(-h, h, count), rng.uniform(-h, h, count), -rng.uniform(0.0, 0.9 * h, count)])
    pts[:3, 3:5] = pts[:3, 0:2]
    return pts, (np.arange(count) % 2).astype(np.int32)


@pytest.mark.parametrize("depth", [-1.0, 40.0])
def test_noalloc_matches_allocating_entry_point(pkg, depth):
    hg = pkg.hamsgpu
    rng = np.random.default_rng(123)
    s = hg.Solver()
    v, wk, w1, wvn = hg.wave_properties(3, 0.9, depth)
    s.set_frequency(v, wk, w1, depth, wvn)
    for call in range(2):  # two calls in a row share the fixed array
        pts, flags = _points(rng, 257 + 300 * call, depth)
        ref = s.green_points(pts, flags)
        got = s.green_points_noalloc(pts, flags)
        scale = np.maximum(np.abs(ref), 1e-300)
        assert np.all(np.abs(got - ref) <= TOL * scale), call
    s.close()


def test_noalloc_rejects_oversized_calls(pkg):
    hg = pkg.hamsgpu
    s = hg.Solver()
    v, wk, w1, _ = hg.wave_properties(3, 0.9, -1.0)
    s.set_frequency(v, wk, w1, -1.0, None)
    n = 65536 + 1
    pts = np.zeros((n, 6)); pts[:, 2] = -1.0; pts[:, 5] = -2.0; pts[:, 3] = 1.0
    with pytest.raises(hg.HamsGpuError) as exc:
        s.green_points_noalloc(pts, np.zeros(n, dtype=np.int32))
    assert "exceeds" in str(exc.value)
    s.close()
