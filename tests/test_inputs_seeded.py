"""The seeded synthetic inputs reproduce the committed fixtures
(``tests/golden/inputs_seeded.npz``, written by ``make_inputs.py``):
integer data exactly, floating data to 1e-12 relative (FFT and sine
results may differ in the last bits across CPU architectures)."""
import numpy as np

from tests.golden.make_inputs import make


def test_seeded_inputs_reproduce_fixtures(golden):
    g = golden("inputs_seeded.npz")
    now = make()
    assert set(g) == set(now)
    for k in g:
        a, b = g[k], now[k]
        assert a.shape == b.shape and a.dtype == b.dtype, k
        if np.issubdtype(a.dtype, np.integer):
            assert np.array_equal(a, b), k
        else:
            assert np.allclose(a, b, rtol=1e-12, atol=1e-15 * np.abs(a).max()), k


def test_bench_config_picks_are_the_stated_instances():
    """The instances test_gpu_bench_configs.py compares with the oracle are
    the ones its comment names: in the seed-0 batch the largest side and
    the largest kappa_max / kappa_min x N^2; in the held-out seed-1 batch
    the largest side."""
    from easier_gb300 import mesh
    from easier_gb300.numeric.batched import p1_sides
    from tests.test_gpu_bench_configs import CONFIG3_PICKS, CONFIG4_PICKS
    sides = p1_sides(256, 32, 512, seed=0)
    assert CONFIG3_PICKS[0] == int(np.argmax(sides)) and CONFIG3_PICKS[2] == int(np.argmin(sides))
    spread = []
    for i, n in enumerate(sides):
        k = mesh.kappa_from_field(mesh.gaussian_random_field(int(n), 2 * i, 0.1, 1.0))
        spread.append(float(k.max() / k.min()) * int(n) ** 2)
    assert CONFIG3_PICKS[1] == int(np.argmax(spread))
    assert CONFIG4_PICKS[0] == int(np.argmax(p1_sides(256, 32, 512, seed=1)))
