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
