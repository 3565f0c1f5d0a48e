"""Host-side quadrature weights of the device (mu, T) sweeps: the Simpson
weights of the Correlator's integral (kwant/kpm.py:627, scipy's composite
rule for irregular points with Cartwright's last-interval correction) must
reproduce scipy.integrate.simpson on the Chebyshev nodes and on random
points, for odd and even counts (CPU only)."""

import numpy as np
import pytest
from scipy.integrate import simpson


@pytest.mark.parametrize('n', [2, 3, 4, 5, 6, 33, 96, 97, 512, 4000])
def test_simpson_weights_match_scipy(n):
    from kwant_gb300.kpm import _simpson_weights, _chebyshev_nodes
    rng = np.random.default_rng(n)
    for x in (np.sort(rng.random(n)), _chebyshev_nodes(n)):
        w = _simpson_weights(x)
        for _ in range(3):
            y = rng.standard_normal(n) + 1j * rng.standard_normal(n)
            ref = simpson(y, x=x)
            assert abs(np.dot(w, y) - ref) <= 1e-13 * max(1.0, abs(ref))
