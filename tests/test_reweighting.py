"""The reweighting estimator of the uptake sensitivity (CPU): for snapshot
energies linear in a parameter, the derivative of the reweighted mean guest
count at theta = 0 equals -beta (<N g> - <N><g>)."""
import numpy as np

from fastmc_gb300.adjoint import uptake_sensitivity


def test_uptake_sensitivity_matches_reweighting():
    rng = np.random.default_rng(4)
    n = rng.integers(0, 50, size=4000).astype(float)
    g = rng.normal(size=(4000, 3)) + 0.02 * n[:, None]
    beta = 1.0 / (1.9872041e-3 * 293.0)

    def mean_n(theta):
        w = np.exp(-beta * (g @ theta))
        return (n * w).sum() / w.sum()

    est = uptake_sensitivity(n, g, beta)
    h = 1e-6
    for k in range(3):
        d = np.zeros(3)
        d[k] = h
        fd = (mean_n(d) - mean_n(-d)) / (2 * h)
        assert abs(fd - est[k]) <= 1e-6 * max(abs(est[k]), 1.0)
