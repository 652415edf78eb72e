"""CPU: the h-network reference's analytic gradient against finite
differences (FP64)."""
import numpy as np

from oracle import hnet_ref


def test_hnet_reference_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    w = rng.normal(0, 0.3, hnet_ref.NP)
    x = rng.normal(0, 1, (64, 3))
    y = rng.normal(0, 1, 64)
    _, g = hnet_ref.loss_grad(w, x, y)
    gf = hnet_ref.fd_grad(w, x, y)
    np.testing.assert_allclose(g, gf, rtol=1e-6, atol=1e-9)


def test_hnet_reference_shapes():
    assert hnet_ref.NP == 32 * 3 + 32 + 32 * 32 + 32 + 32 + 1
    w = np.zeros(hnet_ref.NP)
    assert np.all(hnet_ref.forward(w, np.ones((5, 3))) == 0)
