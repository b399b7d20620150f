"""CPU checks of the flow oracle: analytic gradients against finite differences,
sampling against the density direction, and the parameter layout of the C ABI."""
import numpy as np
import pytest

from oracle import flow_ref as F


@pytest.mark.parametrize("kind", [0, 1])
def test_oracle_gradient_vs_finite_differences(kind):
    rng = np.random.default_rng(3)
    D, L, H, K = 8, 6, 16, 16
    th = F.init_params(D, L, H, K, seed=2) + rng.normal(0, 0.3, F.n_params(D, L, H, K))
    x = rng.random((48, D))
    coef = rng.random(48) + 0.5
    _, g, _ = F.loss_and_grad(x, coef, th, kind, D, L, H, K, bf=False)
    idx = rng.choice(len(th), 120, replace=False)
    eps = 1e-6
    fd = []
    for i in idx:
        tp, tm = th.copy(), th.copy()
        tp[i] += eps
        tm[i] -= eps
        fd.append((F.loss_and_grad(x, coef, tp, kind, D, L, H, K, bf=False)[0] -
                   F.loss_and_grad(x, coef, tm, kind, D, L, H, K, bf=False)[0]) / (2 * eps))
    fd = np.array(fd)
    assert np.abs(fd - g[idx]).max() <= 1e-6 * np.abs(g[idx]).max()


def test_oracle_sample_inverts_density():
    rng = np.random.default_rng(4)
    D, L, H, K = 8, 6, 32, 16
    th = F.init_params(D, L, H, K, seed=5) + rng.normal(0, 0.2, F.n_params(D, L, H, K))
    z = rng.random((500, D))
    x, lq = F.sample(z, th, D, L, H, K, bf=False)
    assert x.min() >= 0 and x.max() <= 1
    lq2, z2 = F.log_density(x, th, D, L, H, K, bf=False)
    assert np.max(np.abs(z2 - z)) < 1e-10
    assert np.max(np.abs(lq2 - lq)) < 1e-10


def test_oracle_identity_at_initialisation():
    """Zero last-layer weights and the derivative bias give the identity map."""
    th = F.init_params(8, 6, 128, 16, seed=1)
    x = np.random.default_rng(1).random((64, 8))
    lq, z = F.log_density(x, th, bf=True)
    assert np.max(np.abs(z - x)) < 1e-12
    assert np.max(np.abs(lq)) < 1e-12


def test_density_normalised_by_quadrature():
    """q integrates to 1: Monte Carlo over uniform x, 1-sigma-scaled bound."""
    rng = np.random.default_rng(6)
    th = F.init_params(8, 6, 16, 16, seed=3) + rng.normal(0, 0.2, F.n_params(8, 6, 16, 16))
    x = rng.random((20000, 8))
    lq, _ = F.log_density(x, th, 8, 6, 16, 16, bf=False)
    q = np.exp(lq)
    assert abs(q.mean() - 1) < 5 * q.std() / np.sqrt(len(q))


def test_bf16_rounding_is_round_to_nearest_even():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.0e-3])
    r = F.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -7 and r[3] == -2.5
    assert abs(r[4] - 3.0e-3) < 3.0e-3 * 2 ** -8
