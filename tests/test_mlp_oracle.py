"""CPU checks of the network's host restatement (oracle/mlp_oracle.py): its analytic gradient
against central finite differences, and its BF16 rounding."""
import numpy as np

from oracle import mlp_oracle as mo


def _problem(seed=0, n=64):
    rng = np.random.default_rng(seed)
    params = np.concatenate([
        rng.normal(0, 1 / np.sqrt(8), 64 * 8), rng.normal(0, 0.1, 64),
        rng.normal(0, 1 / np.sqrt(64), 64 * 64), rng.normal(0, 0.1, 64),
        rng.normal(0, 1 / np.sqrt(64), 64 * 64), rng.normal(0, 0.1, 64),
        rng.normal(0, 1 / np.sqrt(64), 64), rng.normal(0, 0.1, 1)])
    norm = np.concatenate([rng.normal(0, 1, 8), rng.uniform(0.5, 2, 8), [1.7, 1.0]])
    feat = rng.normal(0, 1.5, (n, 8))
    target = rng.normal(0, 1, n)
    return params, norm, feat, target


def test_param_count():
    assert mo.N_PARAMS == 8961 and mo.N_NORM == 18


def test_gradient_matches_finite_differences():
    params, norm, feat, target = _problem()
    g, _ = mo.gradient(params, norm, feat, target, emulate=False)
    rng = np.random.default_rng(1)
    idx = np.concatenate([rng.choice(mo.N_PARAMS, 60, replace=False), [mo.N_PARAMS - 1]])
    eps = 1e-6
    for k in idx:
        p1, p0 = params.copy(), params.copy()
        p1[k] += eps
        p0[k] -= eps
        fd = (mo.loss(p1, norm, feat, target) - mo.loss(p0, norm, feat, target)) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-6 + 1e-5 * abs(fd), (k, fd, g[k])


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -2.5, 3.0e-5], np.float32)
    r = mo.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                   # tie to even (down)
    assert r[2] == 1.0 + 4 * 2 ** -8     # tie to even (up)
    assert r[3] == 1.0                   # below half an ulp
    assert r[4] == -2.5
    assert abs(r[5] - 3.0e-5) <= 3.0e-5 * 2 ** -8
