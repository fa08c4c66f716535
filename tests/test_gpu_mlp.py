"""The learned-lambda network's tensor-core kernels against the host restatement
(oracle/mlp_oracle.py, which reproduces the kernels' BF16 rounding points).

Tolerances: the kernels evaluate SiLU through the hardware tanh approximation (relative error
about 2^-11 per activation) where the restatement uses exact float64; a few BF16 roundings of
activations then land on the other side of a rounding boundary.  Forward outputs agree to 1e-2 of
the largest output (mean 2e-3), gradients to 1e-2 in relative L2 norm per parameter tensor."""
import numpy as np
import pytest

from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu


def _problem(seed, n):
    from akuaengine_gb300.warm_start import init_params

    rng = np.random.default_rng(seed)
    params = init_params(seed)
    b = mo.unpack(params)
    for name in ("b1", "b2", "b3", "b4"):
        b[name] = rng.normal(0, 0.2, b[name].shape)
    params = mo.pack(b).astype(np.float32)
    mean = rng.normal(0, 1, 8).astype(np.float32)
    inv_std = rng.uniform(0.5, 2.0, 8).astype(np.float32)
    scale = np.float32(3.0e-4)
    feat = (rng.normal(0, 1.3, (n, 8)) / inv_std + mean).astype(np.float32)
    target = (rng.normal(0, 1, n) * scale).astype(np.float32)
    return params, mean, inv_std, scale, feat, target


@pytest.fixture
def net(cuda_lib):
    from akuaengine_gb300.warm_start import LambdaNet

    n = LambdaNet()
    yield n
    n.close()


@pytest.mark.parametrize("n", [1, 127, 1000, 40000])
def test_forward_matches_oracle(net, n):
    import torch

    params, mean, inv_std, scale, feat, _ = _problem(3, n)
    net.set_params(params)
    net.set_normalization(mean, inv_std, scale)
    out = net.forward(torch.from_numpy(feat).cuda()).cpu().numpy().astype(np.float64)
    norm = np.concatenate([mean, inv_std, [scale, 1.0]])
    want, _ = mo.forward(params, norm, feat, emulate=True)
    err = np.abs(out - want)
    ref = np.abs(want).max()
    print("forward n=%d: max err %.3g, mean err %.3g, of max |y| %.3g" % (n, err.max(), err.mean(), ref))
    assert err.max() <= 1e-2 * ref
    assert err.mean() <= 2e-3 * ref


@pytest.mark.parametrize("n", [128, 1000, 20000])
def test_gradient_matches_oracle(net, n):
    import torch

    params, mean, inv_std, scale, feat, target = _problem(5, n)
    net.set_params(params)
    net.set_normalization(mean, inv_std, scale)
    g, loss = net.gradient(torch.from_numpy(feat).cuda(), torch.from_numpy(target).cuda())
    norm = np.concatenate([mean, inv_std, [scale, 1.0]])
    gw, lw = mo.gradient(params, norm, feat, target, emulate=True)
    assert abs(loss - lw) <= 1e-2 * lw
    got, want = mo.unpack(g), mo.unpack(gw)
    for name, _ in mo.SIZES:
        d = np.linalg.norm(got[name] - want[name])
        r = np.linalg.norm(want[name])
        print("grad %s: rel l2 err %.3g (|g| %.3g)" % (name, d / max(r, 1e-30), r))
        assert d <= 1e-2 * r + 1e-9, name


def test_adam_fits_a_smooth_function(net):
    import torch

    from akuaengine_gb300.warm_start import train

    rng = np.random.default_rng(11)
    n = 65536
    feat = rng.normal(0, 1, (n, 8)).astype(np.float32)
    target = (np.sin(feat[:, 0]) + 0.5 * feat[:, 1] * feat[:, 2] - 0.3 * feat[:, 3] ** 2)
    target = (target * 1e-3).astype(np.float32)
    f = torch.from_numpy(feat).cuda()
    t = torch.from_numpy(target).cuda()
    net.fit_normalization(f, t)
    _, loss0 = net.gradient(f, t)
    losses = train(net, f, t, epochs=40, batch=4096, lr=3e-3, lr_final=1e-4)
    print("adam: loss %.4g -> %s" % (loss0, ["%.4g" % v for v in losses]))
    assert losses[-1] < 0.05 * loss0


def test_network_argument_errors(net):
    import torch

    from akuaengine_gb300 import AkuaError

    with pytest.raises(ValueError):
        net.set_params(np.zeros(10, np.float32))
    with pytest.raises(AkuaError):
        net.set_normalization(np.zeros(8), np.ones(8), 0.0)
    with pytest.raises(AkuaError):
        net.set_normalization(np.zeros(8), np.ones(8), 1.0, float("nan"))
    bad = np.zeros(8961, np.float32)
    bad[5] = np.nan
    with pytest.raises(AkuaError):
        net.set_params(bad)
    f = torch.zeros((4, 8), device="cuda")
    with pytest.raises(ValueError):
        net.forward(f[:, :4].contiguous())
