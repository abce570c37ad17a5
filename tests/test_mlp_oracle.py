"""CPU checks of the FP64 MLP oracle used to verify the learned warm start."""
import numpy as np

from oracle import mlp_oracle as M


def _data(n=64, seed=0):
    rng = np.random.default_rng(seed)
    f = rng.normal(size=(n, M.N_IN))
    t = np.sin(f[:, 0]) + 0.3 * f[:, 4] - 0.1 * f[:, 1] ** 2
    norm = np.concatenate([f.mean(0), f.std(0), [t.mean(), t.std()]])
    return f, t, norm


def test_gradient_matches_finite_differences():
    f, t, norm = _data()
    p = M.init_params(1)
    _, g = M.loss_and_grad(p, norm, f, t)
    rng = np.random.default_rng(2)
    for i in rng.choice(M.N_PARAMS, 40, replace=False):
        e = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[i] += e
        pm[i] -= e
        fd = (M.loss_and_grad(pp, norm, f, t)[0] - M.loss_and_grad(pm, norm, f, t)[0]) / (2 * e)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def test_adam_reduces_loss():
    f, t, norm = _data(256)
    opt = M.Adam(M.init_params(3), lr=1e-2)
    l0 = M.loss_and_grad(opt.p, norm, f, t)[0]
    for _ in range(200):
        opt.step(M.loss_and_grad(opt.p, norm, f, t)[1])
    assert M.loss_and_grad(opt.p, norm, f, t)[0] < 0.2 * l0


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.01171875, 3.14159, -2.5e-3])
    r = M.bf16_round(x)
    # bf16 spacing at 1 is 2^-7: 1 + 2^-8 and 1 + 3 * 2^-8 are ties -> even mantissa
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.015625
    assert np.all(np.abs(r - x) <= np.abs(x) * 2**-8)
