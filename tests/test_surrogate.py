"""CPU tests of the rank-surrogate oracle (oracle/surrogate.py): the analytic
gradient is pinned by central finite differences, the BF16 rounding by known
values, and the Adam step by a hand-computed first update."""
import numpy as np

from oracle import surrogate as S


def _data(n=96, seed=0):
    rng = np.random.default_rng(seed)
    F = np.stack([rng.integers(0, 6, n), rng.uniform(1, 60, n), rng.uniform(1, 4, n),
                  np.log1p(rng.integers(8, 4000, n))], axis=1)
    T = np.log(5 + 0.3 * F[:, 1] + 2 * F[:, 0]) + 0.05 * rng.standard_normal(n)
    return F, T


def test_gradient_matches_finite_differences():
    F, T = _data()
    w = S.init_weights(F, seed=1).astype(np.float64)
    w[8:] += 0.05 * np.random.default_rng(2).standard_normal(S.NW - 8)  # nonzero biases too
    loss, g = S.loss_and_grad(w, F, T, round_bf16=False, dtype=np.float64)
    rng = np.random.default_rng(3)
    idx = np.concatenate([[S.NW - 1], rng.choice(np.arange(8, S.NW), 60, replace=False)])
    h = 1e-6
    for i in idx:
        wp, wm = w.copy(), w.copy()
        wp[i] += h
        wm[i] -= h
        fd = (S.loss_and_grad(wp, F, T, False, np.float64)[0] -
              S.loss_and_grad(wm, F, T, False, np.float64)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])
    assert np.all(g[:8] == 0.0)


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.1415927], np.float32)
    r = S.bf16_round(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                 # halfway: ties to even
    assert r[2] == 1.0 + 2 ** -7       # above halfway: up
    assert r[3] == -2.5
    assert abs(r[4] - 3.140625) < 1e-7


def test_adam_first_step_is_sign_times_lr():
    w = np.ones(S.NW, np.float32)
    g = np.linspace(-1, 1, S.NW).astype(np.float32)
    m = np.zeros_like(w)
    v = np.zeros_like(w)
    S.adam_step(w, g, m, v, t=1, lr=0.01)
    expect = 1.0 - 0.01 * np.sign(g[8:]) * (np.abs(g[8:]) / (np.abs(g[8:]) + 1e-8))
    assert np.allclose(w[8:], expect, atol=1e-6)
    assert np.all(w[:8] == 1.0)
