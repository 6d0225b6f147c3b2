"""The surrogate network's CPU oracle: BF16 rounding, GELU and finite-difference gradients (no GPU)."""
import numpy as np

from oracle import mlp_oracle as M


def test_bf16_rounding_ties_to_even_and_specials():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -2.5, 0.0, np.inf, 65504.0],
                 dtype=np.float32)
    r = M.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                        # halfway: ties to the even mantissa (1.0)
    assert r[2] == 1.0 + 4 * 2 ** -8          # halfway: rounds up to the even neighbour
    assert r[3] == 1.0
    assert r[4] == -2.5 and r[5] == 0.0 and np.isinf(r[6])
    assert r[7] == 65536.0
    assert np.isnan(M.bf16(np.array([np.nan], dtype=np.float32)))[0]


def test_gelu_grad_matches_finite_difference():
    u = np.linspace(-6, 6, 101)
    h = 1e-6
    fd = (M.gelu(u + h) - M.gelu(u - h)) / (2 * h)
    assert np.max(np.abs(fd - M.gelu_grad(u))) < 1e-8


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    params = [p.astype(np.float64) for p in M.init_params(1)]
    x = M.pad_features(rng.uniform(-1, 1, size=(5, M.N_FEATURES))).astype(np.float64)
    t = rng.dirichlet(np.ones(1024), size=5)
    loss, grads = M.backward(params, x, t, rnd=M._exact, dtype=np.float64)
    h = 1e-6
    for pi, idx in [(0, (3, 2)), (1, (7,)), (2, (10, 200)), (4, (0, 0)), (6, (900, 17)), (7, (512,))]:
        p = params[pi]
        old = p[idx]
        p[idx] = old + h
        lp = M.kl_loss(M.forward(params, x, M._exact, np.float64)[2], t)
        p[idx] = old - h
        lm = M.kl_loss(M.forward(params, x, M._exact, np.float64)[2], t)
        p[idx] = old
        fd = (lp - lm) / (2 * h)
        assert abs(fd - grads[pi][idx]) < 1e-7 + 1e-5 * abs(fd), (pi, idx, fd, grads[pi][idx])
    # padded inputs receive no gradient
    assert not grads[0][:, M.N_FEATURES:].any()


def test_adam_step_reduces_loss_and_ensemble_stats():
    rng = np.random.default_rng(2)
    params = M.init_params(3)
    x = M.pad_features(rng.uniform(-1, 1, size=(64, M.N_FEATURES)))
    t = rng.dirichlet(np.ones(1024) * 0.5, size=64)
    m = [np.zeros_like(p) for p in params]
    v = [np.zeros_like(p) for p in params]
    l0, _ = M.backward(params, x, t)
    for step in range(1, 31):
        _, g = M.backward(params, x, t)
        M.adam(params, g, m, v, step, lr=1e-3)
    l1, _ = M.backward(params, x, t)
    assert l1 < l0
    qs = [M.forward(M.init_params(s), x)[2] for s in range(3)]
    mean, spread = M.ensemble_stats(qs)
    assert np.allclose(mean.sum(axis=1), 1.0) and spread.shape == (64,) and (spread > 0).all()
    assert np.allclose(M.tv(qs[0], qs[0]), 0.0)
