"""The learned initial guess's network: the tcgen05 forward pass, loss and gradients
against the CPU reference (oracle/mlp_ref.py, same BF16 rounding points), the
reference's gradient against finite differences, and training."""
import numpy as np
import pytest

from oracle import mlp_ref as ref


def random_params(seed):
    rng = np.random.default_rng(seed)
    p = np.zeros(ref.P_TOTAL)
    W1 = np.zeros((ref.NH, ref.KIN))
    W1[:, :ref.NIN] = rng.uniform(-1, 1, (ref.NH, ref.NIN)) * np.sqrt(6 / (ref.NIN + ref.NH))
    W3 = np.zeros((ref.NO, ref.NH))
    W3[:ref.NOUT] = rng.uniform(-1, 1, (ref.NOUT, ref.NH)) * np.sqrt(6 / (ref.NH + ref.NOUT))
    p[ref.P_W1:ref.P_B1] = W1.ravel()
    p[ref.P_B1:ref.P_W2] = 0.1 * rng.standard_normal(ref.NH)
    p[ref.P_W2:ref.P_B2] = rng.uniform(-1, 1, ref.NH * ref.NH) * np.sqrt(6 / (2 * ref.NH))
    p[ref.P_B2:ref.P_W3] = 0.1 * rng.standard_normal(ref.NH)
    p[ref.P_W3:ref.P_B3] = W3.ravel()
    p[ref.P_B3:ref.P_B3 + ref.NOUT] = 0.1 * rng.standard_normal(ref.NOUT)
    norm = np.concatenate([rng.standard_normal(ref.NIN), rng.uniform(0.5, 2.0, ref.NIN),
                           rng.standard_normal(ref.NOUT), rng.uniform(0.5, 2.0, ref.NOUT)])
    return p.astype(np.float32), norm.astype(np.float32)


def data(n, seed, fseed=0):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, ref.NIN)).astype(np.float32)
    # a smooth target the network can learn (the function is fixed by fseed)
    A = np.random.default_rng(1000 + fseed).standard_normal((ref.NIN, ref.NOUT)) / np.sqrt(ref.NIN)
    T = (np.tanh(X @ A) + 0.1 * np.sin(3 * X[:, :ref.NOUT])).astype(np.float32)
    return X, T


def test_reference_gradient_matches_finite_differences():
    p, norm = random_params(1)
    p = p.astype(np.float64)
    X, T = data(64, 2)
    loss, g = ref.loss_grad(p, norm, X, T, rnd=ref.exact)
    rng = np.random.default_rng(3)
    live = np.flatnonzero(p != 0)
    for k in rng.choice(live, 40, replace=False):
        h = 1e-6 * max(1.0, abs(p[k]))
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (ref.loss_grad(pp, norm, X, T, rnd=ref.exact)[0] -
              ref.loss_grad(pm, norm, X, T, rnd=ref.exact)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1e-3, abs(g[k])) + 1e-9, (k, fd, g[k])


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


@pytest.mark.gpu
def test_forward_matches_reference(gpulib):
    m = gpulib.Mlp(0)
    p, norm = random_params(4)
    m.set_params(p, norm)
    X, _ = data(1000, 5)  # 8 tiles, the last one partial
    Y = m.forward(X)
    Yr, _ = ref.forward(p.astype(np.float64), norm, X)
    assert rel(Y, Yr) < 2e-3, rel(Y, Yr)


@pytest.mark.gpu
def test_loss_and_gradient_match_reference(gpulib):
    m = gpulib.Mlp(0)
    p, norm = random_params(6)
    m.set_params(p, norm)
    X, T = data(300, 7)
    loss, g = m.loss_grad(X, T)
    lr_, gr = ref.loss_grad(p.astype(np.float64), norm, X, T)
    assert abs(loss - lr_) <= 2e-3 * lr_
    for name, a, b in (("W1", ref.P_W1, ref.P_B1), ("b1", ref.P_B1, ref.P_W2),
                       ("W2", ref.P_W2, ref.P_B2), ("b2", ref.P_B2, ref.P_W3),
                       ("W3", ref.P_W3, ref.P_B3), ("b3", ref.P_B3, ref.P_TOTAL)):
        assert rel(g[a:b], gr[a:b]) < 1e-2, (name, rel(g[a:b], gr[a:b]))


@pytest.mark.gpu
def test_training_reduces_loss(gpulib):
    m = gpulib.Mlp(11)
    X, T = data(20000, 8)
    l0 = m.train(X, T, epochs=1, batch_tiles=8, lr=1e-3, seed=1)
    l1 = m.train(X, T, epochs=10, batch_tiles=8, lr=1e-3, seed=2)
    assert l1 < 0.25 * l0, (l0, l1)
    # held-out data: the trained network generalises
    Xv, Tv = data(4000, 9)
    p, norm = m.params()
    Yv = m.forward(Xv)
    mu, sd = norm[2 * ref.NIN:2 * ref.NIN + ref.NOUT], norm[2 * ref.NIN + ref.NOUT:]
    lv = (((Yv - Tv) / sd) ** 2).mean()
    assert lv < 2 * l1 + 0.05, (lv, l1)
