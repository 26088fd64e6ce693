"""The FP64 surrogate oracle: its gradient against central differences and
its Adam step against torch.optim.Adam (CPU)."""
import numpy as np
import pytest

from oracle import oracle as O


def rand_model(seed=0, layers=3):
    rng = np.random.default_rng(seed)
    P = np.zeros(O.OracleMLP.NPARAM)
    P[0:1024] = rng.uniform(-0.6, 0.6, 1024)
    P[1024:1088] = rng.uniform(-0.1, 0.1, 64)
    P[1088:5184] = rng.uniform(-0.3, 0.3, 4096)
    P[5184:5248] = rng.uniform(-0.1, 0.1, 64)
    P[5248:9344] = rng.uniform(-0.3, 0.3, 4096)
    P[9344:9408] = rng.uniform(-0.1, 0.1, 64)
    P[9408:9472] = rng.uniform(-0.2, 0.2, 64)
    P[9472] = 0.1
    mu = rng.uniform(-1, 1, 16)
    sd = rng.uniform(0.5, 2, 16)
    return O.OracleMLP(P, mu, sd, tau_scale=0.7, layers=layers), rng


# blocks [lo, hi) of the hidden layers a network of `layers` does not use
FROZEN = {1: (1088, 9408), 2: (5248, 9408), 3: (0, 0)}


def numpy_forward(m, f):
    """Independent restatement: h <- silu(W h + b) per hidden layer, y = W4 h + b4."""
    P = m.P
    h = (f - m.mu) / m.sd
    blocks = [(0, 1024, 1088, 16), (1088, 5184, 5248, 64), (5248, 9344, 9408, 64)]
    for w0, b0, b1, nin in blocks[:m.layers]:
        z = h @ P[w0:b0].reshape(64, nin).T + P[b0:b1]
        h = z / (1.0 + np.exp(-z))
    return h @ P[9408:9472] + P[9472]


@pytest.mark.parametrize("layers", [1, 2, 3])
def test_forward_matches_numpy(layers):
    m, rng = rand_model(3, layers)
    f = rng.uniform(-2, 2, (40, 16))
    np.testing.assert_allclose(m.forward(f), numpy_forward(m, f), rtol=1e-12, atol=1e-13)


@pytest.mark.parametrize("layers", [1, 2, 3])
def test_gradient_matches_central_differences(layers):
    m, rng = rand_model(0, layers)
    f = rng.uniform(-2, 2, (24, 16))
    tau = rng.uniform(0, 2, 24)
    sigma = 1.5
    loss, g = m.loss_grad(f, tau, sigma)
    assert loss > 0
    lo, hi = FROZEN[layers]
    assert not g[lo:hi].any()  # unused layers: exactly zero
    idx = list(rng.choice(9473, 60, replace=False)) + [0, 1024, 1088, 5248, 9408, 9472]
    h = 1e-6
    for i in idx:
        Pp = m.P.copy()
        Pp[i] += h
        Pm = m.P.copy()
        Pm[i] -= h
        num = (m.loss_grad(f, tau, sigma, Pp)[0] - m.loss_grad(f, tau, sigma, Pm)[0]) / (2 * h)
        assert g[i] == pytest.approx(num, rel=1e-5, abs=1e-9), i


@pytest.mark.parametrize("layers", [1, 2, 3])
def test_forward_consistent_with_loss(layers):
    m, rng = rand_model(1, layers)
    f = rng.uniform(-2, 2, (5, 16))
    y = m.forward(f)
    sigma = 2.0
    tau = np.zeros(5)
    loss, _ = m.loss_grad(f, tau, sigma)
    expect = np.mean((np.exp(-sigma * m.tau_scale * np.logaddexp(0.0, y)) - 1.0) ** 2)
    assert loss == pytest.approx(expect, rel=1e-12)


def test_adam_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(2)
    w0 = rng.normal(size=50)
    grads = [rng.normal(size=50) for _ in range(3)]
    p = torch.nn.Parameter(torch.tensor(w0, dtype=torch.float64))
    opt = torch.optim.Adam([p], lr=1e-3, betas=(0.9, 0.999), eps=1e-8)
    w, m, v = w0.copy(), np.zeros(50), np.zeros(50)
    for t, g in enumerate(grads, start=1):
        opt.zero_grad()
        p.grad = torch.tensor(g, dtype=torch.float64)
        opt.step()
        w, m, v = O.adam_step(w, m, v, g, 1e-3, 0.9, 0.999, 1e-8, t)
    np.testing.assert_allclose(w, p.detach().numpy(), rtol=1e-12, atol=1e-14)
