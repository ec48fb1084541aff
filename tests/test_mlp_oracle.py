"""The radiance-cache network's CPU oracle (no GPU): backward pass against
central finite differences of the loss, in fp32 mode."""
import numpy as np


def random_samples(n, seed):
    rng = np.random.default_rng(seed)
    s = np.zeros((n, 16), np.float32)
    s[:, :12] = rng.uniform(0.0, 1.0, (n, 12))
    s[:, 12:15] = rng.uniform(0.0, 2.0, (n, 3))
    return s


def random_weights(seed):
    rng = np.random.default_rng(seed)
    w = rng.uniform(-0.3, 0.3, 4 * 4096 + 8 * 64).astype(np.float32)
    w[4 * 4096 + 3 * 64:] = 0.0
    return w


def fd_check(oracle, W, S, dW, idx, h):
    y0 = oracle.mlp_forward(W, S, bf16=False).astype(np.float64)
    den = y0 ** 2 + 0.01          # the gradient holds the denominator at the current prediction
    t = S[:, 12:15].astype(np.float64)

    def L(w):
        y = oracle.mlp_forward(w, S, bf16=False).astype(np.float64)
        return np.mean((y - t) ** 2 / den)
    errs = []
    for i in idx:
        Wp, Wm = W.copy(), W.copy()
        Wp[i] += h
        Wm[i] -= h
        fd = (L(Wp) - L(Wm)) / (2 * h)
        errs.append(abs(fd - dW[i]) / max(abs(fd), 1e-4))
    return np.array(errs)


def test_gradient_matches_finite_differences(oracle):
    S = random_samples(24, 1)
    W = random_weights(2)
    dW, loss = oracle.mlp_gradient(W, S, bf16=False)
    assert loss > 0
    rng = np.random.default_rng(3)
    # output layer: the loss is quadratic in these weights, central differences are exact
    out_idx = 4 * 4096 + rng.integers(0, 3 * 64, 20)
    assert fd_check(oracle, W, S, dW, out_idx, 1e-2).max() < 1e-3
    # hidden layers: piecewise linear (ReLU); a perturbation may cross a kink
    hid_idx = rng.integers(0, 4 * 4096, 60)
    e = fd_check(oracle, W, S, dW, hid_idx, 1e-3)
    assert np.mean(e < 2e-2) >= 0.8 and np.median(e) < 1e-2, e


def test_adam_step_moves_against_gradient(oracle):
    W = random_weights(4)
    S = random_samples(64, 5)
    dW, l0 = oracle.mlp_gradient(W, S, bf16=False)
    W1, m, v = oracle.mlp_adam(W, dW, np.zeros_like(W), np.zeros_like(W), 1e-3, 1)
    _, l1 = oracle.mlp_gradient(W1, S, bf16=False)
    assert l1 < l0
    assert np.all(W1[4 * 4096 + 3 * 64:] == 0.0)
