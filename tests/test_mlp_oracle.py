"""CPU checks of the MLP oracle: exact gradients against central finite
differences, and the BF16-rounded gradients close to the exact ones."""
import numpy as np

from oracle.mlp_oracle import bf16, grads_exact, loss_and_grads, loss_exact


def _net(seed=0, dims=(10, 16, 16, 6), B=20):
    rng = np.random.default_rng(seed)
    Ws = [rng.normal(size=(k, n)) * np.sqrt(2.0 / k) for k, n in zip(dims[:-1], dims[1:])]
    bs = [rng.normal(size=n) * 0.1 for n in dims[1:]]
    X = rng.normal(size=(B, dims[0]))
    T = rng.normal(size=(B, dims[-1]))
    return Ws, bs, X, T


def test_exact_gradients_match_finite_differences():
    Ws, bs, X, T = _net()
    gW, gb = grads_exact(Ws, bs, X, T)
    h = 1e-6
    rng = np.random.default_rng(3)
    for l in range(len(Ws)):
        for _ in range(5):
            i, j = rng.integers(Ws[l].shape[0]), rng.integers(Ws[l].shape[1])
            Wp = [w.copy() for w in Ws]
            Wm = [w.copy() for w in Ws]
            Wp[l][i, j] += h
            Wm[l][i, j] -= h
            fd = (loss_exact(Wp, bs, X, T) - loss_exact(Wm, bs, X, T)) / (2 * h)
            assert abs(fd - gW[l][i, j]) < 1e-6 * max(1.0, abs(fd))
        k = rng.integers(bs[l].size)
        bp = [b.copy() for b in bs]
        bm = [b.copy() for b in bs]
        bp[l][k] += h
        bm[l][k] -= h
        fd = (loss_exact(Ws, bp, X, T) - loss_exact(Ws, bm, X, T)) / (2 * h)
        assert abs(fd - gb[l][k]) < 1e-6 * max(1.0, abs(fd))


def test_bf16_rounding_and_rounded_gradients():
    assert bf16(np.array([1.0, 1.0 + 2 ** -9, 1.0 + 3 * 2 ** -9]))[1] == 1.0       # ties to even
    assert bf16(np.array([1.0 + 3 * 2 ** -9]))[0] == 1.0 + 2 ** -7
    Ws, bs, X, T = _net(seed=1)
    _, gW, gb = loss_and_grads(Ws, bs, X, T)
    eW, eb = grads_exact(Ws, bs, X, T)
    for a, b in zip(gW + gb, eW + eb):
        assert np.linalg.norm(a - b) < 0.05 * np.linalg.norm(b)
