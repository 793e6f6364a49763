"""The MLP oracle itself: its gradients against central finite differences
(CPU only)."""
import numpy as np

from oracle import mlp_oracle as M


def test_bf16_rounding_ties_to_even():
    x = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.0e38], dtype=np.float64)
    r = M.to_bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0  # 1 + 2^-8 is a tie: rounds to even (1.0)
    assert r[2] == 1.0078125             # above the tie: rounds up
    assert r[3] == -2.5


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    sizes = [5, 7, 6, 3]
    Ws = [rng.normal(0, 0.5, (o, i)) for i, o in zip(sizes[:-1], sizes[1:])]
    bs = [rng.normal(0, 0.1, o) for o in sizes[1:]]
    # exactly representable weights so that BF16 rounding is the identity
    Ws = [M.to_bf16(W) for W in Ws]
    X = rng.normal(size=(4, 5))
    T = rng.normal(size=(4, 3))
    loss, gW, gb = M.loss_and_grads(Ws, bs, X, T)
    h = 1e-6
    for l in range(len(bs)):
        for j in range(bs[l].size):
            bp = [b.copy() for b in bs]
            bp[l][j] += h
            bm = [b.copy() for b in bs]
            bm[l][j] -= h
            fd = (M.loss_and_grads(Ws, bp, X, T)[0] - M.loss_and_grads(Ws, bm, X, T)[0]) / (2 * h)
            assert abs(fd - gb[l][j]) < 1e-7
