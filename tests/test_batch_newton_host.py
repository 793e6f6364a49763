"""Host parts of the lock-step batched Newton driver: the block-diagonal
pattern and order given to the device LDL^T, the topology check, and the
batched learned-start features / targets / proposals against the
one-problem functions they restate."""
import numpy as np
import pytest
import scipy.sparse as sp

from nla3d_gb300 import batch_newton as BN
from nla3d_gb300 import learned as L


def _upper_csr(n, seed):
    rng = np.random.default_rng(seed)
    A = sp.random(n, n, density=0.3, random_state=rng) + sp.eye(n)
    U = sp.triu(A + A.T).tocsr()
    U.sort_indices()
    return (U.indptr + 1).astype(np.uint32), (U.indices + 1).astype(np.uint32), U


def test_block_diagonal_pattern_is_scipy_block_diag():
    io, co, U = _upper_csr(9, 1)
    io_bd, co_bd = BN.block_diagonal_pattern(io, co, 4)
    ref = sp.block_diag([U] * 4, format="csr")
    ref.sort_indices()
    assert np.array_equal(io_bd.astype(np.int64) - 1, ref.indptr)
    assert np.array_equal(co_bd.astype(np.int64) - 1, ref.indices)


def test_block_diagonal_order_permutes_every_copy():
    perm = np.array([2, 0, 3, 1])
    out = BN.block_diagonal_order(perm, 4, 3)
    assert out.tolist() == [2, 0, 3, 1, 6, 4, 7, 5, 10, 8, 11, 9]
    assert np.array_equal(np.sort(out), np.arange(12))


def test_same_topology():
    a = L.block_problem(2, 0.5, 1000.0, 1.5)
    b = L.block_problem(2, 0.9, 3000.0, 1.2)     # other material and stretch: same topology
    c = L.block_problem(3, 0.5, 1000.0, 1.5)
    d = L.block_problem(2, 0.5, 1000.0, 1.5, n_loadsteps=10)
    assert BN.same_topology([a, b])
    assert not BN.same_topology([a, c])
    assert not BN.same_topology([a, d])


class _Basis:
    """A CoarseBasis stand-in: random orthonormal Q on n - nc free DoFs."""

    def __init__(self, n, nc, k, seed):
        rng = np.random.default_rng(seed)
        self.nc, self.n = nc, n
        self.Q, _ = np.linalg.qr(rng.normal(size=(n - nc, k)))

    project = L.CoarseBasis.project


def test_batched_features_targets_and_proposals_match_single():
    rng = np.random.default_rng(5)
    B, n, nc = 5, 300, 20
    basis = _Basis(n, nc, 64, 2)
    dU1, dU2 = rng.normal(size=(B, n)), rng.normal(size=(B, n))
    dU = 0.8 * dU1 - 0.1 * dU2 + rng.normal(size=(B, n)) * 0.05
    c10, kb = rng.uniform(0.2, 1.0, B), rng.uniform(500, 5000, B)
    X, s = L.batch_features(basis, dU1, dU2, 0.35, 0.5, c10, kb)
    Y = L.batch_target(basis, dU1, dU2, dU, s)
    P = L.batch_compose(basis, dU1, dU2, s, Y)
    for j in range(B):
        x, sj = L.features(basis, dU1[j], dU2[j], 0.35, 0.5, c10[j], kb[j])
        assert np.allclose(X[j], x, rtol=1e-12, atol=1e-14) and np.isclose(s[j], sj, rtol=1e-13)
        y = L.target(basis, dU1[j], dU2[j], dU[j], sj)
        assert np.allclose(Y[j], y, rtol=1e-8, atol=1e-10 * np.abs(y).max()), j
        p = L.compose(basis, dU1[j], dU2[j], sj, y)
        assert np.allclose(P[j], p, rtol=1e-8, atol=1e-10 * np.abs(p).max())


def test_batch_history_collects_samples_of_completed_steps():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(7)
    B, n, nc = 3, 120, 10
    basis = _Basis(n, nc, 64, 3)

    class _Drv:
        failed = np.array([False, True, False])

    h = L.BatchHistory(B, n, basis, np.full(B, 0.5), np.full(B, 1000.0), collect=True,
                       offset=10)
    states = [rng.normal(size=(B, n)) for _ in range(5)]
    for k, U in enumerate(states):
        d = _Drv()
        d.U = torch.from_numpy(U)
        h(d, (k + 1) / 5)
    # samples for the steps n = 3, 4, 5 of the two problems that did not fail
    assert len(h.X) == 3 and all(x.shape == (2, L.N_IN) for x in h.X)
    assert all(o.tolist() == [10, 12] for o in h.owner)
    assert len(h.U) == 4
    Us = [np.zeros((B, n))] + states
    dU1, dU2 = Us[2] - Us[1], Us[1] - Us[0]
    x0, _ = L.features(basis, dU1[2], dU2[2], 3 / 5, 1.0, 0.5, 1000.0)
    assert np.allclose(h.X[0][1], x0, rtol=1e-12, atol=1e-14)
