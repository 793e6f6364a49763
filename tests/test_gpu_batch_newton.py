"""Lock-step batched Newton on the GPU: every problem of a batch takes the
same Newton iterations per load step as the one-problem driver (device
LDL^T, FP64 fronts), with and without the secant-extrapolation start, and the
learned start trained on batched solves cuts the iterations on held-out
problems at the unchanged 1e-8 residual tolerance."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _single(pb, start):
    from nla3d_gb300 import learned as L
    from nla3d_gb300.storage import FEStorage
    be = FEStorage(pb.mesh, "fp64").initSolutionData()
    factory = (lambda sv, h: L.ExtrapolationPredictor(h)) if start == "extrapolation" else None
    s, _ = L.solve(pb, be, factory, linear_solver="gpu")
    return [r.iterations for r in s.records], [r.predicted for r in s.records], s.U


@pytest.mark.parametrize("start", ["plain", "extrapolation"])
def test_batch_matches_single_problem_driver(start):
    pytest.importorskip("torch")
    from nla3d_gb300 import learned as L
    from nla3d_gb300.batch_newton import BatchNewton
    problems = L.sample_block_problems(3, n=3, seed=21)
    drv = BatchNewton(problems, precision="fp64", fronts="fp64")
    hist = L.BatchHistory(drv.B, drv.n)
    pred = L.BatchExtrapolationPredictor(hist) if start == "extrapolation" else None
    drv.solve(predictor=pred, on_converged=hist)
    assert not drv.failed.any()
    U = drv.U.cpu().numpy()
    for j, pb in enumerate(problems):
        its, used, Us = _single(pb, start)
        assert drv.iterations[j].tolist() == its, (j, drv.iterations[j], its)
        if start == "extrapolation":
            assert drv.predicted[j].tolist() == used
        assert np.abs(U[j] - Us).max() <= 1e-8 * np.abs(Us).max()
    drv.close()


def test_batched_learned_start_reduces_newton_iterations():
    pytest.importorskip("torch")
    from nla3d_gb300 import learned as L
    solvers = {}
    X, Y, iters, failed, owner = L.generate_batched(L.sample_block_problems(24, n=3, seed=11),
                                                    batch_size=12, solvers=solvers)
    assert failed == 0 and iters.shape == (24, 20)
    # 20 load steps: one sample per step from the third on
    assert np.array_equal(np.bincount(owner), np.full(24, 18))
    assert X.shape == (24 * 18, L.N_IN) and Y.shape == (24 * 18, L.N_OUT)
    mlp = L.MLP(seed=0)
    hist = mlp.fit(X, Y, epochs=300, batch=128, lr=2e-3)
    assert hist[-1][1] < hist[0][1]
    res = L.evaluate_batched(L.sample_block_problems(4, n=3, seed=99), mlp, batch_size=4,
                             solvers=solvers)
    assert res["failed"] == {"plain": 0, "extrapolation": 0, "learned": 0}
    assert res["learned"] < res["plain"], res


def test_batch_matches_single_problem_driver_with_mpc_rows():
    """Torsion bars with a rigid-body MPC end (Lagrange multiplier rows in
    K(2)): the batched residual removes the multipliers' forces per problem
    as the one-problem driver does, so the iteration counts agree."""
    pytest.importorskip("torch")
    import math
    from nla3d_gb300 import learned as L
    from nla3d_gb300.batch_newton import BatchNewton
    from nla3d_gb300.storage import FEStorage
    problems = [L.bar_problem(2, 6, c10, 1000.0, st, math.radians(tw), n_loadsteps=10)
                for c10, st, tw in ((0.4, 1.3, 30.0), (0.6, 1.5, 45.0))]
    drv = BatchNewton(problems, precision="fp64", fronts="fp64")
    assert drv.nm > 0
    drv.solve()
    assert not drv.failed.any()
    U = drv.U.cpu().numpy()
    for j, pb in enumerate(problems):
        be = FEStorage(pb.mesh, "fp64").initSolutionData()
        s, _ = L.solve(pb, be, linear_solver="gpu")
        s.close()
        assert drv.iterations[j].tolist() == [r.iterations for r in s.records], j
        assert np.abs(U[j] - s.U).max() <= 1e-8 * np.abs(s.U).max()
    drv.close()
