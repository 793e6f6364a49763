"""Learned Newton start on the GPU: the MLP kernels' gradients against the
CPU oracle, and a trained network reducing Newton iterations per load step on
held-out problems at the unchanged 1e-8 residual tolerance."""
import numpy as np
import pytest

from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu


def test_mlp_kernel_gradients_match_cpu_oracle():
    torch = pytest.importorskip("torch")
    from nla3d_gb300.learned import MLP, N_IN, N_OUT
    mlp = MLP(seed=3)
    rng = np.random.default_rng(4)
    X = rng.normal(size=(37, N_IN)).astype(np.float32)
    T = rng.normal(size=(37, N_OUT)).astype(np.float32)
    Xd = torch.from_numpy(X).cuda()
    Td = torch.from_numpy(T).cuda()
    acts = mlp.forward(Xd)
    gW, gb = mlp.backward(acts, mlp.loss_grad(acts[-1], Td))
    torch.cuda.synchronize()
    Ws, bs = mlp.weights()
    loss, oW, ob = M.loss_and_grads(Ws, bs, X.astype(np.float64), T.astype(np.float64))
    out = acts[-1].cpu().numpy()
    ref_out = M.forward(Ws, bs, X.astype(np.float64))[-1]
    assert np.abs(out - ref_out).max() <= 1e-4 * np.abs(ref_out).max()
    for l in range(len(gW)):
        g, o = gW[l].cpu().numpy(), oW[l]
        assert np.abs(g - o).max() <= 2e-3 * np.abs(o).max(), l
        g, o = gb[l].cpu().numpy(), ob[l]
        assert np.abs(g - o).max() <= 2e-3 * np.abs(o).max(), l


def test_learned_start_reduces_newton_iterations():
    pytest.importorskip("torch")
    from nla3d_gb300 import learned as L
    train = L.sample_block_problems(24, n=3, seed=11)
    X, Y, _ = L.generate(train)
    mlp = L.MLP(seed=0)
    hist = mlp.fit(X, Y, epochs=300, batch=128, lr=2e-3)
    assert hist[-1][1] < hist[0][1]
    held_out = L.sample_block_problems(4, n=3, seed=99)
    res = L.evaluate(held_out, mlp)
    assert res["learned"] < res["plain"], res
