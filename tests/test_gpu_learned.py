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


@pytest.mark.parametrize("m,n,k,a_bf16,b_bf16,act", [
    (37, 256, 132, 0, 1, 1),     # forward, first layer: X W^T + b, tanh
    (128, 66, 256, 0, 1, 0),     # forward, output layer
    (256, 132, 37, 0, 0, 0),     # dW = dZ^T X (both FP32), K not a multiple of 32
    (300, 256, 256, 0, 1, 0),    # dX = dZ W, M over three tiles
    (5, 8, 0, 0, 1, 1),          # K = 0: act(bias)
])
def test_mlp_gemm_tensor_cores_against_fp64(m, n, k, a_bf16, b_bf16, act):
    """nla3d_mlp_gemm (tcgen05, BF16 operands, FP32 accumulation) against a
    float64 product of the same inputs: an FP32 operand enters as a BF16 pair
    (2^-16 relative), so the error stays within a few 2^-16 of sum |a b|."""
    torch = pytest.importorskip("torch")
    import ctypes
    from nla3d_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(m * 7 + n + k)
    A = torch.from_numpy(rng.normal(size=(m, k)).astype(np.float32)).cuda()
    Bt = torch.from_numpy(rng.normal(size=(n, k)).astype(np.float32)).cuda()   # B[k, n] = Bt[n, k]
    if b_bf16:
        Bt = Bt.to(torch.bfloat16)
    if a_bf16:
        A = A.to(torch.bfloat16)
    bias = torch.from_numpy(rng.normal(size=n).astype(np.float32)).cuda()
    C = torch.full((m, n), 7.0, dtype=torch.float32, device="cuda")
    rc = lib.nla3d_mlp_gemm(m, n, k, A.data_ptr(), a_bf16, k, 1, Bt.data_ptr(), b_bf16, 1, k,
                            C.data_ptr(), n, bias.data_ptr(), act, None)
    assert rc == 0
    torch.cuda.synchronize()
    t = ctypes.c_uint32()
    assert lib.nla3d_mlp_status(ctypes.byref(t)) == 0 and t.value == 0
    a = A.float().cpu().numpy().astype(np.float64)
    b = Bt.float().cpu().numpy().astype(np.float64).T
    z = a @ b + bias.cpu().numpy()
    ref = np.tanh(z) if act else z
    scale = (np.abs(a) @ np.abs(b)).max() + 1.0
    assert np.abs(C.cpu().numpy() - ref).max() <= 8 * 2.0 ** -16 * scale
