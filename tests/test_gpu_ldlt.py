"""The device LDL^T (nla3d_ldlt_*) on K(2) blocks assembled on the GPU:
solutions equal SciPy's sparse LU solution to 1e-10 (relative) and the
refined residual ||b - K x|| / ||b|| reaches 1e-13 (FP64 fronts) or 1e-12
(FP32 fronts + FP64 refinement); u/p blocks, MPC and CE equations, rigid-body
masters, thermal blocks; fronts above 256 rows (the blocked path); bitwise
reproducible; and the Newton driver on the reference's rigid-body test with
the solve on the device."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

import cases
from nla3d_gb300 import ldlt
from nla3d_gb300 import meshgen as mg
from nla3d_gb300.newton import NewtonSolver, csr_full, nested_dissection
from nla3d_gb300.storage import FEStorage

pytestmark = pytest.mark.gpu


def _storage(mesh, u, p, extra, do_update):
    s = FEStorage(mesh).initSolutionData()
    ne, ee = s.eq_numbers()
    s.setU(mg.u_to_vector(ne, ee, u, p, s.n_total, extra))
    if do_update:
        s.updateResults()
    s.assembleGlobalEqMatrices()
    s.synchronize()
    return s


def _order(s):
    io, co = s.pattern(2)
    n2 = io.size - 1
    K = csr_full(io, co, np.ones(co.size), n2, n2, True)
    pts = np.random.default_rng(1).random((n2, 3))
    return ldlt.saddle_order(io, co, nested_dissection(K, pts, leaf=16), s.n_unk)


def _check(s, precision="fp64", tol=1e-13, seed=0, max_refine=10):
    io, co = s.pattern(2)
    n2 = io.size - 1
    A = csr_full(io, co, s.K(2), n2, n2, True).tocsc()
    b = np.random.default_rng(seed).standard_normal(n2)
    solver = ldlt.DeviceLDLT.for_storage(s, _order(s), precision)
    solver.factor(s)
    x = solver.solve_host(s, b, max_refine=max_refine, tol=tol)
    assert solver.info()["nonfinite"] == 0
    xr = spla.spsolve(A, b)
    assert np.linalg.norm(b - A @ x) <= tol * np.linalg.norm(b) * 1.01
    assert np.abs(x - xr).max() <= 1e-10 * np.abs(xr).max()
    return solver, x


@pytest.mark.parametrize("name", ["cube4_nh_clamped", "biderman_3x3x3_clamped", "bar_mpc_2x2x3",
                                  "bar_mpc_ce_2x2x3", "plane41_mr_4x3_clamped",
                                  "tetra0_3x3x3", "quadth_lines_6x5"])
def test_small_cases_match_scipy(name):
    # (ce_block_3x3x2 is left out: its K(2) is singular -- free rigid-body modes)
    s = _storage(*cases.FULL_CASES[name]())
    _check(s)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-13), ("fp32", 1e-12)])
def test_blocked_fronts_twisted_block(precision, tol):
    """12^3 twisted Mooney-Rivlin block, z = 0 clamped: the top separators
    exceed 256 rows, so the blocked panel path runs."""
    mesh = mg.solid81_block(12, 12, 12, 1.0 / 12, mg.MAT_MOONEY_RIVLIN, (0.4, 0.1, 2000.0),
                            clamp_z0=True)
    u, p = mg.twist_state(mesh, angle_deg=20.0, stretch=1.3, noise_frac=0.005, seed=2)
    s = _storage(mesh, u, p, None, True)
    solver, x = _check(s, precision, tol)
    assert solver.info()["max_front"] > 256
    # bitwise reproducible
    solver.factor(s)
    b = np.random.default_rng(0).standard_normal(x.size)
    x2 = solver.solve_host(s, b, max_refine=10, tol=tol)
    assert np.array_equal(x.view(np.uint64), x2.view(np.uint64))


def test_newton_rigid_body_with_device_solver():
    """The reference's rigid_body_mpc_block_ROTX test through the Newton driver
    with K(2) factored on the device (MPC equations and the master node
    last): the reaction curve passes the reference's 1e-4 and equals the
    host-solve curve to 1e-8."""
    import rigid_body_case as rb
    mesh, fixes, ref = rb.load_case()
    curves = {}
    for solver in ("direct", "gpu", "gpu-fp32"):
        s = FEStorage(mesh).initSolutionData()
        n = NewtonSolver(s, fixes, n_loadsteps=20, n_iterations=15, solver=solver).solve()
        assert rb.curve_error(n, mesh, ref) < rb.THRESHOLD
        curves[solver] = np.concatenate([r for r in n.reactions])
    for k in ("gpu", "gpu-fp32"):
        assert np.abs(curves[k] - curves["direct"]).max() <= 1e-8 * np.abs(curves["direct"]).max()


def test_fp32_fronts_on_a_nearly_incompressible_block():
    """K/G = 1e6 (Neo-Hookean), twisted: the FP32 factor alone is far from
    1e-12; the refinement (steps, then GMRES preconditioned by the factor)
    reaches it and agrees with SciPy."""
    mesh = mg.solid81_block(6, 6, 6, 1.0 / 6, mg.MAT_NEO_HOOKEAN, (1.0, 1.0e6), clamp_z0=True)
    u, p = mg.twist_state(mesh, angle_deg=30.0, stretch=1.2, noise_frac=0.01, seed=4)
    s = _storage(mesh, u, p, None, True)
    solver, x = _check(s, "fp32", 1e-12)
    assert solver.last_steps >= 2


@pytest.mark.parametrize("precision", ["fp32", "fp32-tc"])
def test_fp32_fronts_nearly_incompressible_blocked(precision):
    """K/G = 1e6 on a 12^3 block: FP32 fronts above 256 rows (the blocked
    solve, its plain steps with compensated FP32 products, then GMRES with
    FP64 products), refined to 1e-12 and equal to SciPy's solution."""
    mesh = mg.solid81_block(12, 12, 12, 1.0 / 12, mg.MAT_NEO_HOOKEAN, (1.0, 1.0e6), clamp_z0=True)
    u, p = mg.twist_state(mesh, angle_deg=30.0, stretch=1.2, noise_frac=0.01, seed=4)
    s = _storage(mesh, u, p, None, True)
    solver, x = _check(s, precision, 1e-12, max_refine=60)
    assert solver.info()["max_front"] > 256
    assert solver.last_steps >= 2


@pytest.mark.parametrize("m", [200, 700])
def test_tensor_core_trailing_update_matches_fma(m):
    """The tcgen05 trailing update (split TF32, FP32 accumulation) against the
    FMA kernel on the same random front: FP32-level agreement."""
    from nla3d_gb300 import _lib
    out = np.zeros(2)
    assert _lib.load().nla3d_ldlt_tc_check(m, out.ctypes.data) == 0
    assert out[0] <= 1e-5 * out[1]


@pytest.mark.parametrize("name", ["cube4_nh_clamped", "bar_mpc_2x2x3", "quadth_lines_6x5"])
def test_tensor_core_fronts_small_cases(name):
    s = _storage(*cases.FULL_CASES[name]())
    _check(s, "fp32-tc", 1e-12)


def test_tensor_core_fronts_twisted_block():
    mesh = mg.solid81_block(12, 12, 12, 1.0 / 12, mg.MAT_MOONEY_RIVLIN, (0.4, 0.1, 2000.0),
                            clamp_z0=True)
    u, p = mg.twist_state(mesh, angle_deg=20.0, stretch=1.3, noise_frac=0.005, seed=2)
    s = _storage(mesh, u, p, None, True)
    solver, x = _check(s, "fp32-tc", 1e-12)
    assert solver.info()["max_front"] > 256
