"""Newton driver (nla3d_gb300.newton) on the CPU oracle backend: reproduces
the reference's own rigid-body MPC reaction-curve test."""
from nla3d_gb300.newton import NewtonSolver, TimeControl
from oracle import oracle as O

import rigid_body_case as rb


def test_time_control_matches_reference_stepping():
    tc = TimeControl()
    steps = 0
    while tc.next_step(1.0 / 20):
        steps += 1
    assert steps == 20 and abs(tc.t - 1.0) < 1e-12
    tc = TimeControl()
    ts = []
    while tc.next_step(0.3):        # 0.3, 0.6, then (1-0.6)/2 twice (FESolver.cpp:43-47)
        ts.append(round(tc.t, 12))
    assert ts == [0.3, 0.6, 0.8, 1.0]


def test_rigid_body_mpc_rotx_reaction_curve_oracle_backend():
    mesh, fixes, ref = rb.load_case()
    m = O.OracleModel(mesh, "port")
    s = NewtonSolver(m, fixes, n_loadsteps=20, n_iterations=15).solve()
    err = rb.curve_error(s, mesh, ref)
    assert err < rb.THRESHOLD, err


def test_residual_criterion_converges_quadratically_and_keeps_the_curve():
    mesh, fixes, ref = rb.load_case()
    s = NewtonSolver(O.OracleModel(mesh, "port"), fixes, n_loadsteps=20, n_iterations=25,
                     residual_tol=1e-10).solve()
    assert rb.curve_error(s, mesh, ref) < rb.THRESHOLD
    for rec in s.records:
        assert rec.residuals[-1] < 1e-10 and rec.iterations <= 4
