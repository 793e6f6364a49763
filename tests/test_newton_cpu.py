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
    # host time per phase: every phase accounted, the host solve none of the
    # device ones (factor / solve are the device LDL^T's)
    assert set(s.timing) == {"assemble", "factor", "solve", "update", "vectors"}
    assert all(v >= 0.0 for v in s.timing.values())
    assert s.timing["assemble"] > 0.0 and s.timing["factor"] == 0.0


def test_residual_criterion_converges_quadratically_and_keeps_the_curve():
    mesh, fixes, ref = rb.load_case()
    s = NewtonSolver(O.OracleModel(mesh, "port"), fixes, n_loadsteps=20, n_iterations=25,
                     residual_tol=1e-10).solve()
    assert rb.curve_error(s, mesh, ref) < rb.THRESHOLD
    for rec in s.records:
        assert rec.residuals[-1] < 1e-10 and rec.iterations <= 4


def test_nested_dissection_solve_gives_the_direct_iterates():
    """The geometric nested-dissection ordering changes only the fill of the
    host factorisation: a 3x3x8 bar clamped at z = 0 whose end face follows a
    rigid-body master pulled along z and twisted takes the same iterations
    and reaches the same state and reactions as the plain direct solve."""
    import numpy as np
    from nla3d_gb300 import meshgen as mg
    mesh = mg.solid81_bar_mpc(3, 3, 8, 1.0)
    master = mesh.n_nodes
    fixes = [(int(n), int(d), 0.0) for n, d in zip(mesh.fix_nodes, mesh.fix_dofs)]
    fixes += [(master, mg.UZ, 2.0), (master, mg.ROTZ, 0.5)]
    fixes += [(master, d, 0.0) for d in (mg.UX, mg.UY, mg.ROTX, mg.ROTY)]
    mesh.fix_nodes = np.concatenate([mesh.fix_nodes, np.full(6, master, np.uint32)])
    mesh.fix_dofs = np.concatenate([mesh.fix_dofs,
                                    np.array([mg.UZ, mg.ROTZ, mg.UX, mg.UY, mg.ROTX, mg.ROTY],
                                             np.int32)])
    runs = [NewtonSolver(O.OracleModel(mesh, "port"), fixes, n_loadsteps=5,
                         solver=solver).solve() for solver in ("direct", "nd")]
    assert [r.iterations for r in runs[0].records] == [r.iterations for r in runs[1].records]
    for a, b in zip(runs[0].reactions, runs[1].reactions):
        assert np.abs(a - b).max() <= 1e-8 * max(np.abs(a).max(), 1e-300)
    assert np.abs(runs[1].U - runs[0].U).max() <= 1e-8 * np.abs(runs[0].U).max()
    s = runs[1]
    assert s.nu + s.nm > 64                      # the ordering really splits
    assert sorted(s._perm.tolist()) == list(range(s.nu + s.nm))
