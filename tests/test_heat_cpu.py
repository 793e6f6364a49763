"""The reference's QUADTH heat-transfer tests (test/QUADTH_test.cpp,
test/QUADTH_transient.cpp) run on the oracle backend: the steady solution
matches ANSYS within the reference's own 1e-3 at every node, and the
transient probe history within its average-error bound 5e-2."""
import numpy as np

import cases
from nla3d_gb300 import meshgen as mg
from nla3d_gb300.linear import LinearFESolver, LinearTransientFESolver
from oracle import oracle as O


def test_steady_heat_matches_ansys():
    mesh, loads, probe, g = cases.heat_model()
    s = LinearFESolver(O.OracleModel(mesh, "port"), loads=loads)
    s.solve()
    T = np.array([s.node_solution(n, mg.TEMP) for n in range(1, mesh.n_nodes + 1)])
    assert np.abs(T - g["ansys_temp"]).max() < 1e-3


def test_transient_heat_probe_matches_ansys():
    mesh, loads, probe, g = cases.heat_model(transient=True)
    s = LinearTransientFESolver(O.OracleModel(mesh, "port"), loads=loads)
    s.time1, s.numberOfTimesteps, s.initValue = 30000.0, 100, -6.0
    t, v = s.solve(probes=[(probe, mg.TEMP)])
    assert t.size == 100 and np.allclose(t, g["ansys_time"])
    assert np.abs(v[:, 0] - g["ansys_probe"]).mean() < 5e-2
