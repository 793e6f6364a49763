"""The reference's QUADTH heat-transfer tests (test/QUADTH_test.cpp,
test/QUADTH_transient.cpp) with the assembly on the GPU: QUADTH conduction
and capacity, SurfaceLINETH convection, the .cdb HEAT load.  The steady
temperatures match ANSYS within the reference's 1e-3 at every node and the
oracle-backend solution to 1e-10; the transient probe history matches ANSYS
within the reference's average-error bound 5e-2 and the oracle to 1e-10."""
import numpy as np
import pytest

import cases
from nla3d_gb300 import meshgen as mg
from nla3d_gb300.linear import LinearFESolver, LinearTransientFESolver
from nla3d_gb300.storage import FEStorage
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _steady(backend, loads, solver="host"):
    s = LinearFESolver(backend, loads=loads, solver=solver)
    return s.solve().copy()


@pytest.mark.parametrize("solver", ["host", "gpu", "gpu-fp32"])
def test_steady_heat_gpu_matches_ansys_and_oracle(solver):
    """solver: the K(2) solve by SciPy or by the device LDL^T (FP64 or FP32
    fronts, refined in FP64)."""
    mesh, loads, probe, g = cases.heat_model()
    st = FEStorage(mesh).initSolutionData()
    U = _steady(st, loads, solver)
    Uo = _steady(O.OracleModel(mesh, "port"), loads)
    ne, _ = st.eq_numbers()
    T = U[ne[:, mg.TEMP].astype(np.int64) - 1]
    assert np.abs(T - g["ansys_temp"]).max() < 1e-3
    assert np.abs(U - Uo).max() <= 1e-10 * np.abs(Uo).max()


def _transient(backend, loads, probe, solver="host"):
    s = LinearTransientFESolver(backend, loads=loads, solver=solver)
    s.time1, s.numberOfTimesteps, s.initValue = 30000.0, 100, -6.0
    return s.solve(probes=[(probe, mg.TEMP)])


@pytest.mark.parametrize("solver", ["host", "gpu", "gpu-fp32"])
def test_transient_heat_gpu_matches_ansys_and_oracle(solver):
    mesh, loads, probe, g = cases.heat_model(transient=True)
    st = FEStorage(mesh).initSolutionData()
    t, v = _transient(st, loads, probe, solver)
    _, vo = _transient(O.OracleModel(mesh, "port"), loads, probe)
    assert t.size == 100 and np.abs(v[:, 0] - g["ansys_probe"]).mean() < 5e-2
    assert np.abs(v - vo).max() <= 1e-10 * np.abs(vo).max()
