"""The reference's TETRA0_test (test/TETRA0_test.cpp on test/TETRA0/tetra.cdb):
linear elastic TETRA0 through LinearFESolver; the nodal displacements match
ANSYS within the test's 1e-10 and the element stresses (TETRA0::update) within
its 1e-3, on the oracle backend (CPU) and with the assembly on the GPU."""
import numpy as np
import pytest

import cases
from nla3d_gb300 import meshgen as mg
from nla3d_gb300.linear import LinearFESolver
from oracle import oracle as O


def _solve(backend, fixes, loads, solver="host"):
    s = LinearFESolver(backend, fixes=fixes, loads=loads, solver=solver)
    s.solve()
    ne, _ = backend.eq_numbers()
    U = s.U
    disp = np.stack([U[ne[:, d].astype(np.int64) - 1] for d in (mg.UX, mg.UY, mg.UZ)], axis=1)
    return U, disp


def _stress(mesh, U):
    o = O.OracleModel(mesh, "port")
    o.set_U(U)
    return o.tetra0_stress()


def test_tetra0_matches_ansys_on_the_oracle():
    mesh, fixes, loads, g = cases.tetra0_ansys_model()
    U, disp = _solve(O.OracleModel(mesh, "port"), fixes, loads)
    assert np.abs(disp - g["ansys_disp"]).max() < 1e-10
    assert np.abs(_stress(mesh, U) - g["ansys_stress"]).max() < 1e-3


@pytest.mark.gpu
def test_tetra0_matches_ansys_with_gpu_assembly():
    from nla3d_gb300.storage import FEStorage
    mesh, fixes, loads, g = cases.tetra0_ansys_model()
    U, disp = _solve(FEStorage(mesh).initSolutionData(), fixes, loads)
    assert np.abs(disp - g["ansys_disp"]).max() < 1e-10
    assert np.abs(_stress(mesh, U) - g["ansys_stress"]).max() < 1e-3


@pytest.mark.gpu
@pytest.mark.parametrize("solver", ["gpu", "gpu-fp32"])
def test_tetra0_matches_ansys_with_the_device_solve(solver):
    """The same test with K(2) factored on the device (LinearFESolver(solver=...))."""
    from nla3d_gb300.storage import FEStorage
    mesh, fixes, loads, g = cases.tetra0_ansys_model()
    U, disp = _solve(FEStorage(mesh).initSolutionData(), fixes, loads, solver)
    assert np.abs(disp - g["ansys_disp"]).max() < 1e-10
    assert np.abs(_stress(mesh, U) - g["ansys_stress"]).max() < 1e-3
