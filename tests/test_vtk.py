"""VTK output (nla3d_gb300/vtk.py) against the reference's own VtkProcessor
(VtkProcessor.cpp): the committed fixtures were written by the compiled
reference (tests/golden/make_golden.py, pre() and process(7)); our writer
reproduces them byte for byte from the same vecU / vecR, with the DoF
numbering of the oracle and of the library's host pattern builder."""
import os

import numpy as np
import pytest

import cases
import make_golden as G
from nla3d_gb300.storage import FEStorage
from nla3d_gb300.vtk import VtkProcessor
from oracle import oracle as O

GOLDEN = os.path.dirname(os.path.abspath(G.__file__))


@pytest.mark.parametrize("backend", ["oracle", "library"])
@pytest.mark.parametrize("name", G.VTK_CASES)
def test_matches_reference_vtk_files(name, backend, tmp_path):
    mesh, U, R = G.vtk_state(name)
    be = O.OracleModel(mesh, "port") if backend == "oracle" else FEStorage(mesh).buildPattern()
    v = VtkProcessor(be, str(tmp_path / "out"))
    v.pre(U, R)
    v.process(7, U, R)
    for step in (0, 7):
        want = open(os.path.join(GOLDEN, f"vtk_{name}_{step}.vtk")).read()
        got = (tmp_path / f"out{step}.vtk").read_text()
        assert got == want, (name, step)


def test_live_reference_on_another_state(tmp_path):
    """With the compiled reference present: a different state (larger values,
    negative zeros, exponents) of the rigid-body case, both writers."""
    if not O.ref_available():
        pytest.skip("compiled reference not built here")
    mesh, U, R = G.vtk_state("bar_mpc_2x2x3")
    U = U * 1.0e7 - 3.0
    U[::7] = -0.0
    R = R * 1e-9
    ref = O.OracleModel(mesh, "ref")
    ref.write_vtk(str(tmp_path / "ref"), 2, U, R)
    v = VtkProcessor(O.OracleModel(mesh, "port"), str(tmp_path / "ours"))
    v.process(2, U, R)
    assert (tmp_path / "ours2.vtk").read_text() == (tmp_path / "ref2.vtk").read_text()
