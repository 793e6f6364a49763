"""The reference's a2000_damper BENCH (test/CMakeLists.txt:141-146) end to
end with the GPU assembly: 3101 PLANE41 from the reference's a2000.cdb
(tests/golden/a2000_plane41.npz), Neo-Hookean (1, 500), 20 load steps, UY
reaction of DISP_BC against the ANSYS curve with the test's threshold 0.2
(main.cpp compareCurves).  FP64 and mixed give the CPU oracle's iterations
and curve."""
import numpy as np
import pytest

import bench
from nla3d_gb300.newton import NewtonSolver
from nla3d_gb300.storage import FEStorage

pytestmark = pytest.mark.gpu


def _run(backend):
    mesh, fixes, nodes, ref, thr = bench.cdb_model("a2000")
    if backend == "port":
        from oracle import oracle as O
        b = O.OracleModel(mesh, "port")
    else:
        b = FEStorage(mesh, backend).initSolutionData()
    s = NewtonSolver(b, fixes, n_loadsteps=20, n_iterations=15, kinematic_tol=1e-3,
                     solver="nd").solve()
    ne = s.ne
    curve = np.array([sum(r[int(ne[n - 1, 1]) - 1] for n in nodes) for r in s.reactions])
    return s, curve, ref, thr


def test_a2000_plane41_curve_within_reference_threshold():
    runs = {k: _run(k) for k in ("fp64", "mixed", "port")}
    for k, (s, curve, ref, thr) in runs.items():
        assert np.abs(curve - ref).mean() < thr, k
    its = {k: [r.iterations for r in v[0].records] for k, v in runs.items()}
    assert its["fp64"] == its["port"] and its["mixed"] == its["port"]
    c64, cport = runs["fp64"][1], runs["port"][1]
    assert np.abs(c64 - cport).max() <= 1e-8 * np.abs(cport).max()
