"""Edge cases of the set-up, against the reference where it is built here
(else the oracle): an empty model and a connectivity or constraint that
names something missing are rejected with a status and a message (the
reference aborts with the same condition); a node no element uses gets no
DoF; a single element, a model whose every nodal DoF is constrained, and
very uneven batches keep the reference's numbering and pattern."""
import numpy as np
import pytest

import cases
from nla3d_gb300 import _lib
from nla3d_gb300 import meshgen as mg
from nla3d_gb300.batch import BatchAssembly
from nla3d_gb300.storage import FEStorage
from oracle import oracle as O

REF = "ref" if O.ref_available() else "port"


def _same_setup(mesh):
    s = FEStorage(mesh).buildPattern()
    r = O.OracleModel(mesh, REF)
    assert [s.n_dofs, s.n_con, s.n_unk, s.n_mpc] == [r.n_dofs, r.n_con, r.n_unk, r.n_mpc]
    for a, b in zip(s.eq_numbers(), r.eq_numbers()):
        assert np.array_equal(a, b)
    for blk in (1, 12, 2):
        (io, co), (rio, rco) = s.pattern(blk), r.pattern(blk)
        assert np.array_equal(io, rio) and np.array_equal(co, rco)
    return s


def test_empty_model_is_rejected():
    m = mg.Mesh(mg.ELEM_SOLID81, np.zeros((0, 3)), np.zeros((0, 8), np.uint32), mat_id=1,
                mat_c=(1.0, 100.0))
    with pytest.raises(_lib.Nla3dError, match="No any nodes or elements"):
        FEStorage(m).buildPattern()
    with pytest.raises(O.OracleError, match="No any nodes or elements"):
        O.OracleModel(m, REF)


def test_missing_node_and_unused_dof_are_rejected():
    m = mg.solid81_block(1, 1, 1, 1.0, clamp_z0=False)
    m.conn = m.conn.copy()
    m.conn[0, 0] = 99
    with pytest.raises(_lib.Nla3dError):
        FEStorage(m).buildPattern()
    m = cases.cube3_nh()[0]
    m.fix_nodes, m.fix_dofs = np.array([1], np.uint32), np.array([mg.TEMP], np.int32)
    with pytest.raises(_lib.Nla3dError, match="unregistered DoF"):
        FEStorage(m).buildPattern()


def test_unused_node_single_element_and_all_fixed():
    m = cases.cube3_nh()[0]
    m.xyz = np.vstack([m.xyz, [[9.0, 9.0, 9.0]]])           # a node no element uses
    s = _same_setup(m)
    assert not s.eq_numbers()[0][-1].any()
    _same_setup(mg.solid81_block(1, 1, 1, 1.0, clamp_z0=False))
    _same_setup(mg.tetra0_block(1, 1, 1, 1.0, clamp_z0=False))
    m = cases.cube3_nh()[0]
    m.fix_nodes = np.repeat(np.arange(1, m.n_nodes + 1, dtype=np.uint32), 3)
    m.fix_dofs = np.tile(np.array([mg.UX, mg.UY, mg.UZ], np.int32), m.n_nodes)
    s = _same_setup(m)
    assert s.n_unk == m.n_elems                             # only the pressures are free


def test_uneven_batch_keeps_each_mesh_pattern():
    meshes = [mg.solid81_block(1, 1, 1, 1.0, clamp_z0=True), mg.solid81_block(9, 2, 5, 0.3),
              mg.solid81_block(1, 7, 1, 0.5, clamp_z0=True)]
    b = BatchAssembly(meshes, "fp64").build_pattern()
    for i, m in enumerate(meshes):
        r = O.OracleModel(m, REF)
        for blk in (1, 12, 2):
            io, co = b.pattern(i, blk)
            rio, rco = r.pattern(blk)
            assert np.array_equal(io, rio) and np.array_equal(co, rco)


def test_mixed_precision_rejects_inputs_outside_the_float_range():
    """The mixed SOLID81 kernel computes in floats and float pairs: a mesh
    whose material constants or extent leave the range it supports is
    rejected at nla3d_create (NLA3D_ERR_RANGE); FP64 takes the same mesh."""
    big = mg.solid81_block(1, 1, 1, 1.0, mg.MAT_MOONEY_RIVLIN, (4e22, 1e22, 2e24))
    tiny = mg.solid81_block(1, 1, 1, 1e-8, mg.MAT_NEO_HOOKEAN, (1.0, 100.0))
    for m in (big, tiny):
        with pytest.raises(_lib.Nla3dError) as ei:
            FEStorage(m, "mixed")
        assert ei.value.code == 5
        FEStorage(m, "fp64").buildPattern()
    FEStorage(mg.solid81_block(1, 1, 1, 1.0), "mixed").buildPattern()
