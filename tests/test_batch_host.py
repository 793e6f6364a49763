"""Batch context, host side (no GPU): each mesh of a batch keeps exactly the
numbering and CSR pattern it gets on its own (one reference FEStorage each)."""
import numpy as np

import cases
from nla3d_gb300 import meshgen as mg
from nla3d_gb300.batch import BatchAssembly
from nla3d_gb300.storage import FEStorage


def small_batch():
    out = []
    for i, (n, clamp) in enumerate([((2, 3, 2), False), ((3, 1, 2), True), ((1, 1, 1), False),
                                    ((2, 2, 3), True)]):
        mat = [(mg.MAT_NEO_HOOKEAN, (1.0 + i, 900.0)), (mg.MAT_MOONEY_RIVLIN, (0.4, 0.1, 2000.0))][i % 2]
        out.append(mg.solid81_block(*n, 0.5, mat[0], mat[1], clamp_z0=clamp))
    out.append(mg.solid81_bar_mpc(2, 2, 3, 1.0))
    # meshes with linear (CE) MPC equations, one of them also with a rigid body
    out.append(cases.ce_block_3x3x2()[0])
    out.append(cases.bar_mpc_ce_2x2x3()[0])
    return out


def test_batch_pattern_equals_single_mesh_patterns():
    meshes = small_batch()
    b = BatchAssembly(meshes, "fp64").build_pattern()
    for i, m in enumerate(meshes):
        s = FEStorage(m).buildPattern()
        ne1, ee1 = b.eq_numbers(i)
        ne2, ee2 = s.eq_numbers()
        assert np.array_equal(ne1, ne2) and np.array_equal(ee1, ee2)
        for blk in (1, 12, 2):
            a, c = b.pattern(i, blk), s.pattern(blk)
            assert np.array_equal(a[0], c[0]) and np.array_equal(a[1], c[1])
    # offsets are the running sums of the meshes' sizes
    sizes = [FEStorage(m).buildPattern().n_total for m in meshes]
    assert list(b.u_off) == list(np.concatenate([[0], np.cumsum(sizes)]))


def test_batched_workload_generator_is_seeded():
    a = mg.batched_meshes(6, seed=3)
    b = mg.batched_meshes(6, seed=3)
    for (m1, u1, p1), (m2, u2, p2) in zip(a, b):
        assert m1.n_elems == m2.n_elems and np.array_equal(u1, u2) and np.array_equal(p1, p2)
        assert m1.mat_c == m2.mat_c
