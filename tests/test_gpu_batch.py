"""Batched assembly on the GPU: one launch per kernel over many meshes, CUDA
graph replay and the autotuner must all give exactly the per-mesh results of
the single-mesh path (bitwise: the same kernels do the same arithmetic per
element and per CSR slot, whatever the launch shape)."""
import numpy as np
import pytest

from nla3d_gb300 import meshgen as mg
from nla3d_gb300.batch import BatchAssembly
from nla3d_gb300.storage import assemble_state

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint64)


def _batch_and_states(precision):
    from test_batch_host import small_batch
    meshes = small_batch()
    states = []
    for i, m in enumerate(meshes):
        u, p = mg.twist_state(m, angle_deg=10.0 + i, stretch=1.2, noise_frac=0.01, seed=i)
        extra = None
        if m.rigid_bodies:
            extra = {(m.n_nodes, mg.UZ): 0.3, (m.n_nodes, mg.ROTZ): 0.2}
        states.append((u, p, extra))
    b = BatchAssembly(meshes, precision).init()
    return meshes, states, b


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_equals_single_mesh_results(precision):
    meshes, states, b = _batch_and_states(precision)
    b.set_U(b.state_vector(states))
    b.update()
    b.assemble()
    K, F = b.K_all(), b.F()
    assert b.element_status() == (0, 0)
    for i, (m, st) in enumerate(zip(meshes, states)):
        _, _, Ks, Fs = assemble_state(m, st[0], st[1], precision, st[2])
        for blk in (1, 12, 2):
            assert np.array_equal(_bits(b.mesh_K(K, i, blk)), _bits(Ks[blk])), (i, blk)
        assert np.array_equal(_bits(b.mesh_F(F, i)), _bits(Fs)), i


def test_graph_replay_and_autotune_keep_results_bitwise():
    meshes, states, b = _batch_and_states("mixed")
    U = b.state_vector(states)
    b.set_U(U)
    b.update()
    b.assemble()
    K0, F0 = b.K_all(), b.F()
    tuned = b.autotune(reps=2)
    assert tuned["warps_per_block"] in (2, 4, 8) and tuned["gather_block"] in (128, 256, 512, 1024)
    b.update()
    b.assemble()
    assert np.array_equal(_bits(b.K_all()), _bits(K0))
    b.capture_graph()
    for _ in range(3):
        b.graph_launch()
    b.synchronize()
    assert np.array_equal(_bits(b.K_all()), _bits(K0))
    assert np.array_equal(_bits(b.F()), _bits(F0))
    # a new vecU is picked up by the replay (the graph reads the U buffer)
    b.set_U(0.5 * U)
    b.graph_launch()
    b.synchronize()
    assert not np.array_equal(_bits(b.K_all()), _bits(K0))
