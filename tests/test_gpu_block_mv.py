"""GPU sparse block products (nla3d_block_mv) against the reference.

matBVprod / matBTVprod (SparseMatrix.cpp:497-558) on the assembled K, as the
Newton iteration uses them (FESolver.cpp:454-466): the GPU result must equal
the vectors that the compiled reference produced (tests/golden/*.npz, made by
tests/golden/make_golden.py) when the device K holds the reference's K values
(compared with ==, bit for bit up to the sign of a zero), and stay within
1e-12 of them on the GPU-assembled K; and equal the bit-exact CPU oracle on a
larger mesh.
"""
import os

import numpy as np
import pytest

import cases
from nla3d_gb300 import meshgen as mg
from nla3d_gb300.storage import FEStorage
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
MV_PRODUCTS = ((1, 0), (2, 0), (12, 0), (12, 1))


def _assembled(case, precision="fp64"):
    mesh, u, p, extra, do_update = case()
    s = FEStorage(mesh, precision).initSolutionData()
    ne, ee = s.eq_numbers()
    s.setU(mg.u_to_vector(ne, ee, u, p, s.n_total, extra))
    if do_update:
        s.updateResults()
    s.assembleGlobalEqMatrices()
    return s


class _DeviceView:
    """A device array of the library (pointer, length) as a torch tensor."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<f8", "data": (ptr, False),
                                         "version": 2}


def _load_reference_K(s, g):
    import torch
    torch.cuda.synchronize()
    s.synchronize()
    for blk in (1, 12, 2):
        ptr, n = s.device_K(blk)
        if n:
            dev = torch.as_tensor(_DeviceView(ptr, n), device="cuda")
            dev.copy_(torch.from_numpy(np.ascontiguousarray(g[f"K_{blk}"])))
    torch.cuda.synchronize()


@pytest.mark.parametrize("name", sorted(cases.FULL_CASES))
def test_block_products_bitwise_on_reference_K(name):
    """With the reference's own K values in the device K, every product
    equals the reference's vector (compared with ==)."""
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    s = _assembled(cases.FULL_CASES[name])
    _load_reference_K(s, g)
    coef = float(g["mv_coef"])
    for blk, trans in MV_PRODUCTS:
        x, y0 = g[f"mv_{blk}_{trans}_x"], g[f"mv_{blk}_{trans}_y0"]
        if y0.size == 0:
            continue
        y = s.block_mv(blk, trans, x, coef, y0)
        assert np.array_equal(y, g[f"mv_{blk}_{trans}_y"]), (blk, trans)


@pytest.mark.parametrize("name", sorted(cases.FULL_CASES))
def test_block_products_on_gpu_K_within_tolerance(name):
    """On the GPU-assembled K (<= 1e-12 from the reference's) the products
    stay within 1e-12 of the reference's vectors, relative to max |y|."""
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    s = _assembled(cases.FULL_CASES[name])
    coef = float(g["mv_coef"])
    for blk, trans in MV_PRODUCTS:
        x, y0 = g[f"mv_{blk}_{trans}_x"], g[f"mv_{blk}_{trans}_y0"]
        if y0.size == 0:
            continue
        y = s.block_mv(blk, trans, x, coef, y0)
        want = g[f"mv_{blk}_{trans}_y"]
        assert np.abs(y - want).max() <= 1e-12 * np.abs(want).max(), (blk, trans)


def test_block_products_twisted_block_vs_oracle():
    """8x7x9 twisted Mooney-Rivlin block clamped at z = 0 (all three blocks
    populated), the oracle's K loaded into the device K: GPU == oracle port
    for every product, twice in a row (the walk lists are built once and
    reused)."""
    mesh = mg.solid81_block(8, 7, 9, 0.2, mg.MAT_MOONEY_RIVLIN, (0.4, 0.1, 2000.0),
                            clamp_z0=True)
    u, p = mg.twist_state(mesh, angle_deg=25.0, stretch=1.3, noise_frac=0.01, seed=21)
    s = _assembled(lambda: (mesh, u, p, None, True))
    m = O.OracleModel(mesh, "port")
    ne, ee = m.eq_numbers()
    m.set_U(mg.u_to_vector(ne, ee, u, p, m.n_total))
    m.update()
    m.assemble()
    _load_reference_K(s, {f"K_{b}": m.K(b) for b in (1, 12, 2)})
    rng = np.random.default_rng(3)
    for blk, trans in MV_PRODUCTS:
        rows, cols, _ = m.blocks[blk]
        nx = cols if (blk == 12 and not trans) else rows
        ny = cols if (blk == 12 and trans) else rows
        for rep in range(2):
            x = rng.standard_normal(nx)
            x[::5] = 0.0
            y0 = rng.standard_normal(ny)
            assert np.array_equal(s.block_mv(blk, trans, x, 0.75, y0),
                                  m.block_mv(blk, trans, x, 0.75, y0)), (blk, trans, rep)


def test_block_mv_rejects_bad_arguments():
    s = _assembled(cases.cube3_nh)
    with pytest.raises(Exception):
        s.block_mv_device(7, 0, 0, 1.0, 0)
    with pytest.raises(Exception):
        s.block_mv_device(12, 2, 0, 1.0, 0)
