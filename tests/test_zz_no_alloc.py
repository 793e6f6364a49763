"""nla3d_assemble_solid81_noalloc: the SOLID81 assembly for callers that may
not allocate device memory (a host framework that owns every device byte
through its own pool, or a time-critical loop that cannot pay for
cudaMalloc's implicit synchronisation).  The caller owns all inputs and
outputs; the library's only intermediate storage is its fixed scratch array.

Checked through the C ABI against the context path (nla3d_assemble) at the
FP64 parity tolerance, on two calls in a row with different states -- the
second call must not see anything the first one left in the shared scratch.
This file is collected last so that a failure here does not hide the others;
it also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from nla3d_gb300 import _lib
from nla3d_gb300 import meshgen as mg
from nla3d_gb300.storage import FEStorage

pytestmark = pytest.mark.gpu
TOL_FP64 = 1e-12


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def inverse_lists(slot, n_slots):
    """Gather lists from an element -> slot map: ascending contribution ids per slot."""
    flat = slot.ravel()
    ids = np.argsort(flat, kind="stable").astype(np.uint32)
    ptr = np.zeros(n_slots + 1, np.uint32)
    ptr[1:] = np.cumsum(np.bincount(flat, minlength=n_slots))
    return ptr, ids


def context_result(mesh, U):
    s = FEStorage(mesh, "fp64").initSolutionData()
    s.setU(U)
    s.updateResults()
    s.assembleGlobalEqMatrices()
    K = np.concatenate([s.K(b) for b in (1, 12, 2)])
    return K, s.F()


def test_noalloc_matches_context_path_on_two_calls():
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    mesh, u, p = mg.config_cube(10, seed=1)            # 1000 SOLID81 elements
    host = FEStorage(mesh).buildPattern()              # host-only: numbering, pattern, slot maps
    ne, ee = host.eq_numbers()
    ks, fs = host.slot_maps()
    nnz = sum(host.blocks[b][2] for b in (1, 12, 2))
    n_eq = host.n_total
    k_ptr, k_ids = inverse_lists(ks, nnz)
    f_ptr, f_ids = inverse_lists(fs, n_eq)
    node_eq = np.zeros((mesh.n_nodes, 4), np.uint32)
    node_eq[:, :3] = ne[:, :3]
    p_eq = ee[:, mg.HYDRO_PRESSURE].copy()

    dev = torch.device("cuda:0")
    # every device buffer belongs to the caller (here: torch's allocator)
    as_t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    d_xyz = as_t(mesh.xyz.astype(np.float64))
    d_conn = as_t(mesh.conn.astype(np.int32))
    d_neq = as_t(node_eq.astype(np.int32))
    d_peq = as_t(p_eq.astype(np.int32))
    d_kptr, d_kids = as_t(k_ptr.astype(np.int32)), as_t(k_ids.astype(np.int32))
    d_fptr, d_fids = as_t(f_ptr.astype(np.int32)), as_t(f_ids.astype(np.int32))
    d_K = torch.empty(nnz, dtype=torch.float64, device=dev)
    d_F = torch.empty(n_eq, dtype=torch.float64, device=dev)
    assert d_neq.data_ptr() % 16 == 0

    states = [mg.u_to_vector(ne, ee, u, p, n_eq),
              mg.u_to_vector(ne, ee, 0.6 * u, p - 0.03, n_eq)]
    stream = torch.cuda.current_stream()
    for U in states:                                   # two calls in a row
        d_U = as_t(U)
        a = _lib.NoAllocArgs()
        a.n_elems, a.n_nodes, a.n_eq, a.nnz = mesh.n_elems, mesh.n_nodes, n_eq, nnz
        a.xyz, a.conn, a.node_eq, a.p_eq = (d_xyz.data_ptr(), d_conn.data_ptr(),
                                            d_neq.data_ptr(), d_peq.data_ptr())
        a.U = d_U.data_ptr()
        a.k_ptr, a.k_ids = d_kptr.data_ptr(), d_kids.data_ptr()
        a.f_ptr, a.f_ids = d_fptr.data_ptr(), d_fids.data_ptr()
        a.mat_id = mesh.mat_id
        for i, c in enumerate(mesh.mat_c):
            a.mat_c[i] = c
        a.K, a.F = d_K.data_ptr(), d_F.data_ptr()
        flagged = ctypes.c_uint32(99)
        rc = lib.nla3d_assemble_solid81_noalloc(ctypes.byref(a),
                                                ctypes.c_void_p(stream.cuda_stream),
                                                ctypes.byref(flagged))
        assert rc == _lib.NLA3D_OK and flagged.value == 0
        torch.cuda.synchronize()
        K_ref, F_ref = context_result(mesh, U)
        assert rel(d_K.cpu().numpy(), K_ref) <= TOL_FP64
        assert rel(d_F.cpu().numpy(), F_ref) <= TOL_FP64


def test_noalloc_rejects_meshes_larger_than_its_scratch():
    lib = _lib.load()
    a = _lib.NoAllocArgs()
    a.n_elems = _lib.NOALLOC_MAX_ELEMS + 1
    rc = lib.nla3d_assemble_solid81_noalloc(ctypes.byref(a), None, None)
    assert rc == 5  # NLA3D_ERR_RANGE, before any pointer is looked at
