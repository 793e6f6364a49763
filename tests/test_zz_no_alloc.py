"""nla3d_assemble_solid81_noalloc: the SOLID81 assembly for callers that may
not allocate device memory (a host framework that owns every device byte
through its own pool, or a time-critical loop that cannot pay for
cudaMalloc's implicit synchronisation).  The caller owns all inputs and
outputs; the library's only intermediate storage is its fixed scratch array.

Checked through the C ABI against the context path (nla3d_assemble) at the
FP64 parity tolerance, on two calls in a row with different states -- the
second call must not see anything the first one left in the shared scratch --
and on a smaller mesh after a larger one.  The status word that every call
clears is checked by a call with inverted elements followed by a clean one,
and the device-side input check by a connectivity id past the last node
(nothing is written, the call reports NLA3D_ERR_ARG, the next call is clean).
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
NLA3D_ERR_ARG, NLA3D_ERR_ELEMENT = 1, 6


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


class CallerBuffers:
    """Everything the caller owns on the device for one mesh (allocated by
    torch's allocator here, standing in for a host framework's pool)."""

    def __init__(self, torch, mesh, conn=None):
        host = FEStorage(mesh).buildPattern()          # host-only: numbering, pattern, slot maps
        self.ne, self.ee = host.eq_numbers()
        ks, fs = host.slot_maps()
        self.mesh = mesh
        self.nnz = sum(host.blocks[b][2] for b in (1, 12, 2))
        self.n_eq = host.n_total
        k_ptr, k_ids = inverse_lists(ks, self.nnz)
        f_ptr, f_ids = inverse_lists(fs, self.n_eq)
        node_eq = np.zeros((mesh.n_nodes, 4), np.uint32)
        node_eq[:, :3] = self.ne[:, :3]
        p_eq = self.ee[:, mg.HYDRO_PRESSURE].copy()
        dev = torch.device("cuda:0")
        self.as_t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
        self.xyz = self.as_t(mesh.xyz.astype(np.float64))
        self.conn = self.as_t((mesh.conn if conn is None else conn).astype(np.int32))
        self.neq = self.as_t(node_eq.astype(np.int32))
        self.peq = self.as_t(p_eq.astype(np.int32))
        self.kptr, self.kids = self.as_t(k_ptr.astype(np.int32)), self.as_t(k_ids.astype(np.int32))
        self.fptr, self.fids = self.as_t(f_ptr.astype(np.int32)), self.as_t(f_ids.astype(np.int32))
        self.K = torch.empty(self.nnz, dtype=torch.float64, device=dev)
        self.F = torch.empty(self.n_eq, dtype=torch.float64, device=dev)
        assert self.neq.data_ptr() % 16 == 0

    def U(self, u, p):
        return mg.u_to_vector(self.ne, self.ee, u, p, self.n_eq)

    def call(self, lib, torch, U):
        d_U = self.as_t(U)
        a = _lib.NoAllocArgs()
        m = self.mesh
        a.n_elems, a.n_nodes, a.n_eq, a.nnz = m.n_elems, m.n_nodes, self.n_eq, self.nnz
        a.xyz, a.conn, a.node_eq, a.p_eq = (self.xyz.data_ptr(), self.conn.data_ptr(),
                                            self.neq.data_ptr(), self.peq.data_ptr())
        a.U = d_U.data_ptr()
        a.k_ptr, a.k_ids = self.kptr.data_ptr(), self.kids.data_ptr()
        a.f_ptr, a.f_ids = self.fptr.data_ptr(), self.fids.data_ptr()
        a.mat_id = m.mat_id
        for i, c in enumerate(m.mat_c):
            a.mat_c[i] = c
        a.K, a.F = self.K.data_ptr(), self.F.data_ptr()
        flagged = ctypes.c_uint32(99)
        stream = torch.cuda.current_stream()
        rc = lib.nla3d_assemble_solid81_noalloc(ctypes.byref(a),
                                                ctypes.c_void_p(stream.cuda_stream),
                                                ctypes.byref(flagged))
        torch.cuda.synchronize()
        return rc, flagged.value


def test_noalloc_matches_context_path_on_two_calls():
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    mesh, u, p = mg.config_cube(10, seed=1)            # 1000 SOLID81 elements
    buf = CallerBuffers(torch, mesh)
    for U in (buf.U(u, p), buf.U(0.6 * u, p - 0.03)):  # two calls in a row
        rc, flagged = buf.call(lib, torch, U)
        assert rc == _lib.NLA3D_OK and flagged == 0
        K_ref, F_ref = context_result(mesh, U)
        assert rel(buf.K.cpu().numpy(), K_ref) <= TOL_FP64
        assert rel(buf.F.cpu().numpy(), F_ref) <= TOL_FP64
    # a smaller mesh after the larger one: it must read none of the first
    # call's scratch
    small, us, ps = mg.config_cube(4, seed=5)
    sb = CallerBuffers(torch, small)
    U = sb.U(us, ps)
    rc, flagged = sb.call(lib, torch, U)
    assert rc == _lib.NLA3D_OK and flagged == 0
    K_ref, F_ref = context_result(small, U)
    assert rel(sb.K.cpu().numpy(), K_ref) <= TOL_FP64
    assert rel(sb.F.cpu().numpy(), F_ref) <= TOL_FP64


def test_noalloc_status_cleared_between_calls():
    """Inverted elements are flagged (NLA3D_ERR_ELEMENT), and the next clean
    call reports none: the status word is cleared by every call."""
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    mesh, u, p = mg.config_cube(6, seed=2)
    buf = CallerBuffers(torch, mesh)
    inverted = u.copy()
    inverted[:, 0] = -2.0 * mesh.xyz[:, 0]             # x -> -x: det F < 0 everywhere
    rc, flagged = buf.call(lib, torch, buf.U(inverted, p))
    assert rc == NLA3D_ERR_ELEMENT and flagged == mesh.n_elems
    U = buf.U(u, p)
    rc, flagged = buf.call(lib, torch, U)
    assert rc == _lib.NLA3D_OK and flagged == 0
    K_ref, F_ref = context_result(mesh, U)
    assert rel(buf.K.cpu().numpy(), K_ref) <= TOL_FP64


def test_noalloc_input_check_writes_nothing():
    """A node id past the last node is caught by the device-side input check:
    the call returns NLA3D_ERR_ARG and leaves K and F untouched; a valid call
    afterwards assembles normally."""
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    mesh, u, p = mg.config_cube(4, seed=3)
    conn = mesh.conn.copy()
    conn[5, 3] = mesh.n_nodes + 1
    bad = CallerBuffers(torch, mesh, conn=conn)
    bad.K.fill_(7.0)
    bad.F.fill_(7.0)
    rc, _ = bad.call(lib, torch, bad.U(u, p))
    assert rc == NLA3D_ERR_ARG
    assert bool((bad.K == 7.0).all()) and bool((bad.F == 7.0).all())
    good = CallerBuffers(torch, mesh)
    U = good.U(u, p)
    rc, flagged = good.call(lib, torch, U)
    assert rc == _lib.NLA3D_OK and flagged == 0
    K_ref, F_ref = context_result(mesh, U)
    assert rel(good.K.cpu().numpy(), K_ref) <= TOL_FP64
    assert rel(good.F.cpu().numpy(), F_ref) <= TOL_FP64


def test_noalloc_rejects_meshes_larger_than_its_scratch():
    lib = _lib.load()
    a = _lib.NoAllocArgs()
    a.n_elems = _lib.NOALLOC_MAX_ELEMS + 1
    rc = lib.nla3d_assemble_solid81_noalloc(ctypes.byref(a), None, None)
    assert rc == 5  # NLA3D_ERR_RANGE, before any pointer is looked at
