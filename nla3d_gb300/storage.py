"""Python front end of the GPU assembly, shaped like the reference's FEStorage.

The method names follow FEStorage (FEStorage.h:38-378) so that code written
against the reference reads the same:

    s = FEStorage(mesh)                  # nodes, elements, material (createNodes/createElements)
    s.setConstrainedNodeDof(node, dof)   # FEStorage.h:159
    s.addMpcCollection(rigid_body)       # FEStorage.h:200
    s.initSolutionData()                 # initDofs + assignEquationNumbers + initSolutionData
    s.setU(U)                            # writes vecU (getU(), FEStorage.h:109)
    s.updateResults()                    # FEStorage.h:270
    s.assembleGlobalEqMatrices()         # FEStorage.h:115
    K = s.getK(); K.block(2).getValuesArray(); s.getF()

All work runs in libnla3d_gpu.so through its C ABI (include/nla3d_gpu.h);
there is no CPU fallback.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from . import meshgen as mg


def _p(a):
    return None if a is None else a.ctypes.data


class SparseBlock:
    """One CSR block of K (SparseMatrix.h:134-186): 1-based iofeir / columns."""

    def __init__(self, rows, cols, iofeir, columns, values):
        self.rows, self.cols = rows, cols
        self._iofeir, self._columns, self._values = iofeir, columns, values

    def getValuesArray(self):
        return self._values

    def getColumnsArray(self):
        return self._columns

    def getIofeirArray(self):
        return self._iofeir

    def nValues(self):
        return int(self._columns.size)

    def nRows(self):
        return self.rows

    def nColumns(self):
        return self.cols

    def to_scipy(self, symmetric_upper: bool):
        import scipy.sparse as sp
        ind = self._iofeir.astype(np.int64) - 1
        m = sp.csr_matrix((self._values, self._columns.astype(np.int64) - 1, ind),
                          shape=(self.rows, self.cols))
        if symmetric_upper:
            m = m + sp.triu(m, 1).T
        return m.tocsr()


class BlockSparseSymMatrix:
    """Host view of K = [block(1) block(1,2); . block(2)] (BlockSparseMatrix.h:39-69)."""

    def __init__(self, blocks):
        self._b = blocks

    def block(self, i, j=None):
        if j is None:
            return self._b[i]
        return self._b[12]


class FEStorage:
    def __init__(self, mesh: mg.Mesh, precision: str = "fp64", stream=None):
        self.lib = _lib.load()
        self.mesh = mesh
        self.precision = precision
        prec = {"fp64": _lib.PREC_FP64, "mixed": _lib.PREC_MIXED}[precision]
        self._xyz = np.ascontiguousarray(mesh.xyz, dtype=np.float64)
        self._conn = np.ascontiguousarray(mesh.conn, dtype=np.uint32)
        self._ep, n_ep = mg.elem_params_array(mesh)
        d = _lib.MeshDesc()
        d.elem_type = mesh.elem_type
        d.n_nodes = mesh.n_nodes
        d.n_elems = mesh.n_elems
        d.xyz = _p(self._xyz)
        d.conn = _p(self._conn)
        d.mat_id = mesh.mat_id
        for i, c in enumerate(mesh.mat_c[:5]):
            d.mat_c[i] = c
        d.elem_params = _p(self._ep)
        d.n_elem_params = n_ep
        h = ctypes.c_void_p()
        rc = self.lib.nla3d_create(ctypes.byref(d), prec, ctypes.byref(h))
        if rc:
            raise _lib.Nla3dError(rc, "nla3d_create rejected the mesh")
        self.h = h
        self.ready = False
        self.transient = False
        if stream is not None:
            self._check(self.lib.nla3d_set_stream(self.h, ctypes.c_void_p(stream)))
        if mesh.fix_nodes is not None and len(mesh.fix_nodes):
            self._add_fix(mesh.fix_nodes, mesh.fix_dofs)
        for q in mesh.mpcs:
            self.addMpc(q)
        for rb in mesh.rigid_bodies:
            self.addMpcCollection(rb)
        if mesh.lines is not None and mesh.lines.n:
            self.add_surface_lines(mesh.lines)
        if mesh.transient:
            self.setTransient(True)

    # ---- lifecycle ----
    def _check(self, rc):
        if rc:
            msg = self.lib.nla3d_last_error(self.h)
            raise _lib.Nla3dError(rc, msg.decode() if msg else "")

    def close(self):
        if getattr(self, "h", None):
            self.lib.nla3d_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- set-up (before initSolutionData) ----
    def _add_fix(self, nodes, dofs):
        n = np.ascontiguousarray(nodes, dtype=np.uint32)
        d = np.ascontiguousarray(dofs, dtype=np.int32)
        self._check(self.lib.nla3d_add_fix(self.h, n.size, _p(n), _p(d)))

    def setConstrainedNodeDof(self, node, dof):
        self._add_fix([node], [dof])

    def addMpc(self, q: mg.LinearMpc):
        """FEStorage::addMpc: a linear MPC equation (numbered before rigid-body ones)."""
        n = np.ascontiguousarray(q.nodes, dtype=np.uint32)
        d = np.ascontiguousarray(q.dofs, dtype=np.int32)
        cf = np.ascontiguousarray(q.coefs, dtype=np.float64)
        self._check(self.lib.nla3d_add_mpc(self.h, n.size, _p(n), _p(d), _p(cf), float(q.b)))

    def addMpcCollection(self, rb: mg.RigidBody):
        s = np.ascontiguousarray(rb.slaves, dtype=np.uint32)
        d = np.ascontiguousarray(np.asarray(rb.dofs, dtype=np.int32))
        self._check(self.lib.nla3d_add_rigid_body(self.h, rb.master, s.size, _p(s), d.size, _p(d)))

    def add_surface_lines(self, lines: mg.SurfaceLines):
        """SurfaceLINETH elements (convection htc to etemp, flux) created after
        the QUADTH elements."""
        c = np.ascontiguousarray(lines.conn, dtype=np.uint32)
        h = np.ascontiguousarray(lines.htc, dtype=np.float64)
        f = np.ascontiguousarray(lines.flux, dtype=np.float64)
        t = np.ascontiguousarray(lines.etemp, dtype=np.float64)
        self._check(self.lib.nla3d_add_surface_lines(self.h, lines.n, _p(c), _p(h), _p(f),
                                                     _p(t)))

    def setTransient(self, on: bool = True):
        """FEStorage::setTransient: assembly also builds C and M on K's pattern."""
        self._check(self.lib.nla3d_set_transient(self.h, 1 if on else 0))
        self.transient = bool(on)

    def set_pattern_builder(self, mode):
        """Where initSolutionData builds the pattern: "host", "device" or
        "auto" (device for single meshes of >= 65,536 elements)."""
        self._check(self.lib.nla3d_set_pattern_builder(self.h, {"host": 0, "device": 1,
                                                                 "auto": -1}[mode]))
        return self

    def pattern_on_device(self):
        return bool(self.lib.nla3d_pattern_on_device(self.h))

    def buildPattern(self):
        """Host-only: initDofs + assignEquationNumbers + the CSR pattern and slot maps."""
        self._check(self.lib.nla3d_build_pattern(self.h))
        self._read_info()
        return self

    def slot_maps(self):
        ks = np.zeros((self.mesh.n_elems, self.n_kc), np.uint32)
        fs = np.zeros((self.mesh.n_elems, max(self.n_fc, 1)), np.uint32)
        self._check(self.lib.nla3d_slot_maps(self.h, _p(ks), _p(fs)))
        return ks, fs[:, :self.n_fc]

    def initSolutionData(self):
        self._check(self.lib.nla3d_init_solution_data(self.h))
        self._read_info()
        self.ready = True
        return self

    def _read_info(self):
        info = np.zeros(16, np.uint32)
        self._check(self.lib.nla3d_info(self.h, _p(info)))
        self.n_dofs, self.n_con, self.n_unk, self.n_mpc = (int(v) for v in info[:4])
        self.blocks = {}
        for b, name in zip(range(3), (1, 12, 2)):
            self.blocks[name] = tuple(int(v) for v in info[4 + 3 * b: 7 + 3 * b])
        self.n_total = self.n_dofs + self.n_mpc
        self.n_kc, self.n_fc = int(info[13]), int(info[14])

    # ---- reference-shaped getters ----
    def nDofs(self):
        return self.n_dofs

    def nConstrainedDofs(self):
        return self.n_con

    def nUnknownDofs(self):
        return self.n_unk

    def nMpc(self):
        return self.n_mpc

    def eq_numbers(self):
        ne = np.zeros((self.mesh.n_nodes, 8), np.uint32)
        ee = np.zeros((self.mesh.n_elems, 8), np.uint32)
        self._check(self.lib.nla3d_eq_numbers(self.h, _p(ne), _p(ee)))
        return ne, ee

    def getNodeDofEqNumber(self, node, dof):
        return int(self.eq_numbers()[0][node - 1, dof])

    def getElementDofEqNumber(self, el, dof):
        return int(self.eq_numbers()[1][el - 1, dof])

    def pattern(self, block):
        rows, cols, nnz = self.blocks[block]
        io = np.zeros(rows + 1, np.uint32)
        co = np.zeros(max(nnz, 1), np.uint32)
        self._check(self.lib.nla3d_pattern(self.h, block, _p(io), _p(co)))
        return io, co[:nnz]

    # ---- per iteration ----
    def setU(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64)
        self._check(self.lib.nla3d_set_U(self.h, _p(U), U.size))

    def setU_device(self, ptr: int, n: int):
        self._check(self.lib.nla3d_set_U_device(self.h, ctypes.c_void_p(ptr), n))

    def updateResults(self):
        self._check(self.lib.nla3d_update_results(self.h))

    # short names shared with the oracle model (the Newton driver's backend API)
    def set_U(self, U):
        self.setU(U)

    def update(self):
        self.updateResults()

    def assemble(self):
        self.assembleGlobalEqMatrices()

    def assembleGlobalEqMatrices(self):
        self._check(self.lib.nla3d_assemble(self.h))

    def synchronize(self):
        self._check(self.lib.nla3d_synchronize(self.h))

    def K(self, block):
        v = np.zeros(self.blocks[block][2])
        if v.size:
            self._check(self.lib.nla3d_get_K(self.h, block, _p(v)))
        return v

    def F(self):
        v = np.zeros(self.n_total)
        self._check(self.lib.nla3d_get_F(self.h, _p(v)))
        return v

    def C(self, block):
        """Capacity matrix values of a transient storage (K's pattern)."""
        v = np.zeros(self.blocks[block][2])
        if v.size:
            self._check(self.lib.nla3d_get_C(self.h, block, _p(v)))
        return v

    def M(self, block):
        """Mass matrix values of a transient storage (K's pattern)."""
        v = np.zeros(self.blocks[block][2])
        if v.size:
            self._check(self.lib.nla3d_get_M(self.h, block, _p(v)))
        return v

    def getK(self):
        out = {}
        for b in (1, 12, 2):
            io, co = self.pattern(b)
            out[b] = SparseBlock(self.blocks[b][0], self.blocks[b][1], io, co, self.K(b))
        return BlockSparseSymMatrix(out)

    def getF(self):
        return self.F()

    def assemble_to_host(self, K1, K12, K2, F, n_chunks=8):
        """nla3d_assemble_to_host: assemble and copy the K blocks and F into
        the given host arrays (float64, contiguous; page-locked for overlap)."""
        for a in (K1, K12, K2, F):
            assert a.dtype == np.float64 and a.flags.c_contiguous
        self._check(self.lib.nla3d_assemble_to_host(self.h, n_chunks, _p(K1) if K1.size else None,
                                                    _p(K12) if K12.size else None,
                                                    _p(K2) if K2.size else None, _p(F)))

    def block_mv_device(self, block, trans, x_ptr, coef, y_ptr, mesh=0):
        """y += coef * op(block) x on device arrays (nla3d_block_mv): the
        reference's matBVprod / matBTVprod on this context's K, asynchronous
        on the context's stream."""
        self._check(self.lib.nla3d_block_mv(self.h, mesh, block, int(trans),
                                            ctypes.c_void_p(x_ptr), float(coef),
                                            ctypes.c_void_p(y_ptr)))

    def block_mv(self, block, trans, x, coef, y):
        """Host-array form of block_mv_device: copies x and y to the device
        (PyTorch allocations), runs the product, returns the new y."""
        import torch
        xd = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64)).cuda()
        yd = torch.from_numpy(np.array(y, dtype=np.float64, copy=True)).cuda()
        torch.cuda.synchronize()
        self.block_mv_device(block, trans, xd.data_ptr(), coef, yd.data_ptr())
        self.synchronize()
        return yd.cpu().numpy()

    def device_K(self, block):
        p = ctypes.c_void_p()
        n = ctypes.c_uint64()
        self._check(self.lib.nla3d_device_K(self.h, block, ctypes.byref(p), ctypes.byref(n)))
        return p.value, n.value

    def device_F(self):
        p = ctypes.c_void_p()
        n = ctypes.c_uint64()
        self._check(self.lib.nla3d_device_F(self.h, ctypes.byref(p), ctypes.byref(n)))
        return p.value, n.value

    def element_status(self):
        c = ctypes.c_uint32()
        f = ctypes.c_uint32()
        rc = self.lib.nla3d_element_status(self.h, ctypes.byref(c), ctypes.byref(f))
        if rc not in (0, 6):
            self._check(rc)
        return c.value, f.value

    def set_contrib_layout(self, layout):
        self._check(self.lib.nla3d_set_contrib_layout(self.h, layout))

    def autotune(self, reps=3):
        chosen = np.zeros(4, np.int32)
        ms = ctypes.c_float()
        self._check(self.lib.nla3d_autotune(self.h, reps, _p(chosen), ctypes.byref(ms)))
        return {"warps_per_block": int(chosen[0]), "blocks_per_sm": int(chosen[1]),
                "gather_block": int(chosen[2]), "layout": int(chosen[3]), "ms": float(ms.value)}

    def set_timing(self, on=True):
        self._check(self.lib.nla3d_set_timing(self.h, 1 if on else 0))

    def kernel_times(self):
        """Mean per-assembly kernel times (ms) since the last call:
        element, K gather, F gather, MPC; and the number of assemblies."""
        ms = np.zeros(4, np.float32)
        n = ctypes.c_uint32()
        self._check(self.lib.nla3d_kernel_times(self.h, _p(ms), ctypes.byref(n)))
        return ms, n.value

    def kernel_launches(self):
        return int(self.lib.nla3d_kernel_launches(self.h))

    @property
    def stream(self):
        return self.lib.nla3d_get_stream(self.h)


def probe_fma_peak(fp64=True):
    """Measured FMA throughput (FLOP/s) of the current GPU."""
    lib = _lib.load()
    v = ctypes.c_double()
    rc = lib.nla3d_probe_fma_peak(1 if fp64 else 0, ctypes.byref(v))
    if rc:
        raise _lib.Nla3dError(rc, "FMA probe failed")
    return v.value


def assemble_state(mesh, u, p, precision="fp64", extra=None, do_update=True):
    """Convenience: build, number, set (u, p), update + assemble; returns
    (storage, U, {block: K}, F)."""
    s = FEStorage(mesh, precision).initSolutionData()
    ne, ee = s.eq_numbers()
    U = mg.u_to_vector(ne, ee, u, p, s.n_total, extra)
    s.setU(U)
    if do_update:
        s.updateResults()
    s.assembleGlobalEqMatrices()
    return s, U, {b: s.K(b) for b in (1, 12, 2)}, s.F()
