"""Batched assembly: many independent SOLID81 meshes in one context.

Each mesh is what the reference would hold in its own FEStorage (own
equation numbering, CSR pattern, K and F); here all of them are assembled by
one launch of each kernel (nla3d_create_batch), optionally replayed as a CUDA
graph (nla3d_graph_capture / nla3d_graph_launch) with the launch shape picked
by the library's autotuner (nla3d_autotune).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from . import meshgen as mg


def _p(a):
    return None if a is None else a.ctypes.data


class BatchAssembly:
    def __init__(self, meshes, precision: str = "mixed", stream=None):
        self.lib = _lib.load()
        self.meshes = list(meshes)
        prec = {"fp64": _lib.PREC_FP64, "mixed": _lib.PREC_MIXED}[precision]
        self.precision = precision
        self._keep = []
        descs = (_lib.MeshDesc * len(self.meshes))()
        for i, m in enumerate(self.meshes):
            if (m.lines is not None and m.lines.n) or m.transient:
                raise ValueError("surface lines and transient C, M are single-mesh (FEStorage) "
                                 "features")
            xyz = np.ascontiguousarray(m.xyz, dtype=np.float64)
            conn = np.ascontiguousarray(m.conn, dtype=np.uint32)
            ep, n_ep = mg.elem_params_array(m)
            self._keep += [xyz, conn, ep]
            d = descs[i]
            d.elem_type, d.n_nodes, d.n_elems = m.elem_type, m.n_nodes, m.n_elems
            d.xyz, d.conn, d.mat_id = _p(xyz), _p(conn), m.mat_id
            for k, c in enumerate(m.mat_c[:5]):
                d.mat_c[k] = c
            d.elem_params = _p(ep)
            d.n_elem_params = n_ep
        h = ctypes.c_void_p()
        rc = self.lib.nla3d_create_batch(descs, len(self.meshes), prec, ctypes.byref(h))
        if rc:
            raise _lib.Nla3dError(rc, "nla3d_create_batch rejected the meshes")
        self.h = h
        if stream is not None:
            self._check(self.lib.nla3d_set_stream(self.h, ctypes.c_void_p(stream)))
        for i, m in enumerate(self.meshes):
            if m.fix_nodes is not None and len(m.fix_nodes):
                n = np.ascontiguousarray(m.fix_nodes, np.uint32)
                dd = np.ascontiguousarray(m.fix_dofs, np.int32)
                self._check(self.lib.nla3d_mesh_add_fix(self.h, i, n.size, _p(n), _p(dd)))
            for q in m.mpcs:
                qn = np.ascontiguousarray(q.nodes, np.uint32)
                qd = np.ascontiguousarray(q.dofs, np.int32)
                qc = np.ascontiguousarray(q.coefs, np.float64)
                self._check(self.lib.nla3d_mesh_add_mpc(self.h, i, qn.size, _p(qn), _p(qd),
                                                        _p(qc), float(q.b)))
            for rb in m.rigid_bodies:
                s = np.ascontiguousarray(rb.slaves, np.uint32)
                dd = np.ascontiguousarray(np.asarray(rb.dofs, np.int32))
                self._check(self.lib.nla3d_mesh_add_rigid_body(self.h, i, rb.master, s.size, _p(s),
                                                               dd.size, _p(dd)))

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

    # ---- set-up ----
    def build_pattern(self):
        self._check(self.lib.nla3d_build_pattern(self.h))
        self._read_offsets()
        return self

    def init(self):
        self._check(self.lib.nla3d_init_solution_data(self.h))
        self._read_offsets()
        return self

    def _read_offsets(self):
        M = len(self.meshes)
        self.info = np.zeros((M, 16), np.uint32)
        self.offsets = np.zeros((M, 5), np.uint64)
        for i in range(M):
            self._check(self.lib.nla3d_mesh_info(self.h, i, _p(self.info[i]), _p(self.offsets[i])))
        n_tot = self.info[:, 0].astype(np.int64) + self.info[:, 3]
        nnz = self.info[:, 6].astype(np.int64) + self.info[:, 9] + self.info[:, 12]
        self.n_total = int(n_tot.sum())
        self.nnz_total = int(nnz.sum())
        self.u_off = np.append(self.offsets[:, 2].astype(np.int64), self.n_total)
        self.k_off = np.append(self.offsets[:, 3].astype(np.int64), self.nnz_total)
        self.n_elems = int(sum(m.n_elems for m in self.meshes))

    def eq_numbers(self, i):
        m = self.meshes[i]
        ne = np.zeros((m.n_nodes, 8), np.uint32)
        ee = np.zeros((m.n_elems, 8), np.uint32)
        self._check(self.lib.nla3d_mesh_eq_numbers(self.h, i, _p(ne), _p(ee)))
        return ne, ee

    def pattern(self, i, block):
        b = {1: 4, 12: 7, 2: 10}[block]
        rows, nnz = int(self.info[i, b]), int(self.info[i, b + 2])
        io = np.zeros(rows + 1, np.uint32)
        co = np.zeros(max(nnz, 1), np.uint32)
        self._check(self.lib.nla3d_mesh_pattern(self.h, i, block, _p(io), _p(co)))
        return io, co[:nnz]

    def state_vector(self, states):
        """Concatenated vecU from per-mesh (u, p[, extra]) states."""
        U = np.zeros(self.n_total)
        for i, st in enumerate(states):
            u, p = st[0], st[1]
            extra = st[2] if len(st) > 2 else None
            ne, ee = self.eq_numbers(i)
            lo, hi = self.u_off[i], self.u_off[i + 1]
            U[lo:hi] = mg.u_to_vector(ne, ee, u, p, hi - lo, extra)
        return U

    # ---- per iteration ----
    def set_U(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64)
        self._check(self.lib.nla3d_set_U(self.h, _p(U), U.size))

    def set_U_device(self, ptr, n):
        self._check(self.lib.nla3d_set_U_device(self.h, ctypes.c_void_p(ptr), n))

    def update(self):
        self._check(self.lib.nla3d_update_results(self.h))

    def assemble(self):
        self._check(self.lib.nla3d_assemble(self.h))

    def K_all(self):
        v = np.zeros(self.nnz_total)
        self._check(self.lib.nla3d_get_K_all(self.h, _p(v)))
        return v

    def F(self):
        v = np.zeros(self.n_total)
        self._check(self.lib.nla3d_get_F(self.h, _p(v)))
        return v

    def mesh_K(self, K_all, i, block):
        """One block of mesh i out of the concatenated K values."""
        n1, n12 = int(self.info[i, 6]), int(self.info[i, 9])
        base = self.k_off[i]
        start = {1: 0, 12: n1, 2: n1 + n12}[block]
        n = int(self.info[i, {1: 6, 12: 9, 2: 12}[block]])
        return K_all[base + start: base + start + n]

    def mesh_F(self, F_all, i):
        return F_all[self.u_off[i]: self.u_off[i + 1]]

    # ---- launch shape, graph ----
    def set_launch_shape(self, warps_per_block=4, blocks_per_sm=0, gather_block=256):
        self._check(self.lib.nla3d_set_launch_shape(self.h, warps_per_block, blocks_per_sm,
                                                    gather_block))

    def autotune(self, reps=3):
        chosen = np.zeros(4, np.int32)
        ms = ctypes.c_float()
        self._check(self.lib.nla3d_autotune(self.h, reps, _p(chosen), ctypes.byref(ms)))
        return {"warps_per_block": int(chosen[0]), "blocks_per_sm": int(chosen[1]),
                "gather_block": int(chosen[2]), "layout": int(chosen[3]), "ms": float(ms.value)}

    def set_contrib_layout(self, layout):
        self._check(self.lib.nla3d_set_contrib_layout(self.h, layout))

    def capture_graph(self):
        self._check(self.lib.nla3d_graph_capture(self.h))

    def graph_launch(self):
        self._check(self.lib.nla3d_graph_launch(self.h))

    def synchronize(self):
        self._check(self.lib.nla3d_synchronize(self.h))

    def element_status(self):
        c = ctypes.c_uint32()
        f = ctypes.c_uint32()
        rc = self.lib.nla3d_element_status(self.h, ctypes.byref(c), ctypes.byref(f))
        if rc not in (0, 6):
            self._check(rc)
        return c.value, f.value

    def set_timing(self, on=True):
        self._check(self.lib.nla3d_set_timing(self.h, 1 if on else 0))

    def kernel_times(self):
        ms = np.zeros(4, np.float32)
        n = ctypes.c_uint32()
        self._check(self.lib.nla3d_kernel_times(self.h, _p(ms), ctypes.byref(n)))
        return ms, n.value

    def kernel_launches(self):
        return int(self.lib.nla3d_kernel_launches(self.h))
