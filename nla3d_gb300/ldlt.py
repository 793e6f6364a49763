"""Sparse LDL^T of K(2) on the device (nla3d_ldlt_*): the GPU counterpart of
the reference's EquationSolver (EquationSolver.h:19-34), factoring the K(2)
block that the assembly leaves in HBM.

    solver = DeviceLDLT.for_storage(s, perm)        # symbolic analysis, once
    solver.factor(s)                                # factorizeEquations
    x = solver.solve_host(s, rhs)                   # substituteEquations (+ refinement)

`analyze` runs the symbolic analysis alone on the host (no GPU needed).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib


def _p(a):
    return None if a is None else a.ctypes.data


def _perm_array(perm, n):
    if perm is None:
        return None
    p = np.ascontiguousarray(perm, dtype=np.int32)
    if p.shape != (n,):
        raise ValueError("perm must have one entry per equation")
    return p


def analyze(iofeir, columns, perm=None):
    """Symbolic analysis: supernodes, their rows (factor order, pivots first),
    the final order and the sizes of the factor."""
    lib = _lib.load()
    io = np.ascontiguousarray(iofeir, dtype=np.uint32)
    co = np.ascontiguousarray(columns, dtype=np.uint32)
    n = io.size - 1
    pa = _perm_array(perm, n)
    stats = np.zeros(8)
    rc = lib.nla3d_ldlt_analyze(n, _p(io), _p(co), _p(pa), _p(stats), None, None, None, None)
    if rc:
        raise _lib.Nla3dError(rc, "nla3d_ldlt_analyze rejected the pattern")
    ns, nrows = int(stats[0]), int(stats[7])
    perm_out = np.zeros(n, np.int32)
    sn_first = np.zeros(ns + 1, np.int32)
    row_ptr = np.zeros(ns + 1, np.int64)
    rows = np.zeros(max(nrows, 1), np.int32)
    rc = lib.nla3d_ldlt_analyze(n, _p(io), _p(co), _p(pa), _p(stats), _p(perm_out), _p(sn_first),
                                _p(row_ptr), _p(rows))
    if rc:
        raise _lib.Nla3dError(rc, "nla3d_ldlt_analyze")
    return {"supernodes": ns, "levels": int(stats[1]), "max_front": int(stats[2]),
            "nnz_L": int(stats[3]), "flops": float(stats[4]), "front_entries": int(stats[5]),
            "max_children": int(stats[6]), "perm": perm_out, "sn_first": sn_first,
            "row_ptr": row_ptr, "rows": rows[:nrows]}


def has_diagonal(iofeir, columns):
    """Rows of an upper CSR whose diagonal entry is stored."""
    io = np.asarray(iofeir, dtype=np.int64)
    co = np.asarray(columns, dtype=np.int64)
    n = io.size - 1
    first = io[:-1] - 1
    nonempty = io[1:] > io[:-1]
    out = np.zeros(n, dtype=bool)
    out[nonempty] = co[first[nonempty]] == np.arange(1, n + 1)[nonempty]
    return out


def saddle_order(iofeir, columns, order, n_unknown):
    """A K(2) order for the factorisation without pivoting: the DoFs with a
    stored diagonal in the given fill-reducing order, then the MPC / CE
    equations (rows n_unknown ..), then the DoFs without a diagonal (a
    rigid-body master node, which couples only through its MPC equations).
    Eliminating the DoFs first makes the equations' pivots negative (-c K^-1
    c^T) and the masters' pivots positive afterwards."""
    order = np.asarray(order, dtype=np.int64)
    diag = has_diagonal(iofeir, columns)
    n = diag.size
    dofs = order[order < n_unknown]
    first = dofs[diag[dofs]]
    last = dofs[~diag[dofs]]
    return np.concatenate([first, np.arange(n_unknown, n), last]).astype(np.int32)


def fill_reducing_order(iofeir, columns, points, n_unknown):
    """nla3d_ldlt_order: geometric nested dissection of K(2)'s rows (a point
    per row), then saddle_order's grouping (DoFs with a diagonal, MPC / CE
    equations, DoFs without a diagonal); the same order as
    saddle_order(iofeir, columns, newton.nested_dissection(K, points),
    n_unknown), computed in the library."""
    lib = _lib.load()
    io = np.ascontiguousarray(iofeir, dtype=np.uint32)
    co = np.ascontiguousarray(columns, dtype=np.uint32)
    n = io.size - 1
    pts = np.ascontiguousarray(points, dtype=np.float64)
    if pts.shape != (n, 3):
        raise ValueError("points must be n x 3")
    order = np.zeros(n, np.int32)
    rc = lib.nla3d_ldlt_order(n, _p(io), _p(co), _p(pts), int(n_unknown), _p(order))
    if rc:
        raise _lib.Nla3dError(rc, "nla3d_ldlt_order rejected the pattern")
    return order


class DeviceLDLT:
    def __init__(self, iofeir, columns, perm=None, precision="fp64", stream=None):
        self.lib = _lib.load()
        self.h = None
        io = np.ascontiguousarray(iofeir, dtype=np.uint32)
        co = np.ascontiguousarray(columns, dtype=np.uint32)
        self.n = io.size - 1
        pa = _perm_array(perm, self.n)
        prec = {"fp64": 0, "fp32": 1, "fp32-tc": 2}[precision]
        h = ctypes.c_void_p()
        rc = self.lib.nla3d_ldlt_create(self.n, _p(io), _p(co), _p(pa), prec,
                                        ctypes.c_void_p(stream) if stream else None,
                                        ctypes.byref(h))
        if h.value:
            self.h = h
        if rc:
            msg = self.lib.nla3d_ldlt_last_error(self.h).decode() if self.h else ""
            self.close()
            raise _lib.Nla3dError(rc, msg or "nla3d_ldlt_create rejected the pattern")
        self.last_steps = 0
        self.last_residual = 0.0

    @classmethod
    def for_storage(cls, storage, perm=None, precision="fp64"):
        """On the K(2) pattern of a GPU FEStorage, on its stream."""
        io, co = storage.pattern(2)
        out = cls(io, co, perm, precision, storage.stream)
        out._storage = storage    # the stream is the storage's: keep it alive as long
        return out

    def _check(self, rc):
        if rc:
            msg = self.lib.nla3d_ldlt_last_error(self.h)
            raise _lib.Nla3dError(rc, msg.decode() if msg else "")

    def close(self):
        if self.h:
            self.lib.nla3d_ldlt_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        v = np.zeros(8)
        self._check(self.lib.nla3d_ldlt_info(self.h, _p(v)))
        return {"supernodes": int(v[0]), "levels": int(v[1]), "max_front": int(v[2]),
                "nnz_L": int(v[3]), "flops": float(v[4]), "front_bytes": float(v[5]),
                "perturbed": int(v[6]), "nonfinite": int(v[7])}

    def factor_device(self, values_ptr):
        self._check(self.lib.nla3d_ldlt_factor(self.h, ctypes.c_void_p(values_ptr)))

    def factor(self, storage):
        """factorizeEquations on the storage's device K(2)."""
        self.factor_device(storage.device_K(2)[0])

    def solve_device(self, values_ptr, b_ptr, x_ptr, max_refine=50, tol=1e-13, strict=True):
        """strict=False returns the refined x and its residual even when tol
        was not reached (NLA3D_ERR_RANGE); other errors always raise."""
        steps = ctypes.c_int()
        rel = ctypes.c_double()
        rc = self.lib.nla3d_ldlt_solve(self.h, ctypes.c_void_p(values_ptr), ctypes.c_void_p(b_ptr),
                                       ctypes.c_void_p(x_ptr), int(max_refine), float(tol),
                                       ctypes.byref(steps), ctypes.byref(rel))
        self.last_steps, self.last_residual = steps.value, rel.value
        if rc and (strict or rc != 5):
            self._check(rc)
        return steps.value, rel.value

    def solve_host(self, storage, rhs, max_refine=50, tol=1e-13, strict=True):
        """x = K(2)^-1 rhs for a host vector (PyTorch device buffers as plumbing)."""
        import torch
        b = torch.from_numpy(np.ascontiguousarray(rhs, dtype=np.float64)).cuda()
        x = torch.empty_like(b)
        torch.cuda.synchronize()
        self.solve_device(storage.device_K(2)[0], b.data_ptr(), x.data_ptr(), max_refine, tol,
                          strict)
        return x.cpu().numpy()
