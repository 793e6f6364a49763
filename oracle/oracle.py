"""ctypes front end for the two CPU oracles.  TEST INFRASTRUCTURE ONLY.

* ``kind="port"`` -- oracle/nla3d_oracle.c, the C restatement of the reference
  algorithm (built by ``make -C oracle port`` into oracle/_build/liborc.so).
* ``kind="ref"``  -- the reference's own C++ sources compiled by
  ``make -C oracle ref`` into oracle/_ref/libnla3d_ref.so (only where the
  reference checkout is present).

Both expose the same FEStorage-shaped sequence (FEStorage.h:255-270): build
model -> add fixes / rigid bodies -> setup -> set U -> update -> assemble ->
read K blocks and F.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline import this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "liborc.so")
REF_SO = os.path.join(HERE, "_ref", "libnla3d_ref.so")
REF_WIDE_SO = os.path.join(HERE, "_ref", "libnla3d_ref_wide.so")
# the reference checkout (read-only); NLA3D_REFERENCE overrides the default
REF_ROOT = os.environ.get("NLA3D_REFERENCE", "/root/reference")
REF_SRC = os.path.join(REF_ROOT, "src", "lib")
REF_TEST = os.path.join(REF_ROOT, "test")

_P = ctypes.c_void_p
_libs: dict = {}


def build_port() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT_SO


def build_ref(wide: bool = False) -> str | None:
    """Compile the reference sources (only where the reference checkout exists)."""
    if not os.path.isdir(REF_SRC):
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref_wide" if wide else "ref", f"REF={REF_SRC}"],
                   check=True)
    return REF_WIDE_SO if wide else REF_SO


def ref_available(wide: bool = False) -> bool:
    return os.path.exists(REF_WIDE_SO if wide else REF_SO)


def _load(kind: str):
    if kind in _libs:
        return _libs[kind]
    if kind == "port":
        path, pre = PORT_SO, "orc_"
        if not os.path.exists(path):
            build_port()
    elif kind in ("ref", "ref_wide"):
        path, pre = (REF_SO if kind == "ref" else REF_WIDE_SO), "ref_"
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path} not built (make -C oracle {kind})")
    else:
        raise ValueError(kind)
    lib = ctypes.CDLL(path)
    f = lambda n: getattr(lib, pre + n)  # noqa: E731
    f("new").restype = _P
    f("new").argtypes = [ctypes.c_int, ctypes.c_uint, _P, ctypes.c_uint, _P, ctypes.c_int, _P,
                         ctypes.c_int, _P, ctypes.c_int]
    f("free").argtypes = [_P]
    f("error").restype = ctypes.c_char_p
    f("error").argtypes = [_P]
    f("add_fix").argtypes = [_P, ctypes.c_uint, _P, _P]
    f("add_rigid_body").argtypes = [_P, ctypes.c_uint, ctypes.c_uint, _P, ctypes.c_uint, _P]
    f("add_mpc").argtypes = [_P, ctypes.c_uint, _P, _P, _P, ctypes.c_double]
    f("add_surface_lines").argtypes = [_P, ctypes.c_uint, _P, _P, _P, _P]
    f("set_transient").argtypes = [_P, ctypes.c_int]
    f("get_C").argtypes = [_P, ctypes.c_int, _P]
    f("get_M").argtypes = [_P, ctypes.c_int, _P]
    f("setup").argtypes = [_P] + ([ctypes.c_uint] if kind == "port" else [])
    f("info").argtypes = [_P, _P]
    f("pattern").argtypes = [_P, ctypes.c_int, _P, _P]
    f("eq_numbers").argtypes = [_P, _P, _P]
    f("set_U").argtypes = [_P, _P, ctypes.c_uint]
    if kind == "port":
        f("update").argtypes = [_P]
        f("assemble").argtypes = [_P]
    else:
        f("update").argtypes = [_P, _P]
        f("assemble").argtypes = [_P, _P]
    f("get_K").argtypes = [_P, ctypes.c_int, _P]
    if kind == "port":
        f("block_mv").argtypes = [_P, ctypes.c_int, ctypes.c_int, _P, ctypes.c_double, _P]
    else:
        f("block_mv").argtypes = [_P, ctypes.c_int, ctypes.c_int, _P, ctypes.c_uint,
                                  ctypes.c_double, _P, ctypes.c_uint]
    f("block_mv").restype = ctypes.c_int
    f("get_F").argtypes = [_P, _P]
    for n in ("add_fix", "add_rigid_body", "add_mpc", "setup", "pattern", "eq_numbers", "set_U",
              "update", "assemble", "get_K", "get_F", "add_surface_lines", "set_transient",
              "get_C", "get_M"):
        f(n).restype = ctypes.c_int
    if kind != "port":
        lib.ref_set_R.argtypes = [_P, _P, ctypes.c_uint]
        lib.ref_set_R.restype = ctypes.c_int
        lib.ref_write_vtk.argtypes = [_P, ctypes.c_char_p, ctypes.c_int]
        lib.ref_write_vtk.restype = ctypes.c_int
    if kind == "port":
        lib.orc_tetra0_stress.argtypes = [_P, _P]
        lib.orc_tetra0_stress.restype = ctypes.c_int
        lib.orc_material_S.argtypes = [ctypes.c_int, _P, _P, ctypes.c_double, _P]
        lib.orc_material_D.argtypes = [ctypes.c_int, _P, _P, ctypes.c_double, _P, _P]
        lib.orc_hex_jacobian.argtypes = [_P, ctypes.c_int, _P, _P]
        lib.orc_matBTDBprod.argtypes = [ctypes.c_int, ctypes.c_int, _P, _P, ctypes.c_double, _P]
        lib.orc_matBTVprod.argtypes = [ctypes.c_int, ctypes.c_int, _P, _P, ctypes.c_double, _P]
        lib.orc_matBVprod.argtypes = [ctypes.c_int, ctypes.c_int, _P, _P, ctypes.c_double, _P]
        lib.orc_matABprod.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P,
                                      ctypes.c_double, _P]
        lib.orc_matATBprod.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P,
                                       ctypes.c_double, _P]
    _libs[kind] = (lib, pre)
    return _libs[kind]


class OracleError(RuntimeError):
    pass


def _ptr(a):
    return None if a is None else a.ctypes.data


class OracleModel:
    """One FEStorage-shaped model held by an oracle library."""

    def __init__(self, mesh, kind: str = "port", max_in_row: int = 100):
        self.kind = kind
        self.lib, self.pre = _load(kind)
        self.mesh = mesh
        self._keep = []
        xyz = np.ascontiguousarray(mesh.xyz, dtype=np.float64)
        conn = np.ascontiguousarray(mesh.conn, dtype=np.uint32)
        mc = np.ascontiguousarray(np.asarray(mesh.mat_c, dtype=np.float64).reshape(-1))
        ep, n_ep = None, 0
        if mesh.elem_params is not None:
            ep = np.ascontiguousarray(mesh.elem_params, dtype=np.float64)
            n_ep = int(ep.shape[1]) if ep.ndim == 2 else 1
        self._keep += [xyz, conn, mc, ep]
        self.h = self._f("new")(mesh.elem_type, mesh.n_nodes, _ptr(xyz), mesh.n_elems,
                                _ptr(conn), mesh.mat_id, _ptr(mc) if mc.size else None,
                                int(mc.size), _ptr(ep), n_ep)
        if not self.h:
            raise OracleError("model creation failed")
        lines = getattr(mesh, "lines", None)
        if lines is not None and lines.n:
            lc = np.ascontiguousarray(lines.conn, dtype=np.uint32)
            lh = np.ascontiguousarray(lines.htc, dtype=np.float64)
            lf = np.ascontiguousarray(lines.flux, dtype=np.float64)
            lt = np.ascontiguousarray(lines.etemp, dtype=np.float64)
            self._keep += [lc, lh, lf, lt]
            self._check(self._f("add_surface_lines")(self.h, lines.n, _ptr(lc), _ptr(lh),
                                                     _ptr(lf), _ptr(lt)))
        self.transient = bool(getattr(mesh, "transient", False))
        if self.transient:
            self._check(self._f("set_transient")(self.h, 1))
        if mesh.fix_nodes is not None and len(mesh.fix_nodes):
            fn = np.ascontiguousarray(mesh.fix_nodes, dtype=np.uint32)
            fd = np.ascontiguousarray(mesh.fix_dofs, dtype=np.int32)
            self._check(self._f("add_fix")(self.h, fn.size, _ptr(fn), _ptr(fd)))
        for q in mesh.mpcs:
            qn = np.ascontiguousarray(q.nodes, dtype=np.uint32)
            qd = np.ascontiguousarray(q.dofs, dtype=np.int32)
            qc = np.ascontiguousarray(q.coefs, dtype=np.float64)
            self._check(self._f("add_mpc")(self.h, qn.size, _ptr(qn), _ptr(qd), _ptr(qc),
                                           float(q.b)))
        for rb in mesh.rigid_bodies:
            sl = np.ascontiguousarray(rb.slaves, dtype=np.uint32)
            dd = np.ascontiguousarray(np.asarray(rb.dofs, dtype=np.int32))
            self._check(self._f("add_rigid_body")(self.h, rb.master, sl.size, _ptr(sl), dd.size,
                                                  _ptr(dd)))
        if kind == "port":
            self._check(self._f("setup")(self.h, max_in_row))
        else:
            self._check(self._f("setup")(self.h))
        info = np.zeros(16, np.uint32)
        self._f("info")(self.h, _ptr(info))
        self.n_dofs, self.n_con, self.n_unk, self.n_mpc = (int(v) for v in info[:4])
        self.blocks = {}
        for b, name in zip(range(3), (1, 12, 2)):
            self.blocks[name] = tuple(int(v) for v in info[4 + 3 * b: 7 + 3 * b])
        self.n_total = self.n_dofs + self.n_mpc

    def _f(self, n):
        return getattr(self.lib, self.pre + n)

    def _check(self, rc):
        if rc:
            raise OracleError(self._f("error")(self.h).decode())

    def close(self):
        if self.h:
            self._f("free")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def eq_numbers(self):
        ne = np.zeros((self.mesh.n_nodes, 8), np.uint32)
        ee = np.zeros((self.mesh.n_elems, 8), np.uint32)
        self._check(self._f("eq_numbers")(self.h, _ptr(ne), _ptr(ee)))
        return ne, ee

    def pattern(self, block):
        rows, cols, nnz = self.blocks[block]
        iofeir = np.zeros(rows + 1, np.uint32)
        columns = np.zeros(nnz, np.uint32)
        if rows or nnz:
            self._check(self._f("pattern")(self.h, block, _ptr(iofeir), _ptr(columns)))
        if rows == 0:
            iofeir[0] = 1
        return iofeir, columns

    def set_U(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64)
        self._check(self._f("set_U")(self.h, _ptr(U), U.size))

    def update(self):
        if self.kind == "port":
            self._check(self._f("update")(self.h))
        else:
            t = ctypes.c_double()
            self._check(self._f("update")(self.h, ctypes.byref(t)))

    def assemble(self):
        if self.kind == "port":
            self._check(self._f("assemble")(self.h))
        else:
            t = ctypes.c_double()
            self._check(self._f("assemble")(self.h, ctypes.byref(t)))

    def K(self, block):
        v = np.zeros(self.blocks[block][2])
        if v.size:
            self._check(self._f("get_K")(self.h, block, _ptr(v)))
        return v

    def F(self):
        v = np.zeros(self.n_total)
        self._check(self._f("get_F")(self.h, _ptr(v)))
        return v

    def tetra0_stress(self):
        """Port only: TETRA0 element stresses from the current U (TETRA0.cpp:79-108)."""
        out = np.zeros((self.mesh.n_elems, 6))
        self._check(self.lib.orc_tetra0_stress(self.h, _ptr(out)))
        return out

    def write_vtk(self, prefix, step, U, R):
        """Compiled reference only: its VtkProcessor writes <prefix>0.vtk (and
        <prefix><step>.vtk for step > 0) from vecU = U, vecR = R."""
        if self.kind == "port":
            raise OracleError("the VTK writer is the compiled reference's")
        self.set_U(U)
        R = np.ascontiguousarray(R, dtype=np.float64)
        self._check(self.lib.ref_set_R(self.h, _ptr(R), R.size))
        self._check(self.lib.ref_write_vtk(self.h, prefix.encode(), int(step)))

    def C(self, block):
        """Capacity matrix block of a transient model (K's pattern)."""
        v = np.zeros(self.blocks[block][2])
        if v.size:
            self._check(self._f("get_C")(self.h, block, _ptr(v)))
        return v

    def M(self, block):
        """Mass matrix block of a transient model (K's pattern)."""
        v = np.zeros(self.blocks[block][2])
        if v.size:
            self._check(self._f("get_M")(self.h, block, _ptr(v)))
        return v

    def block_mv(self, block, trans, x, coef, y):
        """y + coef * op(block) x through the model's own sparse products
        (matBVprod / matBTVprod, SparseMatrix.cpp:497-558); returns a new y."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.array(y, dtype=np.float64, copy=True)
        if self.kind == "port":
            self._check(self._f("block_mv")(self.h, block, int(trans), _ptr(x), coef, _ptr(out)))
        else:
            self._check(self._f("block_mv")(self.h, block, int(trans), _ptr(x), x.size, coef,
                                            _ptr(out), out.size))
        return out


def solve_state(mesh, u, p, kind="port", extra=None, max_in_row=100):
    """Convenience: build, set (u, p) through the oracle's own numbering,
    run update + assemble, return (model, U, {block: K}, F)."""
    m = OracleModel(mesh, kind, max_in_row=max_in_row)
    from nla3d_gb300 import meshgen
    ne, ee = m.eq_numbers()
    U = meshgen.u_to_vector(ne, ee, u, p, m.n_total, extra)
    m.set_U(U)
    m.update()
    m.assemble()
    return m, U, {b: m.K(b) for b in (1, 12, 2)}, m.F()


def port_lib():
    return _load("port")[0]
