"""Legacy-ASCII VTK output of a solution state, as the reference's
VtkProcessor writes it (VtkProcessor.cpp:19-301): `pre()` writes
`<file_name>0.vtk`, `process(step)` writes `<file_name><step>.vtk`.

Each file holds the undeformed node positions, the cells (the model's
elements, then its surface lines) with their VTK types, the point data
"disp" (UX, UY, UZ) and "reaction" vectors when a displacement DoF exists and
a scalar per other nodal DoF type (ROTX .. ROTZ of a rigid-body master, TEMP),
and, when the elements carry DoFs, cell scalars of those (HYDRO_PRESSURE).
Numbers are printed as the reference's streams print doubles (six
significant digits, "%g").  Element result queries (stresses and the like)
are element post-processing outside the assembly path and are not written.
"""
from __future__ import annotations

import numpy as np

from . import meshgen as mg

DOF_LABELS = ("UX", "UY", "UZ", "ROTX", "ROTY", "ROTZ", "HYDRO_PRESSURE", "TEMP")
# VTK cell types of the element shapes (VtkProcessor.cpp:150-168)
VTK_CELL = {mg.ELEM_SOLID81: 12, mg.ELEM_TETRA0: 10, mg.ELEM_QUADTH: 9, mg.ELEM_PLANE41: 9}
VTK_LINE = 3


def _g(x) -> str:
    return "%g" % x


class VtkProcessor:
    """backend: anything with `mesh` and `eq_numbers()` (the GPU FEStorage or
    the oracle model); U, R: vecU and vecR (constrained DoFs first)."""

    def __init__(self, backend, file_name: str):
        self.b = backend
        self.file_name = file_name
        self.mesh = backend.mesh
        self.ne, self.ee = backend.eq_numbers()
        used_n = np.nonzero((self.ne > 0).any(axis=0))[0]
        used_e = np.nonzero((self.ee > 0).any(axis=0))[0] if self.ee.size else []
        self.use_disp = any(d in (mg.UX, mg.UY, mg.UZ) for d in used_n)
        self.nodal_types = [int(d) for d in used_n if d not in (mg.UX, mg.UY, mg.UZ)]
        self.element_types = [int(d) for d in used_e]

    # ---- the reference's PostProcessor interface ----
    def pre(self, U=None, R=None):
        self._write(f"{self.file_name}0.vtk", U, R)

    def process(self, step: int, U=None, R=None):
        self._write(f"{self.file_name}{int(step)}.vtk", U, R)

    def post(self, step: int):
        pass

    def hook(self):
        """on_converged hook for NewtonSolver.solve: one file per load step."""
        count = [0]

        def on_converged(solver, t):
            count[0] += 1
            self.process(count[0], solver.U, solver.R)
        return on_converged

    # ---- file sections ----
    def text(self, U=None, R=None) -> str:
        n_total = int(max(self.ne.max(initial=0), self.ee.max(initial=0)))
        U = np.zeros(n_total) if U is None else np.asarray(U, dtype=np.float64)
        R = np.zeros(n_total) if R is None else np.asarray(R, dtype=np.float64)
        out = ["# vtk DataFile Version 2.0\n",
               "This file is generated by nla3D program\nASCII\n",
               "DATASET UNSTRUCTURED_GRID\n"]
        m = self.mesh
        xyz = np.asarray(m.xyz, dtype=np.float64)
        out.append(f"POINTS {xyz.shape[0]} float\n")
        out += [f"{_g(p[0])} {_g(p[1])} {_g(p[2])}\n" for p in xyz]
        cells = [np.asarray(c, dtype=np.int64) for c in m.conn]
        types = [VTK_CELL[m.elem_type]] * len(cells)
        if m.lines is not None and m.lines.n:
            cells += [np.asarray(c, dtype=np.int64) for c in m.lines.conn]
            types += [VTK_LINE] * m.lines.n
        size = sum(c.size + 1 for c in cells)
        out.append(f"CELLS {len(cells)} {size}\n")
        out += [f"{c.size} " + " ".join(str(int(v) - 1) for v in c) + "\n" for c in cells]
        out.append(f"CELL_TYPES {len(cells)}\n")
        out += [f"{t}\n" for t in types]
        nn = xyz.shape[0]
        out.append(f"POINT_DATA {nn}\n")

        def nodal(vec, dof):
            eq = self.ne[:, dof].astype(np.int64)
            v = np.zeros(nn)
            v[eq > 0] = vec[eq[eq > 0] - 1]
            return v

        if self.use_disp:
            for name, vec in (("disp", U), ("reaction", R)):
                cols = [nodal(vec, d) for d in (mg.UX, mg.UY, mg.UZ)]
                out.append(f"VECTORS {name} float\n")
                out += [f"{_g(a)} {_g(b)} {_g(c)}\n" for a, b, c in zip(*cols)]
                out.append("\n")
        for d in self.nodal_types:
            out.append(f"SCALARS {DOF_LABELS[d]} float 1\nLOOKUP_TABLE default\n")
            out += [f"{_g(v)}\n" for v in nodal(U, d)]
            out.append("\n")
        if self.element_types:
            ne_cells = len(cells)
            out.append(f"CELL_DATA {ne_cells}\n")
            for d in self.element_types:
                eq = self.ee[:, d].astype(np.int64)
                v = np.zeros(ne_cells)
                v[: eq.size][eq > 0] = U[eq[eq > 0] - 1]
                out.append(f"SCALARS {DOF_LABELS[d]} float 1\nLOOKUP_TABLE default\n")
                out += [f"{_g(x)}\n" for x in v]
                out.append("\n")
        return "".join(out)

    def _write(self, path, U, R):
        with open(path, "w") as fh:
            fh.write(self.text(U, R))
