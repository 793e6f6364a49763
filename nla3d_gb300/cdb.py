"""ANSYS .cdb input, as the reference reads it (FEReaders.h:23-100,
FEReaders.cpp:35-80, 321-729): a neutral MeshData filled by readCdbFile,
compressNumbers to renumber nodes 1..n, and the attribute queries main.cpp
uses (main.cpp:167-225) to build the model.

Records understood (everything else is skipped, as in the reference):
  NBLOCK   nodes, fixed-width format line such as (3i9,6e20.13); missing
           trailing coordinates are zero;
  EBLOCK   elements, SOLID layout (material, type, real, section, CS, birth,
           solid-model ref, shape, node count, -, number, nodes) or the
           non-SOLID layout (number, type, real, material, CS, nodes);
  D        fixed DoFs with a numeric node and value;
  F        nodal loads with a numeric node and value (HEAT -> TEMP,
           FX/FY/FZ -> UX/UY/UZ, otherwise a DoF label);
  CE       MPC equations, terms two per line (any count; the reference
           handles two-term equations only);
  CMBLOCK  node / element components (names starting with '_' skipped);
           a negative entry closes a range started by the entry before it;
  ET / ETYPE / TYPE / *SET  tracked, unused (as in the reference).
Lines starting with '/' or '!' and empty first fields are skipped.  Lines may
end in LF, CR or CRLF.  An unknown format line or a short field raises
CdbError where the reference aborts (LOG(FATAL)).
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field

import numpy as np

from . import meshgen as mg

DOF_LABELS = ("UX", "UY", "UZ", "ROTX", "ROTY", "ROTZ", "HYDRO_PRESSURE", "TEMP")
COMPONENT_TYPES = ("ELEM", "NODE")      # FEComponent::labelsOfComponent[1..2]
CELL_ATTRIBUTES = ("MAT", "REAL", "SECT", "CS", "SHAPE", "TYPE")


class CdbError(ValueError):
    """A record the reader cannot parse (the reference aborts there)."""


def label2dof(label: str) -> int:
    """Dof::label2dofType (Dof.cpp:14-22): exact, case-sensitive labels.  The
    reference logs an unknown label and returns UNDEFINED, which fails later;
    here it raises at once."""
    try:
        return DOF_LABELS.index(label)
    except ValueError:
        raise CdbError(f"unknown DoF label {label!r}") from None


@dataclass
class FixBC:
    node: int
    node_dof: int
    value: float


@dataclass
class LoadBC:
    node: int
    node_dof: int
    value: float


@dataclass
class MpcTerm:
    node: int
    node_dof: int
    coef: float


@dataclass
class Mpc:
    eq: list = field(default_factory=list)   # MpcTerm
    b: float = 0.0


@dataclass
class FEComponent:
    name: str
    type: str                                # "NODE", "ELEM" or "NOT DEFINED"
    list: list = field(default_factory=list)


@dataclass
class MeshData:
    """The reference's neutral mesh container (FEReaders.h:24-56)."""
    cellNumbers: list = field(default_factory=list)
    cellNodes: list = field(default_factory=list)
    cellIntData: dict = field(default_factory=dict)
    nodesNumbers: list = field(default_factory=list)
    nodesPos: list = field(default_factory=list)
    loadBcs: list = field(default_factory=list)
    fixBcs: list = field(default_factory=list)
    mpcs: list = field(default_factory=list)
    feComps: dict = field(default_factory=dict)

    def clear(self):
        self.__init__()

    def compressNumbers(self):
        """Renumber nodes 1..n in reading order unless they already are
        (FEReaders.cpp:35-80): elements, loads, fixes, MPC terms and node
        components follow."""
        if not self.nodesNumbers or len(self.nodesNumbers) == max(self.nodesNumbers):
            return
        old2new = {o: k + 1 for k, o in enumerate(self.nodesNumbers)}
        self.nodesNumbers = list(range(1, len(self.nodesNumbers) + 1))
        m = lambda n: old2new.get(n, 0)  # noqa: E731  (std::map::operator[] default)
        self.cellNodes = [[m(n) for n in c] for c in self.cellNodes]
        for bc in self.loadBcs:
            bc.node = m(bc.node)
        for bc in self.fixBcs:
            bc.node = m(bc.node)
        for mpc in self.mpcs:
            for t in mpc.eq:
                t.node = m(t.node)
        for comp in self.feComps.values():
            if comp.type == "NODE":
                comp.list = [m(n) for n in comp.list]

    def getDegeneratedCells(self):
        """Cells with a repeated node (FEReaders.cpp:83-92), as indices."""
        return [i for i, c in enumerate(self.cellNodes) if len(set(c)) != len(c)]

    def getCellsByAttribute(self, name: str, value: int):
        """Indices of the cells whose integer attribute `name` equals value
        (FEReaders.cpp:95-103)."""
        return [i for i, v in enumerate(self.cellIntData[name]) if v == value]

    def nodes_array(self) -> np.ndarray:
        return np.array(self.nodesPos, dtype=np.float64).reshape(-1, 3)


_NBLOCK_FMT = re.compile(r"\((\d+)i(\d+),(\d+)e(\d+)\.[0-9e]+\)")
_INT_FMT = re.compile(r"\((\d+)i(\d+)\)")


def _lines(path):
    with open(path, "rb") as fh:
        data = fh.read().decode("latin-1")
    # getLine (FEReaders.cpp:186-217): LF, CR and CRLF all end a line
    return data.replace("\r\n", "\n").replace("\r", "\n").split("\n")


def _fixed_split(line: str, widths, strict=False):
    """ssplit (FEReaders.cpp:143-163): fixed-width fields; a line may stop
    at a field boundary, not inside a field."""
    out, pos = [], 0
    for w in widths:
        if len(line) - pos < w:
            if strict or len(line) - pos != 0:
                raise CdbError(f"incomplete field in line {line!r}")
            return out
        out.append(line[pos:pos + w])
        pos += w
    return out


def _first_not_blank(line: str) -> str:
    s = line.lstrip(" \t")
    return s[:1]


def _int(s: str) -> int:
    return int(s.strip())


def _float(s: str) -> float:
    return float(s.strip())


def readCdbFile(filename: str, md: MeshData) -> bool:
    """Fill `md` from an ANSYS .cdb file; False if the file cannot be opened
    (FEReaders.cpp:321-729)."""
    try:
        lines = _lines(filename)
    except OSError:
        return False
    md.clear()
    for k in CELL_ATTRIBUTES:
        md.cellIntData[k] = []
    n_lines = len(lines)
    # a trailing empty string after the last newline is not a line
    if n_lines and lines[-1] == "":
        n_lines -= 1
    i = 0
    while i < n_lines:
        line = lines[i]
        i += 1
        tok = [t.strip(" \t") for t in line.split(",")]
        key = tok[0]
        if key == "" or key[0] in "/!":
            continue
        ku = key.upper()
        if ku == "NBLOCK":
            fmt = lines[i].strip(" \t").lower() if i < n_lines else ""
            i += 1
            m = _NBLOCK_FMT.fullmatch(fmt)
            if not m:
                raise CdbError(f"NBLOCK format {fmt!r}")
            n_int, w_int, n_flt, w_flt = (int(g) for g in m.groups())
            widths = [w_int] * n_int + [w_flt] * n_flt
            while i < n_lines:
                row = lines[i]
                i += 1
                if _first_not_blank(row) in ("-", "N"):
                    break
                v = _fixed_split(row, widths)
                pos = [0.0, 0.0, 0.0]
                for c in range(3):
                    if len(v) > n_int + c:
                        pos[c] = _float(v[n_int + c])
                md.nodesNumbers.append(_int(v[0]))
                md.nodesPos.append(pos)
        elif ku == "EBLOCK":
            solid = len(tok) > 2 and tok[2].upper() == "SOLID"
            fmt = lines[i].strip(" \t").lower() if i < n_lines else ""
            i += 1
            m = _INT_FMT.fullmatch(fmt)
            if not m:
                raise CdbError(f"EBLOCK format {fmt!r}")
            widths = [int(m.group(2))] * int(m.group(1))
            while i < n_lines:
                row = lines[i]
                i += 1
                if _first_not_blank(row) in ("-", "N"):
                    break
                v = _fixed_split(row, widths)
                if solid:
                    mat, etype, real, sect, cs = (_int(x) for x in v[:5])
                    shape, n_nodes, number = _int(v[7]), _int(v[8]), _int(v[10])
                    st = 11
                else:
                    number, etype, real, mat, cs = (_int(x) for x in v[:5])
                    sect, shape = 0, 0
                    n_nodes, st = len(v) - 5, 5
                if len(v) != st + n_nodes:
                    raise CdbError(f"not enough fields for the element's nodes: {row!r}")
                md.cellNumbers.append(number)
                md.cellNodes.append([_int(x) for x in v[st:st + n_nodes]])
                for k, val in zip(("TYPE", "MAT", "REAL", "SECT", "CS", "SHAPE"),
                                  (etype, mat, real, sect, cs, shape)):
                    md.cellIntData[k].append(val)
        elif ku == "D":
            try:
                node, value = int(tok[1]), float(tok[3])
            except (ValueError, IndexError):
                continue     # 'ALL', a parameter or a table: not handled (as the reference)
            md.fixBcs.append(FixBC(node, label2dof(tok[2]), value))
        elif ku == "F":
            try:
                node, value = int(tok[1]), float(tok[3])
            except (ValueError, IndexError):
                continue
            lab = tok[2].upper()
            dof = {"HEAT": 7, "FX": 0, "FY": 1, "FZ": 2}.get(lab)
            md.loadBcs.append(LoadBC(node, label2dof(tok[2]) if dof is None else dof, value))
        elif ku == "CE":
            mpc = Mpc(b=float(tok[5]))
            n_terms = int(tok[3])
            while n_terms > 0:
                if i >= n_lines:
                    raise CdbError("CE: missing term line")
                t = [x.strip(" \t") for x in lines[i].split(",")]
                i += 1
                # two terms per line, the last line of an odd count one: the
                # reference's bound max(n_terms, 2) (FEReaders.cpp:551) reads
                # past a one-term line and over-reads when more than two
                # terms remain; it agrees with this for 2-term equations
                for k in range(min(n_terms, 2)):
                    mpc.eq.append(MpcTerm(int(t[3 + 3 * k]), label2dof(t[4 + 3 * k]),
                                          float(t[5 + 3 * k])))
                    n_terms -= 1
            md.mpcs.append(mpc)
        elif ku == "CMBLOCK":
            if tok[1][:1] == "_":
                continue
            ctype = tok[2].upper()
            if ctype not in COMPONENT_TYPES:
                ctype = "NOT DEFINED"   # FEComponent::typeFromString logs and returns this
            n_ranges = int(tok[3].split("!")[0])
            fmt = lines[i].strip(" \t").lower() if i < n_lines else ""
            i += 1
            m = _INT_FMT.fullmatch(fmt)
            if not m:
                raise CdbError(f"CMBLOCK format {fmt!r}")
            per_row, width = int(m.group(1)), int(m.group(2))
            vals = []
            while len(vals) < n_ranges:
                if i >= n_lines:
                    raise CdbError("CMBLOCK: missing entries")
                row = _fixed_split(lines[i], [width] * per_row)
                i += 1
                vals += [_int(x) for x in row]
            vals = vals[:n_ranges]
            lst = []
            for k, v in enumerate(vals):
                if v > 0:
                    lst.append(v)
                else:
                    if k == 0 or vals[k - 1] <= 0:
                        raise CdbError("CMBLOCK: a range without a start")
                    lst.extend(range(vals[k - 1] + 1, -v + 1))
            md.feComps[tok[1]] = FEComponent(tok[1], ctype, lst)
        # ET / ETYPE / TYPE / *SET: tracked by the reference, never used
    return True


def read_cdb(filename: str, compress: bool = True) -> MeshData:
    md = MeshData()
    if not readCdbFile(filename, md):
        raise OSError(f"cannot open cdb file {filename}")
    if compress:
        md.compressNumbers()
    return md


def to_mesh(md: MeshData, elem_type: int, mat_id: int = 0, mat_c=(), type_attr: int = 1,
            name: str = "cdb"):
    """The model main.cpp builds from MeshData (main.cpp:189-225): every node,
    the cells of TYPE `type_attr` as elements of `elem_type`, the CE equations
    as linear MPCs, the D records as fixed DoFs.  Returns (mesh, fixes, loads)
    with fixes / loads as (node, dof, value) lists."""
    nodes_per = {mg.ELEM_SOLID81: 8, mg.ELEM_PLANE41: 4, mg.ELEM_TETRA0: 4, mg.ELEM_QUADTH: 4}
    idx = md.getCellsByAttribute("TYPE", type_attr)
    npe = nodes_per[elem_type]
    for k in idx:
        if len(md.cellNodes[k]) != npe:
            raise CdbError(f"cell {md.cellNumbers[k]} has {len(md.cellNodes[k])} nodes, "
                           f"the element type needs {npe}")
    conn = np.array([md.cellNodes[k] for k in idx], dtype=np.uint32).reshape(-1, npe)
    mesh = mg.Mesh(elem_type, md.nodes_array(), conn, mat_id=mat_id, mat_c=tuple(mat_c),
                   name=name)
    for mpc in md.mpcs:
        mesh.mpcs.append(mg.LinearMpc(np.array([t.node for t in mpc.eq], np.uint32),
                                      np.array([t.node_dof for t in mpc.eq], np.int32),
                                      np.array([t.coef for t in mpc.eq], np.float64),
                                      float(mpc.b)))
    mesh.fix_nodes = np.array([f.node for f in md.fixBcs], dtype=np.uint32)
    mesh.fix_dofs = np.array([f.node_dof for f in md.fixBcs], dtype=np.int32)
    fixes = [(f.node, f.node_dof, f.value) for f in md.fixBcs]
    loads = [(f.node, f.node_dof, f.value) for f in md.loadBcs]
    return mesh, fixes, loads
