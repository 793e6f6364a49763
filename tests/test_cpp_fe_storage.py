"""The C++ host side (include/nla3d_fe_storage.hpp, the reference's FEStorage
interface over the C ABI), driven by a C++ program written the way the
reference's own tests are (tests/cpp/fe_storage_example.cpp: createNodes,
createElements, setConstrainedNodeDof, addMpc, addMpcCollection,
initSolutionData, getU, updateResults, assembleGlobalEqMatrices, getK()->
block(..), getF()).  The numbering and the three CSR blocks equal the
compiled reference's fixtures bit for bit (host set-up, no GPU); with the GPU,
K and F equal them within 1e-12."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import cases
from nla3d_gb300 import meshgen as mg

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLDEN = os.path.join(HERE, "golden")
# the C++ interface carries no surface lines or transient switch
CASES = sorted(n for n in cases.FULL_CASES if n not in ("quadth_lines_6x5", "quadth_transient_5x4"))


@pytest.fixture(scope="module")
def example(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no C++ compiler")
    lib_dir = os.path.join(ROOT, "nla3d_gb300")
    if not os.path.exists(os.path.join(lib_dir, "libnla3d_gpu.so")):
        pytest.skip("libnla3d_gpu.so not built")
    exe = str(tmp_path_factory.mktemp("cpp") / "fe_storage_example")
    subprocess.run([gxx, "-O2", "-std=c++17", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"),
                    os.path.join(HERE, "cpp", "fe_storage_example.cpp"), "-L", lib_dir,
                    "-lnla3d_gpu", f"-Wl,-rpath,{lib_dir}", "-o", exe], check=True)
    return exe


def _write_model(path, mesh, U, update):
    ep = np.zeros((mesh.n_elems, 4))
    if mesh.elem_params is not None:
        p = np.asarray(mesh.elem_params, dtype=np.float64)
        ep[:, :p.shape[1]] = p
    mc = list(mesh.mat_c) + [0.0] * (5 - len(mesh.mat_c))
    out = [f"{mesh.elem_type} {mesh.n_nodes} {mesh.n_elems} {mesh.mat_id} "
           + " ".join(repr(float(v)) for v in mc) + " 4"]
    out += [" ".join(repr(float(v)) for v in p) for p in mesh.xyz]
    out += [" ".join(str(int(v)) for v in c) + " " + " ".join(repr(float(v)) for v in q)
            for c, q in zip(mesh.conn, ep)]
    fn = [] if mesh.fix_nodes is None else list(zip(mesh.fix_nodes, mesh.fix_dofs))
    out.append(str(len(fn)))
    out += [f"{int(n)} {int(d)}" for n, d in fn]
    out.append(str(len(mesh.mpcs)))
    for q in mesh.mpcs:
        out.append(f"{len(q.nodes)} {float(q.b)!r} " + " ".join(
            f"{int(n)} {int(d)} {float(c)!r}" for n, d, c in zip(q.nodes, q.dofs, q.coefs)))
    out.append(str(len(mesh.rigid_bodies)))
    for rb in mesh.rigid_bodies:
        out.append(f"{rb.master} {len(rb.slaves)} {len(rb.dofs)} "
                   + " ".join(str(int(s)) for s in rb.slaves) + " "
                   + " ".join(str(int(d)) for d in rb.dofs))
    out.append(f"{U.size} " + " ".join(repr(float(v)) for v in U))
    out.append("1" if update else "0")
    with open(path, "w") as fh:
        fh.write("\n".join(out) + "\n")


def _read_output(path):
    lines = open(path).read().split("\n")
    info = [int(v) for v in lines[0].split()]
    ne = np.array(lines[1].split(), dtype=np.uint32).reshape(-1, 8)
    ee = np.array(lines[2].split(), dtype=np.uint32).reshape(-1, 8)
    blocks, k = {}, 3
    for b in (1, 12, 2):
        shape = tuple(int(v) for v in lines[k].split())
        io = np.array(lines[k + 1].split(), dtype=np.uint32)
        co = np.array(lines[k + 2].split(), dtype=np.uint32)
        va = np.array(lines[k + 3].split(), dtype=np.float64)
        blocks[b] = (shape, io, co, va)
        k += 4
    F = np.array(lines[k + 1].split(), dtype=np.float64)
    return info, ne, ee, blocks, F


def _run(example, tmp_path, name, pattern_only):
    mesh, u, p, extra, do_update = cases.FULL_CASES[name]()
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    model, out = tmp_path / "model.txt", tmp_path / "out.txt"
    _write_model(model, mesh, g["U"], do_update)
    args = [example, str(model), str(out)] + (["pattern"] if pattern_only else [])
    subprocess.run(args, check=True)
    return g, _read_output(out)


@pytest.mark.parametrize("name", CASES)
def test_cpp_numbering_and_pattern_bit_exact(example, tmp_path, name):
    g, (info, ne, ee, blocks, F) = _run(example, tmp_path, name, True)
    assert info == list(g["info"])
    assert np.array_equal(ne, g["node_eq"]) and np.array_equal(ee, g["elem_eq"])
    for b in (1, 12, 2):
        shape, io, co, _ = blocks[b]
        assert shape == tuple(int(v) for v in g[f"shape_{b}"])
        assert np.array_equal(io, g[f"iofeir_{b}"]) and np.array_equal(co, g[f"columns_{b}"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_cpp_assembly_matches_reference_fixtures(example, tmp_path, name):
    g, (info, ne, ee, blocks, F) = _run(example, tmp_path, name, False)
    for b in (1, 12, 2):
        K, want = blocks[b][3], g[f"K_{b}"]
        assert np.abs(K - want).max(initial=0.0) <= 1e-12 * max(np.abs(want).max(initial=0.0), 1e-300)
    assert np.abs(F - g["F"]).max() <= 1e-12 * np.abs(g["F"]).max()


def _order(example, tmp_path, mesh):
    model, out = tmp_path / "model.txt", tmp_path / "out.txt"
    n_total = None
    from nla3d_gb300.storage import FEStorage
    s = FEStorage(mesh).buildPattern()
    n_total = s.n_total
    _write_model(model, mesh, np.zeros(n_total), False)
    subprocess.run([example, str(model), str(out), "order"], check=True)
    lines = open(out).read().split("\n")
    order = np.array(lines[-2].split(), dtype=np.int64)
    assert int(lines[-3]) == order.size
    return s, order


@pytest.mark.parametrize("case", ["bar_mpc_2x2x3", "bar_mpc_4x4x16", "block_12"])
def test_cpp_fill_reducing_order(example, tmp_path, case):
    """fillReducingOrder (the C++ DeviceEquationSolver's default order): a
    permutation of K(2)'s rows with the DoFs that have a diagonal first, the
    MPC equations next and diagonal-less DoFs last, and a fill within 15% of
    the Python driver's nested dissection (same algorithm), well below the
    natural order's on a cube (host symbolic analysis, no GPU)."""
    from nla3d_gb300 import ldlt
    from nla3d_gb300.newton import csr_full, nested_dissection, row_points
    if case == "bar_mpc_4x4x16":
        mesh = mg.solid81_bar_mpc(4, 4, 16, 1.0)
    elif case == "block_12":
        mesh = mg.solid81_block(12, 12, 12, 1.0 / 12, clamp_z0=True)
    else:
        mesh = cases.FULL_CASES[case]()[0]
    s, order = _order(example, tmp_path, mesh)
    io, co = s.pattern(2)
    n = io.size - 1
    assert np.array_equal(np.sort(order), np.arange(n))
    diag = ldlt.has_diagonal(io, co)
    pos = np.empty(n, np.int64)
    pos[order] = np.arange(n)
    rows = np.arange(n)
    dofs_d = rows[(rows < s.n_unk) & diag]
    mpc = rows[rows >= s.n_unk]
    dofs_nd = rows[(rows < s.n_unk) & ~diag]
    if mpc.size:
        assert pos[dofs_d].max(initial=-1) < pos[mpc].min()
    if dofs_nd.size:
        assert pos[mpc].max(initial=-1) < pos[dofs_nd].min()
    K = csr_full(io, co, np.ones(co.size), n, n, True)
    py = ldlt.saddle_order(io, co, nested_dissection(K, row_points(s, s.n_con, s.n_unk, s.n_mpc)),
                           s.n_unk)
    fill_cpp = ldlt.analyze(io, co, order)["nnz_L"]
    fill_py = ldlt.analyze(io, co, py)["nnz_L"]
    fill_nat = ldlt.analyze(io, co, ldlt.saddle_order(io, co, np.arange(n), s.n_unk))["nnz_L"]
    assert fill_cpp <= 1.15 * fill_py
    if case == "block_12":   # (a thin bar's natural order is already banded)
        assert fill_cpp < 0.7 * fill_nat


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["bar_mpc_2x2x3", "cube4_nh_clamped", "biderman_3x3x3_clamped",
                                  "bar_mpc_ce_2x2x3"])
def test_cpp_device_equation_solver(example, tmp_path, name):
    """DeviceEquationSolver::solveEquations(F(2)) after the C++ assembly: the
    solution of the reference's K(2) fixture (SciPy, FP64) within 1e-9, on
    the constrained cases (an unconstrained body's K(2) is singular)."""
    import scipy.sparse.linalg as spla
    from nla3d_gb300.newton import csr_full
    mesh, u, p, extra, do_update = cases.FULL_CASES[name]()
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    model, out = tmp_path / "model.txt", tmp_path / "out.txt"
    _write_model(model, mesh, g["U"], do_update)
    subprocess.run([example, str(model), str(out), "solve"], check=True)
    lines = open(out).read().split("\n")
    head = lines[-3].split()
    x = np.array(lines[-2].split(), dtype=np.float64)
    assert int(head[0]) == x.size
    nc = int(g["info"][1])
    n2 = x.size
    K2 = csr_full(g["iofeir_2"], g["columns_2"], g["K_2"], n2, n2, True).tocsc()
    want = spla.spsolve(K2, g["F"][nc:])
    assert np.abs(x - want).max() <= 1e-9 * np.abs(want).max()
