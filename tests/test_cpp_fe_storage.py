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
