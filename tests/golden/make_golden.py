"""Generate the golden fixtures in tests/golden/ from the COMPILED REFERENCE.

Run in a checkout that has the reference sources (the oracle Makefile compiles
them into oracle/_ref/):

    python tests/golden/make_golden.py

For every case in cases.FULL_CASES it stores the equation numbers, the CSR
pattern of the three K blocks (block(1), block(1,2), block(2)), their values
and F, as produced by the reference's FEStorage::updateResults() +
assembleGlobalEqMatrices().  For cases.DIGEST_CASES (too large to commit) it
stores SHA-256 digests of the exact bytes plus a few norms.
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from oracle import oracle as O  # noqa: E402
from nla3d_gb300 import meshgen as mg  # noqa: E402
import cases  # noqa: E402


def run_reference(case):
    mesh, u, p, extra, do_update = case()
    m = O.OracleModel(mesh, "ref")
    ne, ee = m.eq_numbers()
    U = mg.u_to_vector(ne, ee, u, p, m.n_total, extra)
    m.set_U(U)
    if do_update:
        m.update()
    m.assemble()
    out = {"U": U, "node_eq": ne, "elem_eq": ee, "F": m.F(),
           "info": np.array([m.n_dofs, m.n_con, m.n_unk, m.n_mpc], np.uint32)}
    for b in (1, 12, 2):
        io, co = m.pattern(b)
        out[f"iofeir_{b}"] = io
        out[f"columns_{b}"] = co
        out[f"K_{b}"] = m.K(b)
        out[f"shape_{b}"] = np.array(m.blocks[b], np.uint32)
    return out


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    if not O.build_ref():
        sys.exit("reference sources not found; cannot regenerate goldens")
    for name, case in cases.FULL_CASES.items():
        out = run_reference(case)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
        print("wrote", name)
    lines = []
    for name, case in cases.DIGEST_CASES.items():
        out = run_reference(case)
        for k in sorted(out):
            lines.append(f"{name} {k} {digest(out[k])}")
        lines.append(f"{name} normK2 {float(np.abs(out['K_2']).max()):.17g}")
        lines.append(f"{name} normF {float(np.abs(out['F']).max()):.17g}")
        print("digested", name)
    with open(os.path.join(HERE, "digests.txt"), "w") as f:
        f.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    main()
