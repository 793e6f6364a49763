"""The reference's end-to-end test `rigid_body_mpc_block_ROTX`
(test/CMakeLists.txt:51-57): one SOLID81 hexahedron, Neo-Hookean G=1 K=500,
face x=+1 clamped, face x=-1 slaved to master node 9 by a RigidBodyMpc on
UX UY UZ, master ROTX driven to 0.7853 over 20 load steps; the master's ROTX
reaction must follow the reference curve within a mean abs error of 1e-4."""
import os

import numpy as np

from nla3d_gb300 import meshgen as mg

FIXTURE = os.path.join(os.path.dirname(__file__), "golden", "rigid_body_mpc_block_rotx.npz")
THRESHOLD = 1e-4


def load_case():
    d = np.load(FIXTURE)
    mesh = mg.Mesh(mg.ELEM_SOLID81, d["xyz"], d["conn"], mat_id=mg.MAT_NEO_HOOKEAN,
                   mat_c=(1.0, 500.0), fix_nodes=d["fix_node"], fix_dofs=d["fix_dof"],
                   name="rigid_body_mpc_block_ROTX")
    mesh.rigid_bodies.append(mg.RigidBody(master=int(d["master"][0]), slaves=d["top_side"],
                                          dofs=(mg.UX, mg.UY, mg.UZ)))
    fixes = list(zip(d["fix_node"].tolist(), d["fix_dof"].tolist(), d["fix_value"].tolist()))
    return mesh, fixes, d["ref_curve"]


def curve_error(solver, mesh, ref):
    cur = solver.reaction(int(mesh.rigid_bodies[0].master), mg.ROTX)
    assert cur.size == ref.size, (cur.size, ref.size)
    return float(np.abs(cur - ref).mean())
