"""Small parity cases shared by the golden-fixture script and the tests.

Each case returns (mesh, u, p, extra, do_update):
  u (n_nodes, 3) nodal displacements, p (n_elems,) element pressures,
  extra {(node, dof): value} for DoFs outside the elements (rigid-body master),
  do_update: whether the per-iteration protocol calls updateResults() before
  assembleGlobalEqMatrices() (SOLID81, FESolver.cpp:471 -> :446); the linear
  elements are assembled from their fresh state (FESolver.cpp:364).
"""
import numpy as np

from nla3d_gb300 import meshgen as mg


def cube3_nh():
    mesh, u, p = mg.config_cube(3, seed=1)
    return mesh, u, p, None, True


def cube4_nh_clamped():
    mesh, u, p = mg.config_cube(4, seed=5, clamp_z0=True)
    return mesh, u, p, None, True


def mr_twist_3x2x4():
    m = mg.solid81_block(3, 2, 4, 0.5, mg.MAT_MOONEY_RIVLIN, (0.4, 0.1, 2000.0))
    u, p = mg.twist_state(m, seed=3)
    return m, u, p, None, True


def biderman_3x3x3_clamped():
    m = mg.solid81_block(3, 3, 3, 1.0, mg.MAT_BIDERMAN, (0.5, 0.05, 0.01, 0.1, 800.0),
                         clamp_z0=True)
    u, p = mg.stretch_state(m, 1.3, seed=4)
    return m, u, p, None, True


def bar_mpc_2x2x3():
    m = mg.solid81_bar_mpc(2, 2, 3, 1.0)
    u, p = mg.stretch_state(m, 1.1, seed=7)
    master = m.n_nodes
    extra = {(master, mg.UZ): 0.3, (master, mg.ROTZ): 0.4, (master, mg.ROTX): 0.05,
             (master, mg.UX): 0.01}
    return m, u, p, extra, True


def ce_block_3x3x2():
    """Clamped 3x3x2 Neo-Hookean (10, 5000) block with linear MPC equations of
    the kind readCdbFile builds from CE records (FEReaders.cpp:549-573):
    UX + UZ = 0 on every free node of the x = 3 face, a three-term equation
    with a non-zero right-hand side, one that names the same DoF twice (its
    coefficients accumulate in one K entry), and one on a clamped DoF (its K
    entry lands in block(1,2))."""
    m = mg.solid81_block(3, 3, 2, 1.0, mg.MAT_NEO_HOOKEAN, (10.0, 5000.0), clamp_z0=True)
    x, z = m.xyz[:, 0], m.xyz[:, 2]
    right = np.nonzero((np.abs(x - 3.0) < 1e-12) & (z > 1e-12))[0] + 1
    for n in right:
        m.mpcs.append(mg.LinearMpc(np.array([n, n]), np.array([mg.UX, mg.UZ]),
                                   np.array([1.0, 1.0]), 0.0))
    m.mpcs.append(mg.LinearMpc(np.array([6, 22, 30]), np.array([mg.UY, mg.UX, mg.UZ]),
                               np.array([1.0, -0.5, 0.25]), 0.01))
    m.mpcs.append(mg.LinearMpc(np.array([23, 23, 27]), np.array([mg.UX, mg.UX, mg.UY]),
                               np.array([1.0, 0.5, -1.0]), 0.0))
    m.mpcs.append(mg.LinearMpc(np.array([2]), np.array([mg.UY]), np.array([2.0]), 0.0))
    u, p = mg.stretch_state(m, 1.2, seed=11)
    return m, u, p, None, True


def bar_mpc_ce_2x2x3():
    """The rigid-body bar plus UX + UY = 0 on the free nodes of its x = 0
    face: the CE equations are numbered before the rigid-body ones."""
    m = mg.solid81_bar_mpc(2, 2, 3, 1.0)
    x, z = m.xyz[:-1, 0], m.xyz[:-1, 2]
    side = np.nonzero((np.abs(x) < 1e-12) & (z > 1e-12) & (z < 3.0 - 1e-12))[0] + 1
    for n in side:
        m.mpcs.append(mg.LinearMpc(np.array([n, n]), np.array([mg.UX, mg.UY]),
                                   np.array([1.0, 1.0]), 0.0))
    u, p = mg.stretch_state(m, 1.1, seed=8)
    master = m.n_nodes
    extra = {(master, mg.UZ): 0.3, (master, mg.ROTZ): 0.4, (master, mg.ROTX): 0.05,
             (master, mg.UX): 0.01}
    return m, u, p, extra, True


def plane41_nh_3x2():
    """PLANE41 (4-node plane-strain u/p quad) Neo-Hookean (1, 500) plate of
    3x2 elements, free, stretched and sheared with noise."""
    m = mg.plane41_plate(3, 2, 0.5, mg.MAT_NEO_HOOKEAN, (1.0, 500.0))
    u, p = mg.plane_state(m, stretch=1.2, shear=0.1, seed=3)
    return m, u, p, None, True


def plane41_mr_4x3_clamped():
    """PLANE41 Mooney-Rivlin (0.4, 0.1, 2000) plate of 4x3 elements clamped on y = 0."""
    m = mg.plane41_plate(4, 3, 0.5, mg.MAT_MOONEY_RIVLIN, (0.4, 0.1, 2000.0), clamp_y0=True)
    u, p = mg.plane_state(m, stretch=1.3, shear=-0.15, seed=4)
    return m, u, p, None, True


def tetra0_3x3x3():
    m = mg.tetra0_block(3, 3, 3, 0.5)
    return m, np.zeros((m.n_nodes, 3)), None, None, False


def quadth_5x4():
    m = mg.quadth_plate(5, 4, 0.2, k=3.0)
    return m, np.zeros((m.n_nodes, 3)), None, None, False


def quadth_lines_6x5():
    """QUADTH with volume flux, convection and flux lines (SurfaceLINETH)."""
    m = mg.quadth_thermal_plate(6, 5, 0.1, seed=2)
    return m, np.zeros((m.n_nodes, 3)), None, None, False


def quadth_transient_5x4():
    """Transient QUADTH: K, F and the capacity matrix C (M stays zero)."""
    m = mg.quadth_thermal_plate(5, 4, 0.1, seed=3, transient=True)
    return m, np.zeros((m.n_nodes, 3)), None, None, False


def cube10_nh():
    """The 10^3 unit-cube workload (1000 SOLID81, 4993 equations)."""
    mesh, u, p = mg.config_cube(10, seed=1)
    return mesh, u, p, None, True


FULL_CASES = {f.__name__: f for f in (cube3_nh, cube4_nh_clamped, mr_twist_3x2x4,
                                       biderman_3x3x3_clamped, bar_mpc_2x2x3, ce_block_3x3x2,
                                       bar_mpc_ce_2x2x3, plane41_nh_3x2, plane41_mr_4x3_clamped,
                                       tetra0_3x3x3, quadth_5x4, quadth_lines_6x5,
                                       quadth_transient_5x4)}
DIGEST_CASES = {f.__name__: f for f in (cube10_nh,)}


def heat_model(transient=False):
    """The reference's QUADTH_test / QUADTH_transient model (test/QUADTH/heat.cdb):
    QUADTH k = 0.018 (rho = 1.1e-3, c = 920 when transient), convection lines
    htc = 0.0034 to -6 degrees, the HEAT load of the .cdb; returns (mesh,
    loads, probe node, fixture)."""
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "heat_quadth.npz"))
    E = g["quads"].shape[0]
    ep = np.zeros((E, 4))
    ep[:, 0] = 0.018
    if transient:
        ep[:, 2] = 1.1e-3
        ep[:, 3] = 920.0
    L = g["lines"].shape[0]
    lines = mg.SurfaceLines(g["lines"].astype(np.uint32), np.full(L, 0.0034), np.zeros(L),
                            np.full((L, 2), -6.0))
    mesh = mg.Mesh(mg.ELEM_QUADTH, g["xyz"].astype(np.float64), g["quads"].astype(np.uint32),
                   elem_params=ep, lines=lines, transient=transient, name="heat_quadth")
    loads = [(int(n), int(d), float(v)) for n, d, v in zip(g["load_node"], g["load_dof"],
                                                            g["load_value"])]
    return mesh, loads, int(g["probe"][0]), g


def tetra0_ansys_model():
    """The reference's TETRA0_test model (test/TETRA0/tetra.cdb): 883 TETRA0,
    E = 1e8, my = 0.3, the .cdb's D fixes and F loads; returns (mesh, fixes,
    loads, fixture with the ANSYS displacements and stresses)."""
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "tetra0_ansys.npz"))
    E = g["conn"].shape[0]
    ep = np.zeros((E, 2))
    ep[:, 0], ep[:, 1] = 1.0e8, 0.3
    mesh = mg.Mesh(mg.ELEM_TETRA0, g["xyz"].astype(np.float64), g["conn"].astype(np.uint32),
                   elem_params=ep, name="tetra0_ansys")
    mesh.fix_nodes, mesh.fix_dofs = g["fix_node"], g["fix_dof"]
    fixes = [(int(n), int(d), float(v)) for n, d, v in zip(g["fix_node"], g["fix_dof"],
                                                            g["fix_value"])]
    loads = [(int(n), int(d), float(v)) for n, d, v in zip(g["load_node"], g["load_dof"],
                                                            g["load_value"])]
    return mesh, fixes, loads, g
