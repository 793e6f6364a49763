"""Seeded synthetic meshes for the SOLID81 / TETRA0 / QUADTH assembly path.

The reference reads meshes from ANSYS .cdb files (FEReaders.cpp:321-729); the
workloads here are regular grids generated in memory instead, with the
reference's own conventions:

* nodes at (i, j, k) * h, node id = 1 + i + (nx+1) * (j + (ny+1) * k);
* hexahedron node order (i,j,k), (i+1,j,k), (i+1,j+1,k), (i,j+1,k), then the
  same four at k+1 -- the order of ElementIsoParamHEXAHEDRON::formFunc
  (isoparametric.cpp:191-201);
* elements numbered x-fastest, ids from 1 (FEStorage.h:290-292);
* Neo-Hookean constants passed as (G, K) with G = 2 * C10
  (materials_hyperelastic.cpp:242-263).

All random draws use numpy's PCG64 generator with an explicit seed.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

# Reference enums (sys.h:151-163, MaterialFactory.h:12-18, Dof.h:15-25).
ELEM_PLANE41 = 1
ELEM_SOLID81 = 2
ELEM_TETRA0 = 3
ELEM_QUADTH = 5
MAT_NEO_HOOKEAN = 1
MAT_BIDERMAN = 2
MAT_MOONEY_RIVLIN = 3
UX, UY, UZ, ROTX, ROTY, ROTZ, HYDRO_PRESSURE, TEMP = range(8)

NODES_PER_ELEM = {ELEM_SOLID81: 8, ELEM_TETRA0: 4, ELEM_QUADTH: 4}


@dataclasses.dataclass
class RigidBody:
    """A RigidBodyMpc collection (Mpc.h:51-61): slave nodes follow the master."""
    master: int
    slaves: np.ndarray          # uint32, 1-based node ids
    dofs: tuple = (UX, UY, UZ)


@dataclasses.dataclass
class LinearMpc:
    """An Mpc passed to FEStorage::addMpc (Mpc.h:31-36): sum coefs * u(nodes, dofs) = b."""
    nodes: np.ndarray           # uint32, 1-based node ids
    dofs: np.ndarray            # int32 Dof types
    coefs: np.ndarray           # float64
    b: float = 0.0


@dataclasses.dataclass
class SurfaceLines:
    """SurfaceLINETH elements (QUADTH.h:38-55) on a QUADTH mesh: convection
    (htc, environment temperatures etemp) and flux over 2-node lines."""
    conn: np.ndarray            # (n, 2) uint32, 1-based node ids
    htc: np.ndarray             # (n,) float64
    flux: np.ndarray            # (n,) float64
    etemp: np.ndarray           # (n, 2) float64 (a zero second value takes the first)

    @property
    def n(self) -> int:
        return int(self.conn.shape[0])


@dataclasses.dataclass
class Mesh:
    elem_type: int
    xyz: np.ndarray             # (n_nodes, 3) float64
    conn: np.ndarray            # (n_elems, nodes_per_elem) uint32, 1-based
    mat_id: int = 0
    mat_c: tuple = ()
    # (n_elems, 2..4) float64: TETRA0 (E, my); QUADTH (k[, volFlux, rho, c])
    elem_params: np.ndarray | None = None
    fix_nodes: np.ndarray | None = None     # uint32 1-based
    fix_dofs: np.ndarray | None = None      # int32 Dof types
    rigid_bodies: list = dataclasses.field(default_factory=list)
    mpcs: list = dataclasses.field(default_factory=list)   # LinearMpc, numbered first
    lines: SurfaceLines | None = None       # created after the elements
    transient: bool = False                 # FEStorage::setTransient: assemble C, M too
    name: str = ""

    @property
    def n_nodes(self) -> int:
        return int(self.xyz.shape[0])

    @property
    def n_elems(self) -> int:
        return int(self.conn.shape[0])

    @property
    def bulk_modulus(self) -> float:
        return float(self.mat_c[-1]) if self.mat_c else 0.0


def elem_params_array(mesh: "Mesh"):
    """(contiguous float64 array, columns) of the mesh's element parameters as
    the library takes them: 2 columns (TETRA0 E, my; QUADTH k, volFlux) or 4
    (QUADTH k, volFlux, rho, c); other widths are zero-padded to the next."""
    if mesh.elem_params is None:
        return None, 0
    ep = np.asarray(mesh.elem_params, dtype=np.float64)
    if ep.ndim == 1:
        ep = ep[:, None]
    c = ep.shape[1]
    if c > 4:
        raise ValueError("at most 4 element parameters")
    width = 2 if c <= 2 else 4
    if c < width:
        ep = np.concatenate([ep, np.zeros((ep.shape[0], width - c))], axis=1)
    return np.ascontiguousarray(ep), width


def hex_block(nx: int, ny: int, nz: int, h=1.0) -> tuple[np.ndarray, np.ndarray]:
    """Regular nx*ny*nz hexahedral block: (xyz, conn)."""
    if np.isscalar(h):
        hx = hy = hz = float(h)
    else:
        hx, hy, hz = (float(v) for v in h)
    i = np.arange(nx + 1, dtype=np.float64)
    j = np.arange(ny + 1, dtype=np.float64)
    k = np.arange(nz + 1, dtype=np.float64)
    kk, jj, ii = np.meshgrid(k, j, i, indexing="ij")
    xyz = np.stack([ii.ravel() * hx, jj.ravel() * hy, kk.ravel() * hz], axis=1)

    ei, ej, ek = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    ei = ei.transpose(2, 1, 0).ravel().astype(np.int64)
    ej = ej.transpose(2, 1, 0).ravel().astype(np.int64)
    ek = ek.transpose(2, 1, 0).ravel().astype(np.int64)

    def nid(a, b, c):
        return 1 + a + (nx + 1) * (b + (ny + 1) * c)

    conn = np.stack([
        nid(ei, ej, ek), nid(ei + 1, ej, ek), nid(ei + 1, ej + 1, ek), nid(ei, ej + 1, ek),
        nid(ei, ej, ek + 1), nid(ei + 1, ej, ek + 1), nid(ei + 1, ej + 1, ek + 1),
        nid(ei, ej + 1, ek + 1),
    ], axis=1).astype(np.uint32)
    return xyz, conn


def solid81_block(nx, ny, nz, h=1.0, mat_id=MAT_NEO_HOOKEAN, mat_c=(1.0, 1000.0),
                  clamp_z0=False, name="") -> Mesh:
    xyz, conn = hex_block(nx, ny, nz, h)
    m = Mesh(ELEM_SOLID81, xyz, conn, mat_id=mat_id, mat_c=tuple(float(c) for c in mat_c),
             name=name or f"solid81_{nx}x{ny}x{nz}")
    if clamp_z0:
        base = np.nonzero(np.abs(xyz[:, 2]) < 1e-12)[0].astype(np.uint32) + 1
        m.fix_nodes = np.repeat(base, 3)
        m.fix_dofs = np.tile(np.array([UX, UY, UZ], dtype=np.int32), base.size)
    return m


def solid81_bar_mpc(nx, ny, nz, h=1.0, mat_id=MAT_NEO_HOOKEAN, mat_c=(1.0, 1000.0), name=""):
    """Hex bar clamped on z=0 whose z=L face is slaved to an extra master node
    at the face centre by a RigidBodyMpc on (UX, UY, UZ) (Mpc.h:51-61); the
    master is node n_nodes (the last node) and belongs to no element."""
    xyz, conn = hex_block(nx, ny, nz, h)
    hz = h if np.isscalar(h) else h[2]
    L = nz * float(hz)
    centre = np.array([[0.5 * xyz[:, 0].max(), 0.5 * xyz[:, 1].max(), L]])
    xyz = np.vstack([xyz, centre])
    m = Mesh(ELEM_SOLID81, xyz, conn, mat_id=mat_id, mat_c=tuple(float(c) for c in mat_c),
             name=name or f"solid81_bar_mpc_{nx}x{ny}x{nz}")
    base = np.nonzero(np.abs(xyz[:-1, 2]) < 1e-12)[0].astype(np.uint32) + 1
    m.fix_nodes = np.repeat(base, 3)
    m.fix_dofs = np.tile(np.array([UX, UY, UZ], dtype=np.int32), base.size)
    top = np.nonzero(np.abs(xyz[:-1, 2] - L) < 1e-12)[0].astype(np.uint32) + 1
    m.rigid_bodies.append(RigidBody(master=int(xyz.shape[0]), slaves=top, dofs=(UX, UY, UZ)))
    return m


def tetra0_block(nx, ny, nz, h=1.0, E=1.0e8, my=0.3, clamp_z0=True, name="") -> Mesh:
    """Hex block split into 6 tetrahedra per cube (positive volumes)."""
    xyz, hconn = hex_block(nx, ny, nz, h)
    # Kuhn split of the cube along its 0-6 diagonal.
    split = [(0, 1, 2, 6), (0, 2, 3, 6), (0, 3, 7, 6), (0, 7, 4, 6), (0, 4, 5, 6), (0, 5, 1, 6)]
    tets = []
    for s in split:
        t = hconn[:, list(s)]
        tets.append(t)
    conn = np.stack(tets, axis=1).reshape(-1, 4).astype(np.uint32)
    # orient every tet to positive volume
    p = xyz[conn.astype(np.int64) - 1]
    vol = np.einsum("ij,ij->i", np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0]), p[:, 3] - p[:, 0])
    flip = vol < 0
    conn[flip, 1], conn[flip, 2] = conn[flip, 2].copy(), conn[flip, 1].copy()
    params = np.zeros((conn.shape[0], 2))
    params[:, 0] = E
    params[:, 1] = my
    m = Mesh(ELEM_TETRA0, xyz, conn, elem_params=params, name=name or f"tetra0_{nx}x{ny}x{nz}")
    if clamp_z0:
        base = np.nonzero(np.abs(xyz[:, 2]) < 1e-12)[0].astype(np.uint32) + 1
        m.fix_nodes = np.repeat(base, 3)
        m.fix_dofs = np.tile(np.array([UX, UY, UZ], dtype=np.int32), base.size)
    return m


def quadth_plate(nx, ny, h=1.0, k=1.0, fix_x0=True, name="") -> Mesh:
    """Regular nx*ny QUAD plate in the z=0 plane, TEMP DoF per node."""
    hx = hy = float(h)
    i = np.arange(nx + 1, dtype=np.float64)
    j = np.arange(ny + 1, dtype=np.float64)
    jj, ii = np.meshgrid(j, i, indexing="ij")
    xyz = np.stack([ii.ravel() * hx, jj.ravel() * hy, np.zeros(ii.size)], axis=1)
    ej, ei = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    ei = ei.ravel().astype(np.int64)
    ej = ej.ravel().astype(np.int64)

    def nid(a, b):
        return 1 + a + (nx + 1) * b

    conn = np.stack([nid(ei, ej), nid(ei + 1, ej), nid(ei + 1, ej + 1), nid(ei, ej + 1)],
                    axis=1).astype(np.uint32)
    params = np.zeros((conn.shape[0], 2))
    params[:, 0] = k
    m = Mesh(ELEM_QUADTH, xyz, conn, elem_params=params, name=name or f"quadth_{nx}x{ny}")
    if fix_x0:
        edge = np.nonzero(np.abs(xyz[:, 0]) < 1e-12)[0].astype(np.uint32) + 1
        m.fix_nodes = edge
        m.fix_dofs = np.full(edge.size, TEMP, dtype=np.int32)
    return m


def quadth_thermal_plate(nx, ny, h=0.1, seed=0, transient=False, name="") -> Mesh:
    """QUADTH plate with the thermal loads of the reference's heat-transfer
    model: per-element conductivity k and volume flux (and rho, c when
    transient), convection lines (htc, etemp) on the top edge and flux lines on
    the right edge; interior nodes jittered so that no two elements are equal."""
    m = quadth_plate(nx, ny, h=h, k=1.0, name=name or f"quadth_thermal_{nx}x{ny}")
    rng = np.random.default_rng(seed)
    ep = np.zeros((m.n_elems, 4 if transient else 2))
    ep[:, 0] = 10.0 + 5.0 * rng.random(m.n_elems)
    ep[:, 1] = np.where(rng.random(m.n_elems) < 0.5, 0.0, 1.0e3 * rng.random(m.n_elems))
    if transient:
        ep[:, 2] = 7800.0
        ep[:, 3] = 460.0 + 10.0 * rng.random(m.n_elems)
    m.elem_params = ep
    inner = (m.xyz[:, 0] > 1e-12) & (m.xyz[:, 0] < nx * h - 1e-12) & \
            (m.xyz[:, 1] > 1e-12) & (m.xyz[:, 1] < ny * h - 1e-12)
    m.xyz[inner, :2] += rng.uniform(-0.2 * h, 0.2 * h, (int(inner.sum()), 2))
    top = [1 + i + (nx + 1) * ny for i in range(nx + 1)]
    right = [1 + nx + (nx + 1) * j for j in range(ny + 1)]
    conn = [(top[i + 1], top[i]) for i in range(nx)] + [(right[j], right[j + 1])
                                                        for j in range(ny)]
    htc = np.r_[25.0 + rng.random(nx), np.zeros(ny)]
    flux = np.r_[np.zeros(nx), 300.0 + 50.0 * rng.random(ny)]
    et = np.zeros((nx + ny, 2))
    et[:nx, 0] = 20.0 + rng.random(nx)
    et[:nx:2, 1] = 35.0          # every other line: its own second temperature
    m.lines = SurfaceLines(np.array(conn, np.uint32), htc, flux, et)
    m.transient = transient
    return m


# ---------------------------------------------------------------------------
# Workload states: nodal displacements u (n_nodes, 3) and element pressures p.
# ---------------------------------------------------------------------------

def stretch_state(mesh: Mesh, stretch=1.2, noise_frac=0.01, p_sigma=0.1, seed=0, h=None):
    """u_x=u_y=0, u_z=(stretch-1)*z plus iid U(-noise*h, +noise*h); p ~ N(0, p_sigma)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    if h is None:
        h = _edge_length(mesh)
    u = np.zeros((mesh.n_nodes, 3))
    u[:, 2] = (stretch - 1.0) * mesh.xyz[:, 2]
    u += rng.uniform(-noise_frac * h, noise_frac * h, size=u.shape)
    p = rng.normal(0.0, p_sigma, size=mesh.n_elems)
    return u, p


def twist_state(mesh: Mesh, angle_deg=30.0, stretch=1.5, noise_frac=0.005, p_sigma=0.1,
                seed=0, h=None):
    """x' = R_z(angle * z / L)(x - c) + c, z' = stretch * z, plus U(+-noise*h)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    if h is None:
        h = _edge_length(mesh)
    x = mesh.xyz
    L = float(x[:, 2].max()) or 1.0
    cx = 0.5 * (x[:, 0].min() + x[:, 0].max())
    cy = 0.5 * (x[:, 1].min() + x[:, 1].max())
    th = np.deg2rad(angle_deg) * x[:, 2] / L
    dx, dy = x[:, 0] - cx, x[:, 1] - cy
    xn = np.stack([cx + np.cos(th) * dx - np.sin(th) * dy,
                   cy + np.sin(th) * dx + np.cos(th) * dy,
                   stretch * x[:, 2]], axis=1)
    u = xn - x + rng.uniform(-noise_frac * h, noise_frac * h, size=x.shape)
    p = rng.normal(0.0, p_sigma, size=mesh.n_elems)
    return u, p


def _edge_length(mesh: Mesh) -> float:
    c = mesh.conn[0].astype(np.int64) - 1
    return float(np.linalg.norm(mesh.xyz[c[1]] - mesh.xyz[c[0]]))


# ---------------------------------------------------------------------------
# The benchmark configurations.
# ---------------------------------------------------------------------------

def config_cube(n=10, seed=1, clamp_z0=False):
    """Unit cube of n^3 SOLID81 hexes, Neo-Hookean C10=0.5 (G=1.0), K=1000,
    uniaxial stretch 1.2 along z with +-0.01h noise, p ~ N(0, 0.1)."""
    h = 1.0 / n
    mesh = solid81_block(n, n, n, h, MAT_NEO_HOOKEAN, (1.0, 1000.0), clamp_z0=clamp_z0,
                         name=f"cube{n}_neohookean" + ("_clamped" if clamp_z0 else ""))
    u, p = stretch_state(mesh, 1.2, 0.01, 0.1, seed=seed, h=h)
    return mesh, u, p


def config_twist(n=100, seed=2):
    """Unit-cube block of n^3 SOLID81 hexes, Mooney-Rivlin C10=0.4, C01=0.1,
    K=2000; 30 deg end twist about the block axis plus 1.5 stretch with
    +-0.005h noise; p ~ N(0, 0.1)."""
    h = 1.0 / n
    mesh = solid81_block(n, n, n, h, MAT_MOONEY_RIVLIN, (0.4, 0.1, 2000.0),
                         name=f"block{n}_mooneyrivlin_twist")
    u, p = twist_state(mesh, 30.0, 1.5, 0.005, 0.1, seed=seed, h=h)
    return mesh, u, p


def batched_meshes(n_meshes=256, lo=4, hi=40, seed=3, max_side=None):
    """Uneven hex-block meshes: edge counts per side drawn log-uniform in
    [lo, hi], C10 ~ U(0.2, 1.0), K = C10 * U(500, 5000), stretch ~ U(1.0, 1.8)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for i in range(n_meshes):
        sides = np.rint(np.exp(rng.uniform(math.log(lo), math.log(hi), size=3))).astype(int)
        if max_side is not None:
            sides = np.minimum(sides, max_side)
        c10 = rng.uniform(0.2, 1.0)
        kb = c10 * rng.uniform(500.0, 5000.0)
        lam = rng.uniform(1.0, 1.8)
        h = 1.0 / int(sides.max())
        mesh = solid81_block(*(int(s) for s in sides), h, MAT_NEO_HOOKEAN, (2.0 * c10, kb),
                             name=f"batch{i}")
        u, p = stretch_state(mesh, lam, 0.01, 0.1, seed=int(rng.integers(1 << 31)), h=h)
        out.append((mesh, u, p))
    return out


def plane41_plate(nx, ny, h=1.0, mat_id=MAT_NEO_HOOKEAN, mat_c=(1.0, 500.0), clamp_y0=False,
                  name="") -> Mesh:
    """Regular nx*ny PLANE41 plate (4-node plane-strain u/p quads, UX/UY per
    node, HYDRO_PRESSURE per element) in the z = 0 plane, nodes numbered
    x-fastest, element nodes counter-clockwise; optionally clamped on y = 0."""
    q = quadth_plate(nx, ny, h, fix_x0=False)
    m = Mesh(ELEM_PLANE41, q.xyz, q.conn, mat_id=mat_id, mat_c=tuple(float(c) for c in mat_c),
             name=name or f"plane41_{nx}x{ny}")
    if clamp_y0:
        edge = np.nonzero(np.abs(q.xyz[:, 1]) < 1e-12)[0].astype(np.uint32) + 1
        m.fix_nodes = np.repeat(edge, 2)
        m.fix_dofs = np.tile(np.array([UX, UY], dtype=np.int32), edge.size)
    return m


def plane_state(mesh, stretch=1.2, shear=0.1, noise_frac=0.01, seed=0, p_sigma=0.1):
    """In-plane stretch along y with a simple shear and seeded noise on UX/UY;
    UZ stays 0; element pressures ~ N(0, p_sigma)."""
    rng = np.random.default_rng(seed)
    x = mesh.xyz
    h = float(np.min(np.abs(np.diff(np.unique(x[:, 0]))))) if mesh.n_nodes > 1 else 1.0
    u = np.zeros_like(x)
    u[:, 0] = shear * x[:, 1]
    u[:, 1] = (stretch - 1.0) * x[:, 1]
    u[:, :2] += rng.uniform(-noise_frac * h, noise_frac * h, size=(x.shape[0], 2))
    p = rng.normal(0.0, p_sigma, size=mesh.n_elems)
    return u, p


def u_to_vector(eq_node: np.ndarray, eq_elem: np.ndarray, u: np.ndarray, p: np.ndarray,
                n_total: int, extra_node_values: dict | None = None) -> np.ndarray:
    """Scatter nodal displacements and element pressures into the solution
    vector indexed by equation number (vecU[eq-1], FEStorage.h:338-343).
    eq_node is (n_nodes, 8), eq_elem is (n_elems, 8); 0 marks an unused DoF."""
    U = np.zeros(n_total)
    for d in range(3):
        eq = eq_node[: u.shape[0], d].astype(np.int64)
        ok = eq > 0
        U[eq[ok] - 1] = u[ok, d]
    eqp = eq_elem[:, HYDRO_PRESSURE].astype(np.int64)
    ok = eqp > 0
    if p is not None and ok.any():
        U[eqp[ok] - 1] = p[ok]
    if extra_node_values:
        for (node, dof), val in extra_node_values.items():
            e = int(eq_node[node - 1, dof])
            if e > 0:
                U[e - 1] = val
    return U
