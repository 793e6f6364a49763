"""Quasi-static Newton-Raphson driver around the GPU assembly.

Mirrors NonlinearFESolver::solve (FESolver.cpp:407-508) with TimeControl
(FESolver.cpp:34-56): per load step the fixed DoFs move to value * t, each
equilibrium iteration assembles K and F (on the GPU), solves

    K(2) dU_sl = F_sl + R_sl - K(1,2)^T dU_c          (FESolver.cpp:449-457)

updates U_s += dU_s, U_l = dU_l, recovers the reactions
R_c = K(1) dU_c + K(1,2) dU_sl - F_c (FESolver.cpp:464-467) and calls
updateResults.  The reference's kinematic criterion (mean |dU_s| / tol < tol,
FESolver.cpp:511-521) is kept; a residual criterion ||F_sl + R_sl|| < tol can
be selected instead.  The linear solve runs on the host (SciPy's sparse LU),
standing in for the reference's EquationSolver (EquationSolver.h:19-34).

A predictor may propose each load step's starting state (the learned start);
the plain start (previous converged state) is kept whenever the proposal's
residual is not smaller.
"""
from __future__ import annotations

import dataclasses
import time

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


class TimeControl:
    """Load stepping of the reference (FESolver.h:27-56, FESolver.cpp:34-56)."""

    def __init__(self, start=0.0, end=1.0):
        self.start, self.end = start, end
        self.t = start
        self.dt = 0.0
        self.step = 0
        self.eq_step = 0

    def next_step(self, delta):
        if self.t >= self.end:
            return False
        if self.t + delta >= self.end:
            self.dt = self.end - self.t
        elif self.t + 2 * delta >= self.end:
            self.dt = (self.end - self.t) / 2.0
        else:
            self.dt = delta
        self.t += self.dt
        self.step += 1
        self.eq_step = 0
        return True

    def normalized(self):
        return (self.t - self.start) / (self.end - self.start)


def csr_full(iofeir, columns, values, rows, cols, symmetric_upper):
    ind = iofeir.astype(np.int64) - 1
    m = sp.csr_matrix((values, columns.astype(np.int64) - 1, ind), shape=(rows, cols))
    if symmetric_upper:
        m = (m + sp.triu(m, 1).T).tocsr()
    return m


@dataclasses.dataclass
class StepRecord:
    time: float
    iterations: int
    residuals: list
    criteria: list
    predicted: bool = False
    prediction_residual: float | None = None
    plain_residual: float | None = None


def row_points(backend, nc, n_unk, n_mpc):
    """A point per K(2) row, for nested_dissection: the node of a nodal DoF,
    the element centroid of an element DoF, the first term's node of an MPC
    equation."""
    mesh = backend.mesh
    xyz = np.asarray(mesh.xyz, dtype=np.float64)
    conn = np.asarray(mesh.conn, dtype=np.int64)
    ne, ee = backend.eq_numbers()
    pts = np.zeros((n_unk + n_mpc, 3))
    for d in range(ne.shape[1]):
        eq = ne[:, d].astype(np.int64)
        sel = eq > nc
        pts[eq[sel] - nc - 1] = xyz[sel]
    cen = xyz[conn - 1].mean(axis=1)
    for d in range(ee.shape[1]):
        eq = ee[:, d].astype(np.int64)
        sel = eq > nc
        pts[eq[sel] - nc - 1] = cen[sel]
    first = [int(q.nodes[0]) for q in mesh.mpcs]
    for rb in mesh.rigid_bodies:
        first += [int(n) for n in rb.slaves for _ in rb.dofs]
    for k, n in enumerate(first):
        pts[n_unk + k] = xyz[n - 1]
    return pts


def nested_dissection(K, pts, leaf=64):
    """Fill-reducing order of a symmetric sparse pattern with a point per row:
    split the rows at the median of their longest coordinate extent; the rows
    of the lower half that couple to the upper half form the separator and
    come after both halves; recurse down to `leaf` rows.  K: CSR holding both
    triangles; returns the permutation (new position -> row)."""
    n = K.shape[0]
    order = []

    def rec(idx):
        if len(idx) <= leaf:
            order.extend(idx.tolist())
            return
        P = pts[idx]
        ax = int(np.argmax(P.max(axis=0) - P.min(axis=0)))
        lower = P[:, ax] < np.median(P[:, ax])
        if lower.all() or not lower.any():
            order.extend(idx.tolist())
            return
        li, ri = idx[lower], idx[~lower]
        upper = np.zeros(n, dtype=bool)
        upper[ri] = True
        sub = K[li]
        row = np.repeat(np.arange(len(li)), np.diff(sub.indptr))
        touch = np.zeros(len(li), dtype=bool)
        touch[row[upper[sub.indices]]] = True
        rec(li[~touch])
        rec(ri)
        order.extend(li[touch].tolist())

    rec(np.arange(n))
    return np.asarray(order, dtype=np.int64)


class NewtonSolver:
    """backend: an object with eq_numbers(), pattern(b), K(b), F(), set_U(U),
    update(), assemble(), block_mv(block, trans, x, coef, y), n_con, n_unk,
    n_mpc, n_total, blocks -- the GPU FEStorage (nla3d_gb300.storage, whose
    block_mv runs nla3d_block_mv on the device K) or the CPU oracle model.
    The right-hand side, residual and reactions go through block_mv (the
    reference's matBVprod / matBTVprod); only the solve reads K(2) on the host."""

    def __init__(self, backend, fixes, n_loadsteps=10, n_iterations=15, kinematic_tol=1e-3,
                 residual_tol=None, loads=(), solver="direct"):
        """solver: "direct" factors K(2) every iteration (SciPy SuperLU, standing
        in for the reference's EquationSolver); "nd" does the same after a
        geometric nested-dissection ordering of K(2) (one point per equation
        from backend.mesh), several times less fill on 3D meshes; "lu-gmres"
        keeps the last factorisation as the preconditioner of GMRES and
        refactors only when GMRES needs more than 30 iterations; "gpu" factors
        the device K(2) in place with the library's multifrontal LDL^T
        (nla3d_gb300.ldlt; the same nested-dissection order, the MPC
        equations and master DoFs last), "gpu-fp32" with FP32 fronts, "gpu-tc"
        with FP32 fronts updated on the tensor cores.  Every
        non-default solve is checked to a relative residual of 1e-10."""
        if solver not in ("direct", "nd", "lu-gmres", "gpu", "gpu-fp32", "gpu-tc"):
            raise ValueError(solver)
        self._ldlt = None
        self.inexact_solves = 0
        self.fp64_refactorizations = 0
        self._perm = None
        self.solver = solver
        self._lu = None
        self.factorizations = 0
        self.krylov_iterations = 0
        self.b = backend
        self.n_loadsteps = n_loadsteps
        self.n_iterations = n_iterations
        self.kinematic_tol = kinematic_tol
        self.residual_tol = residual_tol
        ne, ee = backend.eq_numbers()
        self.ne = ne
        self.nc, self.nu, self.nm = backend.n_con, backend.n_unk, backend.n_mpc
        self.n = backend.n_total
        # fixes: (node, dof, value) -- FESolver::addFix; loads: (node, dof, value)
        self.fix_eq = np.array([int(ne[n - 1, d]) for n, d, _ in fixes], dtype=np.int64)
        self.fix_val = np.array([v for _, _, v in fixes], dtype=np.float64)
        assert np.all(self.fix_eq >= 1) and np.all(self.fix_eq <= self.nc), "fix on an unconstrained DoF"
        self.load_eq = np.array([int(ne[n - 1, d]) for n, d, _ in loads], dtype=np.int64)
        self.load_val = np.array([v for _, _, v in loads], dtype=np.float64)
        self.patterns = {blk: backend.pattern(blk) for blk in (1, 12, 2)}
        self.U = np.zeros(self.n)
        self.R = np.zeros(self.n)
        self.records: list[StepRecord] = []
        self.reactions: list[np.ndarray] = [np.zeros(self.nc)]
        # host wall time per phase (s): assemble (set_U + assembly + F to the
        # host), factor, solve (with refinement), update (updateResults),
        # vectors (right-hand side, residual, reactions)
        self.timing = {"assemble": 0.0, "factor": 0.0, "solve": 0.0, "update": 0.0,
                       "vectors": 0.0}

    def close(self):
        """Release the device factorisation (its fronts can take most of HBM)."""
        if self._ldlt is not None:
            self._ldlt.close()
            self._ldlt = None

    # ---- the global system ----
    def _K2(self):
        rows2, cols2, _ = self.b.blocks[2]
        return csr_full(*self.patterns[2], self.b.K(2), rows2, cols2, True)

    def _row_points(self):
        return row_points(self.b, self.nc, self.nu, self.nm)

    def _solve_gpu(self, rhs):
        """The device LDL^T: a solve refined to 1e-10 is used as is; one that
        stops above it (FP32 fronts on a badly conditioned tangent) is still
        used when its residual is below 1e-6 (an inexact Newton step, counted
        in `inexact_solves`); otherwise this iteration is refactored with FP64
        fronts."""
        from .ldlt import DeviceLDLT, fill_reducing_order
        if self._ldlt is None:
            io, co = self.patterns[2]
            self._perm = fill_reducing_order(io, co, self._row_points(), self.nu)
            self._ldlt = DeviceLDLT.for_storage(
                self.b, self._perm, {"gpu": "fp64", "gpu-fp32": "fp32", "gpu-tc": "fp32-tc"}[self.solver])
        t0 = time.perf_counter()
        self._ldlt.factor(self.b)
        t1 = time.perf_counter()
        self.timing["factor"] += t1 - t0
        self.factorizations += 1
        x = self._ldlt.solve_host(self.b, rhs, max_refine=100, tol=1e-10, strict=False)
        self.timing["solve"] += time.perf_counter() - t1
        self.krylov_iterations += self._ldlt.last_steps
        rel = self._ldlt.last_residual
        if rel <= 1e-10:
            return x
        if rel <= 1e-6:
            self.inexact_solves += 1
            return x
        # FP64 fronts for this iteration only: their memory (twice the FP32
        # fronts') is released right after the solve
        ld64 = DeviceLDLT.for_storage(self.b, self._perm, "fp64")
        try:
            ld64.factor(self.b)
            self.fp64_refactorizations += 1
            return ld64.solve_host(self.b, rhs, max_refine=100, tol=1e-10)
        finally:
            ld64.close()

    def _solve(self, K2, rhs):
        if self.solver.startswith("gpu"):
            return self._solve_gpu(rhs)
        if self.solver == "direct":
            self.factorizations += 1
            return spla.spsolve(K2, rhs, permc_spec="MMD_AT_PLUS_A")
        if self.solver == "nd":
            if self._perm is None:
                self._perm = nested_dissection(K2.tocsr(), self._row_points())
            p = self._perm
            lu = spla.splu(K2[p][:, p].tocsc(), permc_spec="NATURAL",
                           options=dict(SymmetricMode=True, DiagPivotThresh=0.001))
            self.factorizations += 1
            x = np.empty_like(rhs)
            x[p] = lu.solve(rhs[p])
            tol = 1e-10 * max(np.linalg.norm(rhs), 1e-300)
            for _ in range(3):          # iterative refinement with the same factors
                r = rhs - K2 @ x
                if np.linalg.norm(r) <= tol:
                    return x
                dx = np.empty_like(rhs)
                dx[p] = lu.solve(r[p])
                x += dx
            if np.linalg.norm(rhs - K2 @ x) <= tol:
                return x
            return spla.spsolve(K2, rhs, permc_spec="MMD_AT_PLUS_A")
        nrm = float(np.linalg.norm(rhs))
        if nrm == 0.0:
            return np.zeros_like(rhs)
        if self._lu is not None:
            its = [0]

            def count(_):
                its[0] += 1

            M = spla.LinearOperator(K2.shape, matvec=self._lu.solve, dtype=np.float64)
            x, info = spla.gmres(K2, rhs, x0=self._lu.solve(rhs), M=M, rtol=1e-13, atol=0.0,
                                 restart=30, maxiter=1, callback=count,
                                 callback_type="pr_norm")
            self.krylov_iterations += its[0]
            if info == 0 and np.linalg.norm(K2 @ x - rhs) <= 1e-11 * nrm:
                return x
        self._lu = spla.splu(K2, permc_spec="COLAMD")
        self.factorizations += 1
        return self._lu.solve(rhs)

    def _rhs(self, F, dUc):
        """FESolver.cpp:449-454: rhs = F_sl + R_sl - K(1,2)^T dUc, the last
        term through the backend's matBTVprod."""
        y = F[self.nc:] + self.R[self.nc:]
        if self.nc == 0:
            return y
        return self.b.block_mv(12, 1, dUc, -1.0, y)

    def _reactions(self, F, dUc, dUsl):
        """FESolver.cpp:463-466: R_c = K(1) dUc + K(1,2) dUsl - F_c (matBVprod)."""
        Rc = np.zeros(self.nc)
        if self.nc == 0:
            return Rc
        Rc = self.b.block_mv(1, 0, dUc, 1.0, Rc)
        Rc = self.b.block_mv(12, 0, dUsl, 1.0, Rc)
        return Rc - F[: self.nc]

    def _apply_bc(self, t):
        """FESolver::applyBoundaryConditions (FESolver.cpp:229-247)."""
        self.R[:] = 0.0
        if self.load_eq.size:
            np.add.at(self.R, self.load_eq - 1, self.load_val * t)
        Uc = self.U[: self.nc].copy()
        Uc[self.fix_eq - 1] = self.fix_val * t
        return Uc

    def _assemble(self, U):
        t0 = time.perf_counter()
        self.b.set_U(U)
        self.b.assemble()
        F = self.b.F()
        self.timing["assemble"] += time.perf_counter() - t0
        return F

    def residual(self, F, dUc):
        """Equilibrium residual of the unknown + MPC rows.  The reference solves
        the Lagrange multipliers as totals (vecUl = deltaUl, FESolver.cpp:461),
        so its right-hand side F_sl + R_sl - K12^T dUc still contains the
        constraint forces; the residual removes them: r = rhs - K2 [0; U_l]."""
        r = self._rhs(F, dUc)
        if self.nm == 0:
            return r
        lam = np.zeros(self.nu + self.nm)
        lam[self.nu:] = self.U[self.nc + self.nu:]
        return self.b.block_mv(2, 0, lam, -1.0, r)

    # ---- the load-step loop ----
    def solve(self, predictor=None, on_converged=None):
        tc = TimeControl()
        delta = (tc.end - tc.start) / self.n_loadsteps
        Ucprev = np.zeros(self.nc)
        self.b.set_U(self.U)
        self.b.update()
        while tc.next_step(delta):
            t = tc.normalized()
            rec = StepRecord(time=t, iterations=0, residuals=[], criteria=[])
            self.current = rec
            Uc_new = self._apply_bc(t)
            if predictor is not None:
                prop = predictor.propose(self, t)
                if prop is not None:
                    # residual of the plain start: F(U_prev) - K12^T dUc (linearised)
                    F0 = self._assemble(self.U)
                    r_plain = self.residual(F0, Uc_new - Ucprev)
                    Up = prop.copy()
                    Up[: self.nc] = Uc_new
                    Uold = self.U
                    self.U = Up
                    self.b.set_U(Up)
                    self.b.update()
                    Fp = self._assemble(Up)
                    r_pred = float(np.linalg.norm(self.residual(Fp, 0.0 * Uc_new)))
                    self.U = Uold
                    rec.prediction_residual, rec.plain_residual = r_pred, float(np.linalg.norm(r_plain))
                    if np.isfinite(r_pred) and r_pred < rec.plain_residual:
                        self.U = Up
                        Ucprev = Uc_new.copy()
                        rec.predicted = True
                    else:
                        self.b.set_U(self.U)
                        self.b.update()
            converged = False
            while True:
                tc.eq_step += 1
                F = self._assemble(self.U)
                Uc = self._apply_bc(t)
                dUc = Uc - Ucprev
                t0 = time.perf_counter()
                rhs = self._rhs(F, dUc)
                rnorm = float(np.linalg.norm(self.residual(F, dUc)))
                self.timing["vectors"] += time.perf_counter() - t0
                rec.residuals.append(rnorm)
                if self.residual_tol is not None and tc.eq_step > 1 and rnorm < self.residual_tol \
                        and not np.any(dUc):
                    # converged without a further solve: reactions for a zero increment
                    sl = np.zeros(self.nu + self.nm)
                    sl[self.nu:] = self.U[self.nc + self.nu:]
                    self.R[: self.nc] = self._reactions(F, np.zeros(self.nc), sl)
                    rec.iterations = tc.eq_step - 1
                    converged = True
                    break
                K2 = None if self.solver.startswith("gpu") else self._K2().tocsc()
                dUsl = self._solve(K2, rhs)
                self.U[: self.nc] = Uc
                self.U[self.nc: self.nc + self.nu] += dUsl[: self.nu]
                self.U[self.nc + self.nu:] = dUsl[self.nu:]
                t0 = time.perf_counter()
                self.R[: self.nc] = self._reactions(F, dUc, dUsl)
                t1 = time.perf_counter()
                self.timing["vectors"] += t1 - t0
                Ucprev = Uc.copy()
                self.b.set_U(self.U)
                self.b.update()
                self.timing["update"] += time.perf_counter() - t1
                crit = float(np.abs(dUsl[: self.nu]).sum() / max(self.nu, 1)) / self.kinematic_tol
                rec.criteria.append(crit)
                if not np.isfinite(crit) or crit > 1e6:
                    raise RuntimeError("The solution is diverged!")
                if self.residual_tol is None and crit < self.kinematic_tol:
                    rec.iterations = tc.eq_step
                    converged = True
                    break
                if tc.eq_step >= self.n_iterations:
                    rec.iterations = tc.eq_step
                    break
            if not converged:
                raise RuntimeError(f"The solution is not converged with {tc.eq_step} equilibrium "
                                   "iterations")
            self.records.append(rec)
            self.reactions.append(self.R[: self.nc].copy())
            if on_converged is not None:
                on_converged(self, t)
        return self

    def reaction(self, node, dof):
        """Reaction history of one constrained DoF (ReactionProcessor, summed per step)."""
        eq = int(self.ne[node - 1, dof])
        return np.array([r[eq - 1] for r in self.reactions])
