"""Lock-step Newton-Raphson over a batch of problems that share one mesh.

Studies such as the learned-start training set solve one mesh thousands of
times with different material constants and boundary values.  Solved one at a
time, a 20^3 block (35,783 equations, small fronts) leaves the GPU mostly
idle, so this driver advances B problems together:

* one batched assembly context holds the B meshes (nla3d_create_batch; each
  keeps its own numbering, pattern, K and F, as one reference FEStorage each),
  so every Newton iteration assembles all of them with one launch of each
  kernel;
* their K(2) blocks form one block-diagonal matrix, factored by one device
  LDL^T (nla3d_ldlt_*).  Its symbolic analysis depends only on the batch
  shape and is shared by every batch of that shape; its supernodal tree is B
  copies of one tree, so every level of the factorisation carries B times
  the fronts of a single solve;
* every problem follows NonlinearFESolver::solve (FESolver.cpp:407-521) with
  the residual criterion exactly as nla3d_gb300.newton.NewtonSolver does:
  its own load-step bookkeeping, right-hand side F_sl + R_sl - K(1,2)^T dU_c
  (the reference's matBTVprod, nla3d_block_mv per mesh), residual, solve and
  update.  A problem that has converged in the current load step waits with
  a zero right-hand side until the others have.

Each problem's right-hand side is scaled to unit norm before the block solve
and the refinement tolerance is divided by sqrt(active problems), so every
problem's own solve meets the single-problem driver's 1e-10 relative
residual.  Vectors live on the device (PyTorch tensors as plumbing; the
library's device arrays are viewed in place, without copies), and all work
runs on one stream: the library's own streams do not synchronise with the
legacy default stream.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib
from .batch import BatchAssembly
from .ldlt import DeviceLDLT, fill_reducing_order
from .newton import TimeControl, row_points


class _CudaArray:
    """Zero-copy view of library-owned device memory (torch.as_tensor)."""

    def __init__(self, ptr, n, typestr="<f8"):
        self.__cuda_array_interface__ = {"shape": (int(n),), "typestr": typestr,
                                         "data": (int(ptr), False), "version": 2,
                                         "strides": None}


def device_view(torch, ptr, n):
    """float64 tensor over n doubles of device memory at ptr (not owned)."""
    return torch.as_tensor(_CudaArray(ptr, n), device="cuda")


def block_diagonal_pattern(iofeir, columns, copies):
    """Upper CSR (1-based) of diag(A, A, ..., A) with `copies` copies of A."""
    io = np.asarray(iofeir, dtype=np.int64)
    co = np.asarray(columns, dtype=np.int64)
    n, nnz = io.size - 1, int(io[-1] - io[0])
    if copies * max(n, nnz) >= 2 ** 32 - 1:
        raise ValueError("block-diagonal pattern exceeds 32-bit indices")
    k = np.arange(copies, dtype=np.int64)[:, None]
    io_bd = np.append((io[None, :-1] + nnz * k).ravel(), io[-1] + nnz * (copies - 1))
    co_bd = (co[None, :] + n * k).ravel()
    return io_bd.astype(np.uint32), co_bd.astype(np.uint32)


def block_diagonal_order(perm, n, copies):
    """The order of diag(A, ..., A) that applies `perm` (perm[new] = row) to
    every copy, copy after copy."""
    p = np.asarray(perm, dtype=np.int64)
    return (p[None, :] + n * np.arange(copies, dtype=np.int64)[:, None]).ravel().astype(np.int32)


def same_topology(problems):
    """Problems that one BatchNewton can hold: one mesh (nodes, elements,
    constraints), one load-step count; materials and fixed values may differ."""
    m0, p0 = problems[0].mesh, problems[0]
    for pb in problems[1:]:
        m = pb.mesh
        if (m.n_nodes != m0.n_nodes or m.n_elems != m0.n_elems
                or not np.array_equal(m.conn, m0.conn) or not np.array_equal(m.xyz, m0.xyz)
                or not np.array_equal(m.fix_nodes, m0.fix_nodes)
                or not np.array_equal(m.fix_dofs, m0.fix_dofs)
                or len(m.mpcs) != len(m0.mpcs) or len(m.rigid_bodies) != len(m0.rigid_bodies)
                or pb.n_loadsteps != p0.n_loadsteps
                or [f[:2] for f in pb.fixes] != [f[:2] for f in p0.fixes]):
            return False
    return True


class BlockSolver:
    """The block-diagonal device LDL^T for batches of one shape (B copies of
    one K(2) pattern); reusable across BatchNewton instances of that shape."""

    def __init__(self, iofeir, columns, perm, copies, fronts="fp32", stream=None):
        """stream: the torch.cuda.Stream every user of this solver runs on (a
        new one if None)."""
        import torch
        self.stream = stream if stream is not None else torch.cuda.Stream()
        self.n = int(np.asarray(iofeir).size - 1)
        self.nnz = int(np.asarray(iofeir)[-1] - np.asarray(iofeir)[0])
        self.copies = copies
        self.fronts = fronts
        io_bd, co_bd = block_diagonal_pattern(iofeir, columns, copies)
        self.perm_bd = block_diagonal_order(perm, self.n, copies)
        self.io_bd, self.co_bd = io_bd, co_bd
        self.ldlt = DeviceLDLT(io_bd, co_bd, self.perm_bd, fronts, self.stream.cuda_stream)
        self._ldlt64 = None
        self.factorizations = 0
        self.fp64_refactorizations = 0

    def fp64(self):
        if self._ldlt64 is None:
            self._ldlt64 = DeviceLDLT(self.io_bd, self.co_bd, self.perm_bd, "fp64",
                                      self.stream.cuda_stream)
        return self._ldlt64


class BatchNewton:
    """B problems (same mesh and constrained DoFs; any material constants and
    fixed values; learned.Problem objects) solved in lock step with the
    residual criterion.  After solve(): `iterations` (B x load steps),
    `predicted` (B x load steps, the learned / extrapolated start kept),
    `failed` (B), `U` (B x n_total, device)."""

    def __init__(self, problems, precision="fp64", fronts="fp32", residual_tol=1e-8,
                 n_iterations=25, kinematic_tol=1e-3, block_solver=None):
        import torch
        if not problems:
            raise ValueError("no problems")
        if not same_topology(problems):
            raise ValueError("BatchNewton needs problems on one mesh with the same constraints")
        if residual_tol is None:
            raise ValueError("BatchNewton runs the residual criterion")
        self.torch = torch
        self.lib = _lib.load()
        self.stream = block_solver.stream if block_solver is not None else torch.cuda.Stream()
        with torch.cuda.stream(self.stream):
            self._init(problems, precision, fronts, residual_tol, n_iterations, kinematic_tol,
                       block_solver)

    def _init(self, problems, precision, fronts, residual_tol, n_iterations, kinematic_tol,
              block_solver):
        torch = self.torch
        self.problems = list(problems)
        self.B = len(problems)
        self.residual_tol = residual_tol
        self.n_iterations = n_iterations
        self.kinematic_tol = kinematic_tol
        self.n_loadsteps = problems[0].n_loadsteps
        self.ba = BatchAssembly([pb.mesh for pb in problems], precision,
                                stream=self.stream.cuda_stream).init()
        info = self.ba.info
        if not (info == info[0]).all():
            raise ValueError("meshes of one batch must number their equations alike")
        n_dofs, self.nc, self.nu, self.nm = (int(v) for v in info[0, :4])
        self.n = n_dofs + self.nm
        self.n2 = self.nu + self.nm
        self.nnz = {1: int(info[0, 6]), 12: int(info[0, 9]), 2: int(info[0, 12])}
        if np.any(np.diff(self.ba.u_off) != self.n):
            raise ValueError("unexpected vecU layout of the batch")
        self.ne, self.ee = self.ba.eq_numbers(0)
        fixes0 = problems[0].fixes
        self.fix_eq = np.array([int(self.ne[nd - 1, d]) for nd, d, _ in fixes0], dtype=np.int64)
        if np.any(self.fix_eq < 1) or np.any(self.fix_eq > self.nc):
            raise ValueError("fix on an unconstrained DoF")
        fix_val = np.array([[v for _, _, v in pb.fixes] for pb in problems], dtype=np.float64)
        dev = torch.device("cuda")
        self.fix_idx = torch.from_numpy(self.fix_eq - 1).to(dev)
        self.fix_val = torch.from_numpy(fix_val).to(dev)
        io2, co2 = self.ba.pattern(0, 2)
        if block_solver is None:
            mesh = problems[0].mesh

            class _Geom:   # what row_points reads of a backend
                pass
            g = _Geom()
            g.mesh = mesh
            g.eq_numbers = lambda: (self.ne, self.ee)
            perm = fill_reducing_order(io2, co2, row_points(g, self.nc, self.nu, self.nm), self.nu)
            block_solver = BlockSolver(io2, co2, perm, self.B, fronts, self.stream)
        if block_solver.copies != self.B or block_solver.n != self.n2 \
                or block_solver.nnz != self.nnz[2]:
            raise ValueError("block solver of another batch shape")
        self.bs = block_solver
        # device views of the batch's K values and F; K(2) gather index
        p, nK = ctypes.c_void_p(), ctypes.c_uint64()
        self._check(self.lib.nla3d_device_K(self.ba.h, 0, ctypes.byref(p), ctypes.byref(nK)))
        self.K_all = device_view(torch, p.value, nK.value)
        pf, nF = ctypes.c_void_p(), ctypes.c_uint64()
        self._check(self.lib.nla3d_device_F(self.ba.h, ctypes.byref(pf), ctypes.byref(nF)))
        self.F_all = device_view(torch, pf.value, nF.value).view(self.B, self.n)
        k2 = (self.ba.k_off[:-1, None].astype(np.int64) + self.nnz[1] + self.nnz[12]
              + np.arange(self.nnz[2], dtype=np.int64)[None, :]).ravel()
        self.k2_idx = torch.from_numpy(k2).to(dev)
        self.K2 = torch.empty(self.B * self.nnz[2], dtype=torch.float64, device=dev)
        self.U = torch.zeros(self.B, self.n, dtype=torch.float64, device=dev)
        self.iterations = np.zeros((self.B, 0), np.int64)
        self.predicted = np.zeros((self.B, 0), bool)
        self.factorizations = 0
        self.inexact_solves = 0
        self.failed = np.zeros(self.B, bool)

    def _check(self, rc):
        if rc:
            msg = self.lib.nla3d_last_error(self.ba.h)
            raise _lib.Nla3dError(rc, msg.decode() if msg else "")

    def close(self):
        self.ba.close()

    # ---- per-mesh block products (the reference's matBVprod / matBTVprod) ----
    def _block_mv(self, mesh, block, trans, x, coef, y):
        self._check(self.lib.nla3d_block_mv(self.ba.h, int(mesh), block, int(trans),
                                            ctypes.c_void_p(x.data_ptr()), float(coef),
                                            ctypes.c_void_p(y.data_ptr())))

    def _assemble(self, U):
        self.ba.set_U_device(U.data_ptr(), U.numel())
        self.ba.assemble()
        return self.F_all

    def _update(self, U):
        self.ba.set_U_device(U.data_ptr(), U.numel())
        self.ba.update()

    def _rhs(self, F, dUc, active):
        """F_sl + R_sl - K(1,2)^T dU_c per problem (FESolver.cpp:449-454); no
        nodal loads (R = 0).  dUc: B x nc device tensor or None (zero).  A
        zero dU_c row skips the product (it would only add -0)."""
        rhs = self.torch.empty((self.B, self.n - self.nc), dtype=F.dtype, device=F.device)
        rhs.copy_(F[:, self.nc:])
        if dUc is not None and self.nc:
            nz = (dUc != 0).any(dim=1).cpu().numpy()
            for j in np.nonzero(nz & active)[0]:
                self._block_mv(j, 12, 1, dUc[j], -1.0, rhs[j])
        return rhs

    def _residual(self, rhs, U, active):
        """rhs - K(2) [0; U_l] (the multipliers' forces removed; MPC meshes)."""
        if self.nm == 0:
            return rhs
        r = rhs.clone()
        lam = self.torch.zeros(self.B, self.n2, dtype=self.torch.float64, device=U.device)
        lam[:, self.nu:] = U[:, self.nc + self.nu:]
        for j in np.nonzero(active)[0]:
            self._block_mv(j, 2, 0, lam[j], -1.0, r[j])
        return r

    def _Uc(self, U, t):
        """FESolver::applyBoundaryConditions: constrained values at load factor t."""
        Uc = U[:, : self.nc].clone()
        Uc[:, self.fix_idx] = self.fix_val * t
        return Uc

    def _solve(self, rhs, active):
        """Block-diagonal solve of the active problems' K(2) dU = rhs."""
        torch = self.torch
        b = rhs.clone()
        b[~torch.from_numpy(active).to(b.device)] = 0.0
        norms = torch.linalg.vector_norm(b, dim=1)
        scale = torch.where(norms > 0, norms, torch.ones_like(norms))
        b /= scale[:, None]
        x = torch.empty_like(b)
        torch.index_select(self.K_all, 0, self.k2_idx, out=self.K2)
        n_act = max(int(active.sum()), 1)
        tol = 1e-10 / math.sqrt(n_act)
        ld = self.bs.ldlt
        ld.factor_device(self.K2.data_ptr())
        self.bs.factorizations += 1
        self.factorizations += 1
        ld.solve_device(self.K2.data_ptr(), b.data_ptr(), x.data_ptr(), max_refine=100, tol=tol,
                        strict=False)
        if ld.last_residual > tol:
            if ld.last_residual <= 1e-6:
                self.inexact_solves += 1
            else:
                ld = self.bs.fp64()
                ld.factor_device(self.K2.data_ptr())
                self.bs.fp64_refactorizations += 1
                ld.solve_device(self.K2.data_ptr(), b.data_ptr(), x.data_ptr(), max_refine=100,
                                tol=tol)
        return x * scale[:, None]

    # ---- the load-step loop ----
    def solve(self, predictor=None, on_converged=None):
        """predictor: object with propose(driver, t) -> (B x n device tensor
        or None, B bool mask of problems with a proposal); on_converged(driver,
        t): called after every load step with self.U.  Both run on the
        driver's stream."""
        with self.torch.cuda.stream(self.stream):
            out = self._solve_steps(predictor, on_converged)
        self.stream.synchronize()
        return out

    def _solve_steps(self, predictor, on_converged):
        torch = self.torch
        tc = TimeControl()
        delta = (tc.end - tc.start) / self.n_loadsteps
        B = self.B
        self.U.zero_()
        Ucprev = torch.zeros(B, self.nc, dtype=torch.float64, device=self.U.device)
        self._update(self.U)
        its, preds = [], []
        while tc.next_step(delta):
            t = tc.normalized()
            eq_step = np.zeros(B, np.int64)
            step_iters = np.zeros(B, np.int64)
            used = np.zeros(B, bool)
            Uc_new = self._Uc(self.U, t)
            if predictor is not None:
                prop, has = predictor.propose(self, t)
                if prop is not None:
                    has = has & ~self.failed
                if prop is not None and has.any():
                    # the plain start's residual F(U_prev) - K12^T dUc against the
                    # proposal's; the smaller one is kept (newton.NewtonSolver.solve)
                    everyone = ~self.failed
                    F0 = self._assemble(self.U)
                    r_plain = self._residual(self._rhs(F0, Uc_new - Ucprev, everyone), self.U,
                                             everyone)
                    n_plain = torch.linalg.vector_norm(r_plain, dim=1).cpu().numpy()
                    Up = self.U.clone()
                    hm = torch.from_numpy(has).to(Up.device)
                    Up[hm] = prop[hm]
                    Up[hm, : self.nc] = Uc_new[hm]
                    self._update(Up)
                    Fp = self._assemble(Up)
                    r_pred = self._residual(self._rhs(Fp, None, everyone), Up, everyone)
                    n_pred = torch.linalg.vector_norm(r_pred, dim=1).cpu().numpy()
                    used = has & np.isfinite(n_pred) & (n_pred < n_plain)
                    um = torch.from_numpy(used).to(Up.device)
                    self.U[um] = Up[um]
                    Ucprev[um] = Uc_new[um]
                    self._update(self.U)
            active = ~self.failed.copy()
            while active.any():
                eq_step[active] += 1
                F = self._assemble(self.U)
                Uc = self._Uc(self.U, t)
                dUc = Uc - Ucprev
                rhs = self._rhs(F, dUc, active)
                r = self._residual(rhs, self.U, active)
                rn = torch.linalg.vector_norm(r, dim=1).cpu().numpy()
                dUc_zero = ~(dUc != 0).any(dim=1).cpu().numpy()
                done = active & (eq_step > 1) & (rn < self.residual_tol) & dUc_zero
                step_iters[done] = eq_step[done] - 1
                active &= ~done
                if not active.any():
                    break
                dU = self._solve(rhs, active)
                crit = (dU[:, : self.nu].abs().sum(dim=1) / max(self.nu, 1)
                        / self.kinematic_tol).cpu().numpy()
                # the single-problem driver raises "diverged" (crit > 1e6) or
                # "not converged" (iteration limit); here the problem is
                # marked failed and reset to the unloaded state, so that its
                # K(2) block stays finite for the others' factorisations
                bad = active & (~np.isfinite(crit) | (crit > 1e6))
                ok = active & ~bad
                am = torch.from_numpy(ok).to(self.U.device)
                Unew = self.U.clone()
                Unew[:, : self.nc] = Uc
                Unew[:, self.nc: self.nc + self.nu] += dU[:, : self.nu]
                Unew[:, self.nc + self.nu:] = dU[:, self.nu:]
                self.U[am] = Unew[am]
                Ucprev[am] = Uc[am]
                over = ok & (eq_step >= self.n_iterations)
                lost = bad | over
                if lost.any():
                    self.failed |= lost
                    step_iters[lost] = eq_step[lost]
                    active &= ~lost
                    fm = torch.from_numpy(lost).to(self.U.device)
                    self.U[fm] = 0.0
                    Ucprev[fm] = 0.0
                self._update(self.U)
            its.append(step_iters)
            preds.append(used)
            if on_converged is not None:
                on_converged(self, t)
        self.iterations = np.stack(its, axis=1)
        self.predicted = np.stack(preds, axis=1)
        return self
