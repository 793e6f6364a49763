"""Linear and linear-transient drivers around the GPU assembly.

LinearFESolver mirrors the reference's LinearFESolver::solve
(FESolver.cpp:337-400): one assembly, the fixed DoFs and nodal loads applied
(FESolver::applyBoundaryConditions, FESolver.cpp:229-247), then

    K(2) U_sl = F_sl + R_sl - K(1,2)^T U_c,
    R_c = K(1) U_c + K(1,2) U_sl - F_c,

and updateResults.  LinearTransientFESolver mirrors
LinearTransientFESolver::solve (FESolver.cpp:532-641): the storage is made
transient so that each assembly also yields C and M, one assembly from the
initial state U = initValue, then Newmark time stepping with the reference's
coefficients a0..a7 (alpha = 0.25, delta = 0.5 by default, FESolver.h:229-230)
on the unknown block:

    Kmod = a0 M(2) + a1 C(2) + K(2)                  (factorised once)
    Kmod U_sl' = F_sl + R_sl + M(2) (a0 U + a2 dU + a3 ddU)_sl
                               + C(2) (a1 U + a4 dU + a5 ddU)_sl
    ddU' = a0 (U' - U) - a2 dU - a3 ddU,   dU' = dU + a6 ddU' + a7 ddU

with U'_c = U_c, as the reference writes them (FESolver.cpp:604-625).

The backend is the GPU FEStorage (nla3d_gb300.storage) or the CPU oracle
model: eq_numbers(), pattern(b), K(b), C(b), M(b), F(), set_U(U), update(),
assemble(), block_mv(...), n_con / n_unk / n_mpc / n_total, blocks.  The
K(1,2) and K(1) products go through block_mv (matBVprod / matBTVprod).  The
linear solve of K(2) runs on the host (SciPy, standing in for the reference's
EquationSolver) or, with solver="gpu" / "gpu-fp32", through the device LDL^T
(nla3d_ldlt_*) on the K(2) values the assembly left in HBM.  The transient
driver factors Kmod by SciPy or, with the same options, by the device LDL^T
(Kmod's values uploaded on K(2)'s pattern); its C / M products run on the
host.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse.linalg as spla

from .newton import csr_full


def _bc_arrays(ne, nc, fixes, loads):
    fix_eq = np.array([int(ne[n - 1, d]) for n, d, _ in fixes], dtype=np.int64)
    fix_val = np.array([v for _, _, v in fixes], dtype=np.float64)
    if fix_eq.size and not (np.all(fix_eq >= 1) and np.all(fix_eq <= nc)):
        raise ValueError("fix on an unconstrained DoF")
    load_eq = np.array([int(ne[n - 1, d]) for n, d, _ in loads], dtype=np.int64)
    load_val = np.array([v for _, _, v in loads], dtype=np.float64)
    if load_eq.size and not np.all(load_eq >= 1):
        raise ValueError("load on an unused DoF")
    return fix_eq, fix_val, load_eq, load_val


class _Driver:
    def __init__(self, backend, fixes=(), loads=()):
        """fixes: (node, dof, value) as FESolver::addFix; loads: (node, dof,
        value) as FESolver::addLoad (FESolver.cpp:250-259).  The fixed DoFs
        must have been constrained in the backend before initSolutionData."""
        self.b = backend
        self.ne, self.ee = backend.eq_numbers()
        self.nc, self.nu, self.nm = backend.n_con, backend.n_unk, backend.n_mpc
        self.n = backend.n_total
        self.fix_eq, self.fix_val, self.load_eq, self.load_val = _bc_arrays(
            self.ne, self.nc, list(fixes), list(loads))
        self.U = np.zeros(self.n)
        self.R = np.zeros(self.n)

    def _apply_bc(self, t):
        """FESolver::applyBoundaryConditions: R += load * t, U_c = fix * t."""
        if self.load_eq.size:
            np.add.at(self.R, self.load_eq - 1, self.load_val * t)
        if self.fix_eq.size:
            self.U[self.fix_eq - 1] = self.fix_val * t

    def _block2(self, values):
        rows2, cols2, _ = self.b.blocks[2]
        return csr_full(*self.b.pattern(2), values, rows2, cols2, True)

    def _device_ldlt(self):
        """The device LDL^T on K(2)'s pattern: nested dissection of the rows'
        points, MPC equations after the DoFs (saddle_order)."""
        from .ldlt import DeviceLDLT, fill_reducing_order
        from .newton import row_points
        io, co = self.b.pattern(2)
        order = fill_reducing_order(io, co, row_points(self.b, self.nc, self.nu, self.nm), self.nu)
        return DeviceLDLT.for_storage(self.b, order, "fp64" if self.solver == "gpu" else "fp32")

    def node_solution(self, node, dof):
        """FEStorage::getNodeDofSolution: vecU at the DoF's equation."""
        return float(self.U[int(self.ne[node - 1, dof]) - 1])


class LinearFESolver(_Driver):
    def __init__(self, backend, fixes=(), loads=(), solver="host"):
        """solver: "host" (SciPy sparse LU) or "gpu" / "gpu-fp32" (the
        library's LDL^T of the device K(2), with a geometric nested-dissection
        order; GPU FEStorage backends only)."""
        super().__init__(backend, fixes, loads)
        if solver not in ("host", "gpu", "gpu-fp32"):
            raise ValueError(solver)
        self.solver = solver

    def _solve_K2(self, rhs):
        if self.solver == "host":
            return spla.spsolve(self._block2(self.b.K(2)).tocsc(), rhs)
        ldlt = self._device_ldlt()
        ldlt.factor(self.b)
        x = ldlt.solve_host(self.b, rhs, max_refine=50, tol=1e-12)
        ldlt.close()
        return x

    def solve(self):
        self.R[:] = 0.0
        self.b.set_U(self.U)
        self.b.assemble()
        F = self.b.F()
        self._apply_bc(1.0)
        nc = self.nc
        Uc = self.U[:nc].copy()
        rhs = F[nc:] + self.R[nc:]
        if nc:
            rhs = self.b.block_mv(12, 1, Uc, -1.0, rhs)
        self.U[nc:] = self._solve_K2(rhs)
        Rc = np.zeros(nc)
        if nc:
            Rc = self.b.block_mv(1, 0, Uc, 1.0, Rc)
            Rc = self.b.block_mv(12, 0, self.U[nc:].copy(), 1.0, Rc)
            Rc = Rc - F[:nc]
        self.R[:nc] = Rc
        self.b.set_U(self.U)
        self.b.update()
        return self.U


class LinearTransientFESolver(_Driver):
    time0 = 0.0
    time1 = 1.0
    numberOfTimesteps = 100
    initValue = 0.0
    alpha = 0.25     # trapezoidal rule
    delta = 0.5

    def __init__(self, backend, fixes=(), loads=(), solver="host"):
        """solver: "host" (SciPy sparse LU of Kmod) or "gpu" / "gpu-fp32"
        (Kmod's values, on K(2)'s pattern, factored once by the device LDL^T
        and every step solved on the device with FP64 refinement)."""
        super().__init__(backend, fixes, loads)
        if solver not in ("host", "gpu", "gpu-fp32"):
            raise ValueError(solver)
        self.solver = solver

    def solve(self, probes=()):
        """Runs the time steps; returns (times, U at the probes per step) for
        probes given as (node, dof) pairs (the reference test's
        ProbeProcessor, one value per completed step)."""
        if not getattr(self.b, "transient", False):
            raise ValueError("the backend must be transient (FEStorage::setTransient) "
                             "before initSolutionData")
        al, de = self.alpha, self.delta
        dt = (self.time1 - self.time0) / self.numberOfTimesteps
        a0 = 1.0 / (al * dt * dt)
        a1 = de / (al * dt)
        a2 = 1.0 / (al * dt)
        a3 = 1.0 / (2.0 * al) - 1.0
        a4 = de / al - 1.0
        a5 = dt / 2.0 * (de / al - 2.0)
        a6 = dt * (1.0 - de)
        a7 = de * dt
        nc = self.nc
        self.R[:] = 0.0
        self.U[:] = self.initValue
        dU = np.zeros(self.n)
        ddU = np.zeros(self.n)
        self.b.set_U(self.U)
        self.b.assemble()
        self._apply_bc(1.0)
        F = self.b.F()
        K2, C2, M2 = self.b.K(2), self.b.C(2), self.b.M(2)
        kmod = a0 * M2 + a1 * C2 + K2
        if self.solver == "host":
            lu = spla.splu(self._block2(kmod).tocsc(), permc_spec="COLAMD")
            solve = lu.solve
        else:
            import torch
            ldlt = self._device_ldlt()
            kmod_d = torch.from_numpy(np.ascontiguousarray(kmod)).cuda()
            b_d = torch.empty(self.nu + self.nm, dtype=torch.float64, device="cuda")
            x_d = torch.empty_like(b_d)
            torch.cuda.synchronize()
            ldlt.factor_device(kmod_d.data_ptr())

            def solve(rhs):
                b_d.copy_(torch.from_numpy(rhs))
                torch.cuda.synchronize()
                ldlt.solve_device(kmod_d.data_ptr(), b_d.data_ptr(), x_d.data_ptr(),
                                  max_refine=50, tol=1e-12)
                return x_d.cpu().numpy()
        Cs, Ms = self._block2(C2), self._block2(M2)
        times, values = [], []
        t = self.time0 + dt
        while t <= self.time1:
            rhs = F[nc:] + self.R[nc:]
            rhs = rhs + Ms @ (a0 * self.U[nc:] + a2 * dU[nc:] + a3 * ddU[nc:])
            rhs = rhs + Cs @ (a1 * self.U[nc:] + a4 * dU[nc:] + a5 * ddU[nc:])
            Un = np.empty(self.n)
            Un[:nc] = self.U[:nc]
            Un[nc:] = solve(rhs)
            ddUn = a0 * (Un - self.U) - a2 * dU - a3 * ddU
            dUn = dU + a6 * ddUn + a7 * ddU
            self.U, dU, ddU = Un, dUn, ddUn
            self.b.set_U(self.U)
            self.b.update()
            times.append(t)
            values.append([self.node_solution(n, d) for n, d in probes])
            t += dt
        self.dU, self.ddU = dU, ddU
        if self.solver != "host":
            ldlt.close()
        return np.array(times), np.array(values)
