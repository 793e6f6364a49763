"""Learned Newton start.

A small MLP proposes each load step's starting state from the last two
converged increments, the load factor and the material constants; the Newton
driver (nla3d_gb300.newton) keeps the reference's plain start (previous
converged state + linearised constrained increment) whenever the proposal's
residual is not smaller, and the unchanged residual tolerance decides
convergence either way.

Proposal:  dU_n = a1 dU_{n-1} + a2 dU_{n-2} + s Q c
  Q   64 orthonormal coarse modes of the free (unknown + MPC) DoFs: Legendre
      polynomials of total degree <= 3 on the normalised geometry for each
      displacement component (60) and degree <= 1 for the element pressure (4);
  s   |Q^T dU_{n-1}|, so that the network sees scale-free inputs;
  (a1, a2, c) = MLP(Q^T dU_{n-1} / s, Q^T dU_{n-2} / s, t, dt_n/dt_{n-1}, C10, log10 K / 4).
Training targets are the least-squares coefficients of the converged dU_n on
[dU_{n-1}, dU_{n-2}, s Q], from solves run with the plain start.

The network (4 hidden layers of 256, tanh, BF16 weights, FP32 accumulation)
is trained on the GPU by the library's own kernels (csrc/mlp.cu) through its
C ABI; torch only provides device memory.
"""
from __future__ import annotations

import ctypes
import dataclasses
import math

import numpy as np

from . import _lib
from . import meshgen as mg

N_MODES = 64
N_IN = 2 * N_MODES + 4
N_OUT = 2 + N_MODES
HIDDEN = (256, 256, 256, 256)


# ---------------------------------------------------------------------------
# coarse modes and features
# ---------------------------------------------------------------------------

def _legendre(k, x):
    return [np.ones_like(x), x, 0.5 * (3 * x * x - 1), 0.5 * (5 * x ** 3 - 3 * x)][k]


class CoarseBasis:
    def __init__(self, mesh: mg.Mesh, ne, ee, nc, n_total):
        self.nc, self.n = nc, n_total
        lo, hi = mesh.xyz.min(axis=0), mesh.xyz.max(axis=0)
        span = np.where(hi - lo > 0, hi - lo, 1.0)
        xn = 2.0 * (mesh.xyz - lo) / span - 1.0
        cen = xn[mesh.conn.astype(np.int64) - 1].mean(axis=1)
        degs = [(i, j, k) for i in range(4) for j in range(4) for k in range(4) if i + j + k <= 3]
        nf = n_total - nc
        phi = []
        for comp in range(3):
            eq = ne[: mesh.n_nodes, comp].astype(np.int64)
            ok = eq > nc
            for (i, j, k) in degs:
                col = np.zeros(nf)
                v = _legendre(i, xn[:, 0]) * _legendre(j, xn[:, 1]) * _legendre(k, xn[:, 2])
                col[eq[ok] - 1 - nc] = v[ok]
                phi.append(col)
        eqp = ee[:, mg.HYDRO_PRESSURE].astype(np.int64)
        okp = eqp > nc
        for f in (np.ones(len(cen)), cen[:, 0], cen[:, 1], cen[:, 2]):
            col = np.zeros(nf)
            col[eqp[okp] - 1 - nc] = f[okp]
            phi.append(col)
        Phi = np.stack(phi, axis=1)
        self.Q, _ = np.linalg.qr(Phi)

    def project(self, dU):
        return self.Q.T @ dU[self.nc:]


def features(basis: CoarseBasis, dU1, dU2, t, ratio, c10, kbulk):
    p1, p2 = basis.project(dU1), basis.project(dU2)
    s = float(np.linalg.norm(p1)) + 1e-300
    x = np.concatenate([p1 / s, p2 / s, [t, ratio, c10, math.log10(kbulk) / 4.0]])
    return x, s


def target(basis: CoarseBasis, dU1, dU2, dU, s):
    nc = basis.nc
    A = np.concatenate([dU1[nc:, None], dU2[nc:, None], s * basis.Q], axis=1)
    y, *_ = np.linalg.lstsq(A, dU[nc:], rcond=None)
    return y


def compose(basis: CoarseBasis, dU1, dU2, s, y):
    out = np.zeros_like(dU1)
    nc = basis.nc
    out[nc:] = y[0] * dU1[nc:] + y[1] * dU2[nc:] + s * (basis.Q @ y[2:])
    return out


# ---------------------------------------------------------------------------
# the MLP on the GPU (library kernels; torch buffers)
# ---------------------------------------------------------------------------

class MLP:
    def __init__(self, sizes=(N_IN,) + HIDDEN + (N_OUT,), seed=0, device="cuda:0"):
        import torch
        self.torch = torch
        self.lib = _lib.load()
        self.sizes = tuple(sizes)
        self.dev = torch.device(device)
        rng = np.random.default_rng(seed)
        self.W, self.Wb, self.b, self.state = [], [], [], []
        for fan_in, fan_out in zip(self.sizes[:-1], self.sizes[1:]):
            lim = math.sqrt(6.0 / (fan_in + fan_out))
            W = torch.from_numpy(rng.uniform(-lim, lim, (fan_out, fan_in)).astype(np.float32)).to(self.dev)
            self.W.append(W)
            self.Wb.append(torch.empty(W.shape, dtype=torch.bfloat16, device=self.dev))
            self.b.append(torch.zeros(fan_out, dtype=torch.float32, device=self.dev))
            self.state.append([torch.zeros_like(W), torch.zeros_like(W),
                               torch.zeros(fan_out, device=self.dev),
                               torch.zeros(fan_out, device=self.dev)])
        for W, Wb in zip(self.W, self.Wb):
            self._ck(self.lib.nla3d_mlp_to_bf16(W.data_ptr(), Wb.data_ptr(), W.numel(), self.stream))
        self.step_count = 0
        self.x_mean = self.x_std = self.y_mean = self.y_std = None

    @property
    def stream(self):
        """The caller's current stream: the kernels run in order with the
        PyTorch work around them, whichever stream that is on."""
        return self.torch.cuda.current_stream(self.dev).cuda_stream

    def _ck(self, rc):
        if rc:
            raise _lib.Nla3dError(rc, "MLP kernel launch failed")

    def check(self):
        """Raise if a tensor-core GEMM tile's bounded MMA wait ran out (its
        outputs were set to NaN) since the last check (synchronises)."""
        t = ctypes.c_uint32()
        self._ck(self.lib.nla3d_mlp_status(ctypes.byref(t)))
        if t.value:
            raise _lib.Nla3dError(5, f"{t.value} MLP GEMM tiles timed out waiting for their MMAs")

    def forward(self, X):
        """X: float32 cuda tensor (B, in).  Returns activations [X, h1, ..., out]."""
        acts = [X]
        L = len(self.W)
        for l in range(L):
            out_dim, in_dim = self.W[l].shape
            Y = self.torch.empty((X.shape[0], out_dim), dtype=self.torch.float32, device=self.dev)
            # Y = act(A W^T + b): A[m,k] at m*in + k; (W^T)[k,n] = W[n,k] at n*in + k
            self._ck(self.lib.nla3d_mlp_gemm(X.shape[0], out_dim, in_dim, acts[-1].data_ptr(), 0,
                                             in_dim, 1, self.Wb[l].data_ptr(), 1, 1, in_dim,
                                             Y.data_ptr(), out_dim, self.b[l].data_ptr(),
                                             1 if l < L - 1 else 0, self.stream))
            acts.append(Y)
        return acts

    def backward(self, acts, dOut):
        """Gradients (dW, db) per layer for the output gradient dOut (B, out)."""
        torch = self.torch
        L = len(self.W)
        B = dOut.shape[0]
        gW, gb = [None] * L, [None] * L
        d = dOut
        for l in range(L - 1, -1, -1):
            out_dim, in_dim = self.W[l].shape
            if l < L - 1:
                self._ck(self.lib.nla3d_mlp_tanh_backward(acts[l + 1].data_ptr(), d.data_ptr(),
                                                          d.numel(), self.stream))
            dW = torch.empty((out_dim, in_dim), dtype=torch.float32, device=self.dev)
            # dW[o,i] = sum_b d[b,o] X[b,i]: A = d^T (A[o,b] at b*out + o), B = X (B[b,i] at b*in + i)
            self._ck(self.lib.nla3d_mlp_gemm(out_dim, in_dim, B, d.data_ptr(), 0, 1, out_dim,
                                             acts[l].data_ptr(), 0, in_dim, 1, dW.data_ptr(), in_dim,
                                             None, 0, self.stream))
            db = torch.empty(out_dim, dtype=torch.float32, device=self.dev)
            self._ck(self.lib.nla3d_mlp_column_sum(d.data_ptr(), B, out_dim, db.data_ptr(),
                                                   self.stream))
            gW[l], gb[l] = dW, db
            if l > 0:
                dX = torch.empty((B, in_dim), dtype=torch.float32, device=self.dev)
                # dX[b,i] = sum_o d[b,o] W[o,i]: A = d (A[b,o] at b*out + o), B = W (B[o,i] at o*in + i)
                self._ck(self.lib.nla3d_mlp_gemm(B, in_dim, out_dim, d.data_ptr(), 0, out_dim, 1,
                                                 self.Wb[l].data_ptr(), 1, in_dim, 1, dX.data_ptr(),
                                                 in_dim, None, 0, self.stream))
                d = dX
        return gW, gb

    def loss_grad(self, out, T):
        """MSE loss gradient 2 (out - T) / n (library kernel)."""
        d = self.torch.empty_like(out)
        self._ck(self.lib.nla3d_mlp_mse_grad(out.data_ptr(), T.data_ptr(), d.data_ptr(), out.numel(),
                                             2.0 / out.numel(), self.stream))
        return d

    def adam(self, gW, gb, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.step_count += 1
        for l in range(len(self.W)):
            mW, vW, mb, vb = self.state[l]
            self._ck(self.lib.nla3d_mlp_adam(self.W[l].data_ptr(), gW[l].data_ptr(), mW.data_ptr(),
                                             vW.data_ptr(), self.W[l].numel(), lr, b1, b2, eps,
                                             self.step_count, self.Wb[l].data_ptr(), self.stream))
            self._ck(self.lib.nla3d_mlp_adam(self.b[l].data_ptr(), gb[l].data_ptr(), mb.data_ptr(),
                                             vb.data_ptr(), self.b[l].numel(), lr, b1, b2, eps,
                                             self.step_count, None, self.stream))

    # ---- training on numpy data ----
    def fit(self, X, Y, epochs=200, batch=256, lr=1e-3, seed=0, log=None):
        torch = self.torch
        self.x_mean, self.x_std = X.mean(0), X.std(0) + 1e-8
        self.y_mean, self.y_std = Y.mean(0), Y.std(0) + 1e-8
        Xn = torch.from_numpy(((X - self.x_mean) / self.x_std).astype(np.float32)).to(self.dev)
        Yn = torch.from_numpy(((Y - self.y_mean) / self.y_std).astype(np.float32)).to(self.dev)
        rng = np.random.default_rng(seed)
        n = X.shape[0]
        history = []
        for ep in range(epochs):
            perm = torch.from_numpy(rng.permutation(n)).to(self.dev)
            for i in range(0, n, batch):
                idx = perm[i:i + batch]
                xb, yb = Xn[idx].contiguous(), Yn[idx].contiguous()
                acts = self.forward(xb)
                gW, gb = self.backward(acts, self.loss_grad(acts[-1], yb))
                self.adam(gW, gb, lr=lr * (0.5 * (1 + math.cos(math.pi * ep / epochs))))
            if ep % 20 == 0 or ep == epochs - 1:
                out = self.forward(Xn)[-1]
                loss = float(((out - Yn) ** 2).mean())
                history.append((ep, loss))
                if log:
                    log(f"epoch {ep} loss {loss:.4e}")
        self.check()
        return history

    def predict(self, X):
        torch = self.torch
        Xn = torch.from_numpy(((np.atleast_2d(X) - self.x_mean) / self.x_std).astype(np.float32)).to(self.dev)
        out = self.forward(Xn)[-1].cpu().numpy().astype(np.float64)
        return out * self.y_std + self.y_mean

    def weights(self):
        return ([W.cpu().numpy().astype(np.float64) for W in self.W],
                [b.cpu().numpy().astype(np.float64) for b in self.b])


# ---------------------------------------------------------------------------
# predictors for the Newton driver
# ---------------------------------------------------------------------------

class History:
    """on_converged hook: converged U and load factors, starting from U = 0 at t = 0."""

    def __init__(self, n_total):
        self.U = [np.zeros(n_total)]
        self.t = [0.0]

    def __call__(self, solver, t):
        self.U.append(solver.U.copy())
        self.t.append(t)


class ExtrapolationPredictor:
    """Secant extrapolation of the last converged increment (a baseline)."""

    def __init__(self, history):
        self.h = history

    def propose(self, solver, t):
        h = self.h
        if len(h.U) < 3:
            return None
        r = (t - h.t[-1]) / (h.t[-1] - h.t[-2])
        return h.U[-1] + r * (h.U[-1] - h.U[-2])


class MLPPredictor:
    def __init__(self, mlp: MLP, basis: CoarseBasis, history: History, c10, kbulk):
        self.mlp, self.basis, self.h = mlp, basis, history
        self.c10, self.kbulk = c10, kbulk

    def propose(self, solver, t):
        h = self.h
        if len(h.U) < 3:
            return None
        dU1, dU2 = h.U[-1] - h.U[-2], h.U[-2] - h.U[-3]
        ratio = (t - h.t[-1]) / (h.t[-1] - h.t[-2])
        x, s = features(self.basis, dU1, dU2, t, ratio, self.c10, self.kbulk)
        y = self.mlp.predict(x)[0]
        return h.U[-1] + compose(self.basis, dU1, dU2, s, y)


# ---------------------------------------------------------------------------
# problem families (seeded)
# ---------------------------------------------------------------------------

@dataclasses.dataclass
class Problem:
    mesh: mg.Mesh
    fixes: list
    c10: float
    kbulk: float
    n_loadsteps: int
    label: str = ""


def block_problem(n, c10, kbulk, stretch, n_loadsteps=20):
    """n^3 block on the unit cube, z=0 clamped, z=1 face pulled to `stretch`
    (UZ prescribed, UX/UY free); Neo-Hookean G = 2 C10, K."""
    m = mg.solid81_block(n, n, n, 1.0 / n, mg.MAT_NEO_HOOKEAN, (2 * c10, kbulk), clamp_z0=True)
    top = (np.nonzero(np.abs(m.xyz[:, 2] - 1.0) < 1e-12)[0] + 1).astype(np.uint32)
    m.fix_nodes = np.concatenate([m.fix_nodes, top])
    m.fix_dofs = np.concatenate([m.fix_dofs, np.full(top.size, mg.UZ, np.int32)])
    fixes = [(int(a), int(b), 0.0) for a, b in zip(m.fix_nodes[:-top.size], m.fix_dofs[:-top.size])]
    fixes += [(int(a), mg.UZ, stretch - 1.0) for a in top]
    return Problem(m, fixes, c10, kbulk, n_loadsteps,
                   f"block{n} C10={c10:.3f} K={kbulk:.0f} stretch={stretch:.3f}")


def bar_problem(nx, nz, c10, kbulk, stretch, twist_rad, n_loadsteps=50):
    """nx x nx x nz bar (h = 1), z=0 clamped, z=L face slaved to a master node
    (RigidBodyMpc) driven to UZ = (stretch-1) L and ROTZ = twist; Neo-Hookean."""
    m = mg.solid81_bar_mpc(nx, nx, nz, 1.0, mg.MAT_NEO_HOOKEAN, (2 * c10, kbulk))
    master = m.n_nodes
    L = float(nz)
    mf = [(master, mg.UX, 0.0), (master, mg.UY, 0.0), (master, mg.UZ, (stretch - 1.0) * L),
          (master, mg.ROTX, 0.0), (master, mg.ROTY, 0.0), (master, mg.ROTZ, twist_rad)]
    m.fix_nodes = np.concatenate([m.fix_nodes, np.full(6, master, np.uint32)])
    m.fix_dofs = np.concatenate([m.fix_dofs, np.arange(6, dtype=np.int32)])
    fixes = [(int(a), int(b), 0.0) for a, b in zip(m.fix_nodes[:-6], m.fix_dofs[:-6])] + mf
    return Problem(m, fixes, c10, kbulk, n_loadsteps,
                   f"bar{nx}x{nx}x{nz} C10={c10:.3f} K={kbulk:.0f} stretch={stretch:.3f} "
                   f"twist={math.degrees(twist_rad):.1f}deg")


def sample_block_problems(count, n=4, seed=0, n_loadsteps=20):
    """C10 ~ U(0.2, 1.0), K ~ U(500, 5000), target stretch ~ U(1.0, 2.0)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return [block_problem(n, rng.uniform(0.2, 1.0), rng.uniform(500.0, 5000.0),
                          rng.uniform(1.0, 2.0), n_loadsteps) for _ in range(count)]


def sample_bar_problems(count, nx=3, nz=12, seed=0, n_loadsteps=50):
    """Around the torsion+stretch bar: C10 ~ U(0.3, 0.7), K ~ U(500, 2000),
    stretch ~ U(1.5, 2.0), twist ~ U(45, 90) deg."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return [bar_problem(nx, nz, rng.uniform(0.3, 0.7), rng.uniform(500.0, 2000.0),
                        rng.uniform(1.5, 2.0), math.radians(rng.uniform(45.0, 90.0)),
                        n_loadsteps) for _ in range(count)]


# ---------------------------------------------------------------------------
# data generation, training and evaluation
# ---------------------------------------------------------------------------

def solve(problem: Problem, backend, predictor_factory=None, residual_tol=1e-8, n_iterations=25,
          linear_solver="direct"):
    """Run the Newton driver; returns (solver, history)."""
    from .newton import NewtonSolver
    solver = NewtonSolver(backend, problem.fixes, n_loadsteps=problem.n_loadsteps,
                          n_iterations=n_iterations, residual_tol=residual_tol,
                          solver=linear_solver)
    hist = History(backend.n_total)
    pred = predictor_factory(solver, hist) if predictor_factory else None
    solver.solve(predictor=pred, on_converged=hist)
    return solver, hist


def samples_from_history(basis, hist, c10, kbulk):
    X, Y = [], []
    for n in range(3, len(hist.U)):
        dU = hist.U[n] - hist.U[n - 1]
        dU1 = hist.U[n - 1] - hist.U[n - 2]
        dU2 = hist.U[n - 2] - hist.U[n - 3]
        t = hist.t[n]
        ratio = (t - hist.t[n - 1]) / (hist.t[n - 1] - hist.t[n - 2])
        x, s = features(basis, dU1, dU2, t, ratio, c10, kbulk)
        X.append(x)
        Y.append(target(basis, dU1, dU2, dU, s))
    return X, Y


def make_backend(problem: Problem, precision="fp64", factory=None):
    """The assembly backend of one solve: the GPU FEStorage, or what
    `factory(mesh)` returns (any object with the FEStorage driver API)."""
    if factory is not None:
        return factory(problem.mesh)
    from .storage import FEStorage
    return FEStorage(problem.mesh, precision).initSolutionData()


def basis_for(problem: Problem, backend):
    ne, ee = backend.eq_numbers()
    return CoarseBasis(problem.mesh, ne, ee, backend.n_con, backend.n_total)


def generate(problems, precision="fp64", linear_solver="direct", backend_factory=None):
    X, Y, iters = [], [], []
    for pb in problems:
        be = make_backend(pb, precision, backend_factory)
        solver, hist = solve(pb, be, linear_solver=linear_solver)
        solver.close()
        x, y = samples_from_history(basis_for(pb, be), hist, pb.c10, pb.kbulk)
        X += x
        Y += y
        iters.append([r.iterations for r in solver.records])
    return np.array(X), np.array(Y), iters


def evaluate(problems, mlp, precision="fp64", linear_solver="direct",
             starts=("plain", "extrapolation", "learned"), log=None, backend_factory=None):
    """Mean Newton iterations per load step: plain start, secant extrapolation
    and the learned start (with the plain-start fallback)."""
    import time
    out = {k: [] for k in starts}
    out["learned_used"] = []
    wall = {}
    phases = {}
    for pb in problems:
        be = make_backend(pb, precision, backend_factory)
        basis = basis_for(pb, be)
        for start in starts:
            if start != "plain":
                be = make_backend(pb, precision, backend_factory)
            factory = None
            if start == "extrapolation":
                factory = lambda sv, h: ExtrapolationPredictor(h)  # noqa: E731
            elif start == "learned":
                factory = lambda sv, h: MLPPredictor(mlp, basis, h, pb.c10, pb.kbulk)  # noqa: E731
            t0 = time.perf_counter()
            s, _ = solve(pb, be, factory, linear_solver=linear_solver)
            wall[start] = wall.get(start, 0.0) + time.perf_counter() - t0
            ph = phases.setdefault(start, {})
            for key, val in getattr(s, "timing", {}).items():
                ph[key] = ph.get(key, 0.0) + val
            s.close()
            out[start] += [r.iterations for r in s.records]
            if start == "learned":
                out["learned_used"] += [r.predicted for r in s.records]
            if log:
                log(f"{pb.label} {start}: {np.mean(out[start]):.3f} it/step, "
                    f"{wall[start]:.1f} s, {s.factorizations} factorisations, "
                    f"{s.inexact_solves} inexact solves, {s.fp64_refactorizations} FP64 refactors")
    res = {k: float(np.mean(v)) for k, v in out.items() if v}
    return res | {"steps": len(out[starts[0]]), "wall_s": wall, "phase_s": phases}


def benchmark(n_block_train=100, n_block_eval=50, block_batch=50, n_bar_train=12, block_n=10,
              bar_nx=20, linear_solver="gpu-tc", log=None):
    """Newton iterations per load step, plain vs learned start, at a 1e-8
    residual tolerance, on the two problem families, with K(2) factored on the
    device (sized so that a run takes a minute or two on one GPU):
      blocks: block_n^3 SOLID81 on the unit cube, C10 ~ U(0.2, 1), K ~ U(500,
              5000), stretch ~ U(1, 2), 20 load steps, solved block_batch at a
              time in lock step (batch_newton.BatchNewton); trained on
              n_block_train solves, evaluated on n_block_eval held-out seeds;
      bar:    bar_nx x bar_nx x 4 bar_nx torsion + stretch bar (rigid-body MPC
              end) at C10 = 0.5, K = 1000, stretch 2.0, 90 deg, 50 load steps;
              the network is trained on 3x3x12 bars with C10 ~ U(0.3, 0.7),
              K ~ U(500, 2000), stretch ~ U(1.5, 2), twist ~ U(45, 90) deg (its
              coarse modes live on the normalised geometry, so it carries over).
    Also FP64 vs mixed assembly iteration counts on that bar."""
    import time
    fronts = {"gpu": "fp64", "gpu-fp32": "fp32", "gpu-tc": "fp32-tc"}[linear_solver]
    out = {}
    t0 = time.perf_counter()
    solvers = {}
    X, Y, train_its, failed, _ = generate_batched(
        sample_block_problems(n_block_train, n=block_n, seed=11), fronts=fronts,
        batch_size=block_batch, solvers=solvers)
    mlp = MLP(seed=0)
    h = mlp.fit(X, Y, epochs=300, batch=128, lr=2e-3)
    out["blocks"] = evaluate_batched(sample_block_problems(n_block_eval, n=block_n, seed=99), mlp,
                                     fronts=fronts, batch_size=block_batch, solvers=solvers)
    out["blocks"].update({"train_samples": int(X.shape[0]), "final_loss": h[-1][1],
                          "mesh": f"{block_n}x{block_n}x{block_n} SOLID81", "load_steps": 20,
                          "train_solves": n_block_train, "train_failed": failed,
                          "train_plain_iterations": float(np.mean(train_its)),
                          "driver": f"batched lock-step Newton, {block_batch} solves per batch"})
    solvers.clear()
    if log:
        log(f"blocks: {out['blocks']}")
    Xb, Yb, _ = generate(sample_bar_problems(n_bar_train, nx=3, nz=12, seed=5, n_loadsteps=50),
                         linear_solver=linear_solver)
    mlpb = MLP(seed=1)
    hb = mlpb.fit(Xb, Yb, epochs=300, batch=128, lr=2e-3)
    cfg = bar_problem(bar_nx, 4 * bar_nx, 0.5, 1000.0, 2.0, math.pi / 2, 50)
    out["bar"] = evaluate([cfg], mlpb, linear_solver=linear_solver)
    out["bar"].update({"train_samples": int(Xb.shape[0]), "final_loss": hb[-1][1],
                       "mesh": f"{bar_nx}x{bar_nx}x{4 * bar_nx} SOLID81 "
                               f"({bar_nx * bar_nx * 4 * bar_nx} elements) + rigid-body MPC end",
                       "load_steps": 50, "trained_on": "3x3x12 bars"})
    # the plain start above ran with the FP64 assembly
    its = {"fp64": out["bar"]["plain"]}
    be = make_backend(cfg, "mixed")
    s, _ = solve(cfg, be, linear_solver=linear_solver)
    s.close()
    its["mixed"] = float(np.mean([r.iterations for r in s.records]))
    out["bar"]["iterations_fp64_assembly"] = its["fp64"]
    out["bar"]["iterations_mixed_assembly"] = its["mixed"]
    out["residual_tol"] = 1e-8
    out["linear_solver"] = linear_solver
    out["seconds"] = time.perf_counter() - t0
    if log:
        log(f"bar: {out['bar']}")
    return out


# ---------------------------------------------------------------------------
# batched studies: many problems on one mesh, solved in lock step
# (nla3d_gb300.batch_newton.BatchNewton)
# ---------------------------------------------------------------------------

def batch_features(basis: CoarseBasis, dU1, dU2, t, ratio, c10, kbulk):
    """features() for B problems at once (dU1, dU2: B x n; c10, kbulk: B)."""
    nc = basis.nc
    P1 = dU1[:, nc:] @ basis.Q
    P2 = dU2[:, nc:] @ basis.Q
    s = np.linalg.norm(P1, axis=1) + 1e-300
    B = dU1.shape[0]
    X = np.concatenate([P1 / s[:, None], P2 / s[:, None], np.full((B, 1), t),
                        np.full((B, 1), ratio), np.asarray(c10, np.float64)[:, None],
                        (np.log10(np.asarray(kbulk, np.float64)) / 4.0)[:, None]], axis=1)
    return X, s


def batch_target(basis: CoarseBasis, dU1, dU2, dU, s):
    """target() for B problems: the least-squares coefficients of dU on
    [dU1, dU2, s Q].  Q is orthonormal, so for any (a1, a2) the Q part is
    fitted exactly by c = (Q^T dU - a1 Q^T dU1 - a2 Q^T dU2) / s, which leaves
    a two-column least-squares problem on the parts of dU1, dU2 and dU
    orthogonal to Q: the same minimiser as the full problem whenever that
    one is unique, at O(n) cost per problem instead of O(n 66^2)."""
    nc, Q = basis.nc, basis.Q
    d1, d2, d = dU1[:, nc:], dU2[:, nc:], dU[:, nc:]
    p1, p2, p = d1 @ Q, d2 @ Q, d @ Q
    r1, r2, r = d1 - p1 @ Q.T, d2 - p2 @ Q.T, d - p @ Q.T
    Y = np.zeros((d.shape[0], 2 + Q.shape[1]))
    for j in range(d.shape[0]):
        a, *_ = np.linalg.lstsq(np.stack([r1[j], r2[j]], axis=1), r[j], rcond=None)
        Y[j, :2] = a
        Y[j, 2:] = (p[j] - a[0] * p1[j] - a[1] * p2[j]) / s[j]
    return Y


def batch_compose(basis: CoarseBasis, dU1, dU2, s, Y):
    """compose() for B problems."""
    nc = basis.nc
    out = np.zeros_like(dU1)
    out[:, nc:] = (Y[:, 0:1] * dU1[:, nc:] + Y[:, 1:2] * dU2[:, nc:]
                   + s[:, None] * (Y[:, 2:] @ basis.Q.T))
    return out


class BatchHistory:
    """on_converged hook of BatchNewton: the last four converged states (host
    copies, B x n) and, with `collect`, the training samples of every load
    step from the third on (rows of problems that have failed are left out;
    `owner` gives each row's problem index, counted from `offset`)."""

    def __init__(self, B, n, basis=None, c10=None, kbulk=None, collect=False, offset=0):
        self.U = [np.zeros((B, n))]
        self.t = [0.0]
        self.basis, self.c10, self.kbulk = basis, c10, kbulk
        self.collect = collect
        self.offset = offset
        self.X, self.Y, self.owner = [], [], []

    def __call__(self, driver, t):
        self.U.append(driver.U.cpu().numpy())
        self.t.append(t)
        if self.collect and len(self.U) >= 4:
            U0, U1, U2, U3 = self.U[-1], self.U[-2], self.U[-3], self.U[-4]
            keep = ~driver.failed
            dU, dU1, dU2 = (U0 - U1)[keep], (U1 - U2)[keep], (U2 - U3)[keep]
            ratio = (self.t[-1] - self.t[-2]) / (self.t[-2] - self.t[-3])
            X, s = batch_features(self.basis, dU1, dU2, self.t[-1], ratio, self.c10[keep],
                                  self.kbulk[keep])
            self.X.append(X)
            self.Y.append(batch_target(self.basis, dU1, dU2, dU, s))
            self.owner.append(np.nonzero(keep)[0] + self.offset)
        del self.U[:-4]


class BatchExtrapolationPredictor:
    """ExtrapolationPredictor for every problem of a BatchNewton."""

    def __init__(self, history: BatchHistory):
        self.h = history

    def propose(self, driver, t):
        h = self.h
        if len(h.t) < 3:
            return None, None
        r = (t - h.t[-1]) / (h.t[-1] - h.t[-2])
        prop = h.U[-1] + r * (h.U[-1] - h.U[-2])
        return driver.torch.from_numpy(prop).to(driver.U.device), np.ones(driver.B, bool)


class BatchMLPPredictor:
    """MLPPredictor for every problem of a BatchNewton (one forward pass of
    the network for the whole batch)."""

    def __init__(self, mlp: MLP, basis: CoarseBasis, history: BatchHistory, c10, kbulk):
        self.mlp, self.basis, self.h = mlp, basis, history
        self.c10, self.kbulk = np.asarray(c10, np.float64), np.asarray(kbulk, np.float64)

    def propose(self, driver, t):
        h = self.h
        if len(h.t) < 3:
            return None, None
        dU1, dU2 = h.U[-1] - h.U[-2], h.U[-2] - h.U[-3]
        ratio = (t - h.t[-1]) / (h.t[-1] - h.t[-2])
        X, s = batch_features(self.basis, dU1, dU2, t, ratio, self.c10, self.kbulk)
        Y = self.mlp.predict(X)
        prop = h.U[-1] + batch_compose(self.basis, dU1, dU2, s, Y)
        return driver.torch.from_numpy(prop).to(driver.U.device), np.ones(driver.B, bool)


def _batches(problems, batch_size):
    for i in range(0, len(problems), batch_size):
        yield problems[i:i + batch_size]


def _batch_driver(group, precision, fronts, solvers):
    from .batch_newton import BatchNewton
    drv = BatchNewton(group, precision=precision, fronts=fronts,
                      block_solver=solvers.get(len(group)))
    solvers[len(group)] = drv.bs
    return drv


def generate_batched(problems, precision="fp64", fronts="fp32", batch_size=100, log=None,
                     solvers=None):
    """generate() with BatchNewton: the plain-start solves of `problems` (one
    mesh), batch_size at a time.  Returns X, Y, the iterations per load step
    (solves x load steps), the number of failed solves and, per sample row,
    the index of the solve it comes from.  `solvers` (a dict) keeps the
    block-diagonal factorisations' symbolic analyses for reuse by later
    calls."""
    import time
    solvers = {} if solvers is None else solvers
    X, Y, owner, iters, failed = [], [], [], [], 0
    t0 = time.perf_counter()
    for k, group in enumerate(_batches(problems, batch_size)):
        drv = _batch_driver(group, precision, fronts, solvers)
        basis = CoarseBasis(group[0].mesh, drv.ne, drv.ee, drv.nc, drv.n)
        hist = BatchHistory(drv.B, drv.n, basis, np.array([pb.c10 for pb in group]),
                            np.array([pb.kbulk for pb in group]), collect=True,
                            offset=k * batch_size)
        drv.solve(on_converged=hist)
        X += hist.X
        Y += hist.Y
        owner += hist.owner
        iters.append(drv.iterations[~drv.failed])
        failed += int(drv.failed.sum())
        drv.close()
        if log:
            log(f"batch {k}: {drv.B} solves, {np.mean(drv.iterations[~drv.failed]):.3f} it/step, "
                f"{drv.factorizations} factorisations, {time.perf_counter() - t0:.1f} s")
    return (np.concatenate(X), np.concatenate(Y), np.concatenate(iters), failed,
            np.concatenate(owner))


def evaluate_batched(problems, mlp, precision="fp64", fronts="fp32", batch_size=100,
                     starts=("plain", "extrapolation", "learned"), log=None, solvers=None):
    """evaluate() with BatchNewton: mean Newton iterations per load step of
    each start on `problems` (one mesh), failed solves left out and counted."""
    import time
    solvers = {} if solvers is None else solvers
    out = {k: [] for k in starts}
    used, wall, failed = [], {}, {k: 0 for k in starts}
    for group in _batches(problems, batch_size):
        c10 = np.array([pb.c10 for pb in group])
        kb = np.array([pb.kbulk for pb in group])
        for start in starts:
            drv = _batch_driver(group, precision, fronts, solvers)
            basis = CoarseBasis(group[0].mesh, drv.ne, drv.ee, drv.nc, drv.n)
            hist = BatchHistory(drv.B, drv.n)
            pred = None
            if start == "extrapolation":
                pred = BatchExtrapolationPredictor(hist)
            elif start == "learned":
                pred = BatchMLPPredictor(mlp, basis, hist, c10, kb)
            t0 = time.perf_counter()
            drv.solve(predictor=pred, on_converged=hist)
            wall[start] = wall.get(start, 0.0) + time.perf_counter() - t0
            ok = ~drv.failed
            out[start].append(drv.iterations[ok])
            failed[start] += int(drv.failed.sum())
            if start == "learned":
                used.append(drv.predicted[ok])
            drv.close()
            if log:
                log(f"{start}: {np.mean(drv.iterations[ok]):.3f} it/step over {int(ok.sum())} "
                    f"solves, {wall[start]:.1f} s")
    res = {k: float(np.mean(np.concatenate(v))) for k, v in out.items() if v}
    if used:
        res["learned_used"] = float(np.mean(np.concatenate(used)))
    res["steps"] = int(np.concatenate(out[starts[0]]).size)
    res["failed"] = failed
    res["wall_s"] = wall
    return res
