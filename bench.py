"""Benchmark of the SOLID81 per-iteration global assembly on GB300.

Workload (one "step" = FEStorage::updateResults + assembleGlobalEqMatrices of
the whole mesh): a 100x100x100 block of SOLID81 u/p hexahedra on the unit cube
(1e6 elements, 1,030,301 nodes, 4,090,903 equations, 149,264,506 upper-CSR
nonzeros), Mooney-Rivlin C10 = 0.4, C01 = 0.1, K = 2000; nodal displacements
from a 30 degree end twist plus 1.5 stretch with seeded +-0.005h noise;
element pressures ~ N(0, 0.1).  Synthetic inputs (no dataset exists).

Arms:
  default            this repo's GPU path (libnla3d_gpu.so through its C ABI)
  --impl reference   the reference's algorithm on the host cores (the oracle
                     port, oracle/nla3d_oracle.c, which reproduces the
                     reference bit for bit), all cores, independent samples

Output: one JSON line (rank 0).  `value` = elements/s / 1e6 with inputs
resident in HBM; `e2e` = the same through the C ABI with host buffers (U
copied in, all K blocks and F copied out every step).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# FP64 flop per SOLID81 element of the algorithm the kernel runs (8 Gauss
# points x 3628: kinematics 189, material + S + wDd 436, -wFS / w cof F 96,
# tangent tensor A 513, h_a = A^T G_a for the 6 blocks i <= k 720, F_u + K_up
# 288, the 231 accumulated K_uu entries 1386; plus 96, and 483 for the 69
# entries of node 7's column and block derived from sum_b G_b = 0).  The
# executed FP64 instruction counters of one ncu capture give 29,467 per
# element (2 DFMA + DMUL + DADD); that figure is used.  The Bh^T D Bh formulation costs 69,072
# (8 x 8634) for the same element.
FLOP_PER_ELEM = 29467
FLOP_PER_ELEM_BTDB = 69072
# FP64 instructions per element in the same capture (12,744 DFMA + 3,096
# DMUL + 883 DADD): a DMUL or DADD takes the pipe as long as a DFMA for half
# the flops, so the pipe's instruction rate is the tighter ceiling.
FP64_INSTR_PER_ELEM = 16723
# DRAM bytes per element of solid81_kernel<double> and of the K gather in one
# ncu capture of a 40^3 block (64,000 elements, 9,675,406 K slots), used to
# scale the traffic to the measured launch; the element kernel's writes are a
# lower bound there (L2 still held part of them when the kernel ended).
DRAM_BYTES_PER_ELEM_SOLID81 = (108.598016e6 + 122.938624e6) / 64000
DRAM_BYTES_PER_ELEM_GATHER_K = (301.560064e6 + 62.591488e6) / 64000
# Executed arithmetic per element of solid81_kernel<float> (mixed), from the
# instruction counters of one ncu capture of a 40^3 block (64,000 elements):
# FP32 2 FFMA + FADD + FMUL and FP64 2 DFMA + DADD + DMUL per element.
MIXED_FP32_FLOP_PER_ELEM = 67044
MIXED_FP64_FLOP_PER_ELEM = 1800
MIXED_WARP_INSTR_PER_ELEM = 2601
METRIC = "SOLID81 assembly Melem/s"  # Newton iterations per load step (plain vs learned) in "newton"
MIXED_DTYPE = ("f32 K_uu / f64 volumetric terms (J, J-1, p/K, K_up, K_pp, F_p) / "
               "float-pair (2^-48) F_u chain / f64 CSR sums")
UNIT = "Melem/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=100, help="hex elements per side")
    ap.add_argument("--cpu-sample-n", type=int, default=30)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--batch-meshes", type=int, default=256)
    ap.add_argument("--no-newton", action="store_true")
    ap.add_argument("--no-solver", action="store_true",
                    help="skip the device LDL^T leg (K(2) of the 20x20x80 bar)")
    ap.add_argument("--model", choices=["3d_damper", "a2000"],
                    help="run one of the reference's BENCH models instead (minutes)")
    ap.add_argument("--model-backend", default="fp64", choices=["fp64", "mixed", "port"])
    ap.add_argument("--cdb", metavar="PATH",
                    help="read the --model mesh from this .cdb file (the reference's "
                         "test/3d_damper/model.cdb or test/a2000_damper/a2000.cdb) with the "
                         "library's reader instead of the committed fixture")
    ap.add_argument("--solver-bench", type=int, default=0, metavar="NX",
                    help="time the device LDL^T of K(2) on the NX x NX x 4NX rigid-body bar "
                         "(40: the 1.07M-equation Newton bar) and exit")
    ap.add_argument("--solver-precisions", default="fp32,fp64")
    ap.add_argument("--newton-bar", type=int, default=0, metavar="NX",
                    help="Newton study on the NX x NX x 4NX torsion + stretch bar (40: the "
                         "256k-element bar): plain vs learned start, FP64 vs mixed assembly, "
                         "K(2) factored on the device; prints one JSON line and exits")
    ap.add_argument("--newton-starts", default="plain,learned")
    ap.add_argument("--learned-blocks", type=int, default=0, metavar="N",
                    help="learned-start study on N^3 blocks (20: the configured size) with "
                         "K(2) factored on the device; prints one JSON line and exits")
    ap.add_argument("--learned-train", type=int, default=2000)
    ap.add_argument("--learned-eval", type=int, default=100)
    ap.add_argument("--learned-batch", type=int, default=100,
                    help="solves advanced in lock step by one batched Newton driver")
    ap.add_argument("--learned-curve", default="50,200,500,1000",
                    help="training-set sizes (solves) for the iterations-saved curve")
    ap.add_argument("--learned-epochs", type=int, default=150)
    ap.add_argument("--newton-solver", default="gpu-fp32", choices=["gpu", "gpu-fp32", "gpu-tc"],
                    help="K(2) solve of --newton-bar and --learned-blocks")
    ap.add_argument("--newton-assembly", default="fp64,mixed",
                    help="assembly precisions of --newton-bar (the mixed run uses the plain start)")
    ap.add_argument("--model-solver", default="nd",
                    choices=["nd", "gpu", "gpu-fp32", "gpu-tc", "direct"],
                    help="K(2) solve of --model runs: host SuperLU after nested dissection, "
                         "or the device LDL^T with FP64 / FP32 fronts")
    ap.add_argument("--e2e-chunks", type=int, default=8,
                    help="element ranges of nla3d_assemble_to_host in the e2e leg")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the full-size parity check against the oracle port")
    ap.add_argument("--no-tune", action="store_true",
                    help="keep the default launch shape and contribution layout")
    return ap.parse_args()


def workload(n):
    from nla3d_gb300 import meshgen as mg
    mesh, u, p = mg.config_twist(n=n, seed=2)
    return mesh, u, p


def workload_config(mesh=None, extra=None, n=None):
    """Config of the n^3 workload (from the mesh, or from n alone)."""
    if mesh is not None:
        n = round(mesh.n_elems ** (1 / 3))
    cfg = {
        "workload": f"SOLID81 u/p hex block {n}^3 on the unit cube, "
                    "Mooney-Rivlin C10=0.4 C01=0.1 K=2000, 30deg twist + 1.5 stretch, "
                    "+-0.005h noise, p~N(0,0.1); step = updateResults + "
                    "assembleGlobalEqMatrices",
        "elements": n ** 3,
        "nodes": (n + 1) ** 3,
        "l2": "no flush: inputs larger than L2 (element contributions 2.6 GB, gather lists "
              "1.9 GB, K 1.2 GB per step at 1e6 elements)",
    }
    if extra:
        cfg.update(extra)
    return cfg


# ---------------------------------------------------------------------------
# CPU side: the reference's algorithm (oracle port), bounded sample.
# ---------------------------------------------------------------------------

def _cpu_sample_worker(args):
    n, reps, budget_s = args
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    from nla3d_gb300 import meshgen as mg
    mesh, u, p = mg.config_twist(n=n, seed=2)
    m = O.OracleModel(mesh, "port")
    ne, ee = m.eq_numbers()
    m.set_U(mg.u_to_vector(ne, ee, u, p, m.n_total))
    m.update()
    m.assemble()                      # warm-up
    times = []
    t_start = time.perf_counter()
    for _ in range(reps):
        t0 = time.perf_counter()
        m.update()
        m.assemble()
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - t_start > budget_s:
            break
    return mesh.n_elems, times


def cpu_baseline_single(n, budget_s=15.0):
    """One host thread, the reference algorithm on an n^3 sample."""
    ne, times = _cpu_sample_worker((n, 50, budget_s))
    t = statistics.median(times)
    return {"value": ne / t / 1e6, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{n}^3 = {ne} SOLID81 elements of the same workload (twist+stretch, "
                      f"Mooney-Rivlin), median of {len(times)} updateResults+assemble calls "
                      "on 1 host thread; oracle/nla3d_oracle.c reproduces the reference "
                      "bit for bit"}


_WORKER = {}


def _worker_init(n):
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    from nla3d_gb300 import meshgen as mg
    mesh, u, p = mg.config_twist(n=n, seed=2)
    m = O.OracleModel(mesh, "port")
    ne, ee = m.eq_numbers()
    m.set_U(mg.u_to_vector(ne, ee, u, p, m.n_total))
    _WORKER["m"], _WORKER["ne"] = m, mesh.n_elems


def _worker_step(_):
    m = _WORKER["m"]
    t0 = time.perf_counter()
    m.update()
    m.assemble()
    return _WORKER["ne"], time.perf_counter() - t0


def run_reference(args):
    """The reference's algorithm on all host cores: one independent sample
    per core (the reference itself is single-threaded)."""
    import multiprocessing as mp
    from oracle import oracle as O
    O.build_port()
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    n = args.cpu_sample_n
    steps = []
    with ctx.Pool(cores, initializer=_worker_init, initargs=(n,)) as pool:
        for i in range(args.warmup + args.steps):
            res = pool.map(_worker_step, range(cores), chunksize=1)
            if i >= args.warmup:
                steps.append((sum(r[0] for r in res), max(r[1] for r in res)))
    ne = steps[0][0]
    t = statistics.median(s[1] for s in steps)
    value = ne / t / 1e6
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "impl": "reference",
        "config": workload_config(None, {"sample": f"each step: {cores} independent {n}^3 "
                                                   "blocks of the same workload, one per host "
                                                   "core (the reference is single-threaded)",
                                         "precision": "fp64"}, n=args.n),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{cores} processes x {n}^3 = {ne // cores} SOLID81 elements, "
                                   "one updateResults+assemble each per step; "
                                   "oracle/nla3d_oracle.c reproduces the reference bit for bit"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# Parity at full size: the oracle port on the bench's own state, in a spawned
# process that runs on one host core while the GPU legs run.
# ---------------------------------------------------------------------------

def _parity_oracle_worker(n, outdir):
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    from nla3d_gb300 import meshgen as mg
    t0 = time.perf_counter()
    mesh, u, p = mg.config_twist(n=n, seed=2)
    m = O.OracleModel(mesh, "port")
    ne, ee = m.eq_numbers()
    m.set_U(mg.u_to_vector(ne, ee, u, p, m.n_total))
    m.update()
    m.assemble()
    np.save(os.path.join(outdir, "ne.npy"), ne)
    np.save(os.path.join(outdir, "ee.npy"), ee)
    for b in (1, 12, 2):
        io, co = m.pattern(b)
        np.save(os.path.join(outdir, f"io{b}.npy"), io)
        np.save(os.path.join(outdir, f"co{b}.npy"), co)
        np.save(os.path.join(outdir, f"K{b}.npy"), m.K(b))
    np.save(os.path.join(outdir, "F.npy"), m.F())
    m.close()
    with open(os.path.join(outdir, "seconds"), "w") as f:
        f.write(str(time.perf_counter() - t0))


def start_parity(n):
    import multiprocessing as mp
    import tempfile
    outdir = tempfile.mkdtemp(prefix="nla3d_parity_")
    proc = mp.get_context("spawn").Process(target=_parity_oracle_worker, args=(n, outdir))
    proc.start()
    return proc, outdir


def _rel(a, b, m=None):
    if m is not None:
        a, b = a[m], b[m]
    if b.size == 0:
        return 0.0
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def finish_parity(proc, outdir, gpu64, gpu_mixed):
    """Compare the GPU results kept on the host with the oracle's arrays.
    gpu64 = (ne, ee, n_con, {b: (io, co)}, {b: K}, F); gpu_mixed = (K2, F) or None."""
    import shutil
    proc.join()
    try:
        if proc.exitcode != 0:
            return {"error": f"oracle process exit code {proc.exitcode}"}
        ld = lambda nm: np.load(os.path.join(outdir, nm + ".npy"), mmap_mode="r")  # noqa: E731
        ne, ee, n_con, pat, K, F = gpu64
        out = {"vs": "oracle port (oracle/nla3d_oracle.c) on the same state, one host core",
               "numbering_equal": bool(np.array_equal(ne, ld("ne")) and np.array_equal(ee, ld("ee"))),
               "pattern_equal": all(np.array_equal(pat[b][0], ld(f"io{b}")) and
                                    np.array_equal(pat[b][1], ld(f"co{b}")) for b in (1, 12, 2)),
               "fp64": {"K_rel": max(_rel(K[b], np.asarray(ld(f"K{b}"))) for b in (1, 12, 2)),
                        "F_rel": _rel(F, np.asarray(ld("F")))},
               "tolerance": 1e-12}
        if gpu_mixed is not None:
            K2m, Fm = gpu_mixed
            Kr, Fr = np.asarray(ld("K2")), np.asarray(ld("F"))
            # entry classes of K(2): u-u, u-p, p-p (pressure equations from ee)
            pres = np.zeros(len(Fr) + 1, bool)
            pe = ee[:, 6].astype(np.int64)
            pres[pe[pe > 0]] = True
            io, co = pat[2]
            rows = np.repeat(np.arange(1, io.size, dtype=np.int64), np.diff(io.astype(np.int64)))
            cls = pres[rows + n_con].astype(np.int8) + pres[co.astype(np.int64) + n_con].astype(np.int8)
            fp = pres[1:len(Fr) + 1]
            out["mixed"] = {"K_uu": _rel(K2m, Kr, cls == 0), "K_up": _rel(K2m, Kr, cls == 1),
                            "K_pp": _rel(K2m, Kr, cls == 2), "F_u": _rel(Fm, Fr, ~fp),
                            "F_p": _rel(Fm, Fr, fp)}
        out["oracle_s"] = float(open(os.path.join(outdir, "seconds")).read())
        out["ok"] = bool(out["numbering_equal"] and out["pattern_equal"] and
                         out["fp64"]["K_rel"] <= 1e-12 and out["fp64"]["F_rel"] <= 1e-12)
        return out
    finally:
        shutil.rmtree(outdir, ignore_errors=True)


# ---------------------------------------------------------------------------
# GPU side
# ---------------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(x, dist):
    """The slowest rank's time (replicas: whole-job time = the max)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(n_units_per_rank, sec, world):
    """Whole-job throughput of `world` independent replicas, in millions of
    units per second, from the slowest rank's time per step."""
    return world * n_units_per_rank / sec / 1e6


def time_steps(st, U_dev, n_total, steps, torch, stream):
    """Device-resident steps: U already in HBM; returns seconds per step."""
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(steps):
        st.setU_device(U_dev.data_ptr(), n_total)
        st.updateResults()
        st.assembleGlobalEqMatrices()
    ev1.record(stream)
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1) / 1e3 / steps


def run_batched(args, torch, stream, local, dist=None, world=1):
    """Batched workload: independent hex blocks with per-side edge counts drawn
    log-uniform in [4, 40], C10 ~ U(0.2, 1.0), K = C10 * U(500, 5000), stretch
    ~ U(1.0, 1.8); FP32 tangent / FP64 residual and CSR sums; all meshes in one
    launch per kernel, replayed as a CUDA graph with the autotuned shape."""
    from nla3d_gb300 import meshgen as mg
    from nla3d_gb300.batch import BatchAssembly
    items = mg.batched_meshes(args.batch_meshes, seed=3)
    meshes = [it[0] for it in items]
    t0 = time.perf_counter()
    b = BatchAssembly(meshes, "mixed", stream=stream.cuda_stream).init()
    setup_s = time.perf_counter() - t0
    U = b.state_vector([(it[1], it[2]) for it in items])
    U_dev = torch.from_numpy(U).to(f"cuda:{local}")
    b.set_U_device(U_dev.data_ptr(), b.n_total)
    b.update()
    b.assemble()
    tuned = b.autotune(reps=2)
    b.capture_graph()
    for _ in range(args.warmup):
        b.graph_launch()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(args.steps):
        b.set_U_device(U_dev.data_ptr(), b.n_total)
        b.graph_launch()
    ev1.record(stream)
    torch.cuda.synchronize()
    sec = max_over_ranks(ev0.elapsed_time(ev1) / 1e3 / args.steps, dist)
    flagged = b.element_status()[0]
    out = {"value": replica_throughput(b.n_elems, sec, world), "unit": UNIT,
           "ms_per_step": sec * 1e3,
           "meshes": len(meshes), "elements": b.n_elems, "equations": b.n_total,
           "nnz_upper": b.nnz_total, "autotuned": tuned, "graph": True,
           "dtype": MIXED_DTYPE,
           "setup_s": setup_s, "element_status": {"flagged": int(flagged)},
           "workload": f"{len(meshes)} hex blocks, sides log-uniform in [4, 40] (seed 3), "
                       "Neo-Hookean C10~U(0.2,1.0), K/C10~U(500,5000), stretch~U(1.0,1.8)"}
    b.close()
    return out


def run_ours(args):
    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    torch.cuda.set_device(local)
    from nla3d_gb300 import meshgen as mg
    from nla3d_gb300.storage import FEStorage, probe_fma_peak

    parity_job = None
    # CPU baseline first (rank 0, N=1 only), before any GPU work
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline_single(args.cpu_sample_n)

    mesh, u, p = workload(args.n)
    stream = torch.cuda.Stream()
    t0 = time.perf_counter()
    st = FEStorage(mesh, "fp64", stream=stream.cuda_stream).initSolutionData()
    setup_s = time.perf_counter() - t0
    ne, ee = st.eq_numbers()
    U = mg.u_to_vector(ne, ee, u, p, st.n_total)
    U_dev = torch.from_numpy(U).to(f"cuda:{local}")
    nnz = sum(st.blocks[b][2] for b in (1, 12, 2))

    # launch shape and contribution layout picked by the library's autotuner
    # (set-up work, outside the timed region), then warm-up
    st.setU_device(U_dev.data_ptr(), st.n_total)
    st.updateResults()
    tuned = None if args.no_tune else st.autotune(reps=2)
    for _ in range(args.warmup):
        st.setU_device(U_dev.data_ptr(), st.n_total)
        st.updateResults()
        st.assembleGlobalEqMatrices()
    torch.cuda.synchronize()
    count, _first = st.element_status()

    # timed region: device-resident inputs, per-kernel CUDA events on the same stream
    st.set_timing(True)
    launches0 = st.kernel_launches()
    if dist:
        dist.barrier()
    with ClockSampler(local) as clk:
        sec = time_steps(st, U_dev, st.n_total, args.steps, torch, stream)
    launches = st.kernel_launches() - launches0
    kt, kcount = st.kernel_times()
    st.set_timing(False)
    sec = max_over_ranks(sec, dist)
    value = replica_throughput(mesh.n_elems, sec, world)
    gpu64 = None
    if rank == 0 and world == 1 and not args.no_parity:
        gpu64 = (ne, ee, st.n_con, {b: st.pattern(b) for b in (1, 12, 2)},
                 {b: st.K(b).copy() for b in (1, 12, 2)}, st.F().copy())

    # e2e through the C ABI with host buffers (pinned): U in, K blocks + F out
    e2e = None
    if not args.no_e2e:
        Uh = torch.from_numpy(U).pin_memory()
        Kh = {b: torch.empty(st.blocks[b][2], dtype=torch.float64).pin_memory() for b in (1, 12, 2)}
        Fh = torch.empty(st.n_total, dtype=torch.float64).pin_memory()
        Uh_np, Fh_np = Uh.numpy(), Fh.numpy()
        Kh_np = {b: Kh[b].numpy() for b in Kh}
        lib, h = st.lib, st.h

        def ptr(a):
            return a.ctypes.data if a.size else None

        def e2e_plain():
            lib.nla3d_set_U(h, Uh_np.ctypes.data, st.n_total)
            lib.nla3d_update_results(h)
            lib.nla3d_assemble(h)
            for b in (1, 12, 2):
                if Kh_np[b].size:
                    lib.nla3d_get_K(h, b, Kh_np[b].ctypes.data)
            lib.nla3d_get_F(h, Fh_np.ctypes.data)

        def e2e_step():
            # set vecU, updateResults, then assembly with the K blocks streamed
            # to the host while later element ranges compute
            lib.nla3d_set_U(h, Uh_np.ctypes.data, st.n_total)
            lib.nla3d_update_results(h)
            rc = lib.nla3d_assemble_to_host(h, args.e2e_chunks, ptr(Kh_np[1]), ptr(Kh_np[12]),
                                            ptr(Kh_np[2]), Fh_np.ctypes.data)
            assert rc == 0, rc

        def time_it(fn):
            for _ in range(max(1, args.warmup)):
                fn()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(args.steps):
                fn()
            torch.cuda.synchronize()
            return (time.perf_counter() - t0) / args.steps

        plain_sec = time_it(e2e_plain)
        K_plain = Kh_np[2].copy()
        e2e_sec = time_it(e2e_step)
        assert np.array_equal(Kh_np[2], K_plain), "chunked copy differs from the plain path"
        e2e_sec = max_over_ranks(e2e_sec, dist)
        e2e = {"value": replica_throughput(mesh.n_elems, e2e_sec, world), "unit": UNIT,
               "h2d_bytes_per_step": int(U.nbytes),
               "d2h_bytes_per_step": int(8 * nnz + 8 * st.n_total),
               "ms_per_step": e2e_sec * 1e3,
               "api": f"nla3d_set_U + nla3d_update_results + nla3d_assemble_to_host "
                      f"({args.e2e_chunks} element ranges, copies overlapped), pinned host buffers",
               "plain_ms_per_step": plain_sec * 1e3,
               "plain_api": "nla3d_set_U + nla3d_update_results + nla3d_assemble + "
                            "nla3d_get_K x3 + nla3d_get_F"}
        assert np.array_equal(Kh_np[2], st.K(2)), "e2e K differs from the device result"

    # full-size parity against the oracle port: a spawned process on one host
    # core, started after the timed FP64 and e2e legs so that it does not
    # compete with their host-side work; it runs while the remaining legs do
    if rank == 0 and world == 1 and not args.no_parity:
        parity_job = start_parity(args.n)

    # mixed precision path on the same workload
    mixed = None
    gpu_mixed = None
    if not args.no_mixed:
        sm = FEStorage(mesh, "mixed", stream=stream.cuda_stream).initSolutionData()
        sm.setU_device(U_dev.data_ptr(), sm.n_total)
        sm.updateResults()
        mtuned = None if args.no_tune else sm.autotune(reps=2)
        for _ in range(args.warmup):
            sm.setU_device(U_dev.data_ptr(), sm.n_total)
            sm.updateResults()
            sm.assembleGlobalEqMatrices()
        sm.set_timing(True)
        msec = time_steps(sm, U_dev, sm.n_total, args.steps, torch, stream)
        mkt, _ = sm.kernel_times()
        K64, K32 = st.K(2), sm.K(2)
        F64, F32 = st.F(), sm.F()
        gpu_mixed = (K32, F32) if parity_job else None
        msec = max_over_ranks(msec, dist)
        mixed = {"value": replica_throughput(mesh.n_elems, msec, world), "unit": UNIT,
                 "ms_per_step": msec * 1e3, "speedup_vs_fp64": sec / msec, "autotuned": mtuned,
                 "kernel_ms": {"element": float(mkt[0]), "gather_K": float(mkt[1]),
                               "gather_F": float(mkt[2])},
                 "K_rel_err_vs_fp64": float(np.abs(K32 - K64).max() / np.abs(K64).max()),
                 "F_rel_err_vs_fp64": float(np.abs(F32 - F64).max() / np.abs(F64).max()),
                 "dtype": MIXED_DTYPE,
                 "bound": "latency of the element kernel (short-scoreboard stalls first), "
                          "the FP64 pipe of its volumetric terms the busiest unit (ncu at "
                          "64,000 elements: FP64 pipe 65%, FP32 FMA 25%, issue 43%, LSU 17%, "
                          "shared wavefronts 18%, DRAM 9%)",
                 "profile": "profiles/solid81_mixed_fp64vol_block40_ncu.md"}
        sm.close()

    batched = None
    if not args.no_batched:
        batched = run_batched(args, torch, stream, local, dist, world)

    newton = None
    if not args.no_newton and rank == 0:
        from nla3d_gb300 import learned
        newton = learned.benchmark()

    ldlt_leg = None
    if not args.no_solver and rank == 0:
        # the consumer of the assembled K(2): its device LDL^T on the 139k-equation bar
        ldlt_leg = solver_bench(20, ("fp32-tc", "fp32", "fp64"))

    parity = None
    if parity_job:
        parity = finish_parity(*parity_job, gpu64, gpu_mixed)

    if rank != 0:
        return
    fp64_peak = probe_fma_peak(True)
    fp32_peak = probe_fma_peak(False)
    if mixed:
        # executed arithmetic of the mixed element kernel against the FMA
        # probes of both pipes, and its warp-instruction issue rate against
        # one instruction per cycle per scheduler
        mel = mixed["kernel_ms"]["element"] * 1e-3
        a32 = MIXED_FP32_FLOP_PER_ELEM * mesh.n_elems / mel
        a64 = MIXED_FP64_FLOP_PER_ELEM * mesh.n_elems / mel
        import torch as _t
        sms = _t.cuda.get_device_properties(local).multi_processor_count
        clk_mhz = (clk.summary().get("sm_mhz") or peaks_sm_mhz())
        issue_peak = sms * 4 * clk_mhz * 1e6
        ai = MIXED_WARP_INSTR_PER_ELEM * mesh.n_elems / mel
        mixed["roofline"] = {
            "bound": "issue", "kernel": "solid81_kernel<float>",
            "achieved": ai / 1e9, "peak": issue_peak / 1e9, "unit": "G warp-instr/s",
            "frac": ai / issue_peak,
            "fp32": {"achieved": a32 / 1e12, "peak": fp32_peak / 1e12, "unit": "TFLOP/s",
                     "frac": a32 / fp32_peak},
            "fp64": {"achieved": a64 / 1e12, "peak": fp64_peak / 1e12, "unit": "TFLOP/s",
                     "frac": a64 / fp64_peak},
            "algorithmic": f"executed per element: {MIXED_FP32_FLOP_PER_ELEM} FP32 flop, "
                           f"{MIXED_FP64_FLOP_PER_ELEM} FP64 flop, {MIXED_WARP_INSTR_PER_ELEM} "
                           "warp instructions (ncu counters of a 64,000-element launch)",
            "peak_source": "FP32 / FP64 FMA throughput probes in this run; issue: SMs x 4 "
                           "schedulers x median SM clock during the timed region",
            "traffic": (112.787712e6 + 122.929664e6) / 64000 * mesh.n_elems,
            "traffic_source": "ncu dram bytes of a 64,000-element launch, scaled by elements"}
    elem_ms = float(kt[0])
    achieved = FLOP_PER_ELEM * mesh.n_elems / (elem_ms * 1e-3)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs")
    gather_ms = float(kt[1] + kt[2])
    # per contribution: its value (8 B) and, in element order, its id (4 B);
    # per slot: the CSR-ordered pointer (4 B) and the result (8 B)
    layout = tuned["layout"] if tuned else 0
    per_contrib = 8 if layout else 12
    gather_bytes = per_contrib * mesh.n_elems * 350 + (4 + 8) * (nnz + st.n_total)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(mesh, {"equations": st.n_total, "nnz_upper": nnz,
                                         "precision": "fp64",
                                         "parallelism": f"replicas x{world}" if world > 1
                                         else "single GPU"}),
        "e2e": e2e,
        "gpu_launches": int(launches),
        "autotuned": tuned,
        "kernel_ms": {"element": elem_ms, "gather_K": float(kt[1]), "gather_F": float(kt[2]),
                      "mpc": float(kt[3]), "assemblies_averaged": int(kcount)},
        "roofline": {"bound": "fp64", "achieved": achieved / 1e12, "peak": fp64_peak / 1e12,
                     "unit": "TFLOP/s", "frac": achieved / fp64_peak,
                     "traffic": DRAM_BYTES_PER_ELEM_SOLID81 * mesh.n_elems,
                     "traffic_source": "ncu dram bytes of a 64,000-element launch, "
                                       "scaled by elements",
                     "kernel": "solid81_kernel<double>",
                     "algorithmic": f"{FLOP_PER_ELEM} FP64 flop/element x {mesh.n_elems}",
                     "btdb_equivalent_tflops": FLOP_PER_ELEM_BTDB * mesh.n_elems
                     / (elem_ms * 1e-3) / 1e12,
                     "fp64_instr_frac": FP64_INSTR_PER_ELEM * mesh.n_elems / (elem_ms * 1e-3)
                     / (fp64_peak / 2),
                     "fp64_instr_note": "executed FP64 instructions per second against the "
                                        "probe's DFMA rate (FMA probe flops / 2)",
                     "peak_source": "FP64 FMA throughput probe in this run "
                                    "(MEASURED_PEAKS.json has no FP64 figure)"},
        "roofline_gather": {"bound": "hbm", "achieved": gather_bytes / (gather_ms * 1e-3) / 1e9,
                            "peak": hbm, "unit": "GB/s",
                            "frac": (gather_bytes / (gather_ms * 1e-3) / 1e9 / hbm) if hbm else None,
                            "traffic": DRAM_BYTES_PER_ELEM_GATHER_K * mesh.n_elems,
                            "kernel": "gather_sorted_kernel<" + ("false" if layout else "true")
                                      + "> (K + F)",
                            "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"},
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "ldlt": ldlt_leg,
        "newton": newton,
        "mixed": mixed,
        "batched": batched,
        "parity": parity,
        "setup_s": setup_s,
        "element_status": {"flagged": int(count)},
    }
    line["summary"] = compact_summary(line)
    print(json.dumps(line), flush=True)


def peaks_sm_mhz():
    try:
        return float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["sm_max_mhz"])
    except Exception:
        return 2070.0


def compact_summary(line):
    """The headline numbers of every leg in a few hundred bytes, last in the
    line (a reader of the line's tail sees them)."""
    def r(x, d=3):
        return None if x is None else round(float(x), d)
    s = {"fp64_melem_s": r(line["value"], 2), "fp64_roofline_frac": r(line["roofline"]["frac"]),
         "e2e_melem_s": r(line["e2e"]["value"], 2) if line.get("e2e") else None}
    m = line.get("mixed")
    if m:
        s["mixed_melem_s"] = r(m["value"], 2)
        s["mixed_speedup"] = r(m["speedup_vs_fp64"], 2)
        if m.get("roofline"):
            s["mixed_issue_frac"] = r(m["roofline"]["frac"])
    b = line.get("batched")
    if b:
        s["batched_melem_s"] = r(b["value"], 2)
    p = line.get("parity")
    if p and "fp64" in p:
        s["parity_fp64"] = {"K": p["fp64"]["K_rel"], "F": p["fp64"]["F_rel"],
                            "pattern_equal": p["pattern_equal"]}
        if "mixed" in p:
            s["parity_mixed"] = {k: float(f"{v:.2e}") for k, v in p["mixed"].items()}
    n = line.get("newton")
    if n:
        for fam in ("blocks", "bar"):
            if fam in n:
                s[f"newton_{fam}"] = {k: r(n[fam].get(k)) for k in ("plain", "learned")} | \
                    {"mesh": n[fam].get("mesh")}
    ld = line.get("ldlt")
    if ld:
        s["ldlt_s"] = {x["precision"]: r(x["value"], 4) for x in ld}
    return s


def cdb_model(name, cdb_path=None):
    """A reference BENCH model, from a .cdb file read by the library's reader
    (nla3d_gb300.cdb, as main.cpp:167-225 builds it) or from its committed
    fixture (tests/golden/, written from the same file):
    3d_damper (test/CMakeLists.txt:148-153): 7016 SOLID81, Neo-Hookean
    (10, 5000), 497 CE equations, UY reaction of TOP_SIDE, threshold 3.0;
    a2000 (test/CMakeLists.txt:141-146): 3101 PLANE41, Neo-Hookean (1, 500),
    UY reaction of DISP_BC, threshold 0.2.  Returns (mesh, fixes, reaction
    nodes, ANSYS curve, threshold).  The ANSYS curve always comes from the
    fixture."""
    from nla3d_gb300 import meshgen as mg
    if cdb_path:
        from nla3d_gb300 import cdb
        md = cdb.read_cdb(cdb_path)
        fx = "damper_3d.npz" if name == "3d_damper" else "a2000_plane41.npz"
        curve = np.load(os.path.join(ROOT, "tests", "golden", fx))["ref_curve"]
        if name == "3d_damper":
            m, fixes, _ = cdb.to_mesh(md, mg.ELEM_SOLID81, mg.MAT_NEO_HOOKEAN, (10.0, 5000.0),
                                      name=name)
            return m, fixes, np.array(md.feComps["TOP_SIDE"].list, np.uint32), curve, 3.0
        m, fixes, _ = cdb.to_mesh(md, mg.ELEM_PLANE41, mg.MAT_NEO_HOOKEAN, (1.0, 500.0), name=name)
        return m, fixes, np.array(md.feComps["DISP_BC"].list, np.uint32), curve, 0.2
    if name == "3d_damper":
        g = np.load(os.path.join(ROOT, "tests", "golden", "damper_3d.npz"))
        m = mg.Mesh(mg.ELEM_SOLID81, g["xyz"], g["conn"], mat_id=mg.MAT_NEO_HOOKEAN,
                    mat_c=(10.0, 5000.0), name=name)
        ptr = g["mpc_ptr"]
        for k in range(len(g["mpc_b"])):
            sl = slice(int(ptr[k]), int(ptr[k + 1]))
            m.mpcs.append(mg.LinearMpc(g["mpc_node"][sl], g["mpc_dof"][sl], g["mpc_coef"][sl],
                                       float(g["mpc_b"][k])))
        nodes, thr = g["top_side"], 3.0
    else:
        g = np.load(os.path.join(ROOT, "tests", "golden", "a2000_plane41.npz"))
        m = mg.Mesh(mg.ELEM_PLANE41, g["xyz"], g["conn"], mat_id=mg.MAT_NEO_HOOKEAN,
                    mat_c=(1.0, 500.0), name=name)
        nodes, thr = g["disp_bc"], 0.2
    m.fix_nodes, m.fix_dofs = g["fix_node"], g["fix_dof"]
    fixes = list(zip(g["fix_node"].tolist(), g["fix_dof"].tolist(), g["fix_value"].tolist()))
    return m, fixes, nodes, g["ref_curve"], thr


def run_cdb_model(args):
    """A reference BENCH run (20 load steps, 15 iterations, kinematic
    criterion 1e-3, UY reaction of the component against the ANSYS curve,
    mean |difference| against the test's threshold as main.cpp compareCurves
    does), with the assembly on the GPU (or on the CPU oracle for
    --model-backend port) and the K(2) solve of --model-solver.
    Prints one JSON line."""
    from nla3d_gb300.newton import NewtonSolver
    mesh, fixes, nodes, ref, thr = cdb_model(args.model, args.cdb)
    if args.model_backend == "port":
        from oracle import oracle as O
        b = O.OracleModel(mesh, "port")
    else:
        from nla3d_gb300.storage import FEStorage
        b = FEStorage(mesh, args.model_backend).initSolutionData()
    t_asm = [0.0]
    assemble = b.assemble

    def timed_assemble():
        t0 = time.perf_counter()
        assemble()
        if hasattr(b, "synchronize"):
            b.synchronize()
        t_asm[0] += time.perf_counter() - t0

    b.assemble = timed_assemble
    t0 = time.perf_counter()
    solver = args.model_solver
    if args.model_backend == "port" and solver.startswith("gpu"):
        raise SystemExit("the device solver needs a GPU backend")
    s = NewtonSolver(b, fixes, n_loadsteps=20, n_iterations=15, kinematic_tol=1e-3,
                     solver=solver).solve()
    wall = time.perf_counter() - t0
    ldlt_info = s._ldlt.info() if s._ldlt is not None else None
    ne = s.ne
    curve = np.array([sum(r[int(ne[n - 1, 1]) - 1] for n in nodes) for r in s.reactions])
    err = float(np.abs(curve - ref).mean())
    print(json.dumps({
        "metric": f"{args.model} reaction curve error vs ANSYS (mean |dF|)", "value": err,
        "higher_is_better": False, "threshold": thr, "passed": err < thr,
        "backend": args.model_backend, "load_steps": 20,
        "iterations": [r.iterations for r in s.records],
        "solver": solver, "ldlt": ldlt_info,
        "factorizations": s.factorizations, "wall_s": wall, "assembly_s": t_asm[0],
        "curve": curve.round(4).tolist(), "ansys": ref.tolist(),
        "model": f"{mesh.n_elems} elements, {mesh.n_nodes} nodes, {len(mesh.mpcs)} CE, "
                 f"{len(fixes)} fixed DoFs"}), flush=True)


def solver_bench(nx, precisions=("fp32", "fp64")):
    """The EquationSolver consumer of the assembled K(2) on the device: the
    nx x nx x 4nx bar of the Newton study (rigid-body MPC end, Neo-Hookean
    G = 1, K = 1000) assembled on the GPU at its initial state, a geometric
    nested-dissection order (MPC equations last), the symbolic analysis on
    the host, then the timed factorisation (CUDA events around
    nla3d_ldlt_factor) and one refined solve.  One dict per front precision."""
    import math
    import torch
    from nla3d_gb300 import learned as L, ldlt
    from nla3d_gb300.newton import NewtonSolver
    from nla3d_gb300.storage import FEStorage
    pb = L.bar_problem(nx, 4 * nx, 0.5, 1000.0, 2.0, math.pi / 2)
    t0 = time.perf_counter()
    s = FEStorage(pb.mesh).initSolutionData()
    ns = NewtonSolver(s, pb.fixes, solver="gpu")
    s.set_U(np.zeros(s.n_total))
    s.assemble()
    s.synchronize()
    io, co = s.pattern(2)
    n2 = io.size - 1
    perm = ldlt.fill_reducing_order(io, co, ns._row_points(), s.n_unk)
    t_order = time.perf_counter() - t0
    rhs = np.random.default_rng(0).standard_normal(n2)
    out = []
    for prec in precisions:
        t1 = time.perf_counter()
        solver = ldlt.DeviceLDLT.for_storage(s, perm, prec)
        t_create = time.perf_counter() - t1
        info = solver.info()
        vals = s.device_K(2)[0]
        times = []
        for _ in range(2):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            solver.factor_device(vals)
            e1.record()
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
        # the first solve also records the solve's CUDA graph; the second is
        # the steady state; a pass without refinement times one forward +
        # backward substitution (with the residual of its result)
        t_solves = []
        for _ in range(2):
            t2 = time.perf_counter()
            x = solver.solve_host(s, rhs, max_refine=20, tol=1e-10)
            t_solves.append(time.perf_counter() - t2)
        steps, resid = solver.last_steps, solver.last_residual
        t2 = time.perf_counter()
        solver.solve_host(s, rhs, max_refine=0, tol=1e-300, strict=False)
        t_pass = time.perf_counter() - t2
        fac = times[-1]
        out.append({
            "metric": "K(2) LDL^T factorisation on the device", "precision": prec,
            "value": fac, "unit": "s", "higher_is_better": False,
            "workload": f"rigid-body bar {nx}x{nx}x{4 * nx}, n={n2}, nnz(upper)={co.size}",
            "flops": info["flops"], "gflops": info["flops"] / fac / 1e9,
            "nnz_L": info["nnz_L"], "front_GB": info["front_bytes"] / 1e9,
            "supernodes": info["supernodes"], "levels": info["levels"],
            "max_front": info["max_front"], "perturbed_pivots": info["perturbed"],
            "factor_s_first": times[0], "solve_s": t_solves[1], "solve_s_first": t_solves[0],
            "solve_pass_s": t_pass, "refine_steps": steps,
            "rel_residual": resid, "order_s": t_order, "symbolic_s": t_create,
            "x_norm": float(np.linalg.norm(x))})
        solver.close()
        del solver
        torch.cuda.empty_cache()
    s.close()
    return out


def run_solver_bench(args):
    for rec in solver_bench(args.solver_bench, tuple(args.solver_precisions.split(","))):
        print(json.dumps(rec), flush=True)


def run_newton_bar(args):
    """Newton-Raphson on the nx x nx x 4nx bar (Neo-Hookean C10 = 0.5, K =
    1000, z = 0 clamped, z = L slaved to a master driven to stretch 2.0 and
    90 deg over 50 load steps, residual tolerance 1e-8) with the assembly on
    the GPU and K(2) factored on the device (FP32 fronts, FP64 refinement).
    The learned start's MLP is trained on small bars (3 x 3 x 12, C10, K,
    stretch and twist drawn around the target) by the library's kernels, then
    used on the large bar through its coarse modes.  Mean Newton iterations
    per load step for each start, and for FP64 vs mixed assembly."""
    import math
    from nla3d_gb300 import learned as L
    nx = args.newton_bar
    log = lambda m: print(m, file=sys.stderr, flush=True)  # noqa: E731
    t0 = time.perf_counter()
    starts = tuple(args.newton_starts.split(","))
    mlp = None
    train = {}
    if "learned" in starts and "fp64" in args.newton_assembly.split(","):
        Xb, Yb, _ = L.generate(L.sample_bar_problems(12, nx=3, nz=12, seed=5, n_loadsteps=50))
        mlp = L.MLP(seed=1)
        hist = mlp.fit(Xb, Yb, epochs=300, batch=128, lr=2e-3)
        train = {"train_samples": int(Xb.shape[0]), "final_loss": hist[-1][1],
                 "train_s": time.perf_counter() - t0}
        log(f"trained: {train}")
    cfg = L.bar_problem(nx, 4 * nx, 0.5, 1000.0, 2.0, math.pi / 2, 50)
    res = {}
    precisions = args.newton_assembly.split(",")
    if "fp64" in precisions:
        res["fp64_assembly"] = L.evaluate([cfg], mlp, precision="fp64",
                                          linear_solver=args.newton_solver, starts=starts, log=log)
    if "mixed" in precisions:
        res["mixed_assembly"] = L.evaluate([cfg], mlp, precision="mixed",
                                           linear_solver=args.newton_solver, starts=("plain",),
                                           log=log)
    print(json.dumps({
        "metric": "Newton iterations per load step (residual 1e-8)", "unit": "iterations",
        "higher_is_better": False,
        "workload": f"torsion + stretch bar {nx}x{nx}x{4 * nx} ({cfg.mesh.n_elems} SOLID81), "
                    "rigid-body MPC end, 50 load steps",
        "linear_solver": f"device LDL^T ({args.newton_solver}), FP64 refinement",
        "results": res, "training": train, "wall_s": time.perf_counter() - t0}), flush=True)


def run_learned_blocks(args):
    """The learned Newton start on n^3 blocks (Neo-Hookean, C10 ~ U(0.2, 1),
    K ~ U(500, 5000), target stretch ~ U(1, 2), 20 load steps, residual
    1e-8), K(2) factored on the device.  Solves run `--learned-batch` at a
    time in lock step (nla3d_gb300.batch_newton: one batched assembly, one
    block-diagonal LDL^T per Newton iteration).  The MLP (4 x 256, BF16
    weights, FP32 accumulation) is trained by the library's kernels on the
    converged increments of the first N of `--learned-train` plain-start
    solves, for each N of `--learned-curve`, and evaluated on
    `--learned-eval` held-out solves against the plain and the
    secant-extrapolation starts."""
    from nla3d_gb300 import learned as L
    n = args.learned_blocks
    fronts = {"gpu": "fp64", "gpu-fp32": "fp32", "gpu-tc": "fp32-tc"}[args.newton_solver]
    log = lambda m: print(m, file=sys.stderr, flush=True)  # noqa: E731
    solvers = {}
    t0 = time.perf_counter()
    X, Y, its, failed, owner = L.generate_batched(
        L.sample_block_problems(args.learned_train, n=n, seed=11), fronts=fronts,
        batch_size=args.learned_batch, log=log, solvers=solvers)
    t_gen = time.perf_counter() - t0
    log(f"generated {X.shape[0]} samples from {args.learned_train} solves in {t_gen:.1f} s")
    held_out = L.sample_block_problems(args.learned_eval, n=n, seed=99)
    base = L.evaluate_batched(held_out, None, fronts=fronts, batch_size=args.learned_batch,
                              starts=("plain", "extrapolation"), log=log, solvers=solvers)
    sizes = sorted({int(v) for v in args.learned_curve.split(",") if v and
                    int(v) < args.learned_train} | {args.learned_train})
    curve = []
    for size in sizes:
        sel = owner < size
        t1 = time.perf_counter()
        mlp = L.MLP(seed=0)
        hist = mlp.fit(X[sel], Y[sel], epochs=args.learned_epochs, batch=128, lr=2e-3)
        t_fit = time.perf_counter() - t1
        res = L.evaluate_batched(held_out, mlp, fronts=fronts, batch_size=args.learned_batch,
                                 starts=("learned",), log=log, solvers=solvers)
        curve.append({"train_solves": size, "train_samples": int(sel.sum()),
                      "learned": res["learned"], "learned_used": res["learned_used"],
                      "saved_vs_plain": base["plain"] - res["learned"],
                      "failed": res["failed"]["learned"], "final_loss": hist[-1][1],
                      "fit_s": t_fit, "eval_s": res["wall_s"]["learned"]})
        log(f"trained on {size} solves: {curve[-1]}")
    full = curve[-1]
    print(json.dumps({
        "metric": "Newton iterations per load step (residual 1e-8), learned vs plain start",
        "unit": "iterations", "higher_is_better": False,
        "workload": f"{n}^3 SOLID81 blocks (C10 ~ U(0.2,1), K ~ U(500,5000), stretch ~ U(1,2)), "
                    "20 load steps",
        "train_solves": args.learned_train, "train_samples": int(X.shape[0]),
        "train_failed": failed, "train_plain_iterations": float(np.mean(its)),
        "eval_solves": args.learned_eval,
        "plain": base["plain"], "extrapolation": base["extrapolation"],
        "learned": full["learned"], "learned_used": full["learned_used"],
        "saved_vs_plain": full["saved_vs_plain"], "eval_failed": base["failed"],
        "curve": curve, "eval_wall_s": base["wall_s"],
        "generate_s": t_gen, "wall_s": time.perf_counter() - t0,
        "batch": args.learned_batch, "epochs": args.learned_epochs,
        "linear_solver": f"block-diagonal device LDL^T ({fronts} fronts), FP64 refinement"}),
        flush=True)


def main():
    args = parse()
    if args.learned_blocks:
        run_learned_blocks(args)
        return
    if args.newton_bar:
        run_newton_bar(args)
        return
    if args.solver_bench:
        run_solver_bench(args)
        return
    if args.model:
        run_cdb_model(args)
        return
    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) != 0:
            return
        run_reference(args)
        return
    run_ours(args)


if __name__ == "__main__":
    main()
