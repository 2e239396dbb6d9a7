"""Benchmark of the butterfly Helmholtz apply on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl bfg|reference]
                    [--config c4|c3|c3s|c2|c2s|c1] [--rhs R]

One step = one apply of the factorization to R right-hand sides (the
workload's synthetic, seeded inputs).  The metric is right-hand sides per
second at <= 1e-6 relative error against a dense FP64 product on sampled
rows: the fastest precision whose error meets that bound is the headline.
The factorization itself runs once before timing (its time is reported).

--impl reference times the reference's own apply algorithm on the host cores
(the C port of the oracle, fed the same block structure) -- the reference
library compiled from source cannot be present on this machine.

Multi-GPU runs are independent replicas (the path needs no exchange): each
rank runs the same workload, value = total RHS / max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# workloads (sizes, geometry, wavenumber, tolerance) and the error bound
CONFIGS = {
    # 4,096 uniform sources / circle r=3 targets, k=64, leaf 64, tol 1e-8, 1 RHS
    "c1": dict(n=4096, k=64.0, curve="circle", a=3.0, b=3.0, leaf=64, tol=1e-8, R=1),
    # 65,536 / ellipse (3,2), k=512, tol 1e-10, 16 RHS
    "c2": dict(n=65536, k=512.0, curve="ellipse", a=3.0, b=2.0, leaf=64, tol=1e-10, R=16),
    # the c2 geometry at 32,768 points and k=256 (kernel profiles: the FP32
    # arena, 0.5 GB, is still larger than L2)
    "c2s": dict(n=32768, k=256.0, curve="ellipse", a=3.0, b=2.0, leaf=64, tol=1e-10, R=16),
    # 262,144 / star r = 3 + 0.5 cos 5 theta, k=2048, tol 1e-7, 256 RHS
    "c4": dict(n=262144, k=2048.0, curve="star", a=3.0, b=3.0, leaf=64, tol=1e-7, R=256),
    # 256 independent problems in one factorization and one apply: N log-uniform
    # in [1,024, 16,384], sources iid uniform in [-1,1]^2, targets equispaced on
    # the circle of radius 3, k = N / 30, leaf 64, tol 1e-8, 8 RHS (opt-in: its
    # factors take ~63 GB in FP64 and minutes to build)
    "c3": dict(batched=True, problems=256, nmin=1024, nmax=16384, leaf=64, tol=1e-8, R=8),
    # the same at 64 problems, N in [1,024, 4,096] (seconds to build)
    "c3s": dict(batched=True, problems=64, nmin=1024, nmax=4096, leaf=64, tol=1e-8, R=8),
}
METRIC = "Butterfly apply RHS/s at 1e-6 rel err vs plain FP64 GPU; GMRES time-to-1e-8"
# DRAM bytes (ncu dram__bytes_read.sum + dram__bytes_write.sum) per algorithmic
# byte of each stage launch of the 16-RHS apply (FP32 pipelined kernel, bf16x3
# tensor-core kernel), from one ncu capture of the c2s workload each; the c2
# workload (same geometry, kernels and stage structure at twice the size)
# reports its dominant launch's traffic as this ratio times its own
# algorithmic bytes
NCU_DRAM_PER_ALG = {("c2", "fp32", 16): [0.7973, 1.0266, 0.9855, 0.7925],
                    ("c2", "bf16x3", 16): [0.8888, 1.0627, 1.0246, 1.0386],
                    ("c2s", "fp32", 16): [0.7973, 1.0266, 0.9855, 0.7925],
                    ("c2s", "bf16x3", 16): [0.8888, 1.0627, 1.0246, 1.0386],
                    ("c2", "bf16x3", 256): [0.537, 1.057],
                    ("c4", "bf16x3", 256): [0.537, 1.057]}
NCU_TRAFFIC_SOURCE = {
    ("c2", 16): "ncu DRAM bytes of the same stage in a capture of the 32,768-point workload, "
                "scaled by algorithmic bytes",
    ("c2s", 16): "ncu capture",
    ("c2", 256): "ncu capture (stages 0 and 1 of the 65,536-point workload at 256 RHS)",
    ("c4", 256): "ncu DRAM bytes per algorithmic byte of the same stage in a capture of the "
                 "65,536-point workload at 256 RHS (stages 0 and 1), times this launch's "
                 "algorithmic bytes"}
ERR_BOUND = 1e-6


def factorization_work(table, st):
    """The factorization's unit counts and rates from its block table
    (rows kind, m, n; kinds 0..3 = FIRST, MIDDLE, LAST, DENSE) and stats.

    Kernel evaluations: m n per LAST/DENSE block (the fill kernel) and
    p^2 + p n per FIRST/MIDDLE block of rank p (Z_equiv p x p and Z_orig
    p x n, evaluated inside the re-expansion kernels; helm2.c:321-365).

    Reference-equivalent SVD work: what the reference's algorithm does, one
    SVD of every FIRST/MIDDLE block's Z_equiv (the model 22 p^3 flops) plus
    16 p^2 n for applying its pseudo-inverse to Z_orig (two complex p x p
    products per column).  The library executes less than this: blocks with
    the same Z_equiv share one SVD, and blocks of large rank take the
    randomized path.  The rate is therefore this work over the time of both
    re-expansion paths, a reference-equivalent rate and not a fraction of a
    hardware peak."""
    kind = table[:, 0]
    m = table[:, 1].astype(np.float64)
    n = table[:, 2].astype(np.float64)
    fm = kind <= 1
    fill = float(np.sum(m[~fm] * n[~fm]))
    proxy = float(np.sum(m[fm] * m[fm] + m[fm] * n[fm]))
    svd = float(np.sum(22.0 * m[fm] ** 3 + 16.0 * m[fm] ** 2 * n[fm]))
    reexp_s = (st["reexpSmemMs"] + st["reexpGlobalMs"] + st.get("sketchMs", 0.0)) / 1e3
    return {"kernel_evals": fill + proxy, "fill_evals": fill, "proxy_evals": proxy,
            "fill_evals_per_s": fill / (st["fillMs"] / 1e3) if st["fillMs"] > 0 else None,
            "first_middle_blocks": int(np.sum(fm)),
            "full_path_svds": st.get("reexpSvds"),
            "sketched_blocks": st.get("numSketched"),
            "reexp_s": reexp_s,
            "svd_flops_reference_equivalent": svd,
            "svd_model": "22 p^3 + 16 p^2 n per FIRST/MIDDLE block (rank p, n columns)",
            "reference_equivalent_tflops": svd / reexp_s / 1e12 if reexp_s > 0 else None}


def gpu_local_cpus(dev=0):
    """The host CPUs of the NUMA node the GPU's PCI device reports, or None
    (one node, or nothing reported)."""
    try:
        import torch
        pr = torch.cuda.get_device_properties(dev)
        addr = "%04x:%02x:%02x.0" % (pr.pci_domain_id, pr.pci_bus_id, pr.pci_device_id)
        node = int(open("/sys/bus/pci/devices/%s/numa_node" % addr).read())
        if node < 0:
            return None
        cpus = set()
        for part in open("/sys/devices/system/node/node%d/cpulist" % node).read().strip().split(","):
            a, _, b = part.partition("-")
            cpus.update(range(int(a), int(b or a) + 1))
        return cpus & os.sched_getaffinity(0) or None
    except Exception:
        return None


def pinned_local(make):
    """make() run with the calling thread on the GPU's NUMA node, so that the
    pinned host pages it first touches sit next to the GPU; (result, node
    CPUs or None)."""
    cpus = gpu_local_cpus()
    if not cpus:
        return make(), None
    old = os.sched_getaffinity(0)
    try:
        os.sched_setaffinity(0, cpus)
        return make(), sorted(cpus)
    finally:
        os.sched_setaffinity(0, old)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="bfg", choices=["bfg", "reference"])
    ap.add_argument("--config", default=os.environ.get("BFG_BENCH_CONFIG", "c4"),
                    choices=sorted(CONFIGS))
    ap.add_argument("--rhs", type=int, default=0)
    ap.add_argument("--dense-rows", type=int, default=4096,
                    help="sampled target rows of the dense FP64 check")
    ap.add_argument("--err-rhs", type=int, default=0,
                    help="right-hand sides in the error check (0: all)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-c2", action="store_true",
                    help="skip the 65,536-point workload's block (1 and 16 RHS)")
    ap.add_argument("--no-c3", action="store_true",
                    help="skip the 256-problem batched workload's block")
    ap.add_argument("--no-cpu-factorization", action="store_true",
                    help="skip the oracle factorization timings on the host cores")
    ap.add_argument("--profile", default="", choices=["", "fp64", "df64", "fp32", "bf16x3", "bf16x2"],
                    help="profiling driver: factorize the workload, then run --warmup + --steps "
                         "applies of this precision to --rhs RHS with no timing (for ncu)")
    ap.add_argument("--cpu-fac-worker", default="", help=argparse.SUPPRESS)
    ap.add_argument("--cpu-fac-budget", type=float, default=0.0, help=argparse.SUPPRESS)
    ap.add_argument("--no-gmres", action="store_true",
                    help="skip the multiple-scattering GMRES time-to-1e-8 measurement")
    ap.add_argument("--no-learned", action="store_true",
                    help="skip the learned preconditioner: training on GMRES solves of other "
                         "scatterer layouts and FGMRES beside block-Jacobi (about a minute)")
    return ap.parse_args()


def workload_inputs(cfg, impl):
    """Sources iid uniform in [-1,1]^2 (seed 0), targets equispaced in the
    curve parameter."""
    if impl == "bfg":
        import butterfly_gb300 as B
        src = B.uniform_square_points(cfg["n"], 0)
        tgt = B.curve_points(cfg["curve"], cfg["n"], cfg["a"], cfg["b"])
    else:
        from oracle import bf_oracle as O
        src = O.uniform_square_points(cfg["n"], 0)
        tgt = O.curve_points(cfg["curve"], cfg["n"], cfg["a"], cfg["b"])
    return src, tgt


def config_json(name, cfg, R):
    return {"workload": "helmholtz2d_butterfly_apply_%s" % name, "n_src": cfg["n"],
            "n_tgt": cfg["n"], "k": cfg["k"], "targets": cfg["curve"], "leaf_size": cfg["leaf"],
            "tolerance": cfg["tol"], "rhs": R,
            "l2": "factor arena and vectors larger than L2 (129 MB); no flush needed"}


class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.proc = None
        self.lines = []
        self.device = device

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("BFG_BENCH_GLOO") is None else "gloo")
        return world, rank, local, dist
    return 1, 0, 0, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(v, dist):
    if dist is None:
        return v
    import torch
    # NCCL reduces device tensors, gloo (the CPU test backend) host ones
    dev = "cpu" if dist.get_backend() == "gloo" else "cuda"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
# timing: one apply captured in a CUDA graph, replayed K times
# ---------------------------------------------------------------------------
def graph_timed(fac, X, Y, R, prec, args, stream, dist):
    """Warm-up applies, then one apply captured in a CUDA graph (the library
    launches on the context's stream, which is `stream`), W warm-up replays
    and K timed replays with a CUDA event between replays.  Returns (total
    ms of the K replays, median ms per replay, captured)."""
    import torch
    for _ in range(max(3, args.warmup)):
        fac.apply_device(X.data_ptr(), R, R, Y.data_ptr(), R, prec)
    stream.synchronize()
    graph = None
    try:
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=stream):
            fac.apply_device(X.data_ptr(), R, R, Y.data_ptr(), R, prec)
    except Exception:                  # an uncapturable apply is timed directly
        graph = None
        torch.cuda.synchronize()

    def step():
        if graph is not None:
            graph.replay()
        else:
            fac.apply_device(X.data_ptr(), R, R, Y.data_ptr(), R, prec)

    with torch.cuda.stream(stream):
        for _ in range(max(3, args.warmup)):
            step()
    stream.synchronize()
    barrier(dist)
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    with torch.cuda.stream(stream):
        ev[0].record(stream)
        for i in range(args.steps):
            step()
            ev[i + 1].record(stream)
    ev[-1].synchronize()
    torch.cuda.synchronize()
    barrier(dist)
    per = [ev[i].elapsed_time(ev[i + 1]) for i in range(args.steps)]
    return ev[0].elapsed_time(ev[-1]), float(np.median(per)), graph is not None


# ---------------------------------------------------------------------------
# Batched problems
# ---------------------------------------------------------------------------
def batched_problems(B, cfg):
    u = B.Rng(3).uniform(cfg["problems"])
    lo, hi = np.log(cfg["nmin"]), np.log(cfg["nmax"])
    sizes = np.floor(np.exp(lo + (hi - lo) * u)).astype(np.int64)
    problems = [(B.uniform_square_points(int(n), 1000 + j), B.curve_points("circle", int(n), 3.0, 3.0))
                for j, n in enumerate(sizes)]
    return sizes, problems, sizes / 30.0


def run_batched(args, cfg):
    """--config c3: one batched factorization of all problems; a step is one
    apply of R RHS to every problem at once (the block-diagonal operator)."""
    import torch

    import butterfly_gb300 as B
    world, rank, local, dist = dist_setup()
    torch.cuda.set_device(local)
    ctx = B.Context(local)
    line = batched_line(args, cfg, B, ctx, world, rank, local, dist)
    if line is not None:
        print(json.dumps(line))


def batched_line(args, cfg, B, ctx, world, rank, local, dist):
    """The batched workload's measurement as a dict (None off rank 0)."""
    import torch
    sizes, problems, ks = batched_problems(B, cfg)
    t0 = time.perf_counter()
    # every problem's two quadtrees in one GPU pass (the same trees as the
    # host build)
    fac = B.make_batched(B.Helm2(1.0), problems, ks, leaf_size=cfg["leaf"], rank_eps=cfg["tol"],
                         pinv_tol=cfg["tol"], context=ctx, tree_on_gpu=True)
    fac_s = time.perf_counter() - t0
    n = int(sizes.sum())
    R = args.rhs or cfg["R"]
    so, to = fac.src_offsets, fac.tgt_offsets
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    Xh = B.Rng(1234 + rank).complex_randn(n * R).reshape(n, R)     # original point order
    with torch.cuda.stream(stream):
        X64 = torch.from_numpy(Xh).to("cuda")
        X32 = X64.to(torch.complex64)
        Y64 = torch.empty((n, R), dtype=torch.complex128, device="cuda")
        Y32 = torch.empty((n, R), dtype=torch.complex64, device="cuda")
    stream.synchronize()
    precs = {"fp64": (X64, Y64), "fp32": (X32, Y32), "bf16x3": (X32, Y32), "bf16x2": (X32, Y32)}
    # dense FP64 rows of 8 sampled problems (64 target rows each) from the
    # oracle on the host cores (glibc Bessel functions, helm2.c:282-319)
    from oracle import bf_oracle as O
    ref = []
    for j in range(0, len(problems), max(1, len(problems) // 8)):
        src, tgt = problems[j]
        rows = np.unique(np.linspace(0, len(tgt) - 1, 64).astype(np.int64))
        K = O.kernel_matrix(O.Helm2(float(ks[j])), src, tgt[rows])
        ref.append((to[j] + rows, K @ Xh[so[j]:so[j + 1]]))
    errs = {}
    for p, (X, Y) in precs.items():
        fac.apply_device(X.data_ptr(), R, R, Y.data_ptr(), R, p, original_order=True)
        stream.synchronize()
        Yh = Y.cpu().numpy().astype(np.complex128)
        num = sum(float(np.linalg.norm(Yh[r] - yd) ** 2) for r, yd in ref)
        den = sum(float(np.linalg.norm(yd) ** 2) for r, yd in ref)
        errs[p] = (num / den) ** 0.5

    clocks = ClockSampler(local)
    clocks.start()
    tm = {p: graph_timed(fac, precs[p][0], precs[p][1], R, p, args, stream, dist) for p in precs}
    clk = clocks.stop()
    total_ms = {p: max_over_ranks(v[0], dist) for p, v in tm.items()}
    median_ms = {p: v[1] for p, v in tm.items()}
    captured = all(v[2] for v in tm.values())
    rhs_s = {p: world * R * args.steps / (total_ms[p] / 1e3) for p in precs}
    ok = [p for p in precs if errs[p] <= ERR_BOUND]
    head = max(ok, key=lambda p: rhs_s[p]) if ok else "fp64"
    X, Y = precs[head]
    per = np.mean([fac.apply_timed(X.data_ptr(), R, R, Y.data_ptr(), R, head) for _ in range(3)],
                  axis=0)
    info = fac.launch_info(precision=head, rhs=R)
    dom = int(np.argmax(per))
    sA = {"fp64": 16, "df64": 16, "fp32": 8, "bf16x3": 12, "bf16x2": 8}[head]
    sv = 16 if head in ("fp64", "df64") else 8
    alg = float(info[dom, 0] * sA + R * sv * (info[dom, 1] + info[dom, 2]))
    try:
        peak, peak_src = float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        peak, peak_src = 6800.0, "fallback"
    achieved = float(alg / (float(per[dom]) / 1e3) / 1e9)
    # end to end with host complex128 operands
    Xp = torch.from_numpy(Xh).pin_memory()
    Yp = torch.empty((n, R), dtype=torch.complex128).pin_memory()
    lib = B.lib()
    ctx.check(lib.bfgFacApplyHost(fac.handle, B.PRECISIONS[head], B._VP(Xp.data_ptr()), R, R,
                                  B._VP(Yp.data_ptr()), R, 0))
    t0 = time.perf_counter()
    e2e_steps = max(1, min(args.steps, 10))
    for _ in range(e2e_steps):
        ctx.check(lib.bfgFacApplyHost(fac.handle, B.PRECISIONS[head], B._VP(Xp.data_ptr()), R, R,
                                      B._VP(Yp.data_ptr()), R, 0))
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist)
    if rank != 0:
        fac.close()
        return None
    st = fac.stats()
    line = {"metric": METRIC, "value": rhs_s[head], "unit": "RHS/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_ms[head] / args.steps, "median_ms_per_step": median_ms[head],
            "graph_captured": captured, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": {"fp64": "complex128", "df64": "double-float (complex128 vectors)",
                      "fp32": "complex64",
                      "bf16x3": "bf16x3 split (complex64 vectors)",
                      "bf16x2": "bf16x2 split (complex64 vectors)"}[head],
            "data": "synthetic",
            "config": {"workload": "helmholtz2d_butterfly_batched_%d" % cfg["problems"],
                       "problems": cfg["problems"], "n_min": int(sizes.min()),
                       "n_max": int(sizes.max()), "n_total": n, "k": "N/30",
                       "targets": "circle r=3", "leaf_size": cfg["leaf"],
                       "tolerance": cfg["tol"], "rhs": R,
                       "l2": "factor arena and vectors larger than L2 (129 MB); no flush needed"},
            "precision": head, "rel_err": errs[head], "rel_err_all": errs,
            "rhs_per_s_all": rhs_s, "problem_rhs_per_s": rhs_s[head] * cfg["problems"],
            "err_bound": ERR_BOUND,
            "err_sample": "64 rows of each of %d problems, oracle rows on the host" % len(ref),
            "factorization": {"wall_s": fac_s, "device_ms": st["factorMs"],
                              "blocks": st["numBlocks"], "bytes_fp64": fac.num_bytes(),
                              "max_rank": st["maxRank"],
                              "work": factorization_work(fac.block_table(), st)},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None, "peak_source": peak_src,
                         "kernel": "apply launch %d of %d" % (dom, len(per)),
                         "launch_ms": float(per[dom]), "alg_bytes": alg},
            "cpu_baseline": None,
            "e2e": {"value": world * R * e2e_steps / e2e_s, "unit": "RHS/s",
                    "h2d_bytes_per_step": n * R * 16, "d2h_bytes_per_step": n * R * 16,
                    "precision": head},
            "clocks": clk, "gpu_launches": len(info) * args.steps}
    fac.close()
    return line


# ---------------------------------------------------------------------------
# GMRES time-to-1e-8 (the metric's second part)
# ---------------------------------------------------------------------------
def gmres_scattering(B, ctx, extra_modes=5):
    """Sound-soft multiple scattering: 64 circles, radii U[0.05, 0.15], seeded
    rejection sampling in [-2,2]^2 with gaps >= 0.05, 12 points per
    wavelength at k = 200; combined-field operator 1/2 I + (D - i k S) diag(w)
    with the order-6 Kapur-Rokhlin correction, butterfly-compressed in FP64
    (leaf 64, tolerance 1e-10); incident plane wave at a seeded uniform angle;
    right-preconditioned FGMRES to a 1e-8 relative residual with
    block-Jacobi (the reference's preconditioner) and with the two-level
    preconditioner (block-Jacobi plus a coarse space of every circle's
    radiating Fourier modes and extra_modes more, bfgSystemBuildCoarse).
    The headline is the two-level solve; its setup (block-Jacobi and the
    coarse space) is reported beside it and in time_to_tol_with_setup_s."""
    import torch
    k = 200.0
    pts, nrm, w, off, _ = B.scattering_geometry(num=64, k=k, ppw=12.0, rmin=0.05, rmax=0.15,
                                                box=2.0, gap=0.05, seed=0)
    helm = B.Helm2(k, B.LayerPot.CombinedField, alpha=-1j * k, beta=1.0)
    t0 = time.perf_counter()
    fac = B.FacHelm2.make_multilevel(helm, B.Quadtree(pts, nrm, leaf_size=64),
                                     B.Quadtree(pts, leaf_size=64), rank_eps=1e-10,
                                     pinv_tol=1e-10, context=ctx)
    fac_s = time.perf_counter() - t0
    system = B.System(fac, pts, nrm, w, off, kr_order=6, diag_shift=0.5)
    t0 = time.perf_counter()
    system.build_block_jacobi()
    torch.cuda.synchronize()
    bj_s = time.perf_counter() - t0
    theta = 2 * np.pi * B.Rng(7).uniform(1)[0]
    d = np.array([np.cos(theta), np.sin(theta)])
    b = torch.from_numpy(-np.exp(1j * k * (pts @ d))).cuda()

    def solve(prec, precond, max_iter):
        system.set_apply_precision(prec)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        x, info = B.solve_gmres(system, b, tol=1e-8, max_num_iter=max_iter, precond=precond)
        torch.cuda.synchronize()
        return {"time_to_tol_s": time.perf_counter() - t0,
                "iterations": int(info["iterations"]), "converged": bool(info["converged"]),
                "true_rel_residual": float(info["trueRelResidual"])}

    # the matvecs in double-float (FP32 arithmetic, ~1e-13 of FP64) and in
    # FP64; the solver's final true residual is FP64 in both
    bj = {"setup_s": bj_s, "df64": solve("df64", "block_jacobi", 3000),
          "fp64": solve("fp64", "block_jacobi", 3000)}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    dim = system.build_coarse(extra_modes)
    torch.cuda.synchronize()
    coarse_s = time.perf_counter() - t0
    solve("df64", "two_level", 500)               # warm: the first solve allocates
    tl = {"extra_modes": extra_modes, "coarse_dim": dim, "coarse_setup_s": coarse_s,
          "block_jacobi_setup_s": bj_s, "df64": solve("df64", "two_level", 500),
          "fp64": solve("fp64", "two_level", 500)}
    head = tl["df64"]
    return {"workload": "cfie_multiple_scattering_64_circles_k200_12ppw", "unknowns": int(len(pts)),
            "tol": 1e-8, "preconditioner": "two_level", "matvec_precision": "df64",
            "iterations": head["iterations"], "converged": head["converged"],
            "time_to_tol_s": head["time_to_tol_s"],
            "time_to_tol_with_setup_s": head["time_to_tol_s"] + coarse_s + bj_s,
            "true_rel_residual": head["true_rel_residual"],
            "two_level": tl, "block_jacobi": bj, "factorization_s": fac_s}


def learned_scattering(B, ctx, train_layouts=6, angles=6, iterates=(0, 20, 60, 150),
                       epochs=30, chunk=64):
    """The learned preconditioner on the C5 problem: a 4 chunk -> 256 -> 256
    -> 2 chunk network trained (hand-written kernels, Adam) on pairs from
    block-Jacobi GMRES solves on other scatterer layouts (seeds 1..6, random
    angles), then FGMRES to 1e-8 on the bench layout (seed 0) and a held-out
    one (seed 7) with block-Jacobi alone and with the network."""
    import torch
    from butterfly_gb300 import learned as L
    k = 200.0

    def build(seed):
        pts, nrm, w, off, _ = B.scattering_geometry(num=64, k=k, ppw=12.0, rmin=0.05,
                                                    rmax=0.15, box=2.0, gap=0.05, seed=seed)
        helm = B.Helm2(k, B.LayerPot.CombinedField, alpha=-1j * k, beta=1.0)
        fac = B.FacHelm2.make_multilevel(helm, B.Quadtree(pts, nrm, leaf_size=64),
                                         B.Quadtree(pts, leaf_size=64), rank_eps=1e-10,
                                         pinv_tol=1e-10, context=ctx)
        system = B.System(fac, pts, nrm, w, off, kr_order=6, diag_shift=0.5)
        system.build_block_jacobi()
        system.set_apply_precision("df64")
        return pts, system

    def rhs(pts, th):
        return torch.from_numpy(-np.exp(1j * k * (pts @ np.array([np.cos(th), np.sin(th)])))).cuda()

    net = L.Mlp(4 * chunk, 256, 2 * chunk, seed=11, context=ctx)
    rng = B.Rng(5)
    t0 = time.perf_counter()
    Fs, Ts = [], []
    for seed in range(1, 1 + train_layouts):
        pts, system = build(seed)
        L.set_learned(system, net, chunk)
        for th in 2 * np.pi * rng.uniform(angles):
            F, T, _ = L.collect_pairs(system, rhs(pts, th), iterates=iterates)
            Fs.append(F)
            Ts.append(T)
    F, T = torch.cat(Fs), torch.cat(Ts)
    data_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    losses = L.train(net, F, T, epochs=epochs, batch=1024, lr=1e-3)
    train_s = time.perf_counter() - t0
    evals = []
    for seed in (0, 7):
        pts, system = build(seed)
        L.set_learned(system, net, chunk)
        for th in (0.4, 3.9):
            b = rhs(pts, th)
            row = {"layout": seed, "angle": th}
            for pc in ("block_jacobi", "learned"):
                B.solve_gmres(system, b, tol=1e-8, max_num_iter=3000, precond=pc)   # warm
                torch.cuda.synchronize()
                t = time.perf_counter()
                _, info = B.solve_gmres(system, b, tol=1e-8, max_num_iter=3000, precond=pc)
                torch.cuda.synchronize()
                row[pc] = {"iterations": int(info["iterations"]), "time_s": time.perf_counter() - t,
                           "true_rel_residual": float(info["trueRelResidual"])}
            evals.append(row)
    return {"network": "%d-256-256-%d ReLU, FP32" % (4 * chunk, 2 * chunk),
            "training_pairs": int(F.shape[0]), "training_solves": train_layouts * angles,
            "pair_collection_s": data_s, "train_s": train_s,
            "loss_first_last_epoch": [losses[0], losses[-1]],
            "target_mean_square": float(T.pow(2).mean().item()), "eval": evals}


# ---------------------------------------------------------------------------
# CPU legs and the accuracy check (the only places bench.py runs the oracle)
# ---------------------------------------------------------------------------
STANDIN_ENTRIES = 1 << 29        # 8 GiB of complex128: the CPU timings' block values


def standin_port(plan_text):
    """The reference's apply algorithm (oracle C port of
    mat_block_dense/mat_product/mat_block_diag/mat_block_coo Mul) over the
    plan's structure, with constant stand-in block values (values do not
    change the cost) in a buffer far larger than the host caches that every
    block reads in turn."""
    from oracle import bf_oracle as O
    entries = O.parse_plan_entries(plan_text)
    data = np.full(min(STANDIN_ENTRIES, entries), 1e-3 + 1e-3j, dtype=np.complex128)
    return O.ApplyPort.from_plan(plan_text, data, True, wrap=entries > data.size), entries


def cpu_port_time(plan_text, X, nthreads, budget_s=20.0):
    """RHS/s of the reference's apply algorithm on host cores, on the number
    of right-hand sides that fits the time budget."""
    port, _ = standin_port(plan_text)
    t0 = time.perf_counter()
    port(X[:, :1], nthreads)
    t1 = time.perf_counter() - t0
    Rs = int(max(1, min(X.shape[1], budget_s / 3 / max(t1, 1e-6))))
    Xs = np.ascontiguousarray(X[:, :Rs])
    times = []
    for _ in range(3):
        t0 = time.perf_counter()
        port(Xs, nthreads)
        times.append(time.perf_counter() - t0)
    t = float(np.median(times))
    return Rs / t, Rs, t


class OracleRows(threading.Thread):
    """Dense FP64 rows of K X from the oracle (glibc Bessel functions, the
    reference's kernel formulas, helm2.c:93-125, 282-319) on the host cores,
    in column chunks; runs beside the GPU timing."""

    def __init__(self, k, src_tree, tgt_tree, rows, X):
        super().__init__(daemon=True)
        self.args = (k, src_tree, tgt_tree, rows, X)
        self.result = None
        self.error = None
        self.seconds = None

    def run(self):
        try:
            from oracle import bf_oracle as O
            k, src_tree, tgt_tree, rows, X = self.args
            t0 = time.perf_counter()
            self.result = O.dense_rows(O.Helm2(k), src_tree, tgt_tree, rows, X)
            self.seconds = time.perf_counter() - t0
        except Exception as exc:       # reported with the line
            self.error = str(exc)[:200]

    def get(self):
        self.join()
        return self.result


def cpu_factorization_worker(name, budget_s):
    """One process, thread counts fixed by its environment: the oracle's
    factorization (the reference's algorithm: glibc kernel fills, scipy
    zgesvd pseudo-inverses; fac_helm2.c:943-1002, helm2.c:321-365) of the
    workload -- in full when `budget_s` <= 0, else an estimate from a
    sample of its blocks drawn with probability proportional to a cost
    model (Horvitz-Thompson: total ~ mean of time / probability)."""
    from oracle import bf_oracle as O
    cfg = CONFIGS[name]
    src, tgt = workload_inputs(cfg, "reference")
    t0 = time.perf_counter()
    fac = O.Factorization(O.Helm2(cfg["k"]), src, tgt, leaf_size=cfg["leaf"], eps=cfg["tol"],
                          rcut="relative", fill=False)
    plan_s = time.perf_counter() - t0
    blocks = fac.blocks()
    if budget_s <= 0:
        t0 = time.perf_counter()
        for b in blocks:
            fac.fill_block(b)
        return {"workload": name, "full": True, "seconds": plan_s + time.perf_counter() - t0,
                "blocks": len(blocks)}
    # strata of equal modelled cost (blocks sorted by cost); a few blocks
    # drawn at random from each, timed, and the stratum's total estimated as
    # its block count times their mean time
    cost = np.array([22.0 * b.m ** 3 + 16.0 * b.m ** 2 * b.n + 300.0 * (b.m * b.m + b.m * b.n)
                     if b.kind in ("first", "middle") else 300.0 * b.m * b.n for b in blocks])
    order = np.argsort(cost)
    cum = np.cumsum(cost[order]) / cost.sum()
    G = 10
    edges = np.searchsorted(cum, np.arange(1, G) / G)
    strata = [s_ for s_ in np.split(order, edges) if len(s_)]
    rng = np.random.default_rng(0)
    times = []
    for st_ in strata:
        # at least two blocks per stratum, more while its share of the budget lasts
        pk = rng.permutation(st_)
        ts = []
        t0s = time.perf_counter()
        for i in pk:
            if len(ts) >= 2 and time.perf_counter() - t0s > budget_s / len(strata):
                break
            b = blocks[int(i)]
            t0 = time.perf_counter()
            fac.fill_block(b)
            ts.append(time.perf_counter() - t0)
            b.data = None
        times.append(ts)
    total, var, n = plan_s, 0.0, 0
    for st_, ts in zip(strata, times):
        n += len(ts)
        total += len(st_) * float(np.mean(ts))
        if len(ts) > 1:
            var += (len(st_) ** 2) * float(np.var(ts, ddof=1)) / len(ts)
    per_stratum = min(len(t_) for t_ in times)
    return {"workload": name, "full": False, "estimated_seconds": total,
            "standard_error_s": var ** 0.5, "sampled_blocks": n, "blocks": len(blocks),
            "sample": "%d strata of equal modelled cost (22 p^3 + 16 p^2 n + 300 kernel "
                      "evaluations per block), random blocks timed in each (at least %d, more while "
                      "its tenth of the budget lasts); estimate = "
                      "sum of stratum size x mean time" % (len(strata), per_stratum)}


def cpu_factorization(jobs):
    """The oracle's factorization timed on the host cores in child processes,
    with one thread and with all of them (OPENBLAS/OMP thread counts set in
    the child's environment before numpy loads)."""
    out = {}
    ncpu = os.cpu_count() or 1
    for name, budget in jobs:
        for threads in (1, ncpu):
            env = dict(os.environ, OPENBLAS_NUM_THREADS=str(threads), OMP_NUM_THREADS=str(threads))
            try:
                r = subprocess.run([sys.executable, os.path.abspath(__file__), "--cpu-fac-worker",
                                    name, "--cpu-fac-budget", str(budget)],
                                   env=env, capture_output=True, text=True, timeout=600)
                res = json.loads(r.stdout.strip().splitlines()[-1])
            except Exception as exc:
                res = {"error": str(exc)[:200]}
            res["threads"] = threads
            out["%s_%dthread" % (name, threads)] = res
    return out


def run_reference(args):
    """--impl reference: the reference's apply (oracle C port of
    mat_block_dense/mat_product/mat_block_diag/mat_block_coo Mul) on host
    cores over the same block structure, built by the oracle planner, with
    stand-in block values.  Each step applies a bounded number of the
    workload's RHS."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import bf_oracle as O
    cfg = CONFIGS[args.config]
    R = args.rhs or cfg["R"]
    src, tgt = workload_inputs(cfg, "reference")
    t0 = time.perf_counter()
    fac = O.Factorization(O.Helm2(cfg["k"]), src, tgt, leaf_size=cfg["leaf"], eps=cfg["tol"],
                          fill=False)
    plan_s = time.perf_counter() - t0
    text = fac.plan_text()
    port, entries = standin_port(text)
    rng = O.RefRng(1)
    Xs = rng.complex_randn(cfg["n"] * 1).reshape(cfg["n"], 1)
    Xs = np.ascontiguousarray(np.repeat(Xs, R, axis=1))
    nthreads = os.cpu_count() or 1
    port(Xs[:, :1], nthreads)
    t0 = time.perf_counter()
    port(Xs[:, :1], nthreads)
    t1 = time.perf_counter() - t0
    # RHS per step: what fits about 5 s (the whole run stays within minutes)
    Rs = int(max(1, min(R, 5.0 / max(t1, 1e-6))))
    times = []
    for _ in range(max(1, args.warmup)):
        port(Xs[:, :Rs], nthreads)
    for _ in range(args.steps):
        t0 = time.perf_counter()
        port(Xs[:, :Rs], nthreads)
        times.append(time.perf_counter() - t0)
    ms = float(np.mean(times)) * 1e3
    value = Rs / (ms / 1e3)
    sample = ("all %d blocks of the factorization's structure (oracle planner; %d entries, "
              "stand-in values), %d of %d RHS per step" % (len(fac.blocks()), entries, Rs, R))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "RHS/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "complex128", "data": "synthetic",
            "config": config_json(args.config, cfg, R),
            "cpu_baseline": {"value": value, "unit": "RHS/s", "cores": nthreads,
                             "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "RHS/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "plan_s": plan_s, "world_size": world}
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# the single-problem workloads
# ---------------------------------------------------------------------------
DTYPES = {"fp64": "complex128", "df64": "double-float (complex128 vectors)",
          "fp32": "complex64", "bf16x3": "bf16x3 split (complex64 vectors)",
          "bf16x2": "bf16x2 split (complex64 vectors)"}
ENTRY_BYTES = {"fp64": 16, "df64": 16, "fp32": 8, "bf16x3": 12, "bf16x2": 8}


def measured_peaks():
    """HBM GB/s and dense bf16 TFLOP/s (burst) measured on the GB300s,
    else the fallback figures."""
    try:
        pk = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(pk["hbm_gbs"]), float(pk["bf16_tflops"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, 1900.0, "fallback"


def hbm_peak():
    hbm, _, src = measured_peaks()
    return hbm, src


# tensor-core products per stored entry and right-hand side: planes of A
# times planes of x kept (bf16x3: hh hm hl mh mm lh; bf16x2: hh hl lh), each
# 8 real flops per complex multiply-add
TC_PRODUCTS = {"bf16x3": 6, "bf16x2": 3}


def launch_roofline(fac, X, Y, R, prec):
    """Per-launch CUDA-event times of one apply (mean of 3) and the
    algorithmic bytes of each launch (entries x bytes per entry + R x vector
    bytes x (rows in + rows out)); the dominant launch against HBM and, for
    the tensor-core precisions, against the bf16 tensor peak (algorithmic
    flops, 8 per complex multiply-add, and the executed plane products).  The
    roof the dominant launch is closer to is the reported bound."""
    per = np.mean(np.array([fac.apply_timed(X.data_ptr(), R, R, Y.data_ptr(), R, prec)
                            for _ in range(3)], dtype=np.float64), axis=0)
    info = fac.launch_info(precision=prec, rhs=R)
    sA = ENTRY_BYTES[prec]
    sv = 16 if prec in ("fp64", "df64") else 8
    alg = [float(e * sA + R * sv * (ri + ro)) for e, ri, ro in info]
    dom = int(np.argmax(per))
    # launches before the first stage (an input gather or tile-major copy:
    # no stored entries)
    lead = 1 if len(info) > 1 and info[0, 0] == 0 else 0
    hbm, bf16, src = measured_peaks()
    t = per[dom] / 1e3
    ach = float(alg[dom] / t / 1e9)
    alg_tf = float(8.0 * info[dom, 0] * R / t / 1e12)
    out = {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
           "peak_source": src, "kernel": "apply launch %d of %d" % (dom, len(per)),
           "stage": dom - lead if lead <= dom < len(per) - 1 else None,
           "launch_ms": float(per[dom]), "alg_bytes": alg[dom],
           "launch_share": [float(v) for v in per / per.sum()],
           "alg_bytes_per_launch": alg, "launch_ms_all": [float(v) for v in per],
           "flops_per_s": alg_tf * 1e12,
           "whole_apply_gbs": float(sum(alg) / (per.sum() / 1e3) / 1e9),
           "hbm": {"achieved_gbs": ach, "peak_gbs": hbm, "frac": ach / hbm}}
    if prec in TC_PRODUCTS:
        exe = alg_tf * TC_PRODUCTS[prec]
        out["tensor"] = {"achieved_alg_tflops": alg_tf, "executed_tflops_min": exe,
                         "peak_tflops": bf16, "frac_alg": alg_tf / bf16, "frac_executed": exe / bf16,
                         "executed": "%d plane products per entry and RHS (tile padding not "
                                     "counted)" % TC_PRODUCTS[prec]}
        if exe / bf16 > ach / hbm:
            out.update({"bound": "tensor", "achieved": alg_tf, "peak": bf16, "unit": "TFLOP/s",
                        "frac": alg_tf / bf16})
    return out


def timed(fac, X, Y, R, prec, steps, warmup, stream, dist):
    """Warm-up applies, one apply captured in a CUDA graph, warm-up replays,
    then `steps` timed replays with a CUDA event between replays (on the
    stream the library launches on).  Returns (total ms, median ms, captured)."""
    import torch
    for _ in range(warmup):
        fac.apply_device(X.data_ptr(), R, R, Y.data_ptr(), R, prec)
    stream.synchronize()
    graph = None
    try:
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=stream):
            fac.apply_device(X.data_ptr(), R, R, Y.data_ptr(), R, prec)
    except Exception:                  # an uncapturable apply is timed directly
        graph = None
        torch.cuda.synchronize()

    def step():
        if graph is not None:
            graph.replay()
        else:
            fac.apply_device(X.data_ptr(), R, R, Y.data_ptr(), R, prec)

    with torch.cuda.stream(stream):
        for _ in range(warmup):
            step()
    stream.synchronize()
    barrier(dist)
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    with torch.cuda.stream(stream):
        ev[0].record(stream)
        for i in range(steps):
            step()
            ev[i + 1].record(stream)
    ev[-1].synchronize()
    torch.cuda.synchronize()
    barrier(dist)
    per = [ev[i].elapsed_time(ev[i + 1]) for i in range(steps)]
    return ev[0].elapsed_time(ev[-1]), float(np.median(per)), graph is not None


def make_fac(B, ctx, cfg, src, tgt):
    t0 = time.perf_counter()
    fac = B.FacHelm2.make_multilevel(
        B.Helm2(cfg["k"]), B.Quadtree(src, leaf_size=cfg["leaf"]),
        B.Quadtree(tgt, leaf_size=cfg["leaf"]), rank_eps=cfg["tol"], pinv_tol=cfg["tol"],
        context=ctx)
    return fac, time.perf_counter() - t0


def fac_summary(fac, wall_s):
    st = fac.stats()
    return {"wall_s": wall_s, "device_ms": st["factorMs"], "blocks": st["numBlocks"],
            "bytes_fp64": fac.num_bytes(), "max_rank": st["maxRank"],
            "jacobi_not_converged": st["jacobiNotConverged"],
            "sketched_blocks": st["numSketched"], "sketch_ms": st["sketchMs"],
            "sketch_mean_width": st["sketchMeanWidth"], "sketch_max_width": st["sketchMaxWidth"],
            "sketch_retries": st["sketchRetries"], "reexp_svds": st["reexpSvds"],
            "sketch_svds": st["sketchGroups"],
            "sketch_phase_ms": dict(zip(("fill", "z_omega", "qr_y", "zh_q", "qr_g", "jacobi",
                                         "weights", "output"), st["sketchPhaseMs"])),
            "fill_ms": st["fillMs"],
            "reexp_shared_ms": st["reexpSmemMs"], "reexp_global_ms": st["reexpGlobalMs"],
            "work": factorization_work(fac.block_table(), st)}


def rel_rows(Y, rows, Re, yd):
    ye = Y[rows][:, :Re].cpu().numpy().astype(np.complex128)
    return float(np.linalg.norm(ye - yd) / np.linalg.norm(yd))


FP64_MEASURED = {"tflops": None}


def small_rhs_block(B, fac, ctx, stream, n, R, precs, steps, yd_rows, Xh, dist):
    """Applies to R (1 or few) right-hand sides: RHS/s, error against the
    oracle rows, and the dominant launch's HBM roofline per precision."""
    import torch
    rows, yd = yd_rows
    out = {}
    with torch.cuda.stream(stream):
        X64 = torch.from_numpy(np.ascontiguousarray(Xh[:, :R])).to("cuda")
        X32 = X64.to(torch.complex64)
        Y64 = torch.empty((n, R), dtype=torch.complex128, device="cuda")
        Y32 = torch.empty((n, R), dtype=torch.complex64, device="cuda")
    stream.synchronize()
    for p in precs:
        X, Y = (X64, Y64) if p in ("fp64", "df64") else (X32, Y32)
        fac.apply_device(X.data_ptr(), R, R, Y.data_ptr(), R, p)
        stream.synchronize()
        err = rel_rows(Y, rows, R, yd[:, :R]) if yd is not None else None
        tot, med, _ = timed(fac, X, Y, R, p, steps, 3, stream, dist)
        roof = launch_roofline(fac, X, Y, R, p)
        tf = float(fac.stats()["flopsPerRhs"] * R / (tot / steps / 1e3) / 1e12)
        out[p] = {"rhs_per_s": R * steps / (tot / 1e3), "ms_per_apply": tot / steps,
                  "rel_err": err, "dominant_launch_gbs": roof["hbm"]["achieved_gbs"],
                  "dominant_launch_frac_of_measured_hbm": roof["hbm"]["frac"],
                  "whole_apply_gbs": roof["whole_apply_gbs"],
                  "whole_apply_tflops": tf}
        if p == "fp64" and FP64_MEASURED["tflops"]:
            out[p]["whole_apply_frac_of_measured_fp64"] = tf / FP64_MEASURED["tflops"]
    return out


def secondary_c2(B, ctx, stream, args, dist):
    """The 65,536-point ellipse workload (k = 512, tolerance 1e-10) in the
    same run: factorization time, 1- and 16-RHS applies with errors against
    oracle rows and HBM rates."""
    cfg = CONFIGS["c2"]
    n = cfg["n"]
    src, tgt = workload_inputs(cfg, "bfg")
    fac, wall = make_fac(B, ctx, cfg, src, tgt)
    sp, tp = fac.perms()
    Xh = B.Rng(99).complex_randn(n * 16).reshape(n, 16)
    rows = np.unique(np.linspace(0, n - 1, min(args.dense_rows, n)).astype(np.int64))
    orows = OracleRows(cfg["k"], src[sp], tgt[tp], rows, Xh)
    orows.start()
    yd = orows.get()
    res = {"workload": "helmholtz2d_butterfly_apply_c2", "n": n, "k": cfg["k"],
           "tolerance": cfg["tol"], "factorization": fac_summary(fac, wall),
           "err_rows": int(len(rows)), "oracle_rows_s": orows.seconds}
    if yd is None:
        res["error"] = orows.error
        yd_rows = (rows, None)
    else:
        yd_rows = (rows, yd)
    res["rhs1"] = small_rhs_block(B, fac, ctx, stream, n, 1, ("fp64", "df64", "fp32", "bf16x3"),
                                  20, yd_rows, Xh, dist)
    res["rhs16"] = small_rhs_block(B, fac, ctx, stream, n, 16,
                                   ("fp64", "df64", "fp32", "bf16x3", "bf16x2"), 10, yd_rows, Xh,
                                   dist)
    fac.close()
    return res


def run_profile(args):
    """--profile: the workload's factorization, then W + K applies of one
    precision on device-resident operands, untimed, for an ncu capture of
    the apply kernels (skip the factorization's and the warm-up applies'
    launches with ncu -s)."""
    import torch

    import butterfly_gb300 as B
    cfg = CONFIGS[args.config]
    R = args.rhs or cfg["R"]
    n = cfg["n"]
    ctx = B.Context(0)
    if args.profile in ("fp64", "df64"):
        print(json.dumps({"fp64_measured_tflops": B.measure_fp64_rate(ctx)}), flush=True)
    src, tgt = workload_inputs(cfg, "bfg")
    fac, wall = make_fac(B, ctx, cfg, src, tgt)
    dt = torch.complex128 if args.profile in ("fp64", "df64") else torch.complex64
    X = torch.from_numpy(B.Rng(5).complex_randn(n * R).reshape(n, R)).to("cuda").to(dt)
    Y = torch.empty_like(X)
    torch.cuda.synchronize()
    for _ in range(args.warmup + args.steps):
        fac.apply_device(X.data_ptr(), R, R, Y.data_ptr(), R, args.profile)
    torch.cuda.synchronize()
    per = fac.apply_timed(X.data_ptr(), R, R, Y.data_ptr(), R, args.profile)
    info = fac.launch_info(precision=args.profile, rhs=R)
    print(json.dumps({"workload": args.config, "rhs": R, "precision": args.profile,
                      "factorization_s": wall, "launches_per_apply": len(info),
                      "entries_per_launch": [int(v) for v in info[:, 0]],
                      "rows_in_out_per_launch": [[int(a), int(b)] for a, b in info[:, 1:]],
                      "launch_ms": [float(v) for v in per]}))


def main():
    args = parse()
    if args.profile:
        run_profile(args)
        return
    if args.cpu_fac_worker:
        print(json.dumps(cpu_factorization_worker(args.cpu_fac_worker, args.cpu_fac_budget)))
        return
    if CONFIGS[args.config].get("batched"):
        if args.impl == "reference":
            if int(os.environ.get("RANK", "0")) == 0:
                print(json.dumps({"impl": "reference", "unavailable":
                                  "the batched workload has no CPU reference timing here "
                                  "(256 CPU factorizations take hours)"}))
            return
        run_batched(args, CONFIGS[args.config])
        return
    if args.impl == "reference":
        run_reference(args)
        return
    import torch

    import butterfly_gb300 as B

    world, rank, local, dist = dist_setup()
    torch.cuda.set_device(local)
    cfg = CONFIGS[args.config]
    R = args.rhs or cfg["R"]
    n = cfg["n"]
    ctx = B.Context(local)
    # the FP64 roof of the FP64 apply and the factorization, measured here
    FP64_MEASURED["tflops"] = B.measure_fp64_rate(ctx)
    src, tgt = workload_inputs(cfg, "bfg")
    fac, fac_wall_s = make_fac(B, ctx, cfg, src, tgt)
    sp, tp = fac.perms()

    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    rng = B.Rng(1234 + rank)
    Xh = rng.complex_randn(n * R).reshape(n, R)           # tree order, as A X takes it
    # accuracy: dense FP64 rows from the oracle on the host cores, computed
    # while the GPU is timed; the library's own GPU evaluator cross-checks it
    Re = min(R, args.err_rhs) if args.err_rhs > 0 else R
    rows = np.unique(np.linspace(0, n - 1, min(args.dense_rows, n)).astype(np.int64))
    orows = None
    if rank == 0:
        orows = OracleRows(cfg["k"], src[sp], tgt[tp], rows, np.ascontiguousarray(Xh[:, :Re]))
        orows.start()
    with torch.cuda.stream(stream):
        X64 = torch.from_numpy(Xh).to("cuda")
        X32 = X64.to(torch.complex64)
        Y64 = torch.empty((n, R), dtype=torch.complex128, device="cuda")
        Y32 = torch.empty((n, R), dtype=torch.complex64, device="cuda")
        Y16 = torch.empty((n, R), dtype=torch.complex64, device="cuda")
        Ydf = torch.empty_like(Y64)
    stream.synchronize()
    # the tensor-core schedules: the RHS tile width and per stage the fastest
    # of several CTA dealings (bfgFacAutotune), before anything is timed
    tuned = {}
    for p in ("bf16x3", "bf16x2"):
        t = fac.autotune(p, R)
        tuned[p] = {"default_ms": [float(v) for v in t[:, 0]], "tuned_ms": [float(v) for v in t[:, 1]],
                    "rhs_tile": fac.rhs_tile(p, R)}
    precs = {"fp64": (X64, Y64), "df64": (X64, Ydf), "fp32": (X32, Y32), "bf16x3": (X32, Y16),
             "bf16x2": (X32, Y16)}
    outs = {}
    apply_ms = {}
    for p, (X, Y) in precs.items():
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fac.apply_device(X.data_ptr(), R, R, Y.data_ptr(), R, p)
        stream.synchronize()
        apply_ms[p] = (time.perf_counter() - t0) * 1e3
        outs[p] = Y[rows][:, :Re].cpu().numpy().astype(np.complex128)
    # GPU evaluator rows (cross-check of the oracle rows)
    Rg = min(Re, 16)
    with torch.cuda.stream(stream):
        yg = fac.dense_rows(rows, X64[:, :Rg].contiguous(), Rg)
    stream.synchronize()
    yg = yg.cpu().numpy()

    # K timed steps for the precisions whose apply takes under a second, 3
    # for the slower FP64 forms (the ratio's denominator), W >= 3 warm-ups
    clocks = ClockSampler(local)
    clocks.start()
    steps_p = {p: (args.steps if apply_ms[p] < 1000 else min(args.steps, 3)) for p in precs}
    warm_p = {p: (max(3, args.warmup) if apply_ms[p] < 1000 else 1) for p in precs}
    tm = {p: timed(fac, precs[p][0], precs[p][1], R, p, steps_p[p], warm_p[p], stream, dist)
          for p in precs}
    clk = clocks.stop()
    total_ms = {p: max_over_ranks(v[0], dist) for p, v in tm.items()}
    median_ms = {p: v[1] for p, v in tm.items()}
    captured = all(v[2] for v in tm.values())
    rhs_s = {p: world * R * steps_p[p] / (total_ms[p] / 1e3) for p in precs}

    yd = orows.get() if orows is not None else None
    err_src = "oracle"
    if yd is None:                     # fall back to the GPU evaluator, and say so
        yd, err_src = yg, "gpu evaluator (oracle rows failed: %s)" % (orows.error if orows else "")
        Re = Rg
    errs = {p: float(np.linalg.norm(outs[p][:, :Re] - yd[:, :Re]) / np.linalg.norm(yd[:, :Re]))
            for p in precs}
    gpu_rows_vs_oracle = (float(np.linalg.norm(yg - yd[:, :Rg]) / np.linalg.norm(yd[:, :Rg]))
                          if err_src == "oracle" else None)
    ok = [p for p in precs if errs[p] <= ERR_BOUND]
    head = max(ok, key=lambda p: rhs_s[p]) if ok else "fp64"

    X, Y = precs[head]
    roof = launch_roofline(fac, X, Y, R, head)
    ratios = NCU_DRAM_PER_ALG.get((args.config, head, R))
    roof["traffic"] = None
    if ratios is not None:
        st = roof["stage"]
        if st is not None and st < len(ratios):
            roof["traffic"] = float(ratios[st] * roof["alg_bytes"])
            roof["traffic_source"] = NCU_TRAFFIC_SOURCE[(args.config, R)]

    # end to end through the C ABI with pinned host complex128 operands, two
    # input/output pairs used in turn: the pipelined call
    # (bfgFacApplyHostAsync: one step's upload and download overlap another
    # step's compute) with one wait at the end, and the synchronous call
    # (bfgFacApplyHost) timed beside it
    e2e_steps = steps_p[head]
    (Xp, Yp), local_cpus = pinned_local(lambda: (
        [torch.from_numpy(Xh).pin_memory() for _ in range(2)],
        [torch.zeros((n, R), dtype=torch.complex128).pin_memory() for _ in range(2)]))
    lib = B.lib()
    P = B.PRECISIONS[head]

    def host_steps(k, pipelined):
        for i in range(k):
            x, y = B._VP(Xp[i & 1].data_ptr()), B._VP(Yp[i & 1].data_ptr())
            if pipelined:
                ctx.check(lib.bfgFacApplyHostAsync(fac.handle, P, x, R, R, y, R, 0))
            else:
                ctx.check(lib.bfgFacApplyHost(fac.handle, P, x, R, R, y, R, 0))
        if pipelined:
            ctx.check(lib.bfgFacApplyHostWait(fac.handle))

    # the raw host<->device copy times of one step's operands, for reading
    # the end-to-end figure against
    dcopy = torch.empty((n, R), dtype=torch.complex128, device="cuda")
    copy_ms = {}
    for name, fn in (("h2d", lambda: dcopy.copy_(Xp[0], non_blocking=True)),
                     ("h2d_second_buffer", lambda: dcopy.copy_(Xp[1], non_blocking=True)),
                     ("d2h", lambda: Yp[0].copy_(dcopy, non_blocking=True)),
                     ("d2h_second_buffer", lambda: Yp[1].copy_(dcopy, non_blocking=True))):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        copy_ms[name] = (time.perf_counter() - t0) / 3 * 1e3
    del dcopy
    e2e_t = {}
    for pipelined in (True, False):
        host_steps(2, pipelined)
        barrier(dist)
        t0 = time.perf_counter()
        host_steps(e2e_steps, pipelined)
        e2e_t[pipelined] = max_over_ranks(time.perf_counter() - t0, dist)
    e2e = {"value": world * R * e2e_steps / e2e_t[True], "unit": "RHS/s",
           "h2d_bytes_per_step": n * R * 16, "d2h_bytes_per_step": n * R * 16,
           "precision": head, "call": "bfgFacApplyHostAsync (pipelined), one wait",
           "steps": e2e_steps,
           "synchronous_call_value": world * R * e2e_steps / e2e_t[False],
           "copy_ms": copy_ms,
           "pinned_on_gpu_node_cpus": len(local_cpus) if local_cpus else None}
    del Xp, Yp

    # one right-hand side: the HBM-bound single-vector apply
    rhs1 = small_rhs_block(B, fac, ctx, stream, n, 1, ("fp64", "df64", "fp32", "bf16x3"), 10,
                           (rows, yd), Xh, dist) if rank == 0 else None
    fac_info = fac_summary(fac, fac_wall_s)
    plan_text = fac.describe()
    launches = len(fac.launch_info(precision=head, rhs=R)) * steps_p[head]
    fac.close()
    del precs, X64, X32, Y64, Y32, Y16, Ydf, X, Y
    torch.cuda.empty_cache()

    if rank != 0:
        return
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        nthreads = os.cpu_count() or 1
        v, Rs, t = cpu_port_time(plan_text, Xh, nthreads)
        cpu = {"value": v, "unit": "RHS/s", "cores": nthreads, "kind": "port",
               "sample": "the reference's apply algorithm (oracle C port) over this "
                         "factorization's structure with stand-in values, %d of %d RHS, "
                         "median of 3" % (Rs, R)}
        # the same on one core (the reference's own apply is single-threaded
        # apart from its BLAS calls)
        v1, Rs1, _ = cpu_port_time(plan_text, Xh, 1, budget_s=12.0)
        cpu["one_thread"] = {"value": v1, "unit": "RHS/s", "cores": 1,
                             "sample": "%d of %d RHS, median of 3" % (Rs1, R)}
    c2 = None
    if world == 1 and not args.no_c2 and args.config != "c2":
        try:
            c2 = secondary_c2(B, ctx, stream, args, dist)
        except Exception as exc:
            c2 = {"error": str(exc)[:200]}
    c3 = None
    if world == 1 and not args.no_c3:
        try:
            c3 = batched_line(args, CONFIGS["c3"], B, ctx, world, rank, local, dist)
            c3 = {k: v for k, v in c3.items() if k not in ("metric", "n_gpus", "steps", "warmup",
                                                           "higher_is_better", "scaling",
                                                           "vs_baseline", "data")}
        except Exception as exc:
            c3 = {"error": str(exc)[:200]}
    cpu_fac = None
    if world == 1 and not args.no_cpu_factorization:
        cpu_fac = cpu_factorization([("c1", 0), ("c2", 10.0)])
        try:
            f1, w1 = make_fac(B, ctx, CONFIGS["c1"], *workload_inputs(CONFIGS["c1"], "bfg"))
            cpu_fac["gpu_c1"] = {"wall_s": w1, "device_ms": f1.stats()["factorMs"]}
            f1.close()
        except Exception as exc:
            cpu_fac["gpu_c1"] = {"error": str(exc)[:200]}
    gm = None
    if world == 1 and not args.no_gmres:
        try:
            gm = gmres_scattering(B, ctx)
        except Exception as exc:       # reported, the apply line still stands
            gm = {"error": str(exc)[:200]}
        if not args.no_learned and "error" not in gm:
            try:
                gm["learned"] = learned_scattering(B, ctx)
            except Exception as exc:
                gm["learned"] = {"error": str(exc)[:200]}
    line = {"metric": METRIC, "value": rhs_s[head], "unit": "RHS/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_ms[head] / steps_p[head], "median_ms_per_step": median_ms[head],
            "graph_captured": captured, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": DTYPES[head],
            "data": "synthetic", "config": config_json(args.config, cfg, R),
            "precision": head, "rel_err": errs[head], "rel_err_all": errs,
            "rhs_per_s_all": rhs_s, "steps_per_precision": steps_p, "err_bound": ERR_BOUND,
            "err_rows": int(len(rows)), "err_rhs": Re, "err_reference": err_src,
            "oracle_rows_s": orows.seconds if orows else None,
            "gpu_rows_vs_oracle": gpu_rows_vs_oracle,
            "fp64_speedup": rhs_s[head] / rhs_s["fp64"],
            "factorization": fac_info, "rhs1": rhs1,
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
            "gpu_launches": launches, "gmres": gm, "autotune": tuned,
            "cpu_factorization": cpu_fac, "c2": c2, "c3": c3,
            "fp64_measured_tflops": FP64_MEASURED["tflops"]}
    print(json.dumps(line))


if __name__ == "__main__":
    main()
