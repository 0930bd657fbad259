"""Benchmark of the PA H1 path on one GB300 (or N replicas).

Workload (default): FP64 PA diffusion operator apply, L-vector to L-vector
(restriction gather fused into the sum-factorised apply, deterministic CSR
scatter), on the jittered Cartesian hex mesh of the unit cube with n = 77
elements per side (interior vertices jittered by U(-0.1h, 0.1h), seed 1),
H1 order p = 4, Gauss-Legendre rule with p + 2 = 6 points per dimension,
29,503,629 DOFs, x ~ U[-1, 1] (seed 2). One step = one operator apply.
Inputs (qdata 4.7 GB) are larger than L2, so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gbpa|reference]

Prints one JSON line. --impl reference times the CPU oracle (the plain-C
restatement of the reference's PA path) on the host cores instead.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "GDOF/s PA diffusion apply; PCG time-to-1e-10 mixed vs FP64, one GB300"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gbpa", choices=["gbpa", "reference"])
    ap.add_argument("--n", type=int, default=77)
    ap.add_argument("--p", type=int, default=4)
    ap.add_argument("--kind", default="diffusion", choices=["diffusion", "mass"])
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--precision", default="f64", choices=["f64", "f32", "x2"],
                    help="arithmetic of the timed operator (x2: FP64 data, double-float on FP32 pipes)")
    ap.add_argument("--layout", default="default", choices=["default", "cuda_core", "tensor_core"],
                    help="FP32 diffusion: the apply layout of the timed operator (default: the tuned one)")
    ap.add_argument("--cpu-sample-n", type=int, default=None,
                    help="mesh of the CPU baseline (default: the GPU workload's n)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0,
                    help="CPU baseline: applies timed for about this long")
    ap.add_argument("--no-pcg", action="store_true", help="skip the precision-form PCG comparison")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the batching- and combined-form blocks of the default run")
    ap.add_argument("--pcg-n", type=int, default=77,
                    help="mesh size of the precision-form PCG comparison (77: ~29.5 M DOFs at p=4)")
    ap.add_argument("--pcg-only", action="store_true", help="run only the precision-form PCG comparison")
    ap.add_argument("--pcg-max-it", type=int, default=20000)
    ap.add_argument("--batched", action="store_true", help="run only the batching-form comparison")
    ap.add_argument("--nprob", type=int, default=256)
    ap.add_argument("--combined", action="store_true", help="run only the combined-form comparison")
    ap.add_argument("--combined-n", type=int, default=24, help="54: ~19.9 M DOFs at p=5")
    ap.add_argument("--no-reference", action="store_true", help="combined form: skip the FP64 reference solve")
    ap.add_argument("--combined-apply-only", action="store_true",
                    help="combined form: only the block apply against single applies (no solves)")
    ap.add_argument("--mg", action="store_true", help="run only the p-multigrid-preconditioned solve")
    ap.add_argument("--sweep", action="store_true", help="run only the p = 1..8 apply sweep")
    ap.add_argument("--sweep-dofs", type=float, default=8e6)
    ap.add_argument("--mg-n", type=int, default=77)
    ap.add_argument("--mg-jacobi", action="store_true", help="p-multigrid form: also time FP64 Jacobi-PCG")
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(ms, world):
    """Slowest rank's time (the job's time): all_reduce MAX over the process
    group (NCCL tensors on the GPU, gloo on the CPU)."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([ms], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(ndofs_per_rank, steps, world, ms):
    """Whole-job GDOF/s: every rank applies its own replica (weak scaling)."""
    return world * ndofs_per_rank * steps / (ms * 1e-3) / 1e9


def algorithmic_bytes(ne, ndofs, D, Q, w, kind, element_only):
    """Algorithmic HBM bytes of one apply: qdata once, index map once, x read
    once; L->L also writes y once; the element kernel alone writes the
    E-vector instead of y."""
    S = 6 if kind == "diffusion" else 1
    qd = ne * S * Q ** 3 * w
    maps = ne * D ** 3 * 4
    if element_only:
        return qd + maps + ndofs * w + ne * D ** 3 * w
    return qd + maps + 2 * ndofs * w


def element_flops(D, Q, kind):
    """Algorithmic floating-point operations (an FMA = 2) of one element's
    sum-factorised apply, in the kernel's contraction order. Diffusion:
    x, y, z forward (2 D^3 Q + 3 D^2 Q^2 + 3 D Q^3 FMA), the symmetric 3x3
    qdata product (9 Q^3), the same contractions backward. Mass: one field,
    D^3 Q + D^2 Q^2 + D Q^3 each way, and Q^3 products."""
    if kind == "diffusion":
        fwd = 2 * D ** 3 * Q + 3 * D ** 2 * Q ** 2 + 3 * D * Q ** 3
        return 2 * (2 * fwd + 9 * Q ** 3)
    fwd = D ** 3 * Q + D ** 2 * Q ** 2 + D * Q ** 3
    return 2 * (2 * fwd) + Q ** 3


def measured_hbm_live_gbs():
    """HBM copy bandwidth measured now, the same way as the pool's peak file:
    b.copy_(a) over 2^30 bf16 elements (read + write bytes), best of 10."""
    import torch
    a = torch.empty(1 << 30, dtype=torch.bfloat16, device="cuda")
    b = torch.empty_like(a)
    b.copy_(a)
    best = float("inf")
    for _ in range(10):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        b.copy_(a)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    nbytes = 2 * a.numel() * a.element_size()
    del a, b
    return nbytes / (best * 1e-3) / 1e9


def measured_fp64_peak_tflops():
    """The FP64 rate of this GPU, measured now: cuBLAS DGEMM 4096^3 (2 N^3
    operations), best of 3 after one warm-up, CUDA events."""
    import torch
    n = 4096
    a = torch.rand(n, n, dtype=torch.float64, device="cuda")
    b = torch.rand(n, n, dtype=torch.float64, device="cuda")
    c = a @ b
    best = float("inf")
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b, out=c)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b, c
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1])); mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def profiled_traffic(precision, kind, p, ne, layout=0):
    """DRAM bytes per launch of the element kernel from the committed ncu
    summary of the same kernel on a small case (profiles/: the 24^3 case, or
    40^3 for the tensor-core kernel), scaled by the element count (traffic
    grows with elements: qdata, map and E-vector are per element, the
    gathered x is ~1 dof per element)."""
    if kind != "diffusion" or p != 4:
        return None, None
    name = {"f64": "f64", "x2": "f64x2", "f32": "f32"}[precision]
    path = os.path.join(REPO, "profiles", f"diffusion_apply_{name}_p4_n24.md")
    if layout == 2:
        path = os.path.join(REPO, "profiles", "diffusion_tc_f32_p4_n40.md")
    try:
        for line in open(path):
            if line.startswith("dram_bytes_per_element:"):
                return float(line.split(":")[1]) * ne, os.path.relpath(path, REPO)
    except OSError:
        pass
    return None, None


def measured_peak_hbm():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def workload_config(args, world=1):
    """The `config` dict of both arms (GPU and reference): the same workload
    described from the command line alone."""
    n, p = args.n, args.p
    ne, ndofs, Q = n ** 3, (p * n + 1) ** 3, p + 2
    S = 6 if args.kind == "diffusion" else 1
    return {"workload": f"PA {args.kind} operator apply L->L (BilinearForm::Mult, AssemblyLevel::PARTIAL), "
                        f"jittered hex mesh n={n}^3 (interior vertices +-0.1h, seed 1), H1 p={p}, "
                        f"Gauss-Lobatto basis, q={Q} Gauss points per direction, coefficient 1, "
                        f"{ndofs} DOFs, x~U[-1,1] (seed 2); one step = one apply",
            "ne": ne, "ndofs": ndofs, "p": p, "q1d": Q, "kind": args.kind,
            "parallelism": f"replicas x{world}",
            "l2": "inputs larger than L2 (qdata %.2f GB in FP64); no flush" % (ne * S * Q ** 3 * 8 / 1e9)}


# ----------------------------------------------------------------- problem set-up
def build_problem(n, p, kind, seed_jitter=1):
    """Mesh, maps and qdata on the device through the library."""
    import torch
    from mfem_gb300 import fem
    from mfem_gb300.pa import (DiffusionIntegrator, FiniteElementSpace, MassIntegrator, PAOperator)
    mesh = fem.CartesianMesh(n, jitter=0.1, seed=seed_jitter)
    fes = FiniteElementSpace(mesh, p)
    integ = DiffusionIntegrator() if kind == "diffusion" else MassIntegrator()
    integ.AssemblePA(fes)
    kind_id = 0 if kind == "diffusion" else 1
    return fes, integ, kind_id


def cpu_oracle_apply_rate(n, p, kind, steps, warmup=1, single_thread=False, seconds=None, keep_y=None):
    """The oracle's L->L apply (gather, element kernel, CSR scatter) on the
    host cores, set up by the oracle itself from the same synthetic mesh.
    seconds: instead of `steps`, time as many applies as fit in about that
    long (at least 3), from the warm-up apply's duration. keep_y: a list that
    receives the oracle's y = A x (the parity check of the GPU arm)."""
    from mfem_gb300 import fem
    from tests import oracle_lib
    o = oracle_lib.load()
    mesh = fem.CartesianMesh(n, jitter=0.1, seed=1)
    sp = fem.H1Space(mesh, p)
    D, Q = p + 1, p + 2
    t = fem.Tables(p, Q)
    off, ind, gm = o.restriction_build(mesh.ne, D ** 3, sp.ndofs, sp.element_dofs(), None)
    gt = fem.Tables(1, Q)
    J = o.geom_jacobians3d(mesh.ne, 2, Q, gt.B, gt.G, mesh.nodes_evector(1))
    if kind == "diffusion":
        qd = o.diffusion_setup3d(mesh.ne, Q, 1, t.W, J, np.array([1.0]))
    else:
        det = o.geom_det3d(mesh.ne, J, Q ** 3)
        qd = o.mass_setup3d(mesh.ne, Q ** 3, t.W, det, np.array([1.0]))
    del J
    x = 2 * fem.u01_array(2, sp.ndofs) - 1
    kid = 0 if kind == "diffusion" else 1
    tw = time.perf_counter()
    for _ in range(max(warmup, 1)):
        y = o.pa_mult(kid, mesh.ne, sp.ndofs, True, D, Q, gm, off, ind, t.B, t.G, qd, x)
    if keep_y is not None:
        keep_y.append(y)
    tw = (time.perf_counter() - tw) / max(warmup, 1)
    if seconds is not None:
        steps = int(min(max(3, seconds / max(tw, 1e-6)), 1000))
    t0 = time.perf_counter()
    for _ in range(steps):
        o.pa_mult(kid, mesh.ne, sp.ndofs, True, D, Q, gm, off, ind, t.B, t.G, qd, x)
    dt = time.perf_counter() - t0
    threads = o.num_threads()
    if not single_thread:
        return sp.ndofs * steps / dt / 1e9, sp.ndofs, threads, dt
    # two applies on one thread
    o.set_num_threads(1)
    try:
        t1 = time.perf_counter()
        for _ in range(2):
            o.pa_mult(kid, mesh.ne, sp.ndofs, True, D, Q, gm, off, ind, t.B, t.G, qd, x)
        dt1 = time.perf_counter() - t1
    finally:
        o.set_num_threads(threads)
    return sp.ndofs * steps / dt / 1e9, sp.ndofs, threads, dt, sp.ndofs * 2 / dt1 / 1e9, steps


# ------------------------------------------------------------------- reference arm
REF_BUILD = os.path.join(REPO, "baseline", "_ref", "build")


def mfem_cpu_apply(n, p, steps, warmup, backend="omp", threads=None, timeout=1200):
    """The reference MFEM's own PA diffusion apply (BilinearForm::Mult,
    AssemblyLevel::PARTIAL) on the host cores: oracle/ref/bench_driver.cpp
    linked to the unmodified reference sources, built for this host by
    build() into baseline/_ref/build. Returns (result dict, None) or (None,
    reason)."""
    exe = os.path.join(REF_BUILD, "bench_driver")
    if not os.path.exists(exe):
        return None, "reference MFEM not built on this host (baseline/_ref/build/bench_driver absent)"
    env = dict(os.environ)
    env["OMP_NUM_THREADS"] = str(threads or os.cpu_count() or 1)
    try:
        r = subprocess.run([exe, str(n), str(p), str(steps), str(warmup), backend], capture_output=True,
                           text=True, env=env, timeout=timeout)
    except subprocess.TimeoutExpired:
        return None, f"reference bench driver exceeded {timeout} s"
    if r.returncode != 0:
        return None, f"reference bench driver rc={r.returncode}: {r.stderr.strip()[-200:]}"
    return json.loads(r.stdout.strip().splitlines()[-1]), None


def mfem_sample_text(res):
    return (f"{res['steps']} applies (after {res['warmup']} warm-up) of BilinearForm::Mult, "
            f"AssemblyLevel::PARTIAL, Device(\"{res['backend']}\"), {res['threads']} OpenMP threads, "
            f"n={round(res['ne'] ** (1 / 3))} p={res['p']} ({res['ndofs']} DOFs): the unmodified reference MFEM "
            f"built from source on this host (g++ -O3, OpenMP); set-up {res['setup_s']:.1f} s untimed")


def run_reference(args):
    """The reference arm: the reference's own CPU implementation of the path,
    timed on the host cores with every thread, on the GPU arm's workload
    (same config dict). It loads no part of the CUDA library."""
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    steps, warm = args.steps, args.warmup
    cfg = workload_config(args, world)
    res, why = (mfem_cpu_apply(args.n, args.p, steps, warm) if args.kind == "diffusion"
                else (None, "the MFEM bench driver times the diffusion operator only"))
    port = None
    try:
        prate, pnd, pthreads, pdt = cpu_oracle_apply_rate(args.n, args.p, args.kind, 3, warmup=1)
        port = {"value": prate, "unit": "GDOF/s", "cores": pthreads, "kind": "port",
                "sample": f"3 applies of the oracle (plain-C restatement of the reference's PA path), "
                          f"n={args.n} p={args.p} ({pnd} DOFs)"}
    except Exception as e:  # reported, never required
        port = {"value": None, "error": str(e)[:200]}
    if res is not None:
        rate = res["ndofs"] * steps / res["total_s"] / 1e9
        ms = res["total_s"] / steps * 1e3
        base = {"value": rate, "unit": "GDOF/s", "cores": res["threads"], "kind": "reference",
                "sample": mfem_sample_text(res), "median_apply_s": res["median_s"], "sum_y": res["sum_y"]}
    else:
        if port.get("value") is None:
            print(json.dumps({"impl": "reference", "unavailable": f"{why}; port: {port.get('error')}"}))
            return 0
        rate, ms = port["value"], None
        base = dict(port, note=why)
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": "GDOF/s", "n_gpus": args.gpus,
        "steps": steps, "warmup": warm, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg,
        "cpu_baseline": base, "port_baseline": port,
        "e2e": {"value": rate, "unit": "GDOF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# -------------------------------------------------------------------- GPU arm
def run_gpu(args):
    import torch
    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    from mfem_gb300 import _lib
    from mfem_gb300.pa import Device, PAOperator
    dev = Device("cuda", local)
    lib = dev.lib
    stream = torch.cuda.current_stream()
    fes, integ, kid = build_problem(args.n, args.p, args.kind)
    ne, ndofs, D, Q = fes.ne, fes.ndofs, integ.D, integ.Q
    prec = {"f64": 0, "f32": 1, "x2": 2}[args.precision]
    wbytes = 4 if prec == 1 else 8
    if args.layout != "default":
        from mfem_gb300 import autotune
        if prec != 1 or args.kind != "diffusion":
            raise SystemExit("--layout selects between the FP32 diffusion layouts (--precision f32)")
        lay = autotune.GBPA_LAYOUT_TC if args.layout == "tensor_core" else 0
        _lib.check(lib.gbpa_set_apply_layout(0, 1, D, Q, lay, 0), "gbpa_set_apply_layout")
    nbl = ctypes.c_int(0)
    layout_used = lib.gbpa_get_apply_layout(kid, prec, D, Q, ctypes.byref(nbl))
    op = PAOperator(kid, fes, D, Q, integ.B, integ.G, integ.qdata, precision=prec)
    from mfem_gb300 import fem
    x = torch.from_numpy(2 * fem.u01_array(2, ndofs) - 1).cuda()
    if prec == 1:
        x = x.float()
    y = torch.empty_like(x)
    P = lambda t: ctypes.c_void_p(t.data_ptr())

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
            torch.cuda.synchronize()

    # ---- device-resident timing of the L->L apply (value)
    for _ in range(max(args.warmup, 3)):
        op.Mult(x, y)
    barrier()
    launches0 = dev.launches()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            op.Mult(x, y)
        e1.record(stream)
        barrier()
    ms = e0.elapsed_time(e1)
    launches = dev.launches() - launches0
    y_check = y.clone()
    ms = max_over_ranks(ms, world)
    value = job_throughput(ndofs, args.steps, world, ms)

    # ---- dominant kernel alone: gather-fused element apply (E-vector out)
    yE = torch.empty(ne * D ** 3, dtype=x.dtype, device="cuda")
    for _ in range(3):
        _lib.check(lib.gbpa_operator_apply_element(op.handle, P(x), P(yE)), "apply_element")
    torch.cuda.synchronize()
    k0, k1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    nk = max(10, args.steps // 2)
    k0.record(stream)
    for _ in range(nk):
        _lib.check(lib.gbpa_operator_apply_element(op.handle, P(x), P(yE)), "apply_element")
    k1.record(stream)
    torch.cuda.synchronize()
    k_ms = k0.elapsed_time(k1) / nk
    kbytes = algorithmic_bytes(ne, ndofs, D, Q, wbytes, args.kind, element_only=True)
    peak, peak_kind = measured_peak_hbm()
    hbm_live = measured_hbm_live_gbs()
    achieved = kbytes / (k_ms * 1e-3) / 1e9
    traffic, traffic_src = profiled_traffic(args.precision, args.kind, args.p, ne, layout_used)
    fp64_roof = None
    if prec == 0:
        fpe = element_flops(D, Q, args.kind)
        fp64_ach = ne * fpe / (k_ms * 1e-3) / 1e12
        fp64_peak = measured_fp64_peak_tflops()
        fp64_roof = {"achieved": fp64_ach, "peak": fp64_peak, "unit": "TFLOP/s", "frac": fp64_ach / fp64_peak,
                     "flops_per_element": fpe,
                     "peak_source": "cuBLAS DGEMM 4096^3 measured in this run (best of 3)"}

    # ---- end to end through the C ABI with host buffers (pinned): the
    # host-buffer Mult, whose kernels gather x from and scatter y to the
    # pinned buffers over NVLink-C2C; it returns when hy holds the result
    hx = torch.empty(ndofs, dtype=x.dtype).pin_memory()
    hx.copy_(x.cpu())
    hy = torch.empty(ndofs, dtype=x.dtype).pin_memory()
    for _ in range(2):
        op.MultHost(hx, hy)
    barrier()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(args.steps):
        op.MultHost(hx, hy)
    t1.record(stream)
    barrier()
    e2e_ms = max_over_ranks(t0.elapsed_time(t1), world)
    e2e = job_throughput(ndofs, args.steps, world, e2e_ms)
    # the same with explicit staging copies (pinned -> device, Mult, device -> pinned)
    dx = torch.empty_like(x)
    for _ in range(2):
        dx.copy_(hx, non_blocking=True); op.Mult(dx, y); hy.copy_(y, non_blocking=True)
    torch.cuda.synchronize()
    t0.record(stream)
    for _ in range(args.steps):
        dx.copy_(hx, non_blocking=True)
        op.Mult(dx, y)
        hy.copy_(y, non_blocking=True)
    t1.record(stream)
    torch.cuda.synchronize()
    e2e_staged = job_throughput(ndofs, args.steps, world, t0.elapsed_time(t1))

    extras = {}
    if not args.no_extras and rank == 0 and prec == 0:
        extras = run_extras(args, fes, integ, op, x, y)
        if not args.no_pcg:
            extras["pcg"] = run_pcg_form(args.pcg_n, args.p, args.pcg_max_it)
            extras["mg"] = run_mg_form(args.pcg_n, args.p, (1, 2, 4))
        if not args.no_forms:
            # the batching and combined forms at their default sizes
            del op
            torch.cuda.empty_cache()
            extras["batched"] = run_batched_form(args.nprob, persistent=False)
            torch.cuda.empty_cache()
            extras["combined"] = run_combined_form(args.combined_n, 5, 8, True)

    line = {
        "metric": METRIC, "value": value, "unit": "GDOF/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": {0: "f64", 1: "f32", 2: "f64x2"}[prec], "data": "synthetic",
        "config": dict(workload_config(args, world), layout=LAYOUT_NAMES.get(layout_used, str(layout_used))),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "traffic_source": traffic_src,
                     "kernel": (f"{args.kind}_apply (gather fused)" if layout_used != 2 else
                                "diffusion_tc (tensor cores, gather fused)"),
                     "kernel_ms": k_ms, "algorithmic_bytes": kbytes, "peak_source": peak_kind,
                     "peak_live": hbm_live, "frac_live": achieved / hbm_live,
                     "note": ("native FP64 is FP64-pipe bound on GB300 (ncu: FP64 pipe 91.5% active); "
                              "fp64 below is the arithmetic roofline; see f64x2_apply for the double-float form")
                     if prec == 0 else None,
                     "fp64": fp64_roof},
        "e2e": {"value": e2e, "unit": "GDOF/s", "h2d_bytes_per_step": ndofs * wbytes,
                "d2h_bytes_per_step": ndofs * wbytes, "api": "gbpa_operator_mult_host (pinned buffers, "
                "read and written in place over the host link)", "staged_copies_value": e2e_staged},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    parity_ok = True
    if rank == 0:
        # the oracle on the same mesh and x (its own maps, geometry and qdata,
        # built on the host): the parity check at the benchmark's full size,
        # and the port's CPU figure
        sample_n = args.cpu_sample_n or args.n
        port = None
        try:
            ys = []
            rate, sn, threads, dt, rate1, csteps = cpu_oracle_apply_rate(
                sample_n, args.p, args.kind, 3, single_thread=True, seconds=args.cpu_seconds, keep_y=ys)
            port = {"value": rate, "unit": "GDOF/s", "cores": threads, "kind": "port",
                    "sample": f"{csteps} applies of the oracle (plain-C restatement of the reference's PA "
                              f"path) on the n={sample_n} p={args.p} mesh ({sn} DOFs), {dt:.1f} s; "
                              f"1 thread: 2 applies", "value_1_thread": rate1}
            if sample_n == args.n:
                yo = ys[0]
                yg = y_check.cpu().double().numpy()
                rel = float(np.linalg.norm(yg - yo) / np.linalg.norm(yo))
                tol = 1e-5 if prec == 1 else 1e-12
                parity_ok = rel <= tol
                line["parity"] = {"rel_l2_vs_oracle": rel, "tol": tol, "ok": parity_ok, "ndofs": sn,
                                  "oracle": "oracle/gbpa_oracle.c (pinned to reference-generated golden "
                                            "vectors), same mesh and x, oracle-side maps, geometry and qdata"}
        except Exception as e:  # the baseline is reported, never required
            port = {"value": None, "error": str(e)[:200]}
        res, why = (mfem_cpu_apply(sample_n, args.p, 10, 1) if args.kind == "diffusion"
                    else (None, "the MFEM bench driver times the diffusion operator only"))
        if res is not None:
            line["cpu_baseline"] = {"value": res["ndofs"] * res["steps"] / res["total_s"] / 1e9,
                                    "unit": "GDOF/s", "cores": res["threads"], "kind": "reference",
                                    "sample": mfem_sample_text(res)}
            line["port_baseline"] = port
        else:
            line["cpu_baseline"] = dict(port or {}, note=why)
        line.update(extras)
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0 if parity_ok else 1


def _event_ms(fn, steps):
    """ms per call of fn, CUDA events on the current stream, 3 warm-up calls."""
    import torch
    for _ in range(3):
        fn()
    torch.cuda.synchronize()
    s = torch.cuda.current_stream()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(s)
    for _ in range(steps):
        fn()
    b.record(s)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / steps


LAYOUT_NAMES = {0: "slab2d", 1: "3d", 2: "tensor_core"}


def run_extras(args, fes, integ, op, x, y):
    """The same apply in FP32 (the inner operator of the mixed-precision form)
    on the CUDA cores and, where the order has one, on the tensor cores
    (GBPA_LAYOUT_TC: two Kronecker GEMMs per tile of 128 elements, fp16 hi/lo
    limbs, FP32 accumulation), each as the L->L Mult and as the element kernel
    alone; then the double-float apply."""
    import ctypes
    import torch
    from mfem_gb300 import autotune
    from mfem_gb300.pa import Device, PAOperator
    lib = Device.get().lib
    kind = 0 if args.kind == "diffusion" else 1
    D, Q = integ.D, integ.Q
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    out = {}
    op.Mult(x, y)
    torch.cuda.synchronize()
    x32 = x.float()
    yE = torch.empty(fes.ne * D ** 3, dtype=torch.float32, device=x.device)
    nb = ctypes.c_int(0)
    prev = lib.gbpa_get_apply_layout(kind, 1, D, Q, ctypes.byref(nb))
    out["fp32_default_layout"] = LAYOUT_NAMES.get(prev, str(prev))
    cuda_core = (prev, nb.value) if prev != autotune.GBPA_LAYOUT_TC else (0, 0)
    runs = [("fp32_apply", cuda_core)]
    if kind == 0 and (D, Q) in autotune.TC:
        runs.append(("fp32_apply_tensor_core", (autotune.GBPA_LAYOUT_TC, 0)))
    peak = measured_peak_hbm()[0]
    try:
        for name, (layout, nbz) in runs:
            if lib.gbpa_set_apply_layout(kind, 1, D, Q, layout, nbz) != 0:
                continue
            op32 = PAOperator(kind, fes, D, Q, integ.B, integ.G, integ.qdata, precision=1)
            y32 = torch.empty_like(x32)
            ms = _event_ms(lambda: op32.Mult(x32, y32), args.steps)
            mse = _event_ms(lambda: lib.gbpa_operator_apply_element(op32.handle, P(x32), P(yE)), args.steps)
            op32.Mult(x32, y32)
            torch.cuda.synchronize()
            rel = float(torch.linalg.norm(y32.double() - y) / torch.linalg.norm(y))
            out[name] = {"value": fes.ndofs / (ms * 1e-3) / 1e9, "unit": "GDOF/s", "ms_per_apply": ms,
                         "layout": LAYOUT_NAMES.get(layout, str(layout)), "rel_l2_vs_f64": rel,
                         "hbm_frac_alg": algorithmic_bytes(fes.ne, fes.ndofs, D, Q, 4, args.kind, False)
                         / (ms * 1e-3) / 1e9 / peak,
                         "element_kernel_ms": mse,
                         "element_kernel_hbm_frac_alg": algorithmic_bytes(fes.ne, fes.ndofs, D, Q, 4, args.kind,
                                                                          True) / (mse * 1e-3) / 1e9 / peak}
            del op32, y32
    finally:
        lib.gbpa_set_apply_layout(kind, 1, D, Q, prev, nb.value)
    del x32, yE
    # FP64 data, double-float arithmetic on the FP32 pipes
    opx = PAOperator(0 if args.kind == "diffusion" else 1, fes, integ.D, integ.Q, integ.B, integ.G,
                     integ.qdata, precision=2)
    yx = torch.empty_like(y)
    ms = _event_ms(lambda: opx.Mult(x, yx), args.steps)
    op.Mult(x, y)
    torch.cuda.synchronize()
    rel = float(torch.linalg.norm(yx - y) / torch.linalg.norm(y))
    out["f64x2_apply"] = {"value": fes.ndofs / (ms * 1e-3) / 1e9, "unit": "GDOF/s", "ms_per_apply": ms,
                          "rel_l2_vs_native_f64": rel,
                          "hbm_frac_alg": algorithmic_bytes(fes.ne, fes.ndofs, integ.D, integ.Q, 8, args.kind,
                                                            False) / (ms * 1e-3) / 1e9 / measured_peak_hbm()[0]}
    return out


def run_pcg_form(n, p, max_it=2000):
    """Precision form on the jittered mesh with kappa = exp(16 random Fourier
    modes, amplitude 0.5), RHS ~ U[0,1] (seed 4), homogeneous Dirichlet
    boundary: plain FP64 Jacobi-PCG, the same with the double-float operator,
    and FP32-apply PCG inside FP64 defect correction. Every solve stops at a
    relative residual of 1e-10 (preconditioned norm for PCG, true FP64
    residual for the defect correction); the true FP64 residual and the
    error against the FP64 solution are reported for each."""
    import torch
    from mfem_gb300 import _lib, fem
    from mfem_gb300.pa import (DiffusionIntegrator, FiniteElementSpace, OperatorJacobiSmoother,
                               PAOperator, Device)
    dev = Device.get()
    mesh = fem.CartesianMesh(n, jitter=0.1, seed=1)
    fes = FiniteElementSpace(mesh, p)
    integ = DiffusionIntegrator("kappa")
    integ.AssemblePA(fes, modes=fem.kappa_modes(3))
    ess = fes.GetBoundaryTrueDofs()
    A64 = PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata, ess=ess)
    M = OperatorJacobiSmoother(A64, ess)
    nd = fes.ndofs
    b = torch.from_numpy(fem.u01_array(4, nd)).cuda()
    b[torch.from_numpy(ess).long().cuda()] = 0.0
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    out = {"workload": f"Dirichlet Poisson, lognormal kappa, jittered n={n}^3, p={p}, q={p + 2}, "
                       f"{nd} DOFs, RHS~U[0,1]", "rel_tol": 1e-10}
    info = _lib.SolveInfo()
    X64 = torch.zeros_like(b)
    st = dev.lib.gbpa_pcg_solve(A64.handle, P(M.dinv), P(b), P(X64), 1e-10, 0.0, max_it, 0,
                                ctypes.byref(info))
    out["fp64_pcg"] = {"status": st, "seconds": info.seconds, "iterations": info.iterations,
                       "true_rel_residual": info.true_rel_residual}
    Ax2 = PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata, ess=ess, precision=2)
    Xx2 = torch.zeros_like(b)
    st = dev.lib.gbpa_pcg_solve(Ax2.handle, P(M.dinv), P(b), P(Xx2), 1e-10, 0.0, max_it, 0,
                                ctypes.byref(info))
    out["f64x2_pcg"] = {"status": st, "seconds": info.seconds, "iterations": info.iterations,
                        "true_rel_residual": info.true_rel_residual,
                        "rel_l2_vs_fp64": float(torch.linalg.norm(Xx2 - X64) / torch.linalg.norm(X64))}
    del Xx2
    A32 = PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata, ess=ess, precision=1)
    d32 = M.dinv.float()
    # the true residual of the defect correction uses the native FP64 operator:
    # the double-float operator's ~1e-14 error, amplified by the condition
    # number, stalls that residual near 2e-10 on this problem
    for name, outer in (("mixed_f32_in_f64", A64),):
        Xm = torch.zeros_like(b)
        st = dev.lib.gbpa_pcg_solve_mixed(outer.handle, A32.handle, P(d32), P(b), P(Xm), 1e-10, 1e-5,
                                          30, max_it, ctypes.byref(info))
        out[name] = {"status": st, "seconds": info.seconds, "outer": info.outer_iterations,
                     "inner_iterations": info.inner_iterations,
                     "true_rel_residual": info.true_rel_residual,
                     "rel_l2_vs_fp64": float(torch.linalg.norm(Xm - X64) / torch.linalg.norm(X64))}
    # one FP32 PCG with FP64 residual replacement (reliable updates, delta 0.1)
    Xr = torch.zeros_like(b)
    st = dev.lib.gbpa_pcg_solve_mixed_reliable(A64.handle, A32.handle, P(d32), P(b), P(Xr), 1e-10, 0.1,
                                               max_it, ctypes.byref(info))
    out["mixed_reliable"] = {"status": st, "seconds": info.seconds, "replacements": info.outer_iterations,
                             "f32_iterations": info.iterations, "true_rel_residual": info.true_rel_residual,
                             "rel_l2_vs_fp64": float(torch.linalg.norm(Xr - X64) / torch.linalg.norm(X64))}
    # the FP64 reference solution: FP64 Jacobi-PCG to 1e-12; every solution's
    # error against it, and every solution's true residual computed by the
    # oracle on the host (plain-C apply, FP64) from the same qdata and maps
    Xref = torch.zeros_like(b)
    st = dev.lib.gbpa_pcg_solve(A64.handle, P(M.dinv), P(b), P(Xref), 1e-12, 0.0, 2 * max_it, 0,
                                ctypes.byref(info))
    out["fp64_reference_solution"] = {"status": st, "rel_tol": 1e-12, "seconds": info.seconds,
                                      "iterations": info.iterations, "true_rel_residual": info.true_rel_residual}
    sols = {"fp64_pcg": X64, "mixed_f32_in_f64": Xm, "mixed_reliable": Xr}
    for name, X in sols.items():
        out[name]["rel_l2_vs_fp64_reference"] = float(torch.linalg.norm(X - Xref) / torch.linalg.norm(Xref))
    try:
        from tests import oracle_lib
        o = oracle_lib.load()
        R = fes.GetElementRestriction()
        gm, off, ind = R.gather_map.cpu().numpy(), R.offsets.cpu().numpy(), R.indices.cpu().numpy()
        Bh, Gh, qh = integ.B.cpu().numpy(), integ.G.cpu().numpy(), integ.qdata.cpu().numpy()
        bh = b.cpu().numpy()
        ess_l = torch.from_numpy(ess).long()
        for name, X in list(sols.items()) + [("fp64_reference_solution", Xref)]:
            xh = X.cpu().clone()
            xh[ess_l] = 0.0
            r = bh - o.pa_mult(0, fes.ne, nd, True, integ.D, integ.Q, gm, off, ind, Bh, Gh, qh, xh.numpy())
            r[ess] = 0.0
            out[name]["oracle_true_rel_residual"] = float(np.linalg.norm(r) / np.linalg.norm(bh))
        del qh
    except Exception as e:  # reported, never required
        out["oracle_check_error"] = str(e)[:200]
    out["error_target"] = "solution rel. L2 error vs the FP64 reference solution <= 1e-9"
    out["mixed_meets_target"] = bool(out["mixed_reliable"]["rel_l2_vs_fp64_reference"] <= 1e-9 and
                                     out["mixed_f32_in_f64"]["rel_l2_vs_fp64_reference"] <= 1e-9)
    t64 = out["fp64_pcg"]["seconds"]
    out["speedup_mixed_vs_fp64"] = t64 / max(out["mixed_f32_in_f64"]["seconds"], 1e-30)
    out["speedup_mixed_vs_f64x2_pcg"] = out["f64x2_pcg"]["seconds"] / max(out["mixed_f32_in_f64"]["seconds"], 1e-30)
    out["speedup_mixed_reliable_vs_fp64"] = t64 / max(out["mixed_reliable"]["seconds"], 1e-30)
    return out


def run_batched_form(nprob=256, seed=5, rel_tol=1e-10, max_it=5000, persistent=True):
    """Batching form: nprob independent Dirichlet Poisson problems, each a
    jittered Cartesian hex mesh of n^3 elements with n uniform in [4, 16] and
    order p uniform in {2,...,6} (splitmix64 stream, seed 5), lognormal kappa
    and RHS ~ U[0,1] per problem; all solved to 1e-10 together (graph
    schedule: per-order grouped launches, K iterations per CUDA graph), in
    double-float arithmetic (FP64 data, FP64-accurate products on the FP32
    pipes: the batch's headline) and in native FP64, against solving them one
    after another with the single-problem device PCG (CUDA-graph captured
    iterations) in the same two arithmetics. With persistent=True the
    one-launch persistent schedule is timed too.
    dof_iterations = sum over problems of DOFs x iterations: the PCG work."""
    import torch
    from mfem_gb300 import _lib, fem
    from mfem_gb300.pa import (DiffusionIntegrator, Device, FiniteElementSpace,
                               OperatorJacobiSmoother, PAOperator)
    dev = Device.get()
    u = fem.u01_stream(seed, 2 * nprob)
    probs, descs = [], []
    total = 0
    for k in range(nprob):
        n = 4 + int(u[2 * k] * 13)
        p = 2 + int(u[2 * k + 1] * 5)
        mesh = fem.CartesianMesh(n, jitter=0.1, seed=1000 + k)
        fes = FiniteElementSpace(mesh, p)
        integ = DiffusionIntegrator("kappa")
        integ.AssemblePA(fes, modes=fem.kappa_modes(3 + k))
        ess = fes.GetBoundaryTrueDofs()
        A = PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata, ess=ess)
        M = OperatorJacobiSmoother(A, ess)
        b = torch.from_numpy(fem.u01_array(100 + k, fes.ndofs)).cuda()
        b[torch.from_numpy(ess).long().cuda()] = 0.0
        e = torch.from_numpy(ess).cuda()
        x = torch.zeros_like(b)
        R = fes.GetElementRestriction()
        probs.append(dict(A=A, dinv=M.dinv, b=b, x=x, ess=e, ess_h=ess, integ=integ, R=R, n=n, p=p))
        descs.append(_lib.ProblemDesc(fes.ne, fes.ndofs, integ.D, integ.Q, integ.B.data_ptr(),
                                      integ.G.data_ptr(), integ.qdata.data_ptr(), R.gather_map.data_ptr(),
                                      R.offsets.data_ptr(), R.indices.data_ptr(), e.data_ptr(), e.numel(),
                                      M.dinv.data_ptr(), b.data_ptr(), x.data_ptr()))
        total += fes.ndofs
    arr = (_lib.ProblemDesc * nprob)(*descs)

    def batched(precision, schedule):
        sec = ctypes.c_double(0)
        cv = (ctypes.c_int * nprob)()
        it = (ctypes.c_int * nprob)()
        st_o = dev.lib.gbpa_batched_pcg_solve_ex(dev.ctx, nprob, arr, precision, schedule, rel_tol, 0.0,
                                                 max_it, it, cv, None, ctypes.byref(sec))
        torch.cuda.synchronize()
        return st_o, sec.value, int(sum(cv)), list(it), [pr["x"].clone() for pr in probs]

    def max_err(sols, ref):
        return max(float(torch.linalg.norm(xs - xr) / torch.linalg.norm(xr)) for xs, xr in zip(sols, ref))

    out_pe = None
    if persistent:
        st_pe, secs_pe, conv_pe, _, pe_sols = batched(_lib.GBPA_F64, _lib.GBPA_BATCH_PERSISTENT)
    st_x2, secs_x2, conv_x2, its_x2, x2_sols = batched(_lib.GBPA_F64X2, _lib.GBPA_BATCH_GRAPH)
    st, secs, conv, its, f64_sols = batched(_lib.GBPA_F64, _lib.GBPA_BATCH_GRAPH)
    if persistent:
        out_pe = {"status": st_pe, "seconds_one_launch": secs_pe, "converged": conv_pe,
                  "max_rel_l2_vs_graph": max_err(pe_sols, f64_sols)}
        del pe_sols
    x2_err = max_err(x2_sols, f64_sols)
    # one after another: the single-problem PCG, native FP64 and double-float
    info = _lib.SolveInfo()
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    seq, seq_x2, worst, worst_x2 = 0.0, 0.0, 0.0, 0.0
    for k, pr in enumerate(probs):
        X = torch.zeros_like(pr["x"])
        dev.lib.gbpa_pcg_solve(pr["A"].handle, P(pr["dinv"]), P(pr["b"]), P(X), rel_tol, 0.0, max_it, 0,
                               ctypes.byref(info))
        seq += info.seconds
        worst = max(worst, float(torch.linalg.norm(f64_sols[k] - X) / torch.linalg.norm(X)))
        integ = pr["integ"]
        Ax2 = PAOperator(0, pr["R"], integ.D, integ.Q, integ.B, integ.G, integ.qdata, ess=pr["ess_h"],
                         precision=_lib.GBPA_F64X2)
        X2 = torch.zeros_like(pr["x"])
        dev.lib.gbpa_pcg_solve(Ax2.handle, P(pr["dinv"]), P(pr["b"]), P(X2), rel_tol, 0.0, max_it, 0,
                               ctypes.byref(info))
        seq_x2 += info.seconds
        worst_x2 = max(worst_x2, float(torch.linalg.norm(x2_sols[k] - X2) / torch.linalg.norm(X2)))
        del Ax2, X, X2
    orders = [pr["p"] for pr in probs]
    dof_its = sum((probs[k]["b"].numel()) * its[k] for k in range(nprob))
    return {"workload": f"{nprob} Dirichlet Poisson problems, n~U[4,16], p~U{{2..6}}, lognormal kappa, "
                        f"{total} DOFs total, each to rel. residual {rel_tol:g}", "schedule": "graph",
            "arithmetic": "double-float (FP64 data; FP64-accurate products on the FP32 pipes)",
            "status": st_x2, "seconds_batched": secs_x2, "converged": conv_x2,
            "speedup_vs_sequential_fp64": seq / max(secs_x2, 1e-30),
            "speedup_vs_sequential_same_arithmetic": seq_x2 / max(secs_x2, 1e-30),
            "max_rel_l2_vs_fp64_batched": x2_err, "max_rel_l2_vs_sequential_same_arithmetic": worst_x2,
            "seconds_sequential_fp64": seq, "seconds_sequential_f64x2": seq_x2,
            "gdof_iterations_per_s": sum(probs[k]["b"].numel() * its_x2[k] for k in range(nprob))
            / max(secs_x2, 1e-30) / 1e9,
            "iterations_max": max(its_x2), "iterations_min": min(its_x2),
            "fp64": {"status": st, "seconds_batched": secs, "converged": conv,
                     "speedup_vs_sequential_fp64": seq / max(secs, 1e-30),
                     "max_rel_l2_vs_sequential": worst, "dof_iterations": dof_its,
                     "iterations_max": max(its), "iterations_min": min(its)},
            "persistent_fp64": out_pe, "dofs_total": total,
            "problems_per_order": {str(q): orders.count(q) for q in range(2, 7)}}


def run_sweep_form(target_dofs=8e6, reps=20, orders=range(1, 9)):
    """The operator-apply sweep: orders p = 1..8 on the jittered hex mesh with
    n = round(target_dofs^(1/3) / p) elements per side, q = p + 2, x ~
    U[-1, 1]; diffusion and mass L->L applies in FP64, double-float and FP32,
    `reps` applies timed with CUDA events after 3 warm-up applies (inputs larger
    than L2). GDOF/s and the algorithmic-bytes HBM
    fraction for each; the double-float and FP32 results' relative L2 error
    against FP64."""
    import torch
    from mfem_gb300 import fem
    from mfem_gb300.pa import PAOperator
    peak = measured_peak_hbm()[0]
    out = {"workload": f"jittered hex mesh, ~{target_dofs:.0e} DOFs per order, q = p + 2, x ~ U[-1,1]"}
    for p in orders:
        n = max(2, int(round(target_dofs ** (1.0 / 3.0) / p)))
        for kind in ("diffusion", "mass"):
            fes, integ, kid = build_problem(n, p, kind)
            x = torch.from_numpy(2.0 * fem.u01_array(2, fes.ndofs) - 1.0).cuda()
            y64 = torch.empty_like(x)
            row = {"n": n, "ndofs": fes.ndofs}
            for name, prec, w in (("f64", 0, 8), ("f64x2", 2, 8), ("f32", 1, 4)):
                op = PAOperator(kid, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata, precision=prec)
                xx = x.float() if prec == 1 else x
                yy = torch.empty_like(xx)
                for _ in range(3):
                    op.Mult(xx, yy)
                torch.cuda.synchronize()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record()
                for _ in range(reps):
                    op.Mult(xx, yy)
                b.record()
                torch.cuda.synchronize()
                ms = a.elapsed_time(b) / reps
                ent = {"ms": round(ms, 4), "gdofs": round(fes.ndofs / (ms * 1e-3) / 1e9, 3),
                       "hbm_frac_alg": round(algorithmic_bytes(fes.ne, fes.ndofs, integ.D, integ.Q, w, kind, False)
                                             / (ms * 1e-3) / 1e9 / peak, 4)}
                if prec == 0:
                    y64.copy_(yy)
                else:
                    ent["rel_l2_vs_f64"] = float(torch.linalg.norm(yy.double() - y64) / torch.linalg.norm(y64))
                row[name] = ent
                del op
            out[f"{kind}_p{p}"] = row
            del fes, integ
            torch.cuda.empty_cache()
    return out


def run_mg_form(n=77, p=4, orders=(1, 2, 4), with_jacobi=False, rel_tol=1e-10):
    """p-multigrid (next step past the Jacobi preconditioner): the precision
    form's problem (jittered n^3 mesh, lognormal kappa, RHS ~ U[0,1], seed 4,
    Dirichlet boundary) solved by CG preconditioned with a V(1,1) p-multigrid
    cycle over the orders `orders` (order-2 Chebyshev smoothing with
    power-method estimates, CG to 1e-2 on the coarsest order), the structure
    of the reference's examples/ex26.cpp (coarse CG without preconditioner,
    at most 200 iterations), and the same with a Jacobi-preconditioned coarse
    CG capped at 50 iterations. Level arithmetic FP64 and double-float, and
    FP32 levels preconditioning the FP64 CG; the true FP64 residual of each
    solution is reported, and, with_jacobi, the plain FP64 Jacobi-PCG solve
    of the same system."""
    import torch
    from mfem_gb300 import _lib, fem
    from mfem_gb300.pa import CGSolver, Device, DiffusionMultigrid, OperatorJacobiSmoother
    dev = Device.get()
    mesh = fem.CartesianMesh(n, jitter=0.1, seed=1)
    out = {"workload": f"Dirichlet Poisson, lognormal kappa, jittered n={n}^3, p={p}, levels p={list(orders)}",
           "rel_tol": rel_tol}
    sols = {}
    A64 = M64 = None
    b = None
    configs = [("fp64", _lib.GBPA_F64, False, 200), ("f64x2", _lib.GBPA_F64X2, False, 200),
               ("fp64_coarse_jacobi", _lib.GBPA_F64, True, 50), ("f64x2_coarse_jacobi", _lib.GBPA_F64X2, True, 50),
               ("f32_levels_coarse_jacobi", _lib.GBPA_F32, True, 50),
               ("f32_levels_x2_outer", _lib.GBPA_F32, True, 50)]
    Ax2_outer = None
    for name, prec, cj, cmax in configs:
        if name == "f32_levels_x2_outer":
            # the outer CG on the double-float fine operator (FP64-accurate, 3x
            # the native FP64 apply rate)
            fes4 = M64.spaces[-1]
            it4 = M64.integs[-1]
            from mfem_gb300.pa import PAOperator
            Ax2_outer = PAOperator(0, fes4, it4.D, it4.Q, it4.B, it4.G, it4.qdata, ess=M64.ess[-1],
                                   precision=_lib.GBPA_F64X2)
        t0 = time.perf_counter()
        M = DiffusionMultigrid(mesh, orders, "kappa", modes=fem.kappa_modes(3), precision=prec,
                               coarse_jacobi=cj, coarse_max_it=cmax)
        torch.cuda.synchronize()
        setup = time.perf_counter() - t0
        fes = M.spaces[-1]
        if b is None:
            b = torch.from_numpy(fem.u01_array(4, fes.ndofs)).cuda()
            b[torch.from_numpy(M.ess[-1]).long().cuda()] = 0.0
        x = torch.zeros_like(b)
        cg = CGSolver(); cg.SetRelTol(rel_tol); cg.SetMaxIter(500)
        # FP32 levels precondition the FP64 iteration on the FP64 (or the
        # double-float) operator
        cg.SetOperator(M.operators[-1] if prec != _lib.GBPA_F32 else (Ax2_outer if Ax2_outer else A64))
        cg.SetPreconditioner(M)
        cg.Mult(b, x)
        info = cg.info
        if prec == _lib.GBPA_F64:
            A64, M64 = M.operators[-1], M
        r = torch.empty_like(b)
        A64.Mult(x, r)
        res = float(torch.linalg.norm(b - r) / torch.linalg.norm(b))
        out[name] = {"seconds": info.seconds, "iterations": info.iterations, "converged": info.converged,
                     "coarse": f"CG{' + Jacobi' if cj else ''} to 1e-2, at most {cmax} iterations",
                     "coarse_cg_iterations": info.inner_iterations, "setup_seconds": setup,
                     "true_rel_residual": res,
                     "max_eig": [M.smoothers[l].GetMaxEigEstimate() for l in range(1, len(orders))]}
        sols[name] = x
        if M is not M64:
            del M
    for name in sols:
        if name != "fp64":
            out[name]["rel_l2_vs_fp64"] = float(torch.linalg.norm(sols[name] - sols["fp64"]) /
                                                torch.linalg.norm(sols["fp64"]))
    if with_jacobi:
        J = OperatorJacobiSmoother(A64, M64.ess[-1])
        xj = torch.zeros_like(b)
        cj = CGSolver(); cj.SetRelTol(rel_tol); cj.SetMaxIter(20000); cj.SetOperator(A64); cj.SetPreconditioner(J)
        cj.Mult(b, xj)
        out["jacobi_fp64"] = {"seconds": cj.info.seconds, "iterations": cj.info.iterations,
                              "rel_l2_mg_vs_jacobi": float(torch.linalg.norm(sols["fp64"] - xj) /
                                                           torch.linalg.norm(xj))}
        for name in sols:
            out[f"speedup_{name}_vs_jacobi_fp64"] = cj.info.seconds / max(out[name]["seconds"], 1e-30)
    return out


def run_combined_form(n=24, p=5, nrhs=8, with_reference=True, apply_only=False):
    """Combined form: unit cube mapped by x -> x + 0.05 sin(2 pi x) sin(2 pi y)
    sin(2 pi z) per component (order-3 geometry), H1 order p, lognormal kappa,
    nrhs right-hand sides ~ U[-1,1] solved together: FP32 block PCG inside FP64
    defect correction to 1e-10 per right-hand side. Reference: FP64 block PCG
    to 1e-12; per-right-hand-side relative L2 error reported."""
    import torch
    from mfem_gb300 import _lib, fem
    from mfem_gb300.pa import (DiffusionIntegrator, Device, FiniteElementSpace,
                               OperatorJacobiSmoother, PAOperator)
    dev = Device.get()
    mesh = fem.CartesianMesh(n, curved=True)
    fes = FiniteElementSpace(mesh, p)
    integ = DiffusionIntegrator("kappa")
    integ.AssemblePA(fes, modes=fem.kappa_modes(3))
    ess = fes.GetBoundaryTrueDofs()
    A64 = PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata, ess=ess)
    A32 = PAOperator(0, fes, integ.D, integ.Q, integ.B, integ.G, integ.qdata, ess=ess, precision=1)
    M = OperatorJacobiSmoother(A64, ess)
    nd = fes.ndofs
    B = torch.from_numpy(2 * fem.u01_array(6, nd * nrhs) - 1).cuda().view(nd, nrhs)
    B[torch.from_numpy(ess).long().cuda()] = 0.0
    B = B.contiguous()
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    # the FP32 block L->L apply (the inner solve's operator) against nrhs
    # single applies of the same vectors
    B32 = B.float().contiguous()
    Y32 = torch.empty_like(B32)
    cols = [B32[:, r].contiguous() for r in range(nrhs)]
    ycol = torch.empty_like(cols[0])
    blk = lambda: _lib.check(dev.lib.gbpa_operator_mult_block(A32.handle, nrhs, P(B32), P(Y32)), "mult_block")
    D, Q = integ.D, integ.Q
    layout = dev.lib.gbpa_get_block_apply_layout(D, Q, nrhs)
    ms_blk = _event_ms(blk, 20)
    ms_cc = None
    if layout == 2:
        # the CUDA-core block kernel on the same vectors, for comparison
        dev.lib.gbpa_set_block_apply_layout(D, Q, nrhs, 0)
        try:
            ms_cc = _event_ms(blk, 20)
        finally:
            dev.lib.gbpa_set_block_apply_layout(D, Q, nrhs, 2)
        blk()
    ms_one = _event_ms(lambda: [A32.Mult(c, ycol) for c in cols], 20)
    block_err = 0.0
    for r in range(nrhs):
        A32.Mult(cols[r], ycol)
        block_err = max(block_err, float(torch.linalg.norm(Y32[:, r] - ycol) / torch.linalg.norm(ycol)))
    apply_cmp = {"ms_block_apply": ms_blk, "block_kernel": LAYOUT_NAMES.get(layout, str(layout)),
                 "ms_block_apply_cuda_core": ms_cc, "ms_single_applies": ms_one,
                 "speedup_per_vector": ms_one / max(ms_blk, 1e-30),
                 "max_rel_l2_block_vs_single": block_err, "arithmetic": "f32"}
    del B32, Y32, cols, ycol
    if apply_only:
        return {"workload": f"curved order-3 geometry, n={n}^3, p={p}, q={p + 2}, {nd} DOFs, lognormal kappa, "
                            f"{nrhs} RHS~U[-1,1]", "block_apply": apply_cmp}
    X = torch.zeros_like(B)
    info = (_lib.SolveInfo * nrhs)()
    st = dev.lib.gbpa_pcg_solve_block_mixed(A64.handle, A32.handle, nrhs, P(M.dinv.float()), P(B), P(X),
                                            1e-10, 1e-5, 30, 20000, info)
    out = {"workload": f"curved order-3 geometry, n={n}^3, p={p}, q={p + 2}, {nd} DOFs, lognormal kappa, "
                       f"{nrhs} RHS~U[-1,1]", "status": st, "seconds_block_mixed": info[0].seconds,
           "outer": [info[r].outer_iterations for r in range(nrhs)],
           "inner_iterations": [info[r].inner_iterations for r in range(nrhs)],
           "true_rel_residual": [info[r].true_rel_residual for r in range(nrhs)],
           "block_apply": apply_cmp}
    # the same right-hand sides one at a time (single-vector mixed solves)
    seq = 0.0
    si = _lib.SolveInfo()
    for r in range(nrhs):
        xr = torch.zeros(nd, dtype=torch.float64, device="cuda")
        b = B[:, r].contiguous()
        dev.lib.gbpa_pcg_solve_mixed(A64.handle, A32.handle, P(M.dinv.float()), P(b), P(xr), 1e-10, 1e-5,
                                     30, 20000, ctypes.byref(si))
        seq += si.seconds
    out["seconds_sequential_mixed"] = seq
    out["speedup_block_vs_sequential"] = seq / max(info[0].seconds, 1e-30)
    # reliable updates (one FP32 PCG, FP64 residual replacement, delta 0.1): block and one at a time
    XR = torch.zeros_like(B)
    ir = (_lib.SolveInfo * nrhs)()
    st3 = dev.lib.gbpa_pcg_solve_block_mixed_reliable(A64.handle, A32.handle, nrhs, P(M.dinv.float()), P(B),
                                                      P(XR), 1e-10, 0.1, 20000, ir)
    seqr = 0.0
    for r in range(nrhs):
        xr = torch.zeros(nd, dtype=torch.float64, device="cuda")
        b = B[:, r].contiguous()
        dev.lib.gbpa_pcg_solve_mixed_reliable(A64.handle, A32.handle, P(M.dinv.float()), P(b), P(xr), 1e-10,
                                              0.1, 20000, ctypes.byref(si))
        seqr += si.seconds
    out["reliable"] = {"status": st3, "seconds_block": ir[0].seconds, "seconds_sequential": seqr,
                       "f32_iterations": [ir[r].iterations for r in range(nrhs)],
                       "replacements": [ir[r].outer_iterations for r in range(nrhs)],
                       "true_rel_residual": [ir[r].true_rel_residual for r in range(nrhs)]}
    if with_reference:
        X64 = torch.zeros_like(B)
        i64 = (_lib.SolveInfo * nrhs)()
        st2 = dev.lib.gbpa_pcg_solve_block(A64.handle, nrhs, P(M.dinv), P(B), P(X64), 1e-12, 0.0, 50000, i64)
        out["fp64_block_pcg"] = {"status": st2, "seconds": i64[0].seconds,
                                 "iterations": [i64[r].iterations for r in range(nrhs)]}
        out["rel_l2_vs_fp64"] = [float(torch.linalg.norm(X[:, r] - X64[:, r]) / torch.linalg.norm(X64[:, r]))
                                 for r in range(nrhs)]
        out["reliable"]["rel_l2_vs_fp64"] = [float(torch.linalg.norm(XR[:, r] - X64[:, r]) /
                                                   torch.linalg.norm(X64[:, r])) for r in range(nrhs)]
    return out


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.pcg_only:
        from mfem_gb300.pa import Device
        Device("cuda", dist_info()[2])
        print(json.dumps({"pcg": run_pcg_form(args.pcg_n, args.p, args.pcg_max_it)}), flush=True)
        return 0
    if args.batched:
        from mfem_gb300.pa import Device
        Device("cuda", dist_info()[2])
        print(json.dumps({"batched": run_batched_form(args.nprob, persistent=True)}), flush=True)
        return 0
    if args.sweep:
        from mfem_gb300.pa import Device
        Device("cuda", dist_info()[2])
        print(json.dumps({"sweep": run_sweep_form(args.sweep_dofs)}), flush=True)
        return 0
    if args.mg:
        from mfem_gb300.pa import Device
        Device("cuda", dist_info()[2])
        print(json.dumps({"mg": run_mg_form(args.mg_n, 4, (1, 2, 4), args.mg_jacobi)}), flush=True)
        return 0
    if args.combined:
        from mfem_gb300.pa import Device
        Device("cuda", dist_info()[2])
        print(json.dumps({"combined": run_combined_form(args.combined_n, 5, 8, not args.no_reference,
                                                        args.combined_apply_only)}), flush=True)
        return 0
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
