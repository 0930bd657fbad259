"""Autotuner for the apply kernels' thread layout and block shape.

For each (integrator, arithmetic, order p) the 2D-slab apply kernel runs with
block (Q, Q, nbz); nbz -- elements per block -- sets the block size, the
shared memory per block and therefore the occupancy. The 3D
layout (block (Q, Q, Q*nbz), one thread per quadrature point) is a
second candidate. The tuner times the gather-fused element kernel on a
synthetic jittered mesh for every feasible (layout, nbz) and keeps the
fastest. The table is saved as JSON (mfem_gb300/tuning.json: "nbz" for the 2D
slab, "layout3d" for the orders where the 3D layout won) and applied by
Device() on start-up through gbpa_set_elements_per_block and
gbpa_set_apply_layout.

FP32 diffusion at the orders with a tensor-core kernel (GBPA_LAYOUT_TC) is
compared separately, on a large mesh (--tc-dofs, 3e7 by default: the kernel
runs persistent CTAs over tiles of 128 elements, so small meshes leave SMs
idle): "tensor_core" lists the orders where it beat the best CUDA-core
layout, with the timings of both.

    python -m mfem_gb300.autotune [--orders 1-8] [--dofs 2e6] [--out path]
    python -m mfem_gb300.autotune --tensor-core-only [--tc-dofs 3e7]   (updates "tensor_core" in place)
"""
import argparse
import ctypes
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))
TUNING = os.path.join(HERE, "tuning.json")

KINDS = {"diffusion": 0, "mass": 1}
PRECS = {"f64": 0, "f32": 1, "f64x2": 2}


def key(kind, prec, D, Q):
    return f"{kind}:{prec}:{D}:{Q}"


def _parse_entry(k, v):
    """(kind id, precision id, D, Q, nbz) of one table entry; raises
    KeyError/ValueError/TypeError/AttributeError on a malformed entry."""
    kind, prec, D, Q = k.split(":")
    return KINDS[kind], PRECS[prec], int(D), int(Q), int(v)


def _parse_table(table, what, skipped):
    """Valid entries of one table section; malformed ones are listed in
    `skipped` and left out."""
    out = []
    for k, v in dict(table).items():
        try:
            out.append(_parse_entry(k, v))
        except (KeyError, ValueError, TypeError, AttributeError):
            skipped.append(f"{what}[{k!r}]")
    return out


def apply_table(lib, table):
    """Install a tuning table into the library (kind/prec names as in KINDS,
    PRECS). Every entry is parsed before any is installed; malformed entries
    are skipped. Returns the number of entries the library accepted."""
    entries = _parse_table(table, "nbz", [])
    return sum(1 for kd, pr, D, Q, nbz in entries
               if lib.gbpa_set_elements_per_block(kd, pr, D, Q, nbz) == 0)


# (D, Q) pairs with a compile-time 3D-layout diffusion kernel (GBPA_DQ3_LIST)
DQ3 = {(2, 2), (2, 3), (3, 3), (3, 4), (4, 4), (4, 5), (5, 5), (5, 6), (6, 6), (6, 7), (7, 7), (7, 8),
       (8, 8), (8, 9), (9, 9), (9, 10), (4, 6), (5, 8)}


# (D, Q) pairs with a tensor-core FP32 diffusion kernel (GBPA_TC_LIST)
TC = {(3, 4), (4, 5), (5, 6)}
GBPA_LAYOUT_TC = 2


def apply_layouts(lib, layout3d):
    """Install the 3D-layout entries {key: nbz} (parsed first, malformed
    entries skipped)."""
    entries = _parse_table(layout3d, "layout3d", [])
    return sum(1 for kd, pr, D, Q, nbz in entries
               if lib.gbpa_set_apply_layout(kd, pr, D, Q, 1, nbz) == 0)


def load_default(lib, path=TUNING):
    """Install a saved table. The whole file is read and every entry parsed
    before anything is installed: a missing, unreadable or non-object file
    leaves the library's defaults in place, and malformed entries are skipped
    one by one, each named in a warning. Returns the number of entries
    installed."""
    import warnings
    if not os.path.exists(path):
        return 0
    try:
        with open(path) as f:
            t = json.load(f)
        if not isinstance(t, dict):
            raise TypeError("the table is not a JSON object")
        skipped = []
        nbz = _parse_table(t.get("nbz", {}), "nbz", skipped)
        lay = _parse_table(t.get("layout3d", {}), "layout3d", skipped)
        tc = _parse_table(t.get("tensor_core", {}), "tensor_core", skipped)
    except (OSError, ValueError, TypeError, AttributeError) as e:
        warnings.warn(f"tuning table {path} not applied ({type(e).__name__}: {e}); using the defaults")
        return 0
    if skipped:
        warnings.warn(f"tuning table {path}: skipped malformed entries {', '.join(skipped)}")
    n = sum(1 for kd, pr, D, Q, v in nbz if lib.gbpa_set_elements_per_block(kd, pr, D, Q, v) == 0)
    n += sum(1 for kd, pr, D, Q, v in lay if lib.gbpa_set_apply_layout(kd, pr, D, Q, 1, v) == 0)
    # tensor-core entries (value 1) come last: they take precedence over a
    # 3D-layout entry for the same key
    n += sum(1 for kd, pr, D, Q, v in tc
             if v == 1 and lib.gbpa_set_apply_layout(kd, pr, D, Q, GBPA_LAYOUT_TC, 0) == 0)
    return n


def candidates_3d(prec, D, Q, kind="diffusion"):
    w = 4 if prec == "f32" else 8
    if kind == "diffusion":
        per = max(D ** 3, 3 * D * Q * Q) + max(2 * D * D * Q, 3 * Q ** 3)
    else:
        per = max(D ** 3, D * Q * Q) + max(D * D * Q, Q ** 3)
    out = []
    for nbz in range(1, 65):
        if nbz * Q ** 3 > 1024 or nbz * Q > 64 or w * (2 * Q * D + nbz * per) > 200 * 1024:
            break
        out.append(nbz)
    return out


def smem_bytes(kind, w, D, Q, nbz):
    if kind == "diffusion":
        per = max(D ** 3, 3 * D * Q * Q) + 2 * D * D * Q
        return w * (2 * Q * D + nbz * per)
    per = max(D ** 3, D * Q * Q) + D * D * Q
    return w * (Q * D + nbz * per)


def candidates(kind, prec, D, Q):
    w = 4 if prec == "f32" else 8
    out = []
    for nbz in range(1, 65):
        if nbz * Q * Q > 1024 or smem_bytes(kind, w, D, Q, nbz) > 200 * 1024:
            break
        out.append(nbz)
    return out


def time_nbz(lib, op, x, yE, reps):
    import torch
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    for _ in range(2):
        lib.gbpa_operator_apply_element(op.handle, P(x), P(yE))
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        st = lib.gbpa_operator_apply_element(op.handle, P(x), P(yE))
        if st != 0:
            return float("inf")
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def tune(orders=range(1, 9), kinds=("diffusion", "mass"), precs=("f64", "f32", "f64x2"),
         target_dofs=2e6, reps=10, verbose=True):
    import torch
    from . import fem
    from .pa import DiffusionIntegrator, Device, FiniteElementSpace, MassIntegrator, PAOperator
    dev = Device.get()
    lib = dev.lib
    table, timings, layout3d = {}, {}, {}
    for p in orders:
        n = max(2, int(round((target_dofs ** (1 / 3) - 1) / p)))
        mesh = fem.CartesianMesh(n, jitter=0.1, seed=1)
        fes = FiniteElementSpace(mesh, p)
        for kind in kinds:
            integ = DiffusionIntegrator() if kind == "diffusion" else MassIntegrator()
            integ.AssemblePA(fes)
            D, Q = integ.D, integ.Q
            for prec in precs:
                if prec == "f64x2" and (D > 10 or Q > 10):
                    continue
                pid = PRECS[prec]
                op = PAOperator(KINDS[kind], fes, D, Q, integ.B, integ.G, integ.qdata, precision=pid)
                dt = torch.float32 if prec == "f32" else torch.float64
                x = (torch.rand(fes.ndofs, device="cuda") - 0.5).to(dt)
                yE = torch.empty(fes.ne * D ** 3, dtype=dt, device="cuda")
                best = (float("inf"), None)
                res = {}
                # time the 2D slab even if a table selected the 3D layout
                lib.gbpa_set_apply_layout(KINDS[kind], pid, D, Q, 0, 0)
                for nbz in candidates(kind, prec, D, Q):
                    lib.gbpa_set_elements_per_block(KINDS[kind], pid, D, Q, nbz)
                    ms = time_nbz(lib, op, x, yE, reps)
                    res[nbz] = ms
                    best = min(best, (ms, nbz))
                lib.gbpa_set_elements_per_block(KINDS[kind], pid, D, Q, 0)
                res3, best3 = {}, (float("inf"), None)
                if (D, Q) in DQ3:
                    for nbz in candidates_3d(prec, D, Q, kind):
                        lib.gbpa_set_apply_layout(KINDS[kind], pid, D, Q, 1, nbz)
                        ms = time_nbz(lib, op, x, yE, reps)
                        res3[nbz] = ms
                        best3 = min(best3, (ms, nbz))
                    lib.gbpa_set_apply_layout(KINDS[kind], pid, D, Q, 0, 0)
                if best[1] is not None:
                    k = key(kind, prec, D, Q)
                    table[k] = best[1]
                    timings[k] = {"ne": fes.ne, "ndofs": fes.ndofs, "ms": res}
                    if res3:
                        timings[k]["ms_3d"] = res3
                    if best3[1] is not None and best3[0] < best[0]:
                        layout3d[k] = best3[1]
                    if verbose:
                        default = lib.gbpa_get_elements_per_block(KINDS[kind], pid, D, Q)
                        l3 = f"; 3D best nbz={best3[1]} {best3[0]:.4f} ms" if res3 else ""
                        print(f"{kind:9s} {prec:6s} p={p} D={D} Q={Q}: best nbz={best[1]} "
                              f"{best[0]:.4f} ms (default nbz={default}: {res.get(default, float('nan')):.4f} ms)"
                              f"{l3}", flush=True)
                del op, x, yE
            del integ
    return table, timings, layout3d


def time_mult(lib, op, x, y, reps):
    """ms per L->L apply (gbpa_operator_mult, the operator's Mult)."""
    import torch
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    for _ in range(2):
        lib.gbpa_operator_mult(op.handle, P(x), P(y))
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        if lib.gbpa_operator_mult(op.handle, P(x), P(y)) != 0:
            return float("inf")
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def tune_tensor_core(orders=range(1, 9), target_dofs=3e7, reps=20, verbose=True):
    """FP32 diffusion: the tensor-core layout against the layout installed for
    the CUDA cores (the tuned slab or 3D entry), both timed through the
    operator's Mult on one jittered mesh of about target_dofs dofs per order.
    Returns ({key: 1} for the orders where the tensor cores won, timings)."""
    import torch
    from . import fem
    from .pa import DiffusionIntegrator, Device, FiniteElementSpace, PAOperator
    lib = Device.get().lib
    won, timings = {}, {}
    for p in orders:
        D, Q = p + 1, p + 2
        if (D, Q) not in TC:
            continue
        n = max(2, int(round((target_dofs ** (1 / 3) - 1) / p)))
        fes = FiniteElementSpace(fem.CartesianMesh(n, jitter=0.1, seed=1), p)
        integ = DiffusionIntegrator()
        integ.AssemblePA(fes)
        x = (torch.rand(fes.ndofs, device="cuda", dtype=torch.float64) - 0.5)
        y64 = torch.empty_like(x)
        PAOperator(0, fes, D, Q, integ.B, integ.G, integ.qdata).Mult(x, y64)
        x32 = x.float()
        ms, rel = {}, {}
        nb = ctypes.c_int(0)
        prev = lib.gbpa_get_apply_layout(0, 1, D, Q, ctypes.byref(nb))
        # the CUDA-core side: the installed layout, or the 2D slab when the
        # installed one is the tensor-core layout
        cuda_core = (prev, nb.value) if prev != GBPA_LAYOUT_TC else (0, 0)
        for name, (layout, nbz) in (("cuda_core", cuda_core), ("tensor_core", (GBPA_LAYOUT_TC, 0))):
            if lib.gbpa_set_apply_layout(0, 1, D, Q, layout, nbz) != 0:
                continue
            op = PAOperator(0, fes, D, Q, integ.B, integ.G, integ.qdata, precision=1)
            y = torch.empty_like(x32)
            ms[name] = time_mult(lib, op, x32, y, reps)
            rel[name] = float(torch.linalg.norm(y.double() - y64) / torch.linalg.norm(y64))
            del op, y
        lib.gbpa_set_apply_layout(0, 1, D, Q, prev, nb.value)
        k = key("diffusion", "f32", D, Q)
        timings[k] = {"ne": fes.ne, "ndofs": fes.ndofs, "mult_ms": ms, "rel_l2_vs_f64": rel}
        if "tensor_core" in ms and ms["tensor_core"] < ms["cuda_core"]:
            won[k] = 1
        if verbose:
            print(f"diffusion f32 p={p}: {ms} (rel vs f64 {rel})", flush=True)
        del fes, integ, x, y64, x32
        torch.cuda.empty_cache()
    return won, timings


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--orders", default="1-8")
    ap.add_argument("--dofs", type=float, default=2e6)
    ap.add_argument("--reps", type=int, default=10)
    ap.add_argument("--kinds", default="diffusion,mass")
    ap.add_argument("--out", default=TUNING)
    ap.add_argument("--tc-dofs", type=float, default=3e7)
    ap.add_argument("--tensor-core-only", action="store_true",
                    help="re-time only the tensor-core layout; keep the rest of the table at --out")
    args = ap.parse_args()
    lo, hi = (int(v) for v in args.orders.split("-"))
    if args.tensor_core_only:
        with open(args.out) as f:
            t = json.load(f)
    else:
        table, timings, layout3d = tune(range(lo, hi + 1), kinds=tuple(args.kinds.split(",")),
                                        target_dofs=args.dofs, reps=args.reps)
        t = {"nbz": table, "layout3d": layout3d, "timings_ms": timings}
    if "diffusion" in args.kinds:
        won, tct = tune_tensor_core(range(lo, hi + 1), target_dofs=args.tc_dofs)
        t["tensor_core"], t["tensor_core_timings"] = won, tct
    with open(args.out, "w") as f:
        json.dump(t, f, indent=1, sort_keys=True)
    print(f"wrote {args.out} ({len(t['nbz'])} entries, 3D layout for {len(t['layout3d'])}, "
          f"tensor cores for {len(t.get('tensor_core', {}))})")


if __name__ == "__main__":
    main()
