"""Benchmark: GDoF/s of the matrix-free hp-FEM operator apply (dohp's ElastShellMatMult / EllipShellMatMult)
on one GB300.

Default workload (--config hp-elasticity-32, the hp-batching configuration): 3-D linear elasticity (E=1, nu=0.3,
ElastPointwiseJacobian at F=I) on a 32^3 structured hex mesh of the unit cube, interior vertices perturbed
U[-0.1h, 0.1h] (seed 1), per-element order drawn i.i.d. uniform from {2..8} (seed 2), min-order shared
faces/edges with interpolation constraints, Gauss (p+1)^3 quadrature, Dirichlet walls, FP64. A step is one
operator apply y = A x on a seeded x ~ U[-1,1]: one persistent kernel over all order buckets plus the
deterministic E^T restriction, replayed from a CUDA graph. The per-order-launch and persistent forms are timed
beside it. Inputs (geometric factors ~3 GB, E ~1 GB) exceed the 129 MB L2: no flush between steps.
A secondary entry times the uniform FP64 Poisson apply (lognormal k, 64^3, p=4; --config poisson-lognormal-64
makes it the headline).

Prints one JSON line: value = explicit scalar dofs / device seconds per apply (CUDA events on the launching
stream); e2e = dOperatorMultHost (host vectors, copies inside the timed region); roofline of the dominant
element kernel; cpu_baseline = the oracle's CPU restatement of the reference apply on the host cores.
"""
import argparse
import json
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIGS = {
    "hp-elasticity-32": dict(ne=32, kind="elasticity", hp=True, p=4, grf=False, label="hp-elasticity-32^3-p2..8"),
    "poisson-lognormal-64": dict(ne=64, kind="diffusion", hp=False, p=4, grf=True, label="poisson-lognormal-64^3-p4"),
    "poisson-8": dict(ne=8, kind="diffusion", hp=False, p=4, grf=False, label="poisson-8^3-p4"),
    # reduced cases of the same kernels for full ncu captures (inputs still above L2)
    "hp-elasticity-16": dict(ne=16, kind="elasticity", hp=True, p=4, grf=False, label="hp-elasticity-16^3-p2..8"),
    "poisson-lognormal-32": dict(ne=32, kind="diffusion", hp=False, p=4, grf=True, label="poisson-lognormal-32^3-p4"),
}
E0, NU = 1.0, 0.3
FP64_PEAK_GFLOPS = 1203.0  # FP64 FMA issue rate measured on this GB300 (FMA-chain probe)


def max_over_ranks(v, dist, device="cuda"):
    """Max of a per-rank time over all ranks: the replicas' only collective (no data-path exchange)."""
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_gdofs(world, dofs_per_rank, seconds):
    """value: dofs of all replicas over the slowest rank's time"""
    return world * dofs_per_rank / seconds / 1e9


def _plain(o):
    """JSON fallback for numpy scalars."""
    return o.item() if hasattr(o, "item") else str(o)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="hp-elasticity-32", choices=sorted(CONFIGS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true")
    ap.add_argument("--secondary", default="all", help="comma list of apply,learned,newton,multigrid,stokes (or all: apply, learned (which includes the multigrid "
                         "solves), newton)")
    ap.add_argument("--learned-ne", type=int, default=64, help="elements per side of the learned-correction solve")
    ap.add_argument("--learned-epochs", type=int, default=24,
                    help="training epochs of the vertex-lattice network: two thirds at lr 1e-3, the rest at 5e-4")
    ap.add_argument("--learned-gll-epochs", type=int, default=8, help="the same for the GLL-lattice network")
    ap.add_argument("--learned-grids", default="vertex,gll",
                    help="lattices of the learned correction: vertex (mesh vertices), gll (GLL nodes, the Q1-embedded grid)")
    ap.add_argument("--newton-ne", type=int, default=48, help="elements per side of the p-Laplacian Newton run")
    ap.add_argument("--newton-pc", default="mg", choices=("mg", "cheb"),
                    help="Newton linear solves: Q1 multigrid (default) or the single-level Chebyshev-Jacobi")
    return ap.parse_args()


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index, self.proc, self.lines = index, None, []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            out, _ = self.proc.communicate(timeout=5)
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def workload_config(cfg, dofs):
    """the `config` object of both arms' lines (identical for the same workload)"""
    return {"workload": cfg["label"], "elements": cfg["ne"] ** 3, "dofs": dofs,
            "block_size": 3 if cfg["kind"] == "elasticity" else 1,
            "orders": "i.i.d. U{2..8}, seed 2" if cfg["hp"] else "p=%d" % cfg["p"], "quadrature": "Gauss (p+1)^3",
            "mesh": "unit cube, interior vertices perturbed U[-0.1h, 0.1h], seed 1",
            "l2": "inputs larger than L2, no flush"}


def elem_orders(cfg, ne):
    import numpy as np
    if not cfg["hp"]:
        return None
    return np.random.default_rng(2).integers(2, 9, size=ne ** 3).astype(np.int32)


def grf_numpy(grf, X):
    """k = exp(g(X)) for the random-Fourier-feature field (same formula as the library and the oracle)."""
    import numpy as np
    nf = int(grf[0])
    W = grf[3:3 + 3 * nf].reshape(nf, 3)
    b = grf[3 + 3 * nf:3 + 4 * nf]
    out = np.empty(len(X))
    for i in range(0, len(X), 1 << 16):
        out[i:i + (1 << 16)] = np.exp(np.sqrt(2.0 * grf[1] / nf) * np.cos(X[i:i + (1 << 16)] @ W.T + b).sum(axis=1))
    return out


def cpu_baseline(cfg, threads, budget_s=20.0, compare=None):
    """Oracle (CPU restatement of the reference apply: per-element geometry recompute, INTERP+GRAD, q-function,
    INTERP_T+GRAD_T, E/E^T) timed on the full workload (same mesh, orders, coefficient and input as the GPU arm),
    all host threads (OpenMP over elements, expand and restrict; the reference runs one MPI rank per core, each
    on its own elements). The median of up to 10 applies after one warm-up, within budget_s."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    po.build()
    ne = cfg["ne"]
    bs = 3 if cfg["kind"] == "elasticity" else 1
    fs = po.FS(ne + 1, ne + 1, ne + 1, degree=cfg["p"], perturb=0.1, seed=1, bs=bs, elem_degree=elem_orders(cfg, ne))
    qd, kind, param = None, 0, None
    if cfg["kind"] == "elasticity":
        kind = 2
        param = np.array([E0 * NU / ((1 + NU) * (1 - 2 * NU)), E0 / (2 * (1 + NU))])
    if cfg["grf"]:
        grf = po.grf_make(64, 2.0, 0.1, 2)
        qd = grf_numpy(grf, fs.qpt_coords())
    x = np.random.default_rng(0).uniform(-1, 1, fs.n * bs)
    fs.apply(x, kind=kind, qdata=qd, param=param, nthreads=threads)  # warm-up
    times = []
    t_start = time.perf_counter()
    while len(times) < 3 or (time.perf_counter() - t_start < budget_s and len(times) < 10):
        t0 = time.perf_counter()
        fs.apply(x, kind=kind, qdata=qd, param=param, nthreads=threads)
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - t_start > budget_s:
            break
    times.sort()
    t = times[len(times) // 2]
    out = {"value": fs.n * bs / t / 1e9, "unit": "GDoF/s", "cores": threads, "kind": "port", "dofs": fs.n * bs,
           "sample": "the full workload, %d^3 elements (%d dofs), median of %d applies, oracle C restatement, %d OpenMP threads"
                     % (ne, fs.n * bs, len(times), threads)}
    if compare:  # the GPU arm's results on the same input against the oracle's apply
        yo = fs.apply(x, kind=kind, qdata=qd, param=param, nthreads=threads)
        out["gpu_rel_err_vs_this_apply"] = {k: float(np.linalg.norm(v - yo) / np.linalg.norm(yo)) for k, v in compare.items()}
    return out


def cpu_time_to_rtol_poisson8(threads):
    """The CPU-runnable configuration (Poisson 8^3, p=4, mass right-hand side of f ~ U[-1,1], CG + Q1
    Chebyshev(3)-Jacobi to rtol 1e-8) solved by the oracle on the host cores: wall seconds."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    o = po.FS(9, 9, 9, degree=4, perturb=0.1, seed=1)
    b = o.apply(np.random.default_rng(0).uniform(-1, 1, o.n), kind=3, nthreads=threads)
    t0 = time.perf_counter()
    csr = o.q1_assemble()
    t1 = time.perf_counter()
    _, its, rn = o.cg_solve(b, csr, rtol=1e-8, maxit=1000, nthreads=threads)
    t2 = time.perf_counter()
    return {"its": its, "solve_s": t2 - t1, "q1_assembly_s": t1 - t0, "rel_residual": rn, "threads": threads}


def gpu_time_to_rtol_poisson8():
    """Same problem on the GPU: mass right-hand side through the batched dRulesetIterator, Q1 assembly on the
    device, CG with Chebyshev(3)-Jacobi, FP64."""
    import numpy as np
    import torch
    import dohp_gb300 as dg
    fs = dg.FS((9, 9, 9), degree=4, perturb=0.1, seed=1)
    f = torch.as_tensor(np.random.default_rng(0).uniform(-1, 1, fs.n), device="cuda")
    it = dg.RulesetIterator(fs)
    it.start(f)
    a = it.get()
    a["v"].copy_(a["jw"][:, None] * a["u"])
    it.commit(dg.INSERT_VALUES, use_v=True, use_dv=False)
    b = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
    it.finish(b)
    op = fs.operator()
    m = fs.matrix()
    m.assemble()
    for _ in range(2):  # warm-up (geometry, kernels); the timed run below includes assembly and set-up
        x = torch.zeros_like(b)
        dg.KSP(op, m, ksp_type=dg.dKSP_CG).solve(b, x, rtol=1e-8, maxit=1000)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    m.assemble()
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    ksp = dg.KSP(op, m, ksp_type=dg.dKSP_CG)
    x = torch.zeros_like(b)
    its, rn = ksp.solve(b, x, rtol=1e-8, maxit=1000)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    return {"its": its, "solve_s": t2 - t1, "q1_assembly_s": t1 - t0, "rel_residual": rn}


def run_reference(args, cfg, rank):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    cb = cpu_baseline(cfg, threads, budget_s=max(10.0, min(60.0, 3.0 * args.steps)))
    line = {"impl": "reference", "metric": "GDoF/s operator apply", "value": cb["value"], "unit": "GDoF/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded mesh perturbation, orders, field and input)",
            "config": workload_config(cfg, cb["dofs"]),
            "arm": {"parallelism": "host threads (%d)" % threads, "implementation": "oracle C restatement of the reference "
                    "apply (EllipShellMatMult / ElastShellMatMult element loop with geometry recompute, E and E^T)",
                    "sample": cb["sample"]},
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "GDoF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def setup(cfg, stream):
    import numpy as np
    import torch
    import dohp_gb300 as dg
    ne = cfg["ne"]
    bs = 3 if cfg["kind"] == "elasticity" else 1
    fs = dg.FS((ne + 1,) * 3, degree=cfg["p"], perturb=0.1, seed=1, bs=bs, elem_degree=elem_orders(cfg, ne),
               stream=stream.cuda_stream)
    if cfg["kind"] == "elasticity":
        op = fs.operator(dg.dOP_ELASTICITY, param=(E0, NU))
    else:
        op = fs.operator(dg.dOP_DIFFUSION)
        if cfg["grf"]:
            kq = torch.empty(fs.nq, dtype=torch.float64, device="cuda")
            fs.lognormal(dg.grf_create(64, 2.0, 0.1, 2), kq)
            op.set_qdata(kq)
    x = torch.as_tensor(np.random.default_rng(0).uniform(-1, 1, fs.n * bs), device="cuda")
    return fs, op, x, bs


def time_loop(fn, steps, stream):
    import torch
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t0.record(stream)
    for a, b in evs:
        a.record(stream)
        fn()
        b.record(stream)
    t1.record(stream)
    torch.cuda.synchronize()
    per = sorted(a.elapsed_time(b) for a, b in evs)
    return t0.elapsed_time(t1) / steps, per[len(per) // 2]


# (kind, hp, p) -> (DRAM bytes per element per launch of the dominant kernel, where the figure comes from)
NCU_DRAM_BYTES_PER_ELEMENT = {
    ("elasticity", True, 4): (231.705600e6 / 4096, "ncu, k_hp_persistent<double,elasticity>, 16^3 elements: 212.5 MB read + 19.2 MB "
                                                   "written per launch, scaled by elements"),
    ("diffusion", False, 4): (253.2e6 / 32768, "ncu, k_uniform<5,double,diffusion>, 32^3 elements: 229.7 MB read + 23.5 MB written "
                                               "per launch, scaled by elements"),
}


def work_per_apply(fs, cfg, bs):
    """Algorithmic bytes and flops per apply (x and y once, the int32 element map and 8 vertex coordinates per
    element; 36 n^4 + 30 n^3 flops per element and component), and the flops the element kernels issue."""
    import numpy as np
    deg = fs.elem_degree()[:, 0].astype(np.float64)
    n1 = deg + 1
    alg_bytes = 16.0 * bs * fs.nc + float(np.sum(4.0 * n1 ** 3 + 192.0))
    alg_flops = float(np.sum(36.0 * n1 ** 4 * bs + 30.0 * n1 ** 3 * bs))
    pw = 150.0 if bs == 3 else 18.0
    issued = float(np.sum(24.0 * n1 ** 4 * bs + pw * n1 ** 3))
    return alg_bytes, alg_flops, issued


def secondary_lognormal_apply(args):
    """uniform FP64 Poisson apply (lognormal k, 64^3, p=4): element kernel + restrict, device-timed."""
    import torch
    cfg = CONFIGS["poisson-lognormal-64"]
    stream = torch.cuda.current_stream()
    fs, op, x, bs = setup(cfg, stream)
    y = torch.empty(fs.n, dtype=torch.float64, device="cuda")
    yexp = torch.empty(fs.nexp, dtype=torch.float64, device="cuda")
    for _ in range(3):
        op.mult_expanded(x, yexp)
        fs.expanded_to_global(yexp, y)
    ms, _ = time_loop(lambda: (op.mult_expanded(x, yexp), fs.expanded_to_global(yexp, y)), max(args.steps // 2, 5), stream)
    _, kms = time_loop(lambda: op.mult_expanded(x, yexp), max(args.steps // 2, 5), stream)
    _, _, issued = work_per_apply(fs, cfg, bs)
    out = {"workload": cfg["label"], "dofs": fs.n, "value": fs.n / (ms * 1e-3) / 1e9, "unit": "GDoF/s", "ms_per_apply": ms,
           "element_kernel_ms": kms, "fp64_gflops": issued / (kms * 1e-3) / 1e9,
           "fp64_frac_of_peak": issued / (kms * 1e-3) / 1e9 / FP64_PEAK_GFLOPS, "dtype": "f64"}
    out["float_float"] = float_float_leg(op, x, y, args, stream)
    out["float_float"]["value"] = fs.n / (out["float_float"]["ms_per_apply"] * 1e-3) / 1e9
    out["bf16_tensor_core"] = bf16_tc_leg(fs, op, x, y, args, stream)
    return out


def bf16_tc_leg(fs, op, x, y64, args, stream):
    """the same apply with dPREC_BF16 (tcgen05 MMAs, BF16 operands, FP32 accumulation in tensor memory; BF16 geometric
    factors; FP32 expanded output restricted in FP64): time, relative difference from the FP64 result, and the HBM rate
    of its algorithmic bytes (x and y once in FP64, the int32 element map, 6 BF16 factors per Gauss point, the FP32
    expanded output written and read once)"""
    import numpy as np
    import torch
    import dohp_gb300 as dg
    op.mult(x, y64)
    op.set_precision(dg.dPREC_BF16)
    yb = torch.empty_like(y64)
    for _ in range(3):
        op.mult(x, yb)
    ms, _ = time_loop(lambda: op.mult(x, yb), max(args.steps, 5), stream)
    err = float(torch.linalg.norm(yb - y64) / torch.linalg.norm(y64))
    op.set_precision(dg.dPREC_FP64)
    n1 = fs.elem_degree()[:, 0].astype(np.float64) + 1
    nbytes = 16.0 * fs.nc + float(np.sum(4.0 * n1 ** 3 + 12.0 * n1 ** 3 + 8.0 * n1 ** 3))
    hbm, src = peaks()
    return {"unit": "GDoF/s", "value": fs.n / (ms * 1e-3) / 1e9, "ms_per_apply": ms, "rel_diff_vs_fp64": err,
            "alg_bytes_per_apply": nbytes, "hbm_gbs": nbytes / (ms * 1e-3) / 1e9, "hbm_frac": nbytes / (ms * 1e-3) / 1e9 / hbm,
            "dtype": "bf16 operands, fp32 accumulation (tcgen05 tensor cores)"}


def float_float_leg(op, x, y64, args, stream, keep=None):
    """the same apply with dPREC_FF (values as FP32 pairs, unit roundoff ~2^-48, FP32 pipe), its time and its
    relative difference from the FP64 result in y64 (computed by the caller with the same operator); with keep (a
    dict) the FP64 and float-float results are left there as host arrays for the comparison with the oracle"""
    import torch
    import dohp_gb300 as dg
    op.mult(x, y64)
    op.set_precision(dg.dPREC_FF)
    yff = torch.empty_like(y64)
    for _ in range(3):
        op.mult(x, yff)
    ms, _ = time_loop(lambda: op.mult(x, yff), max(args.steps, 5), stream)
    err = float(torch.linalg.norm(yff - y64) / torch.linalg.norm(y64))
    op.set_precision(dg.dPREC_FP64)
    if keep is not None:
        keep["fp64"], keep["float_float"] = y64.cpu().numpy(), yff.cpu().numpy()
    return {"unit": "GDoF/s", "ms_per_apply": ms, "rel_diff_vs_fp64": err,
            "dtype": "float-float (2 x fp32 per value, unit roundoff ~2^-48, FP32 pipe)"}


def secondary_newton(args):
    """p-Laplacian Newton-Krylov (exponent 1.5, eps 1e-6, p=6, f ~ U[-1,1] per dof; 48^3 elements by default, the
    mixed-precision configuration's size): FP64, FP32 and BF16 inner applies (Jacobian, and the Q1 multigrid V-cycle
    in the same precision) inside FGMRES with FP64 residuals and orthogonalisation. Each run advances one Newton step
    at a time (wall time per step, the oracle checks between steps are not timed). Per step and per reduced-precision
    run: the relative error of its Jacobian apply against the FP64 oracle's Jacobian apply at that run's own iterate
    (EllipShellMatMult at the store of the iterate, ellip.c:333-377, 442-472), and the iterate's distance from the
    FP64 run's iterate. At the first step and at each run's final iterate: the nonlinear residual ||F(u) - b|| measured
    by the oracle's own EllipFunction (ellip.c:407-440) and the product's FP64 function against it."""
    import numpy as np
    import torch
    import dohp_gb300 as dg
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    threads = os.cpu_count() or 1
    ne, p, pe, eps = args.newton_ne, 6, 1.5, 1e-6
    fs = dg.FS((ne + 1,) * 3, degree=p, perturb=0.1, seed=1)
    o = po.FS(ne + 1, ne + 1, ne + 1, degree=p, perturb=0.1, seed=1)
    bh = np.random.default_rng(0).uniform(-1, 1, fs.n)
    b = torch.as_tensor(bh, device="cuda")
    mg = args.newton_pc == "mg"
    out = {"workload": "plaplace-newton-%d^3-p6: exponent 1.5, eps 1e-6" % ne,
           "dofs": fs.n, "rtol": 1e-8, "lin_rtol": 1e-3, "lin_maxit": 300,
           "ksp": ("FGMRES(30) + Q1 multigrid V-cycle (Chebyshev(2)-Jacobi smoothing) in the inner precision" if mg else
                   "FGMRES(30) + Chebyshev(3)-Jacobi on the Q1-embedded Jacobian") + ", inexact steps at lin_maxit",
           "oracle_threads": threads}

    def oracle_residual(u):
        """||F(u) - b|| by the oracle's EllipFunction, and the product's FP64 function's relative error against it"""
        Fo = o.function(u, 6, (pe, eps), nthreads=threads)
        op = fs.operator(dg.dOP_PLAPLACE_JACOBIAN)
        y = torch.zeros_like(b)
        op.plap_function(torch.as_tensor(u, device="cuda"), pe, eps, y)
        yh = y.cpu().numpy()
        return float(np.linalg.norm(Fo - bh)), float(np.linalg.norm(yh - Fo) / np.linalg.norm(Fo))

    runs = {}
    for name, prec in (("fp64", dg.dPREC_FP64), ("fp32", dg.dPREC_FP32), ("bf16", dg.dPREC_BF16)):
        op = fs.operator(dg.dOP_PLAPLACE_JACOBIAN)
        m = fs.matrix()
        ksp = dg.KSP(op, m, ksp_type=dg.dKSP_FGMRES, inner_prec=prec, restart=30, pc=dg.dPC_MG_Q1 if mg else dg.dPC_CHEBYSHEV_Q1)
        u = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
        runs[name] = dict(op=op, m=m, ksp=ksp, u=u, wall=0.0, fnorm=[], its=[], done=False, prec=prec)
    per = []
    for k in range(30):
        for name, r in runs.items():
            if r["done"]:
                continue
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            _, fn, li = dg.plap_newton(r["op"], r["m"], r["ksp"], b, r["u"], pe, eps, rtol=0.0, lin_rtol=1e-3, lin_maxit=300,
                                       max_it=1)
            torch.cuda.synchronize()
            r["wall"] += time.perf_counter() - t0
            if not r["fnorm"]:
                r["fnorm"].append(float(fn[0]))
            r["fnorm"].append(float(fn[1]))
            r["its"].append(int(li[0]))
            r["done"] = bool(fn[1] <= 1e-8 * r["fnorm"][0])
            r["last_step"] = k + 1
        row = {"step": k + 1}
        r64 = runs["fp64"]
        d = np.random.default_rng(100 + k).uniform(-1, 1, fs.n)
        dd = torch.as_tensor(d, device="cuda")
        for name in ("fp32", "bf16"):
            r = runs[name]
            if r.get("last_step") != k + 1:
                continue
            uh = r["u"].cpu().numpy()
            st = o.plap_stash(uh, pe, eps, nthreads=threads)
            Jo = o.apply(d, kind=1, qdata=st, nthreads=threads)
            op = r["op"]
            op.plap_stash(r["u"], pe, eps)
            yl = torch.empty_like(dd)
            op.set_precision(r["prec"])
            op.mult(dd, yl)
            op.set_precision(dg.dPREC_FP64)
            row[name + "_jacobian_apply_rel_err_vs_oracle"] = float(np.linalg.norm(yl.cpu().numpy() - Jo) / np.linalg.norm(Jo))
            row[name + "_iterate_rel_diff_vs_fp64_run"] = float(torch.linalg.norm(r["u"] - r64["u"]) / torch.linalg.norm(r64["u"]))
        if r64.get("last_step") == k + 1 and k == 0:
            row["fp64_oracle_residual"], row["fp64_function_rel_err_vs_oracle"] = oracle_residual(r64["u"].cpu().numpy())
        per.append(row)
        if all(r["done"] for r in runs.values()):
            break
    f0 = float(np.linalg.norm(bh))  # F(0) = -b: the oracle's function vanishes at u = 0
    for name, r in runs.items():
        res, ferr = oracle_residual(r["u"].cpu().numpy())
        out[name] = {"newton_steps": len(r["its"]), "fnorm": r["fnorm"], "fgmres_its": r["its"], "wall_s": r["wall"],
                     "converged": r["done"], "oracle_final_rel_residual": res / f0,
                     "fp64_function_rel_err_vs_oracle_at_final_iterate": ferr}
    out["per_step"] = per
    out["speedup_vs_fp64"] = {n: runs["fp64"]["wall"] / runs[n]["wall"] for n in ("fp32", "bf16")}
    return out


def multigrid_solves(fs, op, m, b):
    """the Q1 multigrid preconditioner on a lognormal problem (no network): CG with FP64 applies, and FGMRES with
    FP32 inner applies; the V-cycle runs in the preconditioner's precision (FP64 under CG, FP32 inside the FGMRES).
    Set-up (hierarchy, eigenvalue estimates) is timed apart."""
    import torch
    import dohp_gb300 as dg
    out = {}
    for name, ktype, prec in (("multigrid_cg_fp64", dg.dKSP_CG, dg.dPREC_FP64), ("multigrid_mixed_fp32", dg.dKSP_FGMRES, dg.dPREC_FP32)):
        ksp = dg.KSP(op, m, ksp_type=ktype, inner_prec=prec, restart=30, pc=dg.dPC_MG_Q1)
        x = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        try:
            ksp.solve(b, x, rtol=1e-1, maxit=50)
        except dg.DohpError:
            pass
        torch.cuda.synchronize()
        setup = time.perf_counter() - t0
        x.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        its, _ = ksp.solve(b, x, rtol=1e-8, maxit=2000)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        r = torch.empty_like(x)
        op.mult(x, r)
        out[name] = {"its": its, "wall_s": wall, "setup_and_first_solve_s": setup,
                     "true_rel_residual": float(torch.linalg.norm(b - r) / torch.linalg.norm(b))}
    return out


def secondary_multigrid(args):
    """the multigrid solves alone on the time-to-rtol problem (lognormal Poisson, p=4, --learned-ne elements
    per side, fresh field seed 5000)"""
    import numpy as np
    import torch
    import dohp_gb300 as dg
    ne = args.learned_ne
    fs = dg.FS((ne + 1,) * 3, degree=4, perturb=0.1, seed=1)
    grf = dg.grf_create(64, 2.0, 0.1, 5000)
    kq = torch.empty(fs.nq, dtype=torch.float64, device="cuda")
    fs.lognormal(grf, kq)
    op = fs.operator()
    op.set_qdata(kq)
    m = fs.matrix()
    m.assemble(grf=grf)
    b = torch.as_tensor(np.random.default_rng(5000).uniform(-1, 1, fs.n), device="cuda")
    out = {"workload": "lognormal-poisson-%d^3-p4, Q1 multigrid" % ne, "dofs": fs.n, "rtol": 1e-8}
    out.update(multigrid_solves(fs, op, m, b))
    return out


def secondary_stokes(args):
    """Stokes with the power-law rheology (p = 4/3, the Glen exponent n = 3; eps = 0.5, B = 1): the nonlinear
    function and the Jacobian apply at its state on 32^3 elements (Q3-Q2), then Newton from zero with FGMRES and
    the block preconditioner (one Q1 multigrid V-cycle on the velocity block) on Q3-Q1 spaces with the
    divergence-free body force f = 10 (sin(pi y) sin(pi z), sin(pi z) sin(pi x), sin(pi x) sin(pi y))."""
    import math
    import torch
    import dohp_gb300 as dg
    rheo = (1.0, 0.5, 4.0 / 3.0, 0.0)
    out = {"workload": "stokes power law p=4/3 eps=0.5 B=1", "newton": []}

    def spaces(M, k, codim):
        fsu = dg.FS((M + 1,) * 3, degree=k, perturb=0.1, seed=7, bs=3)
        return fsu, dg.FS(None, degree=k - codim, bs=1, dirichlet=(), mesh_of=fsu)

    fsu, fsp = spaces(32, 3, 1)
    st = dg.Stokes(fsu, fsp, rheo)
    g = torch.Generator(device="cuda").manual_seed(3)
    xu = torch.rand(fsu.n * 3, dtype=torch.float64, device="cuda", generator=g) - 0.5
    xp = torch.rand(fsp.n, dtype=torch.float64, device="cuda", generator=g) - 0.5
    yu, yp = torch.zeros_like(xu), torch.zeros_like(xp)
    stream = torch.cuda.default_stream()
    n = fsu.n * 3 + fsp.n
    for _ in range(3):
        st.function(xu, xp, yu, yp)
    tf, _ = time_loop(lambda: st.function(xu, xp, yu, yp), 10, stream)
    tj, _ = time_loop(lambda: st.mult(dg.dSTOKES_MULT_COUPLED, xu=xu, xp=xp, yu=yu, yp=yp), 10, stream)
    out["apply_32^3_q3q2"] = {"dofs": n, "function_ms": tf, "jacobian_ms": tj, "function_gdofs": n / tf / 1e6,
                              "jacobian_gdofs": n / tj / 1e6}
    del st, fsu, fsp, xu, xp, yu, yp
    torch.cuda.empty_cache()
    for M in (8, 16):
        fsu, fsp = spaces(M, 3, 2)
        st = dg.Stokes(fsu, fsp, rheo)
        it = dg.RulesetIterator(fsu)
        it.start(None)
        a = it.get()
        x = a["x"]
        sx, sy, sz = (torch.sin(math.pi * x[:, i]) for i in range(3))
        a["v"].copy_(10.0 * a["jw"][:, None] * torch.stack([sy * sz, sz * sx, sx * sy], 1))
        it.commit(dg.INSERT_VALUES, use_v=True, use_dv=False)
        bu = torch.zeros(fsu.n * 3, dtype=torch.float64, device="cuda")
        it.finish(bu)
        bp = torch.zeros(fsp.n, dtype=torch.float64, device="cuda")
        walls = []
        for rep in range(2):  # the first solve includes the set-up (Q1 matrix, multigrid hierarchy, FGMRES)
            uu, pp = torch.zeros_like(bu), torch.zeros_like(bp)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            k, fn, li = st.newton(bu, bp, uu, pp, rtol=1e-10, lin_rtol=1e-6, lin_maxit=2000, max_it=40)
            torch.cuda.synchronize()
            walls.append(time.perf_counter() - t0)
        out["newton"].append({"elements": "%d^3" % M, "spaces": "Q3-Q1", "dofs": fsu.n * 3 + fsp.n, "steps": k,
                              "fnorm": [float(fn[0]), float(fn[-1])], "fgmres_its": [int(v) for v in li],
                              "wall_s_with_setup": walls[0], "wall_s": walls[1]})
        del st, it, fsu, fsp
        torch.cuda.empty_cache()
    return out


def secondary_learned(args):
    """Lognormal Poisson (64^3, p=4, ~16.6 M dofs), time to rtol 1e-8 on a fresh field: FGMRES(30) with the
    Q1 Chebyshev(3)-Jacobi preconditioner in FP64 (plain), with FP32 inner applies (mixed), and with the
    learned coarse correction added (learned+mixed, learned+FP64). The network is trained first, on this GPU,
    by the library's own kernels on (residual, error) pairs from the plain CG on fresh seeded k fields."""
    import numpy as np
    import torch
    import dohp_gb300 as dg
    ne, nfields, per_field = args.learned_ne, 8, 250

    def problem(seed):
        fs = dg.FS((ne + 1,) * 3, degree=4, perturb=0.1, seed=1)
        grf = dg.grf_create(64, 2.0, 0.1, seed)
        kq = torch.empty(fs.nq, dtype=torch.float64, device="cuda")
        fs.lognormal(grf, kq)
        op = fs.operator()
        op.set_qdata(kq)
        m = fs.matrix()
        m.assemble(grf=grf)
        return fs, op, m, grf

    grids = [g for g in args.learned_grids.split(",") if g]
    out = {"workload": "lognormal-poisson-%d^3-p4, learned correction and multigrid" % ne, "rtol": 1e-8,
           "ksp": "FGMRES(30), Chebyshev(3)-Jacobi on the Q1-embedded matrix",
           "network": "3-level U-Net 16/32/64 ch, 3^3 kernels, BF16 weights, FP32 accumulate; the stride-1 16/32-channel "
                      "convolutions on the tcgen05 tensor cores (BF16 activations at their inputs), the others on CUDA cores"}
    nets = {}
    for grid in grids:  # learned_* keys: the vertex lattice; learned_gll_*: the GLL lattice of the Q1-embedded matrix
        fs0, _, _, _ = problem(1000)
        if grid == "gll":
            net = dg.Learned(fs0, seed=7, grid=dg.LEARNED_GRID_GLL, crop=65)
        else:
            net = dg.Learned(fs0, seed=7)
        del fs0
        info = {"lattice": "x".join(str(v) for v in net.dims)}
        if grid == "gll":
            info["training_window"] = "65^3 windows at origins that are multiples of 4"
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for f in range(nfields):
            fs, op, m, grf = problem(1000 + f)
            net.set_field(grf)
            ksp = dg.KSP(op, m, ksp_type=dg.dKSP_CG)
            b = torch.as_tensor(np.random.default_rng(1000 + f).uniform(-1, 1, fs.n), device="cuda")
            net.collect(ksp, b, rtol=1e-10, every=3, max_pairs=per_field)
            del fs, op, m, ksp, b
        torch.cuda.synchronize()
        info["pairs"] = net.npairs
        info["collect_s"] = time.perf_counter() - t0
        epochs = args.learned_gll_epochs if grid == "gll" else args.learned_epochs
        e1 = (2 * epochs + 2) // 3
        t0 = time.perf_counter()
        losses = list(net.train(epochs=e1, batch=16, lr=1e-3, seed=1))
        if epochs > e1:  # a step down of the learning rate for the last third
            losses += list(net.train(epochs=epochs - e1, batch=16, lr=5e-4, seed=2))
        torch.cuda.synchronize()
        info["train_s"] = time.perf_counter() - t0
        info["epochs"] = epochs
        info["lr_schedule"] = "%d epochs at 1e-3, %d at 5e-4 (Adam, batch 16)" % (e1, epochs - e1)
        info["loss_per_epoch"] = [float(v) for v in losses]
        nets[grid] = net
        if grid == "vertex":
            out.update(info)
        else:
            out["gll_network"] = info
    fs, op, m, grf = problem(5000)
    for net in nets.values():
        net.set_field(grf)
    b = torch.as_tensor(np.random.default_rng(5000).uniform(-1, 1, fs.n), device="cuda")
    out["dofs"] = fs.n
    legs = [("plain_fp64", dg.dPREC_FP64, None), ("mixed_fp32", dg.dPREC_FP32, None), ("mixed_bf16", dg.dPREC_BF16, None)]
    if "vertex" in nets:
        legs += [("learned_mixed", dg.dPREC_FP32, "vertex"), ("learned_bf16", dg.dPREC_BF16, "vertex"),
                 ("learned_fp64", dg.dPREC_FP64, "vertex")]
    if "gll" in nets:
        legs += [("learned_gll_mixed", dg.dPREC_FP32, "gll")]
    for name, prec, learned in legs:
        ksp = dg.KSP(op, m, ksp_type=dg.dKSP_FGMRES, inner_prec=prec, restart=30)
        if learned:
            ksp.set_learned(nets[learned])
        x = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
        try:  # set-up (power iteration, FP32 copies) outside the timed solve
            ksp.solve(b, x, rtol=1e-1, maxit=200)
        except dg.DohpError:
            pass
        x.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        its, _ = ksp.solve(b, x, rtol=1e-8, maxit=5000)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        r = torch.empty_like(x)
        op.mult(x, r)
        applies, rejects, active = ksp.stats()
        out[name] = {"its": its, "wall_s": wall, "true_rel_residual": float(torch.linalg.norm(b - r) / torch.linalg.norm(b)),
                     "correction_dropped": bool(rejects), "correction_active_at_end": active}
    out.update(multigrid_solves(fs, op, m, b))
    if "vertex" in nets:  # the network added to the multigrid preconditioner (trained on Chebyshev-Jacobi pairs)
        ksp = dg.KSP(op, m, ksp_type=dg.dKSP_FGMRES, inner_prec=dg.dPREC_FP32, restart=30, pc=dg.dPC_MG_Q1)
        ksp.set_learned(nets["vertex"])
        x = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
        try:  # set-up outside the timed solve, as the multigrid legs
            ksp.solve(b, x, rtol=1e-1, maxit=50)
        except dg.DohpError:
            pass
        x.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        its, _ = ksp.solve(b, x, rtol=1e-8, maxit=2000)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        r = torch.empty_like(x)
        op.mult(x, r)
        applies, rejects, active = ksp.stats()
        out["learned_multigrid_mixed"] = {"its": its, "wall_s": wall,
                                          "true_rel_residual": float(torch.linalg.norm(b - r) / torch.linalg.norm(b)),
                                          "correction_dropped": bool(rejects), "correction_active_at_end": active}
    out["speedup_vs_plain_fp64"] = {k: out["plain_fp64"]["wall_s"] / out[k]["wall_s"]
                                    for k in ("mixed_fp32", "mixed_bf16", "learned_mixed", "learned_bf16", "learned_fp64",
                                              "learned_gll_mixed", "multigrid_cg_fp64", "multigrid_mixed_fp32",
                                              "learned_multigrid_mixed") if k in out}
    return out


def main():
    args = parse()
    cfg = CONFIGS[args.config]
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, cfg, rank)

    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    import dohp_gb300 as dg
    from dohp_gb300 import build as _b
    _b.build()

    stream = torch.cuda.current_stream()
    fs, op, x, bs = setup(cfg, stream)
    N = fs.n * bs
    y = torch.empty(N, dtype=torch.float64, device="cuda")
    yexp = torch.empty(fs.nexp * bs, dtype=torch.float64, device="cuda")
    forms = {}
    if cfg["hp"]:
        op.autotune(os.path.join(ROOT, "dohp_gb300", "_lib", "autotune.json"))
        op.set_launch(dg.dLAUNCH_PER_ORDER)
        for _ in range(3):
            op.mult(x, y)
        forms["per_order_ms"], _ = time_loop(lambda: op.mult(x, y), max(args.steps // 2, 3), stream)
        op.set_launch(dg.dLAUNCH_PERSISTENT)
        for _ in range(3):
            op.mult(x, y)
        forms["persistent_ms"], _ = time_loop(lambda: op.mult(x, y), max(args.steps // 2, 3), stream)
        _, kms = time_loop(lambda: op.mult_expanded(x, yexp), max(args.steps // 2, 3), stream)
        op.set_launch(dg.dLAUNCH_GRAPH)
        kernel_name = "k_hp_persistent<double,elasticity> (all order buckets)"
    else:
        for _ in range(3):
            op.mult_expanded(x, yexp)
        _, kms = time_loop(lambda: op.mult_expanded(x, yexp), max(args.steps // 2, 3), stream)
        kernel_name = "k_uniform<%d,double,diffusion> (element apply)" % (cfg["p"] + 1)
    for _ in range(max(args.warmup, 3)):
        op.mult(x, y)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    with ClockSampler(local) as clk:
        ms_step, _ = time_loop(lambda: op.mult(x, y), args.steps, stream)
    if cfg["hp"]:
        forms["graph_ms"] = ms_step
    if dist:
        ms_step = max_over_ranks(ms_step, dist)
        dist.barrier()

    # the same apply in float-float arithmetic, reported beside the FP64 headline (not in place of it)
    gpu_results = {}
    ffleg = float_float_leg(op, x, y, args, stream, keep=gpu_results)
    ffleg["value"] = whole_job_gdofs(world, N, ffleg["ms_per_apply"] * 1e-3)

    # end to end through the host-vector entry point (pinned buffers, copies inside the timed region)
    xh = torch.empty(N, dtype=torch.float64).pin_memory()
    yh = torch.empty(N, dtype=torch.float64).pin_memory()
    xh.copy_(x.cpu())
    xn, yn = xh.numpy(), yh.numpy()
    for _ in range(3):
        op.mult_host(xn, yn)
    e2e_steps = max(3, args.steps // 2)
    t_e = time.perf_counter()
    for _ in range(e2e_steps):
        op.mult_host(xn, yn)
    e2e_s = (time.perf_counter() - t_e) / e2e_steps
    if dist:
        e2e_s = max_over_ranks(e2e_s, dist)
    if rank != 0:
        dist.destroy_process_group()
        return

    hbm, src = peaks()
    alg_bytes, alg_flops, issued = work_per_apply(fs, cfg, bs)
    # DRAM bytes per launch of the dominant kernel from one ncu capture (dram__bytes_read.sum +
    # dram__bytes_write.sum) on a smaller case of the same workload, scaled by elements (the traffic is geometry,
    # E map, input and expanded output, all proportional to the element count)
    per_elem = NCU_DRAM_BYTES_PER_ELEMENT.get((cfg["kind"], cfg["hp"], cfg["p"]))
    traffic = per_elem[0] * fs.nelem if per_elem else None
    traffic_src = per_elem[1] if per_elem else "no capture for this workload"

    achieved = alg_bytes / (kms * 1e-3) / 1e9
    value = whole_job_gdofs(world, N, ms_step * 1e-3)
    line = {
        "metric": "GDoF/s operator apply", "value": value, "unit": "GDoF/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded mesh perturbation, orders, field and input)",
        "config": workload_config(cfg, N),
        "arm": {"parallelism": "replicas" if world > 1 else "single GPU",
                "launch": "persistent kernel + restriction in a CUDA graph" if cfg["hp"] else "fused element kernel + restriction"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": traffic, "traffic_source": traffic_src,
                     "peak_source": src + " (MEASURED_PEAKS.json hbm_gbs)", "kernel": kernel_name, "kernel_ms_median": kms,
                     "alg_bytes_per_launch": alg_bytes},
        "fp64_roofline": {"bound": "fp64 pipe", "achieved": issued / (kms * 1e-3) / 1e9, "peak": FP64_PEAK_GFLOPS,
                          "unit": "GFLOP/s", "frac": issued / (kms * 1e-3) / 1e9 / FP64_PEAK_GFLOPS,
                          "issued_flops_per_launch": issued, "alg_flops_per_launch": alg_flops},
        "e2e": {"value": whole_job_gdofs(world, N, e2e_s), "unit": "GDoF/s", "h2d_bytes_per_step": 8 * N, "d2h_bytes_per_step": 8 * N,
                "entry_point": "dOperatorMultHost"},
        "gpu_launches": 2 * args.steps,
        "clocks": clk.summary(),
    }
    line["float_float"] = ffleg
    if cfg["hp"]:
        line["launch_forms"] = forms
        line["tiles"] = op.tiles()
    if not args.no_secondary and args.config == "hp-elasticity-32":
        del fs, op, x, y, yexp
        torch.cuda.empty_cache()
        which = {"apply", "learned", "newton"} if args.secondary == "all" else set(args.secondary.split(","))
        if "multigrid" in which:
            line["multigrid"] = secondary_multigrid(args)
        if "apply" in which:
            line["secondary"] = secondary_lognormal_apply(args)
        if "learned" in which:
            line["time_to_rtol"] = secondary_learned(args)
            torch.cuda.empty_cache()
        if "newton" in which:
            line["newton_mixed_precision"] = secondary_newton(args)
            torch.cuda.empty_cache()
        if "stokes" in which:
            line["stokes_power_law"] = secondary_stokes(args)
            torch.cuda.empty_cache()
    if not args.no_secondary and args.config == "hp-elasticity-32":
        line["time_to_rtol_poisson_8"] = {"workload": "poisson-8^3-p4, mass right-hand side, CG + Q1 Chebyshev(3)-Jacobi, rtol 1e-8",
                                     "gpu": gpu_time_to_rtol_poisson8()}
    if not args.no_cpu_baseline and world == 1:
        line["cpu_baseline"] = cpu_baseline(cfg, os.cpu_count() or 1, compare=gpu_results)
        if "time_to_rtol_poisson_8" in line:
            line["time_to_rtol_poisson_8"]["cpu_oracle"] = cpu_time_to_rtol_poisson8(os.cpu_count() or 1)
    print(json.dumps(line, default=_plain))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
