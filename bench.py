"""Benchmark: GDoF/s of the matrix-free hp-FEM operator apply (dohp's EllipShellMatMult) on one GB300.

Workload (default, --config cfg4): variable-coefficient Poisson -div(k grad u) on a 64^3 structured hex
mesh of the unit cube, interior vertices perturbed U[-0.1h, 0.1h] (seed 1), uniform p=4 on GLL nodes with
Gauss (p+1)^3 quadrature, k = exp(g) with g a lognormal random field (variance 2, correlation length 0.1,
random Fourier features, seed 2), homogeneous Dirichlet on all walls, FP64. 16,581,375 explicit dofs.
A step is one operator apply y = A x (gather through E, element kernel, deterministic E^T restrict) on a
seeded x ~ U[-1,1]. Inputs (x 133 MB, geometric factors 1.57 GB, E map 131 MB) exceed the 129 MB L2, so
no flush is needed between steps.

Prints one JSON line (see the contract in the repository docs): value = explicit dofs / seconds per apply,
device-timed with CUDA events on the launching stream; e2e = the same apply through dOperatorMultHost
(host buffers, H2D and D2H copies inside the timed region); roofline of the dominant (element) kernel;
cpu_baseline = the oracle's CPU restatement of the reference apply on the host cores.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIGS = {
    # name: (elements per direction, degree, lognormal coefficient)
    "cfg4": dict(ne=64, p=4, grf=True, label="poisson-lognormal-64^3-p4"),
    "cfg1": dict(ne=8, p=4, grf=False, label="poisson-8^3-p4"),
    # reduced case of the same kernel for full ncu captures (geometric factors 196 MB, above L2)
    "cfg4_32": dict(ne=32, p=4, grf=True, label="poisson-lognormal-32^3-p4"),
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="cfg4", choices=sorted(CONFIGS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
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
    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, index):
        self.index = index
        self.proc = None

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
        self.lines = []
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            out, _ = self.proc.communicate(timeout=5)
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
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
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


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


def cpu_baseline(cfg, threads, budget_s=20.0):
    """Oracle (CPU restatement of the reference apply: per-element geometry recompute, INTERP+GRAD,
    q-function, INTERP_T+GRAD_T, E/E^T) timed on a bounded sample of the workload: a 32^3-element block
    of the same order and coefficient kind, all host threads (OpenMP)."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    po.build()
    ne = min(cfg["ne"], 32)
    fs = po.FS(ne + 1, ne + 1, ne + 1, degree=cfg["p"], perturb=0.1, seed=1)
    qd = None
    if cfg["grf"]:
        grf = po.grf_make(64, 2.0, 0.1, 2)
        qd = grf_numpy(grf, fs.qpt_coords())
    x = np.random.default_rng(0).uniform(-1, 1, fs.n)
    fs.apply(x, qdata=qd, nthreads=threads)  # warm-up
    times = []
    t_start = time.perf_counter()
    while len(times) < 3 or (time.perf_counter() - t_start < budget_s and len(times) < 10):
        t0 = time.perf_counter()
        fs.apply(x, qdata=qd, nthreads=threads)
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - t_start > budget_s:
            break
    times.sort()
    t = times[len(times) // 2]
    return {"value": fs.n / t / 1e9, "unit": "GDoF/s", "cores": threads, "kind": "port",
            "sample": "%d^3 elements p=%d (%d dofs), median of %d applies, oracle C restatement, %d OpenMP threads"
                      % (ne, cfg["p"], fs.n, len(times), threads)}


def run_reference(args, cfg, rank):
    threads = os.cpu_count() or 1
    if rank != 0:
        return
    cb = cpu_baseline(cfg, threads, budget_s=max(10.0, min(60.0, 3.0 * args.steps)))
    line = {"impl": "reference", "metric": "GDoF/s operator apply", "value": cb["value"], "unit": "GDoF/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": cfg["label"] + " (bounded CPU sample)", "parallelism": "host threads"},
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "GDoF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    args = parse()
    cfg = CONFIGS[args.config]
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, cfg, rank)

    import numpy as np
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
    ne, p = cfg["ne"], cfg["p"]
    fs = dg.FS((ne + 1,) * 3, degree=p, perturb=0.1, seed=1, stream=stream.cuda_stream)
    op = fs.operator(dg.dOP_DIFFUSION)
    if cfg["grf"]:
        grf = dg.grf_create(64, 2.0, 0.1, 2)
        kq = torch.empty(fs.nq, dtype=torch.float64, device="cuda")
        fs.lognormal(grf, kq)
        op.set_qdata(kq)
    x = torch.as_tensor(np.random.default_rng(0).uniform(-1, 1, fs.n), device="cuda")
    y = torch.empty(fs.n, dtype=torch.float64, device="cuda")
    yexp = torch.empty(fs.nexp, dtype=torch.float64, device="cuda")

    def step():
        op.mult_expanded(x, yexp)
        fs.expanded_to_global(yexp, y)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True); t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for a, b, c in ev:
            a.record(stream)
            op.mult_expanded(x, yexp)
            b.record(stream)
            fs.expanded_to_global(yexp, y)
            c.record(stream)
        t1.record(stream)
        torch.cuda.synchronize()
        # keep the sampler alive over a comparable window for the e2e loop below
    total_ms = t0.elapsed_time(t1)
    kern_ms = sorted(a.elapsed_time(b) for a, b, _ in ev)
    rest_ms = sorted(b.elapsed_time(c) for _, b, c in ev)
    ms_step = total_ms / args.steps
    if dist:
        t = torch.tensor([ms_step], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_step = float(t.item())
        dist.barrier()

    # end to end through the host-vector entry point (pinned buffers, copies inside the timed region)
    xh = torch.empty(fs.n, dtype=torch.float64).pin_memory()
    yh = torch.empty(fs.n, dtype=torch.float64).pin_memory()
    xh.copy_(x.cpu())
    xn, yn = xh.numpy(), yh.numpy()
    for _ in range(3):
        op.mult_host(xn, yn)
    torch.cuda.synchronize()
    e2e_steps = max(3, args.steps // 2)
    t_e = time.perf_counter()
    for _ in range(e2e_steps):
        op.mult_host(xn, yn)
    e2e_s = (time.perf_counter() - t_e) / e2e_steps
    if dist:
        t = torch.tensor([e2e_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())

    if rank != 0:
        dist.destroy_process_group()
        return
    hbm, src = peaks()
    nelem = fs.nelem
    closure_dofs = fs.nc  # (64*4+1)^3 nodes incl. Dirichlet
    alg_bytes = 16.0 * closure_dofs + nelem * (4.0 * (p + 1) ** 3 + 192.0)  # survey algorithmic figure per apply
    n1 = p + 1
    alg_flops = nelem * (36.0 * n1 ** 4 + 30.0 * n1 ** 3)
    kmed = kern_ms[len(kern_ms) // 2]
    achieved = alg_bytes / (kmed * 1e-3) / 1e9
    fp64_peak = 1203.0  # GFLOP/s: FP64 FMA issue rate measured on this GB300 by an FMA-chain probe
    actual_flops = nelem * (2 * 12.0 * n1 ** 4 + 2 * 9.0 * n1 ** 3)  # FLOPs the kernel issues (collocation form)
    clocks = clk.summary()
    value = world * fs.n / (ms_step * 1e-3) / 1e9
    line = {
        "metric": "GDoF/s operator apply", "value": value, "unit": "GDoF/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded mesh perturbation, seeded field and input)",
        "config": {"workload": cfg["label"], "elements": nelem, "degree": p, "dofs": fs.n, "closure_dofs": closure_dofs,
                   "quadrature": "Gauss (p+1)^3", "l2": "inputs larger than L2 (1.8 GB per apply), no flush",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": None, "peak_source": src + " (MEASURED_PEAKS.json hbm_gbs)",
                     "kernel": "k_diffusion<5,double> (element apply)", "kernel_ms_median": kmed,
                     "alg_bytes_per_launch": alg_bytes},
        "fp64_roofline": {"bound": "fp64 pipe", "achieved": actual_flops / (kmed * 1e-3) / 1e9, "peak": fp64_peak,
                          "unit": "GFLOP/s", "frac": actual_flops / (kmed * 1e-3) / 1e9 / fp64_peak,
                          "alg_flops_per_launch": alg_flops, "issued_flops_per_launch": actual_flops,
                          "alg_gflops_per_s": alg_flops / (kmed * 1e-3) / 1e9},
        "restrict_ms_median": rest_ms[len(rest_ms) // 2],
        "e2e": {"value": world * fs.n / e2e_s / 1e9, "unit": "GDoF/s", "h2d_bytes_per_step": 8 * fs.n,
                "d2h_bytes_per_step": 8 * fs.n, "entry_point": "dOperatorMultHost"},
        "gpu_launches": 2 * args.steps,
        "clocks": clocks,
    }
    if not args.no_cpu_baseline and world == 1:
        line["cpu_baseline"] = cpu_baseline(cfg, os.cpu_count() or 1)
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
