"""Small fixed workloads for timing and profiling single kernels in isolation:

    python -m dohp_gb300.workloads apply --ne 48 --precision bf16        # scalar Poisson operator applies, degree 4
    python -m dohp_gb300.workloads unet-forward --ne 32 --grid gll      # whole-lattice forwards, (ne*4+1)^3 nodes
    python -m dohp_gb300.workloads unet-train --ne 64 --batch 16         # loss + gradient steps on the vertex lattice
    python -m dohp_gb300.workloads cg --ne 8                             # Poisson CG + Q1 Chebyshev(3)-Jacobi to 1e-8
    python -m dohp_gb300.workloads fgmres --ne 64 --precision fp32       # 2 restart cycles, lognormal Poisson
    python -m dohp_gb300.workloads fgmres --ne 64 --precision fp32 --pc mg   # the same with the Q1 multigrid V-cycle

Seeded random inputs and weights; each workload runs --reps passes after one warm-up pass and prints one JSON line
with the mean time per pass (CUDA events)."""
import argparse
import json

import torch

import dohp_gb300 as dg


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m dohp_gb300.workloads")
    ap.add_argument("workload", choices=["apply", "unet-forward", "unet-train", "cg", "fgmres"])
    ap.add_argument("--ne", type=int, default=32, help="elements per side")
    ap.add_argument("--degree", type=int, default=4)
    ap.add_argument("--precision", choices=["fp64", "fp32", "bf16", "ff"], default="fp64", help="apply workload")
    ap.add_argument("--grid", choices=["vertex", "gll"], default="gll")
    ap.add_argument("--batch", type=int, default=1)
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--tensor-cores", type=int, default=-1, help="1 on, 0 off, -1 the lattice's default")
    ap.add_argument("--pc", choices=["cheb", "mg"], default="cheb", help="fgmres workload: Q1 Chebyshev(3)-Jacobi or Q1 multigrid")
    a = ap.parse_args(argv)
    torch.cuda.set_device(0)
    fs = dg.FS((a.ne + 1,) * 3, degree=a.degree, perturb=0.1, seed=1)
    if a.workload == "apply":
        op = fs.operator()
        op.set_precision({"fp64": dg.dPREC_FP64, "fp32": dg.dPREC_FP32, "bf16": dg.dPREC_BF16, "ff": dg.dPREC_FF}[a.precision])
        gen = torch.Generator(device="cuda").manual_seed(5)
        x = torch.rand(fs.n, dtype=torch.float64, device="cuda", generator=gen) * 2 - 1
        y = torch.zeros_like(x)
        return run(lambda: op.mult(x, y), a, {"workload": "apply", "elements": a.ne ** 3, "degree": a.degree, "dofs": fs.n,
                                               "precision": a.precision})
    if a.workload == "cg":
        return cg(fs, a)
    if a.workload == "fgmres":
        return fgmres(fs, a)
    grid = dg.LEARNED_GRID_GLL if a.grid == "gll" else dg.LEARNED_GRID_VERTEX
    net = dg.Learned(fs, seed=3, grid=grid)
    if a.tensor_cores >= 0:
        net.set_tensor_cores(bool(a.tensor_cores))
    gen = torch.Generator(device="cuda").manual_seed(5)
    x = torch.randn((a.batch, 2) + net.dims, dtype=torch.float32, device="cuda", generator=gen)
    if a.workload == "unet-forward":
        y = torch.zeros((a.batch, 1) + net.dims, dtype=torch.float32, device="cuda")
        step = lambda: net.forward(x, y)
    else:
        t = torch.randn((a.batch, 1) + net.dims, dtype=torch.float32, device="cuda", generator=gen)
        g = torch.zeros(net.nparam, dtype=torch.float32, device="cuda")
        step = lambda: net.loss_grad(x, t, g)
    return run(step, a, {"workload": a.workload, "lattice": list(net.dims), "batch": a.batch, "grid": a.grid})


def cg(fs, a):
    """CG with the Q1 Chebyshev(3)-Jacobi preconditioner on a seeded right-hand side, to rtol 1e-8: the time of a whole
    solve (set-up, first step and the device-looped rest) and, from a second solve cut at 10 iterations on the same
    solver, the time per iteration of the loop alone"""
    gen = torch.Generator(device="cuda").manual_seed(5)
    b = torch.rand(fs.n, dtype=torch.float64, device="cuda", generator=gen) * 2 - 1
    op = fs.operator()
    m = fs.matrix()
    m.assemble()
    ksp = dg.KSP(op, m, ksp_type=dg.dKSP_CG)
    x = torch.zeros_like(b)
    its, rn = ksp.solve(b, x, rtol=1e-8, maxit=1000)  # warm-up: eigenvalue estimate, kernels
    e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    x.zero_()
    e[0].record()
    its, rn = ksp.solve(b, x, rtol=1e-8, maxit=1000)
    e[1].record()
    x.zero_()
    e[2].record()
    try:  # reports non-convergence as an error after its 10 iterations
        ksp.solve(b, x, rtol=1e-8, maxit=10)
    except dg.DohpError:
        pass
    e[3].record()
    its10 = 10
    torch.cuda.synchronize()
    t, t10 = e[0].elapsed_time(e[1]), e[2].elapsed_time(e[3])
    print(json.dumps({"workload": "cg", "elements": a.ne ** 3, "degree": a.degree, "dofs": fs.n, "its": its, "rel_residual": rn,
                      "solve_ms": t, "us_per_iteration": (t - t10) / (its - its10) * 1e3}))


def fgmres(fs, a):
    """FGMRES(30) with the Q1 Chebyshev(3)-Jacobi preconditioner (or the Q1 multigrid V-cycle, --pc mg) and inner
    applies in --precision on the lognormal Poisson problem (field seed 5000), two restart cycles (at most 60
    iterations, fewer when rtol 1e-12 comes first) after one warm-up cycle: ms per iteration"""
    grf = dg.grf_create(64, 2.0, 0.1, 5000)
    kq = torch.empty(fs.nq, dtype=torch.float64, device="cuda")
    fs.lognormal(grf, kq)
    op = fs.operator()
    op.set_qdata(kq)
    m = fs.matrix()
    m.assemble(grf=grf)
    prec = {"fp64": dg.dPREC_FP64, "fp32": dg.dPREC_FP32, "bf16": dg.dPREC_BF16, "ff": dg.dPREC_FF}[a.precision]
    pc = dg.dPC_MG_Q1 if a.pc == "mg" else dg.dPC_CHEBYSHEV_Q1
    ksp = dg.KSP(op, m, ksp_type=dg.dKSP_FGMRES, inner_prec=prec, restart=30, pc=pc)
    gen = torch.Generator(device="cuda").manual_seed(5)
    b = torch.rand(fs.n, dtype=torch.float64, device="cuda", generator=gen) * 2 - 1
    x = torch.zeros_like(b)

    def cycles(k):
        x.zero_()
        try:  # stops at maxit before the tolerance: reported as an error
            return ksp.solve(b, x, rtol=1e-12, maxit=30 * k)[0]
        except dg.DohpError:
            return 30 * k

    cycles(1)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    its = cycles(2)
    e1.record()
    torch.cuda.synchronize()
    print(json.dumps({"workload": "fgmres", "elements": a.ne ** 3, "dofs": fs.n, "precision": a.precision, "pc": a.pc,
                      "iterations": its, "ms_per_iteration": e0.elapsed_time(e1) / its}))


def run(step, a, info):
    step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(a.reps):
        step()
    e1.record()
    torch.cuda.synchronize()
    info["ms_per_pass"] = e0.elapsed_time(e1) / a.reps
    print(json.dumps(info))


if __name__ == "__main__":
    main()
