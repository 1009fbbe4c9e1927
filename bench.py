#!/usr/bin/env python3
"""AMG-PCG benchmark: DOF/s to 1e-8 relative residual on one GB300.

Workload (one "step" = one pass of the hot path): AMG setup (OldMIS aggregation,
smoothed prolongator, Galerkin RAP) + flexible PCG to ||r||/||b|| <= 1e-8 on the
3D Poisson problem on the unit cube, 128^3 cells Kuhn-split into 12,582,912 P1
tets (2,146,689 vertices), kappa_e = exp(2 g_e), g ~ N(0,1) (seed 4), f ~ U[-1,1]
(seed 5), u = 0 on z = 0.  value = free DOF x steps / device time (inputs in HBM);
e2e = the same through femgpu_setup + femgpu_solve with host b/x buffers.

--precision mixed (default): FP32 hierarchy inside the FP64 outer PCG;
--precision fp64: the same code with an FP64 hierarchy.
--impl reference: the reference algorithm's CPU restatement (oracle) on host cores.
--workload batched: 64^3 mesh with 64 seeded right-hand sides solved with one hierarchy
  (femgpu_solve_multi: eight columns at a time in lockstep PCGs with block kernels);
  reports right-hand-side DOF/s, beside the same columns solved one at a time.
--workload meshes: 48 independent cubes of 12^3..40^3 cells (seeded sizes), each with its own
  log-normal coefficient, set up and solved together through femgpu_solve_batch.
--workload differentiation: 96^3 mesh, theta_e = log kappa_e ~ N(0,1), loss over a 1%
  vertex subset; forward solve + adjoint gradient (femgpu_adjoint_grad) timed, gradient
  compared with the FP64-hierarchy gradient solved to 1e-12.
Only the default workload is the headline line.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "sci-solver_fem_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import numpy as np  # noqa: E402

METRIC = "AMG-PCG DOF/s to 1e-8 rel-resid, mixed vs FP64 on 1 GB300; SpMV HBM GB/s"
UNIT = "DOF/s"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def problem(n, sigma):
    from femgpu import meshes
    return meshes.poisson3d_problem(n, sigma=sigma, kappa_seed=4, f_seed=5)


def cpu_problem(n_sample, sigma):
    """The operator, right-hand side and aggregation graph of the workload, built by the oracle."""
    import oracle as O
    from femgpu import meshes
    xyz, conn, kappa, f, mask = problem(n_sample, sigma)
    rp, ci = O.build_pattern(xyz.shape[0], conn)
    v = O.assemble(xyz, conn, rp, ci, coef=kappa, lambda_mass=0.0)
    b = O.load_vector(xyz, conn, f)
    v, b = O.apply_dirichlet(rp, ci, v, mask, b)
    gx, ga = meshes.adjacency_from_pattern(rp, ci)
    return dict(rp=rp, ci=ci, v=v, b=b, gx=gx, ga=ga, free=int(xyz.shape[0] - mask.sum()))


def workload_config(n, sigma, dofs, free, elements, nnz, precision):
    """The `config` of a bench line: the same for the GPU arm and the reference arm."""
    return {"workload": f"poisson3d_kuhn_{n}^3_sigma{sigma:g}", "dofs": int(dofs), "free_dofs": int(free),
            "elements": int(elements), "nnz": int(nnz), "precision": precision, "tolerance": 1e-8,
            "l2": "inputs larger than L2 (A: %.0f MB)" % (12 * nnz / 1e6)}


def cpu_baseline_run(prob, threads, fp64=False):
    """The reference algorithm restated on the CPU (oracle), timed on host cores:
    AMG setup + flexible PCG to 1e-8 on a prebuilt problem."""
    import oracle as O
    t0 = time.perf_counter()
    amg = O.OracleAMG(prob["rp"], prob["ci"], prob["v"], prob["gx"], prob["ga"], seed=1, threads=threads,
                      fp64_hierarchy=1 if fp64 else 0)
    x, st = amg.pcg(prob["b"], tol=1e-8, max_iters=500, flexible=True)
    dt = time.perf_counter() - t0
    return prob["free"] / dt, dt, st


def cpu_baseline(n_sample, sigma, threads):
    return cpu_baseline_run(cpu_problem(n_sample, sigma), threads)


def run_batched(args):
    """64^3 mesh, 64 right-hand sides, one hierarchy: setup + 64 PCG solves per step."""
    import torch
    import femgpu
    xyz, conn, kappa, f, mask = problem(64, 1.0)
    n = xyz.shape[0]
    free = int(n - mask.sum())
    s = femgpu.Solver(solverType=1, tolerance=1e-8, maxIters=500, flexibleCG=1, seed=1)
    s.set_mesh(xyz, conn)
    s.assemble(kappa, 0.0)
    s.set_dirichlet(mask)
    rng = np.random.default_rng(6)
    k = 64
    B = np.stack([np.where(mask.astype(bool), 0.0, s.load_vector(rng.uniform(-1.0, 1.0, n))) for _ in range(k)])
    dB = torch.from_numpy(B).cuda()  # k x n: column j of the solve is row j here
    dX = torch.zeros_like(dB)
    times, iters = [], []
    for step in range(args.warmup + args.steps):
        dX.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.setup()
        st = s.solve_multi_device(k, dB.data_ptr(), n, dX.data_ptr(), n)
        torch.cuda.synchronize()
        if step >= args.warmup:
            times.append(time.perf_counter() - t0)
            iters.append(st["iterations"])
    dt = float(np.mean(times))
    # the same 64 columns one at a time (single-column solves on the same hierarchy)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s.setup()
    it1 = 0
    for j in range(k):
        dX[j].zero_()
        it1 += s.solve_device(dB[j].data_ptr(), dX[j].data_ptr())["iterations"]
    torch.cuda.synchronize()
    dt1 = time.perf_counter() - t0
    rp, ci, _ = s.matrix()
    out = {"metric": "batched AMG-PCG right-hand-side DOF/s (64 RHS, one hierarchy)", "value": k * free / dt,
           "unit": "DOF*RHS/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt,
           "higher_is_better": True, "dtype": "f64+f32", "data": "synthetic",
           "config": {"workload": "poisson3d_kuhn_64^3_64rhs", "dofs": n, "free_dofs": free, "nrhs": k,
                      "block": 8},
           "pcg_iterations_total": int(np.mean(iters)), "relres_max": st["relres"],
           "outer_operator_reads_per_rhs_iteration": 1.0 / 8.0,
           "outer_operator_bytes_per_rhs_iteration": 12.0 * ci.shape[0] / 8.0,
           "single_column_solves_ms": 1e3 * dt1, "single_column_iterations_total": it1,
           "speedup_vs_single_column_solves": dt1 / dt}
    print(json.dumps(out))


def run_meshes(args):
    """48 independent cubes of 12^3..40^3 cells (sizes seeded), each with its own log-normal
    coefficient: setup + PCG of all of them per step through femgpu_solve_batch."""
    import femgpu
    from femgpu import meshes
    sizes = np.random.default_rng(7).integers(12, 41, size=48)
    solvers, bs, free = [], [], 0
    for i, m in enumerate(sizes):
        xyz, conn, kappa, f, mask = meshes.poisson3d_problem(int(m), sigma=1.0, kappa_seed=8 + i, f_seed=1000 + i)
        s = femgpu.Solver(solverType=1, tolerance=1e-8, maxIters=500, flexibleCG=1, seed=1)
        s.set_mesh(xyz, conn)
        s.assemble(kappa, 0.0)
        s.set_dirichlet(mask)
        bs.append(np.where(mask.astype(bool), 0.0, s.load_vector(f)))
        solvers.append(s)
        free += int(xyz.shape[0] - mask.sum())

    def timed(threads):
        times, iters, worst, setup_ms, solve_ms = [], 0, 0.0, 0.0, 0.0
        for step in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            xs, stats, _ = femgpu.solve_batch(solvers, bs, threads=threads)
            dt = time.perf_counter() - t0
            if step >= args.warmup:
                times.append(dt)
                iters = sum(t["iterations"] for t in stats)
                worst = max(t["relres"] for t in stats)
                setup_ms = sum(t["setup_ms"] for t in stats)
                solve_ms = sum(t["solve_ms"] for t in stats)
        return float(np.mean(times)), iters, worst, setup_ms, solve_ms

    dt, iters, worst, setup_sum, solve_sum = timed(0)
    dt1, _, _, setup1, solve1 = timed(1)
    out = {"metric": "DOF/s over a batch of independent meshes (setup + PCG to 1e-8 each)", "value": free / dt,
           "unit": "DOF/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt,
           "higher_is_better": True, "dtype": "f64+f32", "data": "synthetic",
           "config": {"workload": "poisson3d_kuhn_48_meshes_12^3..40^3", "meshes": len(solvers),
                      "cells_per_edge": [int(m) for m in sizes], "free_dofs": free,
                      "timing": "host wall clock around the synchronous batch call"},
           "one_host_thread_ms_per_step": 1e3 * dt1, "pcg_iterations_total": iters, "relres_max": worst,
           "device_ms_summed_over_meshes": {"setup": setup_sum, "solve": solve_sum,
                                            "setup_one_thread": setup1, "solve_one_thread": solve1}}
    print(json.dumps(out))


def run_differentiation(args):
    """96^3 mesh: forward solve + adjoint gradient per step (mixed precision, PCG to 1e-10);
    the gradient is compared with the FP64-hierarchy gradient solved to 1e-12 and with
    central differences (h = 1e-6) on 32 seeded elements."""
    import torch
    import femgpu
    from femgpu import gradcheck, meshes
    xyz, conn = meshes.kuhn_cube(96)
    n, ne = xyz.shape[0], conn.shape[0]
    mask = (xyz[:, 2] == 0.0).astype(np.uint8)
    rng = np.random.default_rng(9)
    theta = rng.standard_normal(ne)
    S = np.random.default_rng(10).choice(n, n // 100, replace=False)
    theta_obs = np.random.default_rng(11).standard_normal(ne)
    f = np.random.default_rng(5).uniform(-1.0, 1.0, n)
    tol = 1e-10

    def forward(th, precision, tol):
        s = femgpu.Solver(solverType=1, tolerance=tol, maxIters=3000, flexibleCG=1, seed=1, precision=precision)
        s.set_mesh(xyz, conn)
        b = np.where(mask.astype(bool), 0.0, s.load_vector(f))
        s.assemble(np.exp(th), 0.0)
        s.set_dirichlet(mask)
        s.setup()
        u, st = s.solve(b)
        return s, u, b

    s_obs, u_obs, _ = forward(theta_obs, 1, 1e-12)
    s_obs.close()
    times, fwd_ms, adj_ms = [], [], []
    for step in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s, u, b = forward(theta, 0, tol)
        t1 = time.perf_counter()
        r = np.zeros(n)
        r[S] = u[S] - u_obs[S]
        g, st = s.adjoint_grad(r, u)
        t2 = time.perf_counter()
        if step >= args.warmup:
            times.append(t2 - t0)
            fwd_ms.append(1e3 * (t1 - t0))
            adj_ms.append(1e3 * (t2 - t1))
        s.close()
    # FP64 hierarchy, 1e-12 forward and adjoint: the reference gradient
    sr, ur, _ = forward(theta, 1, 1e-12)
    rr = np.zeros(n)
    rr[S] = ur[S] - u_obs[S]
    gr, _ = sr.adjoint_grad(rr, ur)
    sr.close()
    rel = float(np.linalg.norm(g - gr) / np.linalg.norm(gr))
    elems = np.random.default_rng(12).choice(ne, 32, replace=False)
    t_fd = time.perf_counter()
    fd = gradcheck.central_differences(xyz, conn, theta, mask, b, S, u_obs, elems, h=1e-6)
    t_fd = time.perf_counter() - t_fd
    fd_rel = float(np.linalg.norm(fd - g[elems]) / np.linalg.norm(fd))
    out = {"metric": "forward + adjoint gradient wall time (96^3, mixed precision)",
           "value": 1e3 * float(np.mean(times)), "unit": "ms", "higher_is_better": False, "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "data": "synthetic",
           "config": {"workload": "poisson3d_kuhn_96^3_adjoint", "dofs": n, "elements": ne, "observed": len(S),
                      "tolerance": tol},
           "forward_ms": float(np.mean(fwd_ms)), "adjoint_ms": float(np.mean(adj_ms)),
           "gradient_rel_error_vs_fp64_1e-12": rel,
           "central_differences": {"elements": len(elems), "h": 1e-6, "rel_error_vs_adjoint": fd_rel,
                                   "seconds": round(t_fd, 1),
                                   "how": "(L(theta+h) - L(theta-h)) / 2h with u+ - u- = -A+^-1 (A+ - A-) u-, "
                                          "FP64-hierarchy solves to 1e-12"}}
    print(json.dumps(out))


def run_reference(args):
    """--impl reference: the reference's algorithm on the host cores (oracle port)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = len(os.sched_getaffinity(0))
    n_sample = args.cpu_sample
    prob = cpu_problem(n_sample, args.sigma)
    fp64 = args.precision == "fp64"
    for _ in range(args.warmup):
        cpu_baseline_run(prob, threads, fp64)
    vals, times = [], []
    for _ in range(args.steps):
        v, dt, st = cpu_baseline_run(prob, threads, fp64)
        vals.append(v)
        times.append(dt)
    value = float(np.mean(vals))
    what = "the full workload" if n_sample == args.n else "a sample of the same Poisson problem family"
    sample = (f"{n_sample}^3-cell Kuhn tet mesh, {what} ({(n_sample + 1) ** 3} vertices), "
              f"AMG setup + PCG to 1e-8 per step, {threads} threads")
    ne = 6 * n_sample ** 3
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(times)),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64+f32" if args.precision == "mixed" else "f64", "data": "synthetic",
           "config": workload_config(n_sample, args.sigma, prob["rp"].shape[0] - 1, prob["free"], ne,
                                     int(prob["ci"].shape[0]), args.precision),
           "execution": f"CPU oracle (the reference algorithm restated), {threads} host threads",
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=128, help="cells per cube edge")
    ap.add_argument("--sigma", type=float, default=2.0)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--cpu-sample", type=int, default=128,
                    help="cells per edge of the CPU oracle's problem (default: the full 128^3 workload)")
    ap.add_argument("--cpu-sample-1t", type=int, default=48,
                    help="cells per edge of the single-thread CPU sample (0: skip)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="poisson", choices=["poisson", "batched", "meshes", "differentiation"])
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload == "batched":
        run_batched(args)
        return
    if args.workload == "meshes":
        run_meshes(args)
        return
    if args.workload == "differentiation":
        run_differentiation(args)
        return

    import torch
    import femgpu

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    # ---- problem (replicas only: each rank solves its own copy) -------------------
    xyz, conn, kappa, f, mask = problem(args.n, args.sigma)
    n = xyz.shape[0]
    free = int(n - mask.sum())
    stream = torch.cuda.Stream()  # the solver and every torch op below share this stream
    torch.cuda.set_stream(stream)
    prec = 0 if args.precision == "mixed" else 1
    s = femgpu.Solver(solverType=1, tolerance=1e-8, maxIters=500, flexibleCG=1, seed=1, precision=prec,
                      device=local, stream=stream.cuda_stream)
    t_asm0 = time.perf_counter()
    s.set_mesh(xyz, conn)
    s.assemble(kappa, 0.0)
    b = s.load_vector(f)
    s.set_dirichlet(mask)
    b[mask.astype(bool)] = 0.0
    torch.cuda.synchronize()
    assembly_ms = 1e3 * (time.perf_counter() - t_asm0)

    d_b = torch.from_numpy(b).cuda()
    d_x = torch.zeros(n, dtype=torch.float64, device="cuda")

    def step():
        s.setup()
        d_x.zero_()
        return s.solve_device(d_b.data_ptr(), d_x.data_ptr())

    for _ in range(args.warmup):
        st = step()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = femgpu.kernel_launches()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    iters, setup_ms, solve_ms = [], [], []
    for _ in range(args.steps):
        st = step()
        iters.append(st["iterations"])
        setup_ms.append(st["setup_ms"])
        solve_ms.append(st["solve_ms"])
    e1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    launches = femgpu.kernel_launches() - launches0
    ms = e0.elapsed_time(e1) / args.steps
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    relres = st["relres"]
    value = world * free / (ms / 1e3)

    # ---- end to end through the C ABI with host buffers ---------------------------
    # page-locked host buffers (numpy views of pinned torch tensors), so the copies inside
    # the timed region are the DMA transfers a caller streaming right-hand sides would use
    b_h = torch.from_numpy(b).pin_memory().numpy()
    x_h = torch.zeros(n, dtype=torch.float64).pin_memory().numpy()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        s.setup()
        x_h[:] = 0.0  # the initial guess
        x_h, st2 = s.solve(b_h, out=x_h)  # in place, as femgpu_solve
    e2e_ms = 1e3 * (time.perf_counter() - t0) / args.steps
    e2e = {"value": world * free / (e2e_ms / 1e3), "unit": UNIT, "h2d_bytes_per_step": 16 * n,
           "d2h_bytes_per_step": 8 * n}
    clk = clocks.stop()

    # ---- the same workload with the FP64 hierarchy (the metric's "mixed vs FP64" half):
    # same problem, same stream, same timing; one solver per precision
    s64 = femgpu.Solver(solverType=1, tolerance=1e-8, maxIters=500, flexibleCG=1, seed=1, precision=1,
                        device=local, stream=stream.cuda_stream)
    s64.set_mesh(xyz, conn)
    s64.assemble(kappa, 0.0)
    s64.set_dirichlet(mask)
    d_x64 = torch.zeros(n, dtype=torch.float64, device="cuda")

    def step64():
        s64.setup()
        d_x64.zero_()
        return s64.solve_device(d_b.data_ptr(), d_x64.data_ptr())

    for _ in range(args.warmup):
        step64()
    torch.cuda.synchronize()
    e0.record(stream)
    st64s = [step64() for _ in range(args.steps)]
    e1.record(stream)
    torch.cuda.synchronize()
    ms64 = e0.elapsed_time(e1) / args.steps
    fp64 = {"ms_per_step": ms64, "value": world * free / (ms64 / 1e3), "unit": UNIT,
            "setup_ms": float(np.mean([t["setup_ms"] for t in st64s])),
            "solve_ms": float(np.mean([t["solve_ms"] for t in st64s])),
            "pcg_iterations": st64s[-1]["iterations"], "relres": st64s[-1]["relres"]}
    s64.close()

    # ---- the same workload with the l1-Jacobi performance smoother (2 sweeps per relax)
    sl1 = femgpu.Solver(solverType=1, tolerance=1e-8, maxIters=500, flexibleCG=1, seed=1, precision=prec,
                        smoother=1, preInnerIters=2, postInnerIters=2, device=local, stream=stream.cuda_stream)
    sl1.set_mesh(xyz, conn)
    sl1.assemble(kappa, 0.0)
    sl1.set_dirichlet(mask)
    d_xl1 = torch.zeros(n, dtype=torch.float64, device="cuda")

    def step_l1():
        sl1.setup()
        d_xl1.zero_()
        return sl1.solve_device(d_b.data_ptr(), d_xl1.data_ptr())

    for _ in range(args.warmup):
        step_l1()
    torch.cuda.synchronize()
    e0.record(stream)
    stl1 = [step_l1() for _ in range(args.steps)]
    e1.record(stream)
    torch.cuda.synchronize()
    msl1 = e0.elapsed_time(e1) / args.steps
    l1_arm = {"ms_per_step": msl1, "value": world * free / (msl1 / 1e3), "unit": UNIT,
              "setup_ms": float(np.mean([t["setup_ms"] for t in stl1])),
              "solve_ms": float(np.mean([t["solve_ms"] for t in stl1])),
              "pcg_iterations": stl1[-1]["iterations"], "relres": stl1[-1]["relres"],
              "options": "smoother=1 (l1-Jacobi), preInnerIters=postInnerIters=2"}
    sl1.close()

    # ---- rooflines: each hot kernel timed with CUDA events on the solver's stream by the
    # library (femgpu_profile_kernel).  The V-cycle's level-0 post-smoother is timed as a
    # PCG iteration runs it (selector 5); the dominant kernel has the largest time per
    # launch among those that run once per PCG iteration.
    peak, peak_kind = peaks()
    rp, ci, _ = s.matrix()
    nnz = int(ci.shape[0])
    cfg = workload_config(args.n, args.sigma, n, free, conn.shape[0], nnz, args.precision)
    traffic, traffic_cmd = {}, None
    tpath = os.path.join(ROOT, "profiles", "dram_traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as fh:
            tr = json.load(fh)
        # measured DRAM bytes per launch apply only to the configuration they were taken on
        key = f"{cfg['workload']}_{args.precision}"
        traffic = tr.get("per_launch", {}).get(key, {})
        traffic_cmd = tr.get("commands", {}).get(key)
    rooflines = []
    for which in (0, 1, 5, 3, 4, 6, 7):
        name = femgpu.Solver.KERNELS[which]
        kms, kbytes = s.profile_kernel(which, reps=20)
        ach = kbytes / (kms / 1e3) / 1e9
        entry = {"bound": "hbm", "kernel": name, "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
                 "frac": round(ach / peak, 4), "traffic": traffic.get(name), "peak_source": peak_kind,
                 "algorithmic_bytes": kbytes, "ms": round(kms, 4),
                 "per": "assembly" if which >= 6 else "PCG iteration"}
        fp64_pipe = traffic.get("_fp64_pipe_active", {}).get(name)
        if fp64_pipe is not None:  # ncu sm__pipe_fp64_cycles_active of the same kernel
            entry["fp64_pipe_active"] = fp64_pipe
        rooflines.append(entry)
    roofline = max((r for r in rooflines if r["per"] == "PCG iteration"), key=lambda r: r["ms"])
    assembly_device_ms = sum(r["ms"] for r in rooflines if r["per"] == "assembly")

    # final error of the timed solve against an FP64-hierarchy PCG solved to 1e-12
    x_mixed = d_x.cpu().numpy()
    ref = femgpu.Solver(solverType=1, tolerance=1e-12, maxIters=2000, flexibleCG=1, seed=1, precision=1,
                        device=local)
    ref.set_matrix_csr(rp, ci, s.matrix()[2])
    ref.setup()
    x_ref, st_ref = ref.solve(b, np.zeros(n))
    final_error = float(np.linalg.norm(x_mixed - x_ref) / np.linalg.norm(x_ref))
    ref.close()

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = len(os.sched_getaffinity(0))
        v, dt, _ = cpu_baseline(args.cpu_sample, args.sigma, threads)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{args.cpu_sample}^3-cell Kuhn mesh of the same problem ({(args.cpu_sample + 1) ** 3} "
                         f"vertices{', the full workload' if args.cpu_sample == args.n else ''}), oracle AMG setup + "
                         f"PCG to 1e-8, {dt:.1f} s"}
        if args.cpu_sample_1t > 0:  # the same algorithm on one core, on a bounded sample
            v1, dt1, _ = cpu_baseline(args.cpu_sample_1t, args.sigma, 1)
            cpu["single_thread"] = {"value": v1, "unit": UNIT, "cores": 1,
                                    "sample": f"{args.cpu_sample_1t}^3-cell Kuhn mesh of the same problem "
                                              f"({(args.cpu_sample_1t + 1) ** 3} vertices), {dt1:.1f} s"}

    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f64+f32" if prec == 0 else "f64", "data": "synthetic",
               "config": cfg, "execution": "replicas" if world > 1 else "1 GPU",
               "pcg_iterations": iters[-1], "relres": relres, "setup_ms": float(np.mean(setup_ms)),
               "solve_ms": float(np.mean(solve_ms)), "assembly_ms": assembly_ms,
               "assembly_device_ms": assembly_device_ms,
               "fp64_hierarchy": fp64, "mixed_speedup_vs_fp64": fp64["ms_per_step"] / ms if prec == 0 else None,
               "l1_jacobi_smoother": l1_arm,
               "error_vs_fp64_1e-12": final_error, "fp64_1e-12_iterations": st_ref["iterations"],
               "e2e": e2e, "gpu_launches": int(launches), "roofline": roofline, "rooflines": rooflines,
               "traffic_source": traffic_cmd, "cpu_baseline": cpu, "clocks": clk}
        print(json.dumps(out))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
