#!/usr/bin/env python3
"""Benchmark: time to solve the 257^3-node cubic polycrystal to 1e-8 FP64
relative residual on one GB300, plus the dominant kernel's roofline.

Workload (seeded, synthetic; no dataset): 256^3 cells on the unit cube, 64
Voronoi grains with uniformly random orientations of cubic C11=1.68,
C12=1.21, C44=0.75; TensionTest uniaxial_stress with u_x = 0.01 on +x.

One step = one full solve from u = 0 through the C ABI (prepareForSolve +
MLMG iterations), run as FP32 cycles inside FP64 iterative refinement.  The
plain FP64 multigrid solve of the same system is timed once beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`--impl reference` times one complete solve of the same system by the CPU
restatement of the reference algorithm (oracle/, FP64 MLMG F-cycles, OpenMP on
every host core), split over the timed steps.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Solve s @257^3 nodes to 1e-8 FP64 residual, learned+FP32 vs plain; Fapply GB/s"
WORKLOAD = ("257^3-node cubic Voronoi polycrystal (64 grains, C11/C12/C44 = 1.68/1.21/0.75), "
            "uniaxial tension u_x=0.01, solve to 1e-8 relative FP64 residual")
BYTES_PER_NODE = {"jacobi_f32_cubic": 132, "fapply_f32_cubic": 108, "jacobi_f64_cubic": 264,
                  "fapply_f64_cubic": 216}
# FP64 operations of one interior node of the damped-Jacobi sweep on cubic
# cells (an FMA counts 2), counted by ncu on the marching kernel (DFMA, DADD,
# DMUL thread instructions over the interior nodes of one 65^3 launch:
# 98 + 129 + 26)
FLOPS_PER_NODE = {"jacobi_f64_cubic": 351, "fapply_f64_cubic": 339}   # Fapply: 95 + 126 + 23


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=256, help="cells per direction")
    ap.add_argument("--grains", type=int, default=64)
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 solve")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-rve", action="store_true", help="c2: skip the batched RVE measurement of the line")
    ap.add_argument("--cycle", default="F", choices=["F", "V"])
    ap.add_argument("--krylov", type=int, default=8,
                    help="c2, rve: stored directions of the flexible GCR over the FP32 cycle (0: the FP32 cycles alone)")
    ap.add_argument("--omega", type=float, default=-1.0,
                    help="c2: Jacobi damping of the FP32 cycles (< 0: the operator's 2/3)")
    ap.add_argument("--pre", type=int, default=2, help="c2: Fsmooth calls before restriction in the FP32 cycles")
    ap.add_argument("--post", type=int, default=2, help="c2: Fsmooth calls after prolongation in the FP32 cycles")
    ap.add_argument("--workload", default="c2", choices=["c2", "rve", "learned", "sweep", "conv"],
                    help="c2: the 257^3 polycrystal (default); rve: batched periodic RVEs; learned: the learned "
                         "correction trained on 64^3 polycrystals and evaluated on the c2 system at 129^3 and 257^3; sweep: the finest-level "
                         "operator kernels of the c2 system alone (Fapply, residual, Jacobi; FP32 and FP64); conv: the "
                         "learned network's tensor-core convolutions and its forward pass on an (n+1)^3 grid")
    ap.add_argument("--rves", type=int, default=512, help="rve workload: number of RVEs")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "f64"], help="rve workload")
    ap.add_argument("--train-problems", type=int, default=16, help="learned workload: 64^3 training problems")
    ap.add_argument("--train-steps", type=int, default=2000, help="learned workload: Adam steps")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# process group (one replica per GPU; no collective on the data path)
# ---------------------------------------------------------------------------
class Dist:
    def __init__(self):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch
            import torch.distributed as dist
            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local)
            dist.init_process_group(backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v):
        if not self.pg:
            return v
        import torch
        dev = "cuda" if self.pg.get_backend() == "nccl" else "cpu"
        t = torch.tensor([float(v)], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v):
        if not self.pg:
            return v
        import torch
        dev = "cuda" if self.pg.get_backend() == "nccl" else "cpu"
        t = torch.tensor([float(v)], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        if not self.proc:
            return out
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                for k, nm in enumerate(names):
                    if r[5 + k].strip().lower().startswith("active"):
                        reasons.add(nm)
            except (ValueError, IndexError):
                pass
        if sm:
            out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                   "samples": len(sm)}
        return out


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic():
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(p) as f:
            return json.load(f)
    except Exception:
        return {}


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------
def workload(n, grains):
    from alamo_gb300 import microstructure as M
    from alamo_gb300.elastic import TensionTest
    ddw, _, _ = M.voronoi_cubic(n, ngrains=grains, seed=20260)
    bc = TensionTest("uniaxial_stress", disp=0.01)
    return ddw, bc


def run_ours(args, dist):
    import numpy as np
    import torch
    from alamo_gb300 import Elastic, Linear, Newton

    torch.cuda.set_device(dist.local)
    n = args.n
    nodes = (n + 1) ** 3
    ddw_h, bc = workload(n, args.grains)
    op = Elastic([n] * 3, None, "majorminor")
    op.SetBC(bc)
    ddw_d = torch.from_numpy(ddw_h).cuda()
    op.SetModel(ddw_d)
    b_h = op.BCInit(np.zeros(3 * nodes))
    rhs_h = op.NewtonRHS(np.zeros(3 * nodes), b_h)
    rhs_d = torch.from_numpy(rhs_h).cuda()
    sol_d = torch.zeros(3 * nodes, dtype=torch.float64, device="cuda")
    maxfmg = 100000000 if args.cycle == "F" else 0
    cyc = {"omega": args.omega, "pre_smooth": args.pre, "post_smooth": args.post}
    mixed = Linear(op, precision=1, max_fmg_iter=maxfmg, krylov=args.krylov, **cyc)

    def one():
        sol_d.zero_()
        mixed.solve(sol_d, rhs_d, 1e-8, 0.0)
        return mixed.report

    for _ in range(args.warmup):
        one()
    torch.cuda.synchronize()
    dist.barrier()
    clocks = Clocks(dist.local)
    clocks.start()
    t0 = time.perf_counter()
    reps = [one() for _ in range(args.steps)]
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    dist.barrier()
    clk = clocks.stop()
    dev_ms = [r.solve_ms for r in reps]
    step_ms = dist.max(statistics.mean(dev_ms))
    kernels = int(sum(r.kernels for r in reps))
    last = reps[-1]
    if any(r.status != 0 for r in reps):
        raise RuntimeError("a timed solve did not converge: statuses %s" % [r.status for r in reps])
    res = {
        "step_ms": step_ms, "wall_ms": wall * 1000 / args.steps, "kernels": kernels, "clocks": clk,
        "mixed": {"cycles": last.iterations, "refinements": last.refinements, "res0": last.res0,
                  "res_final": last.res_final, "rhs_norm": last.rhs_norm, "nlevels": last.nlevels,
                  "res_rel_final": last.res_final / max(last.rhs_norm, last.res0)},
    }
    x_mixed = sol_d.clone()

    # end to end through the reference-facing calls with host buffers:
    # SetModel(host Matrix4 field) + Newton step (host u, host b) -> host u
    if not args.no_e2e:
        ddw_p = torch.from_numpy(ddw_h).pin_memory().numpy()
        b_p = torch.from_numpy(b_h).pin_memory().numpy()
        u_t = torch.zeros(3 * nodes, dtype=torch.float64).pin_memory()
        u_p = u_t.numpy()
        newton = Newton(op, precision=1, max_fmg_iter=maxfmg, krylov=args.krylov, **cyc)

        parts = []

        def e2e_step():
            t_a = time.perf_counter()
            u_t.zero_()   # the caller's zero initial guess (torch fills on the host threads)
            t_b = time.perf_counter()
            op.SetModel(ddw_p)
            t_c = time.perf_counter()
            newton.solve(u_p, b_p, None, 1e-8, 0.0)
            t_d = time.perf_counter()
            parts.append((t_b - t_a, t_c - t_b, t_d - t_c, newton.report.solve_ms / 1e3))

        for _ in range(2):
            e2e_step()
        torch.cuda.synchronize()
        parts.clear()
        t0 = time.perf_counter()
        ke = 3
        for _ in range(ke):
            e2e_step()
        e2e_s = dist.max((time.perf_counter() - t0) / ke)
        res["e2e"] = {"value": e2e_s, "unit": "s",
                      "h2d_bytes_per_step": int(ddw_p.nbytes + b_p.nbytes + u_p.nbytes),
                      "d2h_bytes_per_step": int(u_p.nbytes),
                      "parts_ms": {k: round(1e3 * sum(p[i] for p in parts) / len(parts), 2) for i, k in
                                   enumerate(("zero_host_u", "SetModel", "Newton_step", "Newton_device_solve"))},
                      "SetModel_ms_min_max": [round(1e3 * min(p[1] for p in parts), 2),
                                              round(1e3 * max(p[1] for p in parts), 2)]}
        newton.Clear()
        res["u_check"] = float(np.abs(u_p).max())
        del ddw_p, b_p, u_p, u_t

    # roofline of the dominant kernel: the FP32 damped-Jacobi sweep on the finest level
    ms_j32 = op.time_sweep(0, "f32", 2, 20)
    ms_a32 = op.time_sweep(0, "f32", 0, 20)
    ms_j64 = op.time_sweep(0, "f64", 2, 5)
    ms_a64 = op.time_sweep(0, "f64", 0, 5)
    res["kernels_ms"] = {"jacobi_f32": ms_j32, "fapply_f32": ms_a32, "jacobi_f64": ms_j64, "fapply_f64": ms_a64}
    # the FP64 sweeps are bound by the FP64 pipe: its throughput, measured now
    from alamo_gb300.elastic import fp64_fma_peak
    res["fp64_peak_tflops"] = max(fp64_fma_peak()[0] for _ in range(3))
    res["nodes"] = nodes

    # plain FP64 multigrid of the same system, once
    if not args.no_plain:
        plain = Linear(op, precision=0, max_fmg_iter=maxfmg, omega=2.0 / 3.0)   # MLMG's damping
        sol_d.zero_()
        plain.solve(sol_d, rhs_d, 1e-8, 0.0)
        pr = plain.report
        res["plain"] = {"ms": pr.solve_ms, "iterations": pr.iterations, "res_final": pr.res_final,
                        "status": pr.status, "res_rel_final": pr.res_final / max(pr.rhs_norm, pr.res0)}
        # the timed mixed solution against the plain FP64 solution of the same
        # system (max-norm relative displacement difference)
        res["err_vs_fp64"] = float((x_mixed - sol_d).abs().max().item() / sol_d.abs().max().item())
        plain.Clear()
    res["x_mixed"] = x_mixed.cpu().numpy()
    res["rhs"] = rhs_h
    del x_mixed

    mixed.Clear()
    op.close()
    return res, ddw_h, bc


def oracle_grid(n, bc):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    return O, O.make_grid([n] * 3, sym=O.MAJORMINOR, bc_type=bc.type, bc_val=bc.val)


def cpu_sample(n, ddw_h, bc, rhs, iterations, k=2):
    """Bounded sample of the CPU leg: the oracle on every host core runs
    prepareForSolve and `k` MLMG F-cycle iterations of the same 257^3 solve
    (about 10 s); the full-solve time is that setup plus `iterations` (the
    FP64 F-cycle count the GPU plain solve of the same system took in this
    run; the oracle's count equals it within one, as the parity tests check)
    times the measured time per iteration."""
    O, g = oracle_grid(n, bc)
    t0 = time.perf_counter()
    sess = O.Session(g, ddw_h, rhs, tol_rel=1e-8, tol_abs=0.0)
    t1 = time.perf_counter()
    sess.iterate(k)
    t2 = time.perf_counter()
    _, rep = sess.finish()
    cores = O.lib().orc_num_threads()
    per_iter = (t2 - t1) / max(rep.iterations, 1)
    value = (t1 - t0) + iterations * per_iter
    return {"value": value, "unit": "s", "cores": cores, "kind": "port",
            "sample": "oracle/ CPU restatement, OpenMP %d threads, same %d^3-node system: prepareForSolve (%.2f s) + "
                      "%d F-cycle iterations (%.2f s each) measured, scaled to the %d iterations the plain FP64 "
                      "solve took on the GPU in this run" % (cores, n + 1, t1 - t0, rep.iterations, per_iter,
                                                             iterations)}


def oracle_check(n, ddw_h, bc, x, rhs):
    """The oracle's FP64 residual of the GPU solution (max norm, relative to
    ||rhs||): the checker's verdict on the timed result."""
    O, g = oracle_grid(n, bc)
    r = O.residual(g, ddw_h, x, rhs)
    return float(np.abs(r).max() / np.abs(rhs).max())


def run_sweep(args, dist):
    """The finest-level operator kernels of the c2 system timed alone:
    `--steps` back-to-back launches per kernel after one warm-up launch (each
    launch reads more than L2 holds), CUDA events on the operator's stream.
    GB/s from the algorithmic bytes per node (FP32 cubic: Fapply 108, residual
    120, Jacobi 132; FP64: 216, 240, 264)."""
    import torch
    from alamo_gb300 import Elastic
    torch.cuda.set_device(dist.local)
    n = args.n
    nodes = (n + 1) ** 3
    ddw_h, bc = workload(n, args.grains)
    op = Elastic([n] * 3, None, "majorminor")
    op.SetBC(bc)
    op.SetModel(torch.from_numpy(ddw_h).cuda())
    del ddw_h
    bpn = {("f32", 0): 108, ("f32", 1): 120, ("f32", 2): 132, ("f64", 0): 216, ("f64", 1): 240, ("f64", 2): 264}
    out = {}
    for prec in ("f32", "f64"):
        for mode, name in ((0, "fapply"), (1, "residual"), (2, "jacobi")):
            ms = op.time_sweep(0, prec, mode, max(1, args.steps))
            out["%s_%s" % (name, prec)] = {"ms": round(ms, 4), "gbs": round(bpn[(prec, mode)] * nodes / ms / 1e6, 1)}
    op.close()
    peak, kind = measured_peak_hbm()
    line = {"metric": "finest-level operator sweeps, GB/s (algorithmic bytes)", "workload": "sweep", "n": n,
            "nodes": nodes, "peak_hbm_gbs": peak, "peak_kind": kind, "sweeps": out}
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    dist.close()


def run_conv(args, dist):
    """The learned network's 3x3x3 tensor-core convolutions (tcgen05) timed
    alone, one shape per layer of the U-Net on its grid of an (n+1)^3-node
    box, and the whole forward pass: `--steps` back-to-back launches after
    one warm-up, CUDA events.  FLOP/s = 2 x 27 cin cout per voxel against the
    measured BF16 peak; GB/s from the activations read and written once."""
    import ctypes
    import torch
    from alamo_gb300._lib import check, lib
    from alamo_gb300.learned import UNet, _i3, _vp, grids
    torch.cuda.set_device(dist.local)
    L = lib()
    g0 = (args.n + 1,) * 3
    G = grids(g0)
    peak = None
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak = float(json.load(f)["bf16_tflops"])
    except Exception:
        peak = 1900.0
    reps = max(1, args.steps)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = {}
    net = UNet(seed=0)
    for l, (ci, co, lev) in enumerate(zip(net.cin, net.cout, net.lev)):
        g = G[lev]
        V = int(np.prod(g))
        x = torch.randn(V * ci, device="cuda").to(torch.bfloat16)
        y = torch.empty(V * co, dtype=torch.bfloat16, device="cuda")
        wp = torch.empty(27 * co * ci, dtype=torch.bfloat16, device="cuda")
        check(L.agb_conv3_tc_pack(ci, co, _vp(net.wb[l]), co, 0, _vp(wp), None))

        def run():
            check(L.agb_conv3_tc(_i3(g), ci, co, _vp(x), ci, 0, _vp(wp), _vp(net.b[l]), _vp(y), co, 0, 0, 1, None))
        run()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            run()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        tf = 2.0 * 27 * ci * co * V / ms / 1e9
        out["layer%d_%dx%d_%d^3" % (l, ci, co, g[0])] = {"ms": round(ms, 4), "tflops": round(tf, 1),
                                                          "frac_bf16": round(tf / peak, 4),
                                                          "gbs": round(V * (ci + co) * 2 / ms / 1e6, 1)}
    feat = torch.randn(int(np.prod(G[0])), 16, device="cuda").to(torch.bfloat16)
    net.forward(g0, feat)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        net.forward(g0, feat)
    e1.record()
    torch.cuda.synchronize()
    line = {"metric": "learned network: tcgen05 convolutions and forward pass", "workload": "conv", "n": args.n,
            "bf16_peak_tflops": peak, "forward_ms": round(e0.elapsed_time(e1) / reps, 3), "layers": out}
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    net.close()
    dist.close()


def rve_measure(nprob, precision, krylov, steps, warmup, check=True):
    """Batched RVE homogenization: `nprob` periodic RVEs (edges 32-96 cells,
    diffuse ellipsoidal inclusions, contrast up to 100, uniform eigenstrain),
    microstructures generated on the GPU, all solved together to 1e-8 by the
    agb_batch_* path.  One step = one batch solve (prepareForSolve +
    cycles), device time.  With `check`, the smallest problem's solution is
    compared with the oracle's FP64 solve of the same problem (on the CPU,
    after the timed steps)."""
    import torch
    from alamo_gb300 import microstructure as M
    from alamo_gb300.batch import Batch
    probs = [M.rve_params(q) for q in range(nprob)]
    sizes = [(p[0],) * 3 for p in probs]
    nodes = sum((n + 1) ** 3 for n, _, _ in probs)
    bt = Batch(sizes, precision=precision, krylov=krylov if precision == 1 else 0)
    for q in range(nprob):
        _, ddw, _ = M.rve_problem_device(q)
        bt.SetModel(q, ddw)
        del ddw
    bt.SetEigenstrain(np.stack([p[2] for p in probs]))
    for _ in range(max(1, warmup)):
        bt.solve(1e-8, 0.0, raise_on_fail=False)
    torch.cuda.synchronize()
    ms = []
    t0 = time.perf_counter()
    for _ in range(steps):
        tot = bt.solve(1e-8, 0.0, raise_on_fail=False)
        ms.append(tot.solve_ms)
    torch.cuda.synchronize()
    wall = (time.perf_counter() - t0) / steps
    for q in range(nprob):
        r = bt.reports[q]
        if r.status != 0:
            print("rve %d (edge %d): status %d after %d cycles, |r|/|b| %.3e" %
                  (q, probs[q][0], r.status, r.iterations, r.res_final / max(r.rhs_norm, 1e-300)), file=sys.stderr)
    step_s = statistics.mean(ms) / 1000.0
    its = [bt.reports[q].iterations for q in range(nprob)]
    worst = max(bt.reports[q].res_final / max(bt.reports[q].rhs_norm, 1e-300) for q in range(nprob))
    out = {"rves": nprob, "nodes": nodes, "rve_per_s": nprob / step_s, "ms_per_batch": step_s * 1000.0,
           "wall_s_per_batch": wall, "cycles_min": min(its), "cycles_max": max(its), "worst_rel_residual": worst,
           "not_converged": sum(1 for q in range(nprob) if bt.reports[q].status != 0), "kernels": tot.kernels,
           "method": ("FP32 %s in FP64 refinement, per-problem GCR(%d)" % ("F-cycles" if krylov else "V-cycles", krylov)
                      if precision == 1 else "FP64 V-cycles")}
    if check:
        q = min(range(nprob), key=lambda i: probs[i][0])
        n, _, F0 = probs[q]
        u = bt.solution(q)
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        _, ddw_h, _ = M.rve_problem(q)
        g = O.make_grid([n] * 3, sym=O.ISO, periodic=(1, 1, 1))
        N = O.nodes(g)
        rhs = O.newton_rhs(g, ddw_h, np.tile(np.asarray(F0).reshape(9), N), np.zeros(3 * N), np.zeros(3 * N))
        xo, _ = O.solve(g, ddw_h, rhs, tol_rel=1e-8, tol_abs=0.0, params=O.default_params(max_fmg_iter=0))
        out["err_vs_oracle"] = {"problem": q, "edge": n, "rel_err": float(np.abs(u - xo).max() / np.abs(xo).max())}
    bt.close()
    return out, tot


def run_rve(args, dist):
    """The batched RVE workload alone (rve_measure) as its own benchmark line."""
    import torch
    torch.cuda.set_device(dist.local)
    clocks = Clocks(dist.local)
    clocks.start()
    res, tot = rve_measure(args.rves, 1 if args.precision == "mixed" else 0, args.krylov, args.steps, args.warmup,
                           check=dist.rank == 0)
    clk = clocks.stop()
    step_s = dist.max(res["ms_per_batch"] / 1000.0)
    value = dist.sum(args.rves) / step_s
    line = {"metric": "periodic RVE solves per second to 1e-8 FP64 residual (batched)", "value": value,
            "unit": "RVE/s", "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": step_s * 1000.0, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64" if args.precision == "mixed" else "f64", "data": "synthetic (seeded RVEs)",
            "config": {"workload": "%d periodic RVEs, edges 32-96 cells, 1-8 diffuse ellipsoids of contrast "
                                   "log-uniform in [1,100], uniform eigenstrain, solve to 1e-8" % args.rves,
                       "nodes": res["nodes"], "l2": "inputs larger than L2"},
            "gpu_launches": tot.kernels, "clocks": clk, "rve": res}
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    dist.close()


def run_learned(args, dist):
    """Learned correction: the U-Net trained (untimed) on the GCR gain of
    multigrid residuals of random 64^3 cubic polycrystals, then the c2 system at 129^3 and 257^3
    nodes solved by the benchmark's method (FP32 F-cycles under GCR(8) in
    FP64 refinement) with and without the network's directions (the
    ablation), and by plain FP64 multigrid; solve times are device times of
    the best of two solves."""
    import torch
    from alamo_gb300 import Elastic, Linear
    from alamo_gb300.learned import UNet, gain_samples, learned_stats, train_gain
    torch.cuda.set_device(dist.local)
    log = lambda m: print(m, file=sys.stderr, flush=True)
    t0 = time.perf_counter()
    problems = gain_samples(count=args.train_problems, n=64, seed=777, log=log)
    t1 = time.perf_counter()
    net = UNet(seed=1)
    hist = train_gain(net, problems, 64, steps=args.train_steps, lr=1e-3, warmup=50, log=log)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    nsamples = sum(len(p["items"]) for p in problems)
    del problems
    out = {"train": {"problems": args.train_problems, "samples": nsamples, "n": 64, "steps": args.train_steps,
                     "params": net.nparams(), "data_s": round(t1 - t0, 1), "train_s": round(t2 - t1, 1),
                     "gain_first50": float(np.mean(hist[:50])), "gain_last50": float(np.mean(hist[-50:]))}}
    for n in (128, 256):
        ddw_h, bc = workload(n, args.grains)
        op = Elastic([n] * 3, None, "majorminor")
        op.SetBC(bc)
        op.SetModel(torch.from_numpy(ddw_h).cuda())
        del ddw_h
        N = (n + 1) ** 3
        zero = torch.zeros(3 * N, dtype=torch.float64, device="cuda")
        b = op.BCInit(torch.zeros(3 * N, dtype=torch.float64, device="cuda"))
        rhs = torch.empty(3 * N, dtype=torch.float64, device="cuda")
        op.NewtonRHS(zero, b, out=rhs)
        row = {}
        for name in ("mixed_gcr8", "mixed_gcr8_learned", "plain_f64"):
            s = Linear(op, precision=0) if name == "plain_f64" else Linear(op, precision=1, krylov=8)
            if name == "mixed_gcr8_learned":
                net.attach(s)
            best = None
            for rep in range(2 if name != "plain_f64" else 1):
                x = torch.zeros(3 * N, dtype=torch.float64, device="cuda")
                s.solve(x, rhs, 1e-8, 0.0)
                r = s.report
                if best is None or r.solve_ms < best["ms"]:
                    best = {"ms": round(r.solve_ms, 2), "cycles": r.iterations, "status": r.status,
                            "rel_res": r.res_final / max(r.rhs_norm, r.res0)}
                    if name == "mixed_gcr8_learned":
                        tried, kept, active = learned_stats(s)
                        best.update({"learned_tried": tried, "learned_kept": kept, "learned_active_at_end": active})
            row[name] = best
            s.Clear()
        row["learned_vs_mixed"] = round(row["mixed_gcr8"]["ms"] / row["mixed_gcr8_learned"]["ms"], 3)
        row["learned_vs_plain_f64"] = round(row["plain_f64"]["ms"] / row["mixed_gcr8_learned"]["ms"], 2)
        out["%d^3" % (n + 1)] = row
        op.close()
    line = {"metric": "learned+FP32 solve s @257^3 nodes (c2 system), with the ablation and plain FP64",
            "value": out["257^3"]["mixed_gcr8_learned"]["ms"] / 1000.0, "unit": "s", "n_gpus": 1, "steps": 2,
            "warmup": 0, "higher_is_better": False, "dtype": "bf16 net + f32/f64 solve",
            "data": "synthetic (seeded Voronoi polycrystals)",
            "config": {"workload": "U-Net trained on the GCR gain of %d multigrid residuals of 64^3 cubic "
                                   "polycrystals, evaluated on the 129^3 and 257^3 c2 systems" % nsamples},
            "learned": out}
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    dist.close()


def main():
    args = parse()
    dist = Dist()
    if args.impl == "reference":
        return run_reference(args, dist)
    if args.workload == "rve":
        return run_rve(args, dist)
    if args.workload == "learned":
        return run_learned(args, dist)
    if args.workload == "sweep":
        return run_sweep(args, dist)
    if args.workload == "conv":
        return run_conv(args, dist)
    res, ddw_h, bc = run_ours(args, dist)
    peak, peak_kind = measured_peak_hbm()
    nodes = res["nodes"]
    ms = res["kernels_ms"]["jacobi_f32"]
    achieved = BYTES_PER_NODE["jacobi_f32_cubic"] * nodes / (ms * 1e-3) / 1e9
    traffic = profile_traffic().get("jacobi_f32_cubic_257", {}).get("dram_bytes_per_launch")
    roof = {"kernel": "k_stencil_tma<MajorMinor,Jacobi> + k_stencil_shell (finest level)",
            "bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": traffic, "peak_kind": peak_kind,
            "bytes_per_launch": BYTES_PER_NODE["jacobi_f32_cubic"] * nodes, "ms_per_launch": ms}
    extra = {
        "fapply_f32_gbs": round(BYTES_PER_NODE["fapply_f32_cubic"] * nodes / (res["kernels_ms"]["fapply_f32"] * 1e-3)
                                / 1e9, 1),
        "jacobi_f64_gbs": round(BYTES_PER_NODE["jacobi_f64_cubic"] * nodes / (res["kernels_ms"]["jacobi_f64"] * 1e-3)
                                / 1e9, 1),
        "fapply_f64_gbs": round(BYTES_PER_NODE["fapply_f64_cubic"] * nodes / (res["kernels_ms"]["fapply_f64"] * 1e-3)
                                / 1e9, 1),
        "kernel_ms": res["kernels_ms"],
        "fp64_roofline": {
            "kernel": "k_stencil_march<double,MajorMinor,Jacobi> + k_stencil_shell (finest level)", "bound": "fp64",
            "flops_per_node": FLOPS_PER_NODE["jacobi_f64_cubic"],
            "achieved": round(FLOPS_PER_NODE["jacobi_f64_cubic"] * nodes / (res["kernels_ms"]["jacobi_f64"] * 1e-3)
                              / 1e12, 3),
            "peak": round(res["fp64_peak_tflops"], 3), "unit": "TFLOP/s", "peak_kind": "measured (FP64 FMA loop)",
            "frac": round(FLOPS_PER_NODE["jacobi_f64_cubic"] * nodes / (res["kernels_ms"]["jacobi_f64"] * 1e-3)
                          / 1e12 / res["fp64_peak_tflops"], 4),
            "fapply": {"flops_per_node": FLOPS_PER_NODE["fapply_f64_cubic"],
                       "achieved": round(FLOPS_PER_NODE["fapply_f64_cubic"] * nodes
                                         / (res["kernels_ms"]["fapply_f64"] * 1e-3) / 1e12, 3),
                       "frac": round(FLOPS_PER_NODE["fapply_f64_cubic"] * nodes
                                     / (res["kernels_ms"]["fapply_f64"] * 1e-3) / 1e12 / res["fp64_peak_tflops"], 4)}},
        "mixed": res["mixed"],
    }
    if "plain" in res:
        extra["plain_fp64_s"] = res["plain"]["ms"] / 1000.0
        extra["plain_fp64_iterations"] = res["plain"]["iterations"]
        extra["plain_fp64_res_rel_final"] = res["plain"]["res_rel_final"]
        extra["speedup_vs_plain_fp64"] = round(res["plain"]["ms"] / res["step_ms"], 2)
        extra["err_vs_fp64"] = res["err_vs_fp64"]
    extra["res_rel_final"] = res["mixed"]["res_rel_final"]
    # a replica solves one system per GPU: the value is the time of one solve
    # (max over ranks), not divided by the number of replicas
    line = {
        "metric": METRIC, "value": res["step_ms"] / 1000.0, "unit": "s", "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["step_ms"], "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded Voronoi polycrystal)",
        "config": {"workload": WORKLOAD, "nodes": nodes,
                   "method": ("FP32 %s-cycles under flexible GCR(%d) in FP64 iterative refinement" % (args.cycle, args.krylov)
                              if args.krylov > 0 else "FP32 %s-cycles in FP64 iterative refinement" % args.cycle),
                   "smoother": "2+2 Fsmooth (4+4 damped-Jacobi sweeps)",
                   "l2": "inputs larger than L2 (modulus field 2.9 GB FP64 / 1.4 GB FP32)",
                   "parallelism": "replicas" if dist.world > 1 else "single GPU"},
        "roofline": roof,
        "gpu_launches": res["kernels"],
        "clocks": res["clocks"],
    }
    if "e2e" in res:
        line["e2e"] = res["e2e"]
    line.update(extra)
    if not args.no_rve:
        # the batched-RVE configuration (512 periodic RVEs), measured after the
        # timed region of the line's own workload
        line["rve"], _ = rve_measure(args.rves, 1, args.krylov, 2, 1, check=dist.rank == 0)
    if dist.rank == 0 and not args.no_cpu:
        line["res_rel_oracle"] = oracle_check(args.n, ddw_h, bc, res["x_mixed"], res["rhs"])
        iters = res.get("plain", {}).get("iterations") or 0
        if iters:
            line["cpu_baseline"] = cpu_sample(args.n, ddw_h, bc, res["rhs"], iters)
    dist.barrier()
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    dist.close()


# ---------------------------------------------------------------------------
# reference arm: the CPU restatement of the reference algorithm
# ---------------------------------------------------------------------------
def run_reference(args, dist):
    """One complete FP64 MLMG solve (F-cycles, 2+2 Fsmooth, BiCGStab bottom,
    ||r||_inf <= 1e-8 ||b||_inf) of the same 257^3 system by the oracle on
    every host core, measured, not extrapolated.  The K timed steps together
    run that one solve: step 0 does prepareForSolve, and each step runs up to
    ceil(60 / K) iterations (the last one runs on to convergence), so the
    whole solve lies inside the timed region.  value = the solve's wall time;
    ms_per_step = value / K.  Each of the W warm-up steps is one F-cycle
    iteration of a throw-away solve of the same system."""
    if dist.rank != 0:
        dist.close()
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    n = args.n
    ddw_h, bc = workload(n, args.grains)
    g = O.make_grid([n] * 3, sym=O.MAJORMINOR, bc_type=bc.type, bc_val=bc.val)
    N = O.nodes(g)
    b = O.bc_init(g, np.zeros(3 * N))
    rhs = O.newton_rhs(g, ddw_h, None, np.zeros(3 * N), b)
    if args.warmup > 0:
        w = O.Session(g, ddw_h, rhs, tol_rel=1e-8, tol_abs=0.0)
        w.iterate(args.warmup)
        w.finish()
        del w
    steps = max(1, args.steps)
    chunk = max(1, int(math.ceil(60.0 / steps)))
    step_s = []
    sess = None
    for k in range(steps):
        t0 = time.perf_counter()
        if sess is None:
            sess = O.Session(g, ddw_h, rhs, tol_rel=1e-8, tol_abs=0.0)
        sess.iterate(chunk if k < steps - 1 else 1 << 20)
        step_s.append(time.perf_counter() - t0)
    x, rep = sess.finish()
    cores = O.lib().orc_num_threads()
    v = sum(step_s)
    rel = rep.res_final / max(float(np.abs(rhs).max()), rep.res0)
    sample = ("measured: one complete solve of the %d^3-node system by the oracle/ CPU restatement (FP64 MLMG "
              "F-cycles, OpenMP %d threads) to %.2e relative residual in %d iterations (status %d), "
              "prepareForSolve %.2f s + iterations %.2f s, split over %d timed steps"
              % (n + 1, cores, rel, rep.iterations, rep.status, rep.t_setup, rep.t_iter, steps))
    line = {"metric": METRIC, "value": v, "unit": "s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": v * 1000.0 / steps, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Voronoi polycrystal)",
            "config": {"workload": WORKLOAD, "nodes": N, "method": "MLMG F-cycles, FP64, CPU"},
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "reference_solve": {"iterations": rep.iterations, "status": rep.status, "res_rel_final": rel,
                                "setup_s": rep.t_setup, "iterations_s": rep.t_iter,
                                "step_s": [round(t, 3) for t in step_s]}}
    print(json.dumps(line), flush=True)
    dist.close()


if __name__ == "__main__":
    main()
