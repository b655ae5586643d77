"""Benchmark: SIMP design iterations/s on a 3D hex8 cantilever (160x80x80,
1,024,000 elements), one GB300.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one design iteration (density filter -> solve to rtol 1e-8 ->
compliance + sensitivities -> filter pullback -> OC update), timed with CUDA
events on the stream the library launches on.  `value` is the device-resident
loop; `e2e` is the same loop through the C ABI with the design copied from and
to pinned host memory every step.  N > 1 runs independent replicas (the path
does not shard: one problem per GPU).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "design iters/s, 3D hex8 1M elems: learned+FP32-IR vs plain FP64 PCG @ rel 1e-6"
NELS = (160, 80, 80)
VOLFRAC, RMIN, PEN, XMIN, RTOL, MOVE = 0.3, 1.5, 3.0, 1e-9, 1e-8, 0.2
WORKLOAD = ("3D PointLoadCantilever 160x80x80 hex8, 1,024,000 cells, E_min 1e-9, load at right-face centre, "
            "p=3, V=0.3, rmin=1.5, x0=0.3, OC move 0.2, rtol 1e-8")
# seconds of CPU design iterations the reference arm times at most (whole iterations only)
REF_BUDGET_S = float(os.environ.get("REF_BUDGET_S", "150"))


def config_line():
    """The `config` object both arms print (short values: it is compared between the arms)."""
    return {"workload": WORKLOAD, "unit_of_work": "one design iteration (filter, solve, compliance, pullback, OC)",
            "l2": "working set ~0.3 GB > 129 MB L2 (no flush)"}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def read_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def read_traffic(ncells):
    """DRAM bytes per launch of the PCG operator kernel: the committed ncu summary's
    bytes per cell (captured on a case larger than L2) scaled by the cell count."""
    p = os.path.join(ROOT, "profiles", "k_march3_fp32_pcg_256x128x128.md")
    try:
        for line in open(p):
            if line.startswith("traffic_bytes_per_element:"):
                return float(line.split(":")[1]) * ncells
    except Exception:
        pass
    return None


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.rows = []
        if self.proc:
            self.proc.terminate()
            out, _ = self.proc.communicate(timeout=10)
            for line in out.strip().splitlines():
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    self.rows.append(parts)

    def summary(self):
        if not getattr(self, "rows", None):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(v, ws, device="cuda"):
    """The slowest rank's time (every rank gets it): NCCL on the GPU ranks of the bench,
    gloo on CPU in the tests."""
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(units_per_rank, ws, t_max):
    """Whole-job throughput of N independent replicas: all ranks' units over the slowest
    rank's time (weak scaling, no data-path collective)."""
    return ws * units_per_rank / t_max


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


# --------------------------------------------------------------------------- CPU legs
def cpu_design_iterations(threads, max_iters, budget_s):
    """The oracle port of the reference path (per-element Ke copies, two-phase gather,
    Jacobi PCG from zero to rtol on the recurrence residual as cg!, compliance, filter
    pullback, OC) run as whole design iterations from the uniform start on `threads`
    host threads, each one timed; stops after `max_iters` or once `budget_s` seconds of
    iterations have run.  Returns the per-iteration seconds and PCG counts, and the
    first iteration's filtered densities, displacement, compliance, sensitivities and
    new design (the accuracy reference of the GPU path)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import topopt_oracle as O
    import oracle_cpu as OC
    prob = O.point_load_cantilever(NELS, (1.0, 1.0, 1.0), load="face_centre")
    Ke = O.element_stiffness(3, (1.0, 1.0, 1.0), 1.0, 0.3)
    cs = OC.CPUSolver(prob, Ke, XMIN, PEN, threads=threads)
    n = prob.grid.ncells
    cs.filter_setup(RMIN)
    f = prob.f.copy()
    f[prob.fixed_dofs] = 0.0
    x = np.full(n, VOLFRAC)
    secs, cg, first = [], [], None
    while len(secs) < max_iters and (not secs or sum(secs) < budget_s):
        t0 = time.perf_counter()
        xf = cs.filter_J(x)
        cs.set_vars(xf)
        u, it, _ = cs.pcg(f, rtol=RTOL, abstol=0.0, maxit=200000)
        c, g = cs.compliance(u)
        dc = cs.filter_JT(g)
        dv = cs.filter_JT(np.full(n, 1.0 / n))
        xn, _, _ = cs.oc(x, dc, dv, dv, VOLFRAC, MOVE)
        secs.append(time.perf_counter() - t0)
        cg.append(int(it))
        if first is None:
            first = dict(xf=xf, u=u, c=c, dc=dc, x_new=xn)
        x = xn
    cs.close()
    return dict(seconds=secs, cg_iters=cg, first=first, threads=threads)


def cpu_threads():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_cpu as OC
    return OC.lib().orc_max_threads()


def run_reference(args):
    """The reference's CPU path (the oracle port, all host threads) timed over whole
    design iterations of the same workload: as many as fit in REF_BUDGET_S seconds,
    at most --steps; the line's steps is the number timed."""
    ws, rank, _ = dist_setup()
    if rank != 0:
        return 0
    threads = cpu_threads()
    r = cpu_design_iterations(threads, args.steps, REF_BUDGET_S)
    k = len(r["seconds"])
    t = sum(r["seconds"])
    v = k / t
    sample = ("design iterations 1..%d from the uniform start, each whole (filter, cold Jacobi PCG to rtol 1e-8: "
              "%s iterations, compliance, pullback, OC), %d of the %d steps asked fit in %.0f s"
              % (k, ",".join(map(str, r["cg_iters"])), k, args.steps, REF_BUDGET_S))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "design_iters/s", "n_gpus": args.gpus,
            "steps": k, "warmup": 0, "ms_per_step": 1e3 * t / k, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config_line(),
            "cpu_baseline": {"value": v, "unit": "design_iters/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": "design_iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "steps_requested": args.steps, "warmup_requested": args.warmup,
            "note": "CPU arm: no warm-up iteration (nothing to warm); whole design iterations only"}
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------------------- GPU leg
def batch_leg(tg, stream, peaks, src, steps):
    """Batched 2D SIMP: 256 uneven cantilevers (nelx ~ U{64..512}, nely = nelx/2, load
    node, volume fraction and filter radius drawn from seed 0), every design iteration
    of all problems one graph launch; FP32-IR with previous-step warm start, rtol 1e-8."""
    import torch
    P = tg.uneven_cantilever_set(256, seed=0)
    b = tg.BatchedSIMP(P["nelx"], P["nely"], P["load_j"], P["volfrac"], P["rmin"], rtol=1e-8)
    rows = b.autotune()
    b.set_stream(stream.cuda_stream)
    b.step()   # warm-up (first design iteration)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    loops, refreshes = [], []
    e0.record(stream)
    for _ in range(steps):
        st = b.step()
        loops.append(int(st.pcg_loops))
        refreshes.append(int(st.reliable_updates))
    e1.record(stream)
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3
    c, ch, it = b.results()
    kern = {}
    for k, name in ((0, "bk_march<float, PCG> (operator)"), (1, "bk_update (PCG vectors)"),
                    (2, "bk_march<double, RESID> (FP64 true residual)")):
        us, by = b.bench_kernel(k, 20)
        kern[name] = {"us_per_launch": us, "algorithmic_bytes": by, "achieved_gbs": by / us / 1e3,
                      "frac": by / us / 1e3 / peaks["hbm_gbs"]}
    nodes = int(np.sum((P["nelx"] + 1) * (P["nely"] + 1)))
    out = {"workload": "256 2D cantilevers, nelx ~ U{64..512} even, nely = nelx/2, %d cells, %d nodes "
                       "(seed 0)" % (int(np.sum(P["nelx"] * P["nely"])), nodes),
           "design_iters_per_s": steps / t, "problem_iters_per_s": 256 * steps / t, "steps": steps,
           "warmup": 1, "operator_rows": rows, "pcg_loops_per_step": loops,
           "reliable_updates_per_step": refreshes, "cg_iters_mean_last": float(np.mean(it)),
           "cg_iters_max_last": int(np.max(it)), "kernels_all_problems": kern,
           "peak_source": src}
    b.close()
    return out


WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "topopt.jl_gb300", "weights",
                       "warmstart_96x48x48.npy")


def learned_leg(tg, steps):
    """Learned warm start: 3D cantilever 96x48x48, one held-out seeded run (volume
    fraction, load node on the free face and direction drawn from seed 1000), the same
    trajectory solved with a cold, a previous-step and a learned start (network trained
    by topopt.jl_gb300/learned.py on seeded runs of the same grid, weights committed)."""
    if not os.path.exists(WEIGHTS):
        return {"unavailable": "no trained weights at topopt.jl_gb300/weights/"}
    from topopt_gb300 import learned as LW
    nels = (96, 48, 48)
    net = tg.WarmStartNet(tuple(n + 1 for n in nels), batch=1, seed=0)
    net.set_params(np.load(WEIGHTS))
    run = LW.sample_runs(1, nels, seed=1000)[0]
    ev = LW.evaluate(nels, run, steps, net)
    net.close()
    prev = ev["previous"]
    out = {"workload": "3D cantilever 96x48x48, held-out run %s" % json.dumps(
        {"volfrac": round(run["volfrac"], 4), "node": run["node"],
         "direction": [round(float(v), 4) for v in run["direction"]]}),
           "design_iters": steps, "rtol": 1e-8}
    for m, r in ev.items():
        out[m] = {"cg_iters_mean": r["cg_iters_mean"], "s_per_design_iter": r["s_per_iter"],
                  "cg_iters": r["cg_iters"]}
    out["learned_vs_previous_cg"] = ev["learned"]["cg_iters_mean"] / prev["cg_iters_mean"]
    out["learned_vs_cold_cg"] = ev["learned"]["cg_iters_mean"] / ev["cold"]["cg_iters_mean"]
    out["compliance_spread_last"] = float(np.ptp([r["compliance"][-1] for r in ev.values()]) /
                                          abs(prev["compliance"][-1]))
    # the most any predicted start could save on this run (exact solution blended in)
    out["start_quality_bound"] = LW.start_quality_bound(nels, run, k=8)
    return out


def full_scale_leg(tg, stream, steps):
    """Configuration 5 at full size: 3D cantilever 256x128x128 (4.19M cells), V = 0.2,
    rmin = 2.0, p = 3, rtol 1e-8: FP32-IR with the previous-step start (design iterations
    2..1+steps timed) against plain FP64 PCG, cold started (design iteration 2 timed)."""
    import torch
    L = tg._lib
    prob = tg.PointLoadCantilever((256, 128, 128), (1.0, 1.0, 1.0), load="face_centre")
    out = {"workload": "3D cantilever 256x128x128 hex8 (4,194,304 cells, %d dofs), V 0.2, rmin 2.0" % prob.ndofs}
    for name, prec, warm, k in (("fp32_ir", "fp32_ir", True, steps), ("fp64_pcg", "fp64", False, 1)):
        s = tg.FEASolver(tg.GB300Solver, prob, xmin=XMIN, penalty=tg.PowerPenaltyFun(PEN), rtol=RTOL, abstol=0.0,
                         cg_max_iter=200000, precision=prec, warm_start=warm)
        L.check(L.lib().tog_set_stream(s.handle, L.C.c_void_p(stream.cuda_stream)))
        loop = tg.SIMPLoop(s, volfrac=0.2, rmin=2.0, filter="density", x0=np.full(prob.ncells, 0.2))
        loop.step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        sts = []
        e0.record(stream)
        for _ in range(k):
            sts.append(loop.step())
        e1.record(stream)
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / 1e3
        out[name] = {"design_iters_per_s": k / t, "steps": k, "cg_iters_per_step": [int(x.cg_iterations) for x in sts],
                     "compliance": [float(x.compliance) for x in sts]}
        s.close()
    out["fp32_ir_vs_fp64"] = out["fp32_ir"]["design_iters_per_s"] / out["fp64_pcg"]["design_iters_per_s"]
    return out


def run_ours(args):
    import torch
    ws, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import __graft_entry__ as ge
    tg = ge.load()
    L = tg._lib
    stream = torch.cuda.Stream()
    prob = tg.PointLoadCantilever(NELS, (1.0, 1.0, 1.0), load="face_centre")
    n = prob.ncells

    def make_solver(precision, warm):
        s = tg.FEASolver(tg.GB300Solver, prob, xmin=XMIN, penalty=tg.PowerPenaltyFun(PEN), rtol=RTOL, abstol=0.0,
                         cg_max_iter=200000, precision=precision, warm_start=warm)
        L.check(L.lib().tog_set_stream(s.handle, L.C.c_void_p(stream.cuda_stream)))
        return s

    # ---- optimised path: FP32 K*u / PCG inside FP64 refinement, warm start from the previous step
    solver = make_solver("fp32_ir", True)
    loop = tg.SIMPLoop(solver, volfrac=VOLFRAC, rmin=RMIN, filter="density")
    stats = []
    for _ in range(args.warmup):
        loop.step()
    torch.cuda.synchronize()
    x_w, u_w = loop.x.copy(), solver.u.copy()   # the state the timed window starts from
    barrier(ws)
    l0 = L.lib().tog_launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(args.steps):
                stats.append(loop.step())
            e1.record(stream)
        torch.cuda.synchronize()
    launches = L.lib().tog_launch_count() - l0
    t_dev = e0.elapsed_time(e1) / 1e3
    t_dev = max_over_ranks(t_dev, ws)
    value = replica_rate(args.steps, ws, t_dev)
    clocks = clk.summary()

    if args.no_extra:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": "design_iters/s", "steps": args.steps,
                              "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps,
                              "gpu_launches": int(launches), "clocks": clocks,
                              "partial": "e2e/fp64/roofline legs skipped (--no-extra)",
                              "inner_cg_iters_per_step": [int(s.cg_iterations) for s in stats]}), flush=True)
        return 0

    # ---- e2e: the same design iterations (restarted from the state after the warm-up)
    #      through the C ABI, the design copied from and to pinned host memory every step
    xh = torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
    xh[:] = x_w
    solver.u = u_w
    torch.cuda.synchronize()
    barrier(ws)
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e2e_cg = []
    with torch.cuda.stream(stream):
        f0.record(stream)
        for _ in range(args.steps):
            L.check(L.lib().tog_set_design(solver.handle, L.dptr(xh)))
            st = L.IterStats()
            L.check(L.lib().tog_simp_step(solver.handle, L.TOG_FP32_IR, RTOL, 200000, 1, L.C.byref(st)))
            L.check(L.lib().tog_get_design(solver.handle, L.dptr(xh)))
            e2e_cg.append(int(st.cg_iterations))
        f1.record(stream)
    torch.cuda.synchronize()
    t_e2e = max_over_ranks(f0.elapsed_time(f1) / 1e3, ws)
    e2e = {"value": ws * args.steps / t_e2e, "unit": "design_iters/s", "h2d_bytes_per_step": 8 * n,
           "d2h_bytes_per_step": 8 * n + 8,
           "window": "design iterations %d..%d, as value" % (args.warmup + 1, args.warmup + args.steps),
           "cg_iters_mean": float(np.mean(e2e_cg))}

    # ---- plain FP64 Jacobi PCG (cold start, as the reference) over the same design-iteration window
    s64 = make_solver("fp64", False)
    loop64 = tg.SIMPLoop(s64, volfrac=VOLFRAC, rmin=RMIN, filter="density")
    for _ in range(args.warmup):
        loop64.step(precision="fp64", warm_start=False)
    k64 = max(1, min(args.steps, int(os.environ.get("FP64_STEPS", str(args.steps)))))
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    st64 = []
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        g0.record(stream)
        for _ in range(k64):
            st64.append(loop64.step(precision="fp64", warm_start=False))
        g1.record(stream)
    torch.cuda.synchronize()
    t64 = g0.elapsed_time(g1) / 1e3
    fp64 = {"value": k64 / t64, "unit": "design_iters/s", "steps": k64, "warmup": args.warmup,
            "cg_iters_per_step": [int(s.cg_iterations) for s in st64],
            "window": "design iterations %d..%d of a cold-start FP64 trajectory (FP32-IR: %d..%d)"
                      % (args.warmup + 1, args.warmup + k64, args.warmup + 1, args.warmup + args.steps)}
    fp64["fp32ir_vs_fp64"] = value / fp64["value"]
    fp64["ms_per_pcg_iter_fp64"] = 1e3 * t64 / max(1, sum(fp64["cg_iters_per_step"]))
    fp64["ms_per_pcg_iter_fp32ir"] = 1e3 * t_dev / max(1, sum(int(s.cg_iterations) for s in stats))

    # ---- design iteration 1 on the GPU (FP32-IR and FP64), for the comparison with the oracle
    s64.close()
    x0 = np.full(n, VOLFRAC)
    first = {}
    for name in ("fp32_ir", "fp64"):
        s_ = make_solver(name, False)
        df_ = tg.DensityFilterFun(s_, RMIN)
        xf = df_(tg.PseudoDensities(x0)).x
        comp = tg.ComplianceFun(s_)
        c = comp(tg.PseudoDensities(xf))
        g = comp.pullback(1.0)
        dc = df_.pullback(g)
        dv = df_.pullback(np.full(n, 1.0 / n))
        xn, _, _ = tg.oc_update(s_, x0, dc, dv, dv, VOLFRAC, MOVE)
        first[name] = dict(xf=xf, u=s_.u.copy(), c=c, dc=dc, x_new=xn)
        s_.close()

    # ---- roofline of the dominant kernel (FP32 PCG operator, k_march3) and of the
    #      PCG update, each timed alone with CUDA events on the launching stream
    peaks, src = read_peaks()

    def time_kernel(kernel, nl):
        L.check(L.lib().tog_bench_kernel(solver.handle, kernel, L.TOG_FP32_IR, 10))
        torch.cuda.synchronize()
        h0, h1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            h0.record(stream)
            L.check(L.lib().tog_bench_kernel(solver.handle, kernel, L.TOG_FP32_IR, nl))
            h1.record(stream)
        torch.cuda.synchronize()
        t = h0.elapsed_time(h1) / 1e3 / nl
        nb = L.C.c_double()
        L.check(L.lib().tog_kernel_bytes(solver.handle, kernel, L.TOG_FP32_IR, L.C.byref(nb)))
        return t, nb.value

    t_k, nbytes = time_kernel(0, 200)
    t_u, ubytes = time_kernel(1, 200)
    achieved = nbytes / t_k / 1e9
    roof = {"bound": "hbm", "kernel": "k_march3 (FP32 PCG operator)", "achieved": achieved, "peak": peaks["hbm_gbs"],
            "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"], "traffic": read_traffic(n),
            "algorithmic_bytes_per_launch": nbytes, "us_per_launch": t_k * 1e6,
            "peak_source": src + " (MEASURED_PEAKS.json hbm_gbs, burst copy)" if src == "measured" else src,
            "pcg_update": {"kernel": "k_pcg_update3<float>", "us_per_launch": t_u * 1e6,
                           "achieved_gbs": ubytes / t_u / 1e9, "frac": ubytes / t_u / 1e9 / peaks["hbm_gbs"]}}
    solver.close()
    batched = batch_leg(tg, stream, peaks, src, int(os.environ.get("BATCH_STEPS", "3")))
    learned = learned_leg(tg, int(os.environ.get("LEARNED_STEPS", "12")))
    full = full_scale_leg(tg, stream, int(os.environ.get("FULL_STEPS", "2")))

    cg = [int(s.cg_iterations) for s in stats]
    roof["fp64_pcg_same_window"] = {"design_iters_per_s": fp64["value"], "fp32ir_vs_fp64": fp64["fp32ir_vs_fp64"]}
    line = {"metric": METRIC, "value": value, "unit": "design_iters/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 K*u and PCG inside f64 refinement",
            "data": "synthetic", "config": config_line(),
            "method": "FP32-IR + previous-step warm start", "parallelism": "replicas" if ws > 1 else "single GPU",
            "clocks": clocks, "e2e": e2e, "gpu_launches": int(launches), "roofline": roof,
            "fp64_pcg": fp64, "batched_2d": batched, "learned_warm_start": learned,
            "full_scale_256x128x128": full,
            "inner_cg_iters_per_step": cg,
            "outer_iters_per_step": [int(s.outer_iterations) for s in stats],
            "compliance_last": stats[-1].compliance}
    if rank == 0 and not args.no_cpu:
        threads = cpu_threads()
        r = cpu_design_iterations(threads, 1, 0.0)
        sec = r["seconds"][0]
        line["cpu_baseline"] = {"value": 1.0 / sec, "unit": "design_iters/s", "cores": threads, "kind": "port",
                                "sample": "design iteration 1, whole: filter, cold Jacobi PCG to rtol 1e-8 (%d "
                                          "iterations), compliance, pullback, OC" % r["cg_iters"][0]}
        ref = r["first"]

        def relmax(a, b):
            return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))

        acc = {"oracle": "C port of the reference path, FP64 Jacobi PCG to rtol 1e-8, design iteration 1"}
        for name, g in first.items():
            acc[name] = {"compliance_rel_err": abs(g["c"] - ref["c"]) / abs(ref["c"]),
                         "sens_rel_err": relmax(g["dc"], ref["dc"]),
                         "filtered_density_rel_err": relmax(g["xf"], ref["xf"]),
                         "displacement_rel_err_2norm": float(np.linalg.norm(g["u"] - ref["u"]) /
                                                             np.linalg.norm(ref["u"])),
                         "x_new_max_abs_diff": float(np.max(np.abs(g["x_new"] - ref["x_new"])))}
        line["accuracy_vs_oracle"] = acc
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def run_profile(args):
    """Small profiling driver: three launches each of the FP32 PCG operator and PCG
    update kernels, then one FP64 operator launch, on a uniform design (no timing;
    used under ncu)."""
    import __graft_entry__ as ge
    tg = ge.load()
    L = tg._lib
    nels = tuple(int(v) for v in args.nels.split(","))
    prob = tg.PointLoadCantilever(nels, (1.0,) * len(nels), load="face_centre")
    s = tg.FEASolver(tg.GB300Solver, prob, xmin=XMIN, penalty=tg.PowerPenaltyFun(PEN))
    s.vars = np.full(prob.ncells, VOLFRAC)
    s._push_vars()
    L.check(L.lib().tog_bench_kernel(s.handle, 0, L.TOG_FP32_IR, 3))
    L.check(L.lib().tog_bench_kernel(s.handle, 1, L.TOG_FP32_IR, 3))
    L.check(L.lib().tog_bench_kernel(s.handle, 0, L.TOG_FP64, 1))
    v = np.empty(prob.ndofs)
    L.check(L.lib().tog_get_u(s.handle, L.dptr(v)))   # synchronises
    s.close()
    print("profile driver ok", nels)
    return 0


def run_rows(args):
    """Timings of the entry points beside the headline loop at 160x80x80 (FP32-IR unless
    stated; host wall time around each call after a CUDA synchronize, so the host-array
    calls include their copies): a design iteration of the device SIMP loop with OC and with
    MMA (3 timed after 3 warm-up each), the MMA update and the fixed-element projection /
    pullback on their own, a 3-load mean compliance (three cold solves), and an FP64 solve
    under the residual-norm rule and under EnergyCriteria.  Prints one JSON line."""
    import time
    import torch
    import __graft_entry__ as ge
    tg = ge.load()

    def timed(fn, reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            out = fn()
        torch.cuda.synchronize()
        return 1e3 * (time.perf_counter() - t0) / reps, out

    prob = tg.PointLoadCantilever(NELS, (1.0,) * 3, load="face_centre")
    n = prob.ncells
    out = {"workload": "3D PointLoadCantilever %dx%dx%d, V %.1f, rmin %.1f, p %.0f" % (NELS + (VOLFRAC, RMIN, PEN))}
    for opt in ("oc", "mma"):
        s = tg.FEASolver(tg.GB300Solver, prob, xmin=XMIN, penalty=tg.PowerPenaltyFun(PEN), rtol=RTOL, abstol=0.0,
                         cg_max_iter=200000, precision="fp32_ir", warm_start=True)
        loop = tg.SIMPLoop(s, volfrac=VOLFRAC, rmin=RMIN, filter="density", optimizer=opt)
        for _ in range(3):
            loop.step()
        ms, st = timed(loop.step, 3)
        out["simp_iteration_ms_" + opt] = ms
        out["simp_last_" + opt] = {"compliance": float(st.compliance), "volume": float(st.volume),
                                   "cg_iterations": int(st.cg_iterations)}
        s.close()
    s = tg.FEASolver(tg.GB300Solver, prob, xmin=XMIN, penalty=tg.PowerPenaltyFun(PEN), rtol=RTOL, abstol=0.0,
                     cg_max_iter=200000, precision="fp32_ir")
    rng = np.random.default_rng(0)
    x = rng.uniform(0.2, 0.8, n)
    df0 = -rng.uniform(0.1, 1.0, n)
    dg = np.full(n, 1.0 / n)
    tg.mma_update(s, x, df0, float(np.mean(x)) - VOLFRAC, dg)
    out["mma_update_ms_host_arrays"], _ = timed(lambda: tg.mma_update(s, x, df0, float(np.mean(x)) - VOLFRAC, dg), 5)
    black = [e for e in range(n) if e % NELS[0] == 0]
    g = tg.get_fixed_element_projector(s, black, [])
    xf = np.full(tg.get_free_variable_count(g), 0.5)
    g(xf)
    out["fixed_project_ms_host_arrays"], _ = timed(lambda: g(xf), 5)
    out["fixed_pullback_ms_host_arrays"], _ = timed(lambda: g.pullback(x), 5)
    g.detach()
    rules = [((NELS[0], NELS[1] / 2, NELS[2] / 2), lambda: np.array([0.0, -1.0, 0.0])),
             ((NELS[0], NELS[1], NELS[2] / 2), lambda: np.array([0.0, 0.0, 1.0])),
             ((NELS[0] / 2, NELS[1], NELS[2]), lambda: np.array([1.0, 0.0, 0.0]))]
    ml = tg.MultiLoad(prob, 1, rules[:1])
    import scipy.sparse as sp
    ml.F = sp.hstack([tg.MultiLoad(prob, 1, [r]).F for r in rules]).tocsc()
    mc = tg.MeanComplianceFun(ml, s, method="exact")
    xs = np.full(n, VOLFRAC)
    out["mean_compliance_3_loads_ms"], c = timed(lambda: mc(tg.PseudoDensities(xs)), 1)
    out["mean_compliance_3_loads_pcg_iterations"] = int(mc._ml.last_stats.iterations)
    s.close()
    for name, conv in (("default", tg.DefaultCriteria()), ("energy", tg.EnergyCriteria())):
        s = tg.FEASolver(tg.GB300Solver, prob, xmin=XMIN, penalty=tg.PowerPenaltyFun(PEN), rtol=RTOL, abstol=0.0,
                         cg_max_iter=200000, precision="fp64", conv=conv)
        s.vars = xs
        ms, _ = timed(s, 1)
        out["fp64_solve_" + name] = {"ms": ms, "iterations": int(s.last_stats.iterations)}
        s.close()
    print(json.dumps(out))
    return 0


def run_lengths(args):
    """The configurations at their own run lengths (opt-in, several minutes): the 3D
    cantilever 160x80x80 for 50 design iterations, the 256 uneven 2D cantilevers for 100,
    the 3D cantilever 256x128x128 for 200.  FP32-IR with the previous-step start; the
    compliance trajectory is kept, and at sampled iterations the compliance of the
    FP32-IR design is recomputed with a cold plain FP64 PCG solve (the FP32-IR error).
    Plain FP64 PCG runs the first design iterations of each 3D configuration for its
    rate.  Prints one JSON line per configuration."""
    import torch
    import __graft_entry__ as ge
    tg = ge.load()
    L = tg._lib
    stream = torch.cuda.Stream()

    def run3d(nels, volfrac, rmin, iters, samples, fp64_iters):
        prob = tg.PointLoadCantilever(nels, (1.0, 1.0, 1.0), load="face_centre")
        n = prob.ncells

        def mk(prec, warm):
            s = tg.FEASolver(tg.GB300Solver, prob, xmin=XMIN, penalty=tg.PowerPenaltyFun(PEN), rtol=RTOL,
                             abstol=0.0, cg_max_iter=400000, precision=prec, warm_start=warm)
            L.check(L.lib().tog_set_stream(s.handle, L.C.c_void_p(stream.cuda_stream)))
            return s
        s = mk("fp32_ir", True)
        loop = tg.SIMPLoop(s, volfrac=volfrac, rmin=rmin, filter="density", x0=np.full(n, volfrac))
        chk = mk("fp64", False)
        comp64 = tg.ComplianceFun(chk)
        traj, cg, errs, t_run = [], [], {}, 0.0
        for k in range(1, iters + 1):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            st = loop.step()
            e1.record(stream)
            torch.cuda.synchronize()
            t_run += e0.elapsed_time(e1) / 1e3
            traj.append(float(st.compliance))
            cg.append(int(st.cg_iterations))
            if k in samples:
                c64 = comp64(tg.PseudoDensities(loop.physical))
                errs[k] = abs(st.compliance - c64) / abs(c64)
        s.close()
        chk.close()
        s64 = mk("fp64", False)
        loop64 = tg.SIMPLoop(s64, volfrac=volfrac, rmin=rmin, filter="density", x0=np.full(n, volfrac))
        torch.cuda.synchronize()
        g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        g0.record(stream)
        cg64 = [int(loop64.step(precision="fp64", warm_start=False).cg_iterations) for _ in range(fp64_iters)]
        g1.record(stream)
        torch.cuda.synchronize()
        t64 = g0.elapsed_time(g1) / 1e3
        s64.close()
        return {"design_iters": iters, "fp32ir_design_iters_per_s": iters / t_run,
                "fp32ir_cg_iters_mean": float(np.mean(cg)), "compliance_first_last": [traj[0], traj[-1]],
                "compliance_every_10": traj[9::10], "fp32ir_vs_fp64_compliance_rel_err": errs,
                "fp64_pcg": {"design_iters": fp64_iters, "design_iters_per_s": fp64_iters / t64,
                             "cg_iters": cg64}}

    out = run3d((160, 80, 80), VOLFRAC, RMIN, 50, {1, 10, 25, 50}, 5)
    print(json.dumps({"config": "3D cantilever 160x80x80, V 0.3, rmin 1.5", **out}), flush=True)
    P = tg.uneven_cantilever_set(256, seed=0)
    b = tg.BatchedSIMP(P["nelx"], P["nely"], P["load_j"], P["volfrac"], P["rmin"], rtol=RTOL)
    rows = b.autotune()
    b.set_stream(stream.cuda_stream)
    comps, t_run = [], 0.0
    for k in range(100):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st = b.step()
        e1.record(stream)
        torch.cuda.synchronize()
        t_run += e0.elapsed_time(e1) / 1e3
        comps.append(b.results()[0].copy())
    res, nref, status = b.solve_info()
    b.close()
    comps = np.array(comps)
    print(json.dumps({"config": "256 uneven 2D cantilevers (seed 0)", "design_iters": 100, "tile_rows": rows,
                      "design_iters_per_s": 100 / t_run, "problem_design_iters_per_s": 25600 / t_run,
                      "compliance_sum_first_last": [float(comps[0].sum()), float(comps[-1].sum())],
                      "max_final_residual": float(np.max(res)), "failed": int(np.sum(status != 0))}), flush=True)
    out = run3d((256, 128, 128), 0.2, 2.0, 200, {1, 50, 100, 200}, 2)
    print(json.dumps({"config": "3D cantilever 256x128x128, V 0.2, rmin 2.0", **out}), flush=True)
    return 0


def run_profile_loop(args):
    """Launch-list driver of the device SIMP loop: one FP32-IR design iteration of the
    benchmark workload (160x80x80); prints its PCG iteration and refresh counts so that
    the kernels ncu lists can be checked against them (no timing; used under ncu)."""
    import __graft_entry__ as ge
    tg = ge.load()
    prob = tg.PointLoadCantilever(NELS, (1.0, 1.0, 1.0), load="face_centre")
    s = tg.FEASolver(tg.GB300Solver, prob, xmin=XMIN, penalty=tg.PowerPenaltyFun(PEN), rtol=RTOL, abstol=0.0,
                     cg_max_iter=200000, precision="fp32_ir", warm_start=True)
    loop = tg.SIMPLoop(s, volfrac=VOLFRAC, rmin=RMIN, filter="density")
    st = loop.step()
    print(json.dumps({"design_iterations": 1, "pcg_iterations": int(st.cg_iterations),
                      "fp64_refreshes": int(st.outer_iterations)}))
    s.close()
    return 0


def run_profile_batch(args):
    """Profiling driver of the batched 2D operator: the benchmark's 256 uneven cantilevers,
    the band height pinned to args.profile_batch rows, five launches of the FP32 operator
    over all problems and five of the update, outside the graph (ncu cannot profile kernels
    inside conditional graph nodes); no timing, used under ncu."""
    import __graft_entry__ as ge
    tg = ge.load()
    P = tg.uneven_cantilever_set(256, seed=0)
    b = tg.BatchedSIMP(P["nelx"], P["nely"], P["load_j"], P["volfrac"], P["rmin"], rtol=1e-8)
    b.set_tile_rows(int(args.profile_batch))
    for k in (0, 1):
        b.bench_kernel(k, 5)
    print("batch profile driver ok", int(args.profile_batch))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the e2e, accuracy, FP64 and roofline legs")
    ap.add_argument("--profile", action="store_true", help="run the small ncu driver instead of the benchmark")
    ap.add_argument("--nels", default="256,128,128", help="grid of --profile")
    ap.add_argument("--rows", action="store_true", help="time the entry points beside the headline loop")
    ap.add_argument("--profile-loop", action="store_true", help="run the device-loop launch-list driver")
    ap.add_argument("--runs", action="store_true",
                    help="run the configurations at their own lengths (50 / 100 / 200 design iterations)")
    ap.add_argument("--profile-batch", type=int, default=0, metavar="ROWS",
                    help="run the batched-operator ncu driver with this band height instead of the benchmark")
    args = ap.parse_args()
    if args.profile:
        return run_profile(args)
    if args.profile_batch:
        return run_profile_batch(args)
    if args.rows:
        return run_rows(args)
    if args.runs:
        return run_lengths(args)
    if args.profile_loop:
        return run_profile_loop(args)
    if args.warmup < 3:
        log("warmup raised to 3 (timing rule)")
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
