"""Learned warm start for 3D SIMP solves (no counterpart in TopOpt.jl).

The network (WarmStartNet, tensor-core kernels of libtopopt_gb300) maps the
state of a design iteration (new filtered densities and their change, the
previous displacement and its residual r0 = f - K(new densities) u_prev) to a
correction d of the previous displacement; the exact correction is K^-1 r0, so
the network learns an approximate inverse of K(rho) applied to the residual.  The solver moves u_prev along d by the Galerkin step
alpha = d.r0 / d.K d before its PCG solve, so a poor prediction can never make
the start worse in the energy norm, and every solve still finishes to the same
residual tolerance: plain PCG stays both the fallback and the measure of the result.

Training data are the solver's own trajectories: seeded cantilever runs with
random volume fraction, load node on the free face and load direction
(LoadedCantilever), recorded on the device one design iteration at a time.
"""
import time

import numpy as np

from . import topopt_api as api


def sample_runs(n, nels, seed, volfrac=(0.2, 0.5)):
    """n seeded run descriptions: volume fraction U[volfrac], load node uniform on the
    free face (x = nelx), load direction uniform on the unit sphere."""
    rng = np.random.default_rng(seed)
    runs = []
    for _ in range(n):
        d = rng.standard_normal(3)
        runs.append({"volfrac": float(rng.uniform(*volfrac)),
                     "node": (int(rng.integers(0, nels[1] + 1)), int(rng.integers(0, nels[2] + 1))),
                     "direction": d / np.linalg.norm(d)})
    return runs


def make_loop(nels, run, rmin, rtol, warm_start):
    prob = api.LoadedCantilever(nels, (1.0, 1.0, 1.0), run["node"], run["direction"])
    s = api.FEASolver(api.GB300Solver, prob, xmin=1e-9, penalty=api.PowerPenaltyFun(3.0), rtol=rtol, abstol=0.0,
                      cg_max_iter=200000, precision="fp32_ir", warm_start=warm_start)
    return s, api.SIMPLoop(s, volfrac=run["volfrac"], rmin=rmin, filter="density")


def generate(nels, runs, steps, rmin=1.5, rtol=1e-8, device="cuda"):
    """Record (input, target) pairs of design iterations 2..steps of every run into
    CUDA tensors X (N, nz, ny, nx, 8) and Y (N, nz, ny, nx, 3)."""
    import torch
    nx, ny, nz = (n + 1 for n in nels)
    cap = len(runs) * (steps - 1)
    X = torch.empty((cap, nz, ny, nx, 8), dtype=torch.float32, device=device)
    Y = torch.empty((cap, nz, ny, nx, 3), dtype=torch.float32, device=device)
    k = 0
    for run in runs:
        s, loop = make_loop(nels, run, rmin, rtol, True)
        s.enable_previous_state()   # from the first iteration on, so the second one records
        for it in range(steps):
            if it > 0:
                s.record_next_step(X[k:k + 1], Y[k:k + 1])
            loop.step()
            if it > 0 and s.record_status():
                # target: the density-weighted correction rho~ (u_new - u_prev) (near-void
                # displacements are barely constrained and unpredictable), of unit RMS:
                # only its direction matters, the solver rescales it by the Galerkin step
                Y[k].mul_(X[k, ..., 0:1])
                Y[k].div_(Y[k].pow(2).mean().sqrt().clamp_min(1e-30))
                k += 1
        s.close()
    torch.cuda.synchronize()
    return X[:k], Y[:k]


def train(net, X, Y, epochs, lr=1e-3, seed=0, lr_min=1e-4):
    """Adam over the samples in a seeded random order; cosine learning-rate decay.
    Returns the mean loss of every epoch."""
    rng = np.random.default_rng(seed)
    n = X.shape[0]
    total = epochs * n
    hist, step = [], 0
    for _ in range(epochs):
        acc = 0.0
        for i in rng.permutation(n):
            lr_t = lr_min + 0.5 * (lr - lr_min) * (1.0 + np.cos(np.pi * step / total))
            acc += net.train_step(X[i:i + 1], Y[i:i + 1], lr_t)
            step += 1
        hist.append(acc / n)
    return hist


def evaluate(nels, run, steps, net=None, rmin=1.5, rtol=1e-8, modes=("cold", "previous", "extrapolate", "learned")):
    """Run the same seeded SIMP trajectory once per warm-start mode and report, per
    mode, the inner PCG iterations of every design iteration and the wall time per
    design iteration (the first iteration excluded: it has no previous state)."""
    import torch
    out = {}
    for mode in modes:
        s, loop = make_loop(nels, run, rmin, rtol, mode)
        if mode == "learned":
            s.attach_network(net)
        elif mode == "extrapolate":
            s.enable_previous_state()
        its, comp, t = [], [], []
        for _ in range(steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            st = loop.step()
            t.append(time.perf_counter() - t0)
            its.append(int(st.cg_iterations))
            comp.append(float(st.compliance))
        s.close()
        out[mode] = {"cg_iters": its, "compliance": comp, "s_per_iter": float(np.mean(t[1:])),
                     "cg_iters_mean": float(np.mean(its[1:]))}
    return out


def start_quality_bound(nels, run, k=8, thetas=(0.0, 0.5, 0.9, 0.99, 0.999), rmin=1.5, rtol=1e-8):
    """What any predicted start can save at most.  After k design iterations of the run,
    the solve of iteration k + 1 (densities rho, previous solution u_prev, exact solution
    u* = the FP64 solve to rtol 1e-13) is repeated from u_prev + theta (u* - u_prev) for
    every theta, i.e. from a prediction that removes the fraction theta of the error of
    the previous-step start (theta = 0), and from a cold start.  Returns the inner PCG
    iterations of FP32-IR to rtol (relative to ||f||) and the relative energy-norm error
    ||u0 - u*||_K / ||u*||_K of each start."""
    s, loop = make_loop(nels, run, rmin, rtol, True)
    for _ in range(k):
        loop.step()
    u_prev = s.u
    loop.step()
    rho = loop.physical
    s.close()
    prob = api.LoadedCantilever(nels, (1.0, 1.0, 1.0), run["node"], run["direction"])
    t = api.FEASolver(api.GB300Solver, prob, xmin=1e-9, penalty=api.PowerPenaltyFun(3.0), rtol=1e-13, abstol=0.0,
                      cg_max_iter=400000, precision="fp64", warm_start=True)
    t.vars = rho
    t.u = u_prev
    t()
    ustar = t.u
    t.rtol = rtol
    kstar = float(ustar @ t.matvec(ustar))
    out = {"design_iteration": k + 1, "rtol": rtol, "starts": []}
    for name, u0 in [("cold", np.zeros_like(ustar))] + [("theta=%g" % th, u_prev + th * (ustar - u_prev))
                                                        for th in thetas]:
        e = u0 - ustar
        t.u = u0
        t(precision="fp32_ir", warm_start=True)
        out["starts"].append({"start": name, "pcg_iters": int(t.last_stats.iterations),
                              "energy_error": float(np.sqrt(max(e @ t.matvec(e), 0.0) / kstar))})
    t.close()
    return out


def main(argv=None):
    """Train the warm-start network for one grid and evaluate it:
        python -m topopt_gb300.learned --nels 96,48,48 --runs 40 --steps 26 --epochs 8 \\
            --out weights_96x48x48.npy
    (the package is importable as topopt_gb300 after __graft_entry__.load()).  Writes the
    FP32 parameter vector (.npy) and a JSON log (training losses, evaluation) beside it."""
    import argparse
    import json
    import torch
    ap = argparse.ArgumentParser()
    ap.add_argument("--nels", default="96,48,48")
    ap.add_argument("--runs", type=int, default=40)
    ap.add_argument("--steps", type=int, default=26)
    ap.add_argument("--epochs", type=int, default=24)
    ap.add_argument("--lr", type=float, default=3e-4)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--eval-runs", type=int, default=2)
    ap.add_argument("--eval-steps", type=int, default=20)
    ap.add_argument("--out", default="weights.npy")
    a = ap.parse_args(argv)
    nels = tuple(int(v) for v in a.nels.split(","))
    t0 = time.time()
    X, Y = generate(nels, sample_runs(a.runs, nels, a.seed), a.steps)
    t_gen = time.time() - t0
    net = api.WarmStartNet(tuple(n + 1 for n in nels), batch=1, seed=a.seed)
    torch.cuda.synchronize()
    t0 = time.time()
    hist = train(net, X, Y, a.epochs, lr=a.lr, seed=a.seed)
    torch.cuda.synchronize()
    t_train = time.time() - t0
    np.save(a.out, net.get_params())
    Xv, Yv = generate(nels, sample_runs(a.eval_runs, nels, a.seed + 1000), a.steps)
    val = float(np.mean([net.gradients(Xv[i:i + 1], Yv[i:i + 1])[0] for i in range(Xv.shape[0])]))
    del Xv, Yv
    evals = [evaluate(nels, r, a.eval_steps, net) for r in sample_runs(a.eval_runs, nels, a.seed + 1000)]
    log = {"nels": nels, "runs": a.runs, "steps": a.steps, "samples": int(X.shape[0]), "epochs": a.epochs,
           "lr": a.lr, "seed": a.seed, "generate_s": t_gen, "train_s": t_train,
           "train_ms_per_step": 1e3 * t_train / (a.epochs * X.shape[0]), "loss_per_epoch": hist,
           "target_mean_square": float(Y.pow(2).mean()), "validation_loss_heldout_runs": val,
           "evaluation": evals}
    with open(a.out.rsplit(".", 1)[0] + ".json", "w") as f:
        json.dump(log, f, indent=1)
    print(json.dumps({k: v for k, v in log.items() if k != "evaluation"}))
    for e in evals:
        print({m: (round(r["cg_iters_mean"]), round(r["s_per_iter"], 4)) for m, r in e.items()})


if __name__ == "__main__":
    main()
