"""Train the outer-iteration accelerator and write data/mlp_accel.npy.

    python -m staticbtesolver_gb300.train_accel [--problems 40] [--steps 4000] [--out path]

Training data are the solver's own temperature histories on seeded 2D
problems (learned.training_problems): plain, Aitken-accelerated, and, in each
further round, accelerated by the network of the round before.  The network
is trained on the GPU by the project's kernels (bte_mlp_train).  The held-out evaluation solves the
square20k workload with and without the accelerator.
"""
from __future__ import annotations

import argparse
import json
import os
import tempfile
import time

import numpy as np

from . import learned, synth


def evaluate(params, name="square20k", everies=(4, 6, 8), tol=1e-5):
    """Outer iterations and wall time to margin <= tol on a held-out workload: plain,
    Aitken and learned at each extrapolation interval, with each field's relative L2
    distance (of T - T_ref) to the plain run and to the field converged to 1e-10."""
    import staticbtesolver_gb300 as S

    with tempfile.TemporaryDirectory() as tmp:
        p = synth.make_problem(name, tmp)
        prob = S.Problem(p.geo, p.bc_file, p.band_file, p.DM, p.num_theta, p.num_phi, p.T_ref, p.L_x, p.L_y, p.L_z)
        out = {}
        runs = [("converged", 0, 8, 1e-10), ("plain", 0, 8, tol)]
        runs += [(f"{lab}_every{e}", a, e, tol) for e in everies for lab, a in (("learned", 1), ("aitken", 2))]
        for label, accel, every, t in runs:
            ctx = S.Context(0).load(prob)
            if accel == 1:
                ctx.set_mlp(params)
            ctx.solve(max_iter=20000, tol=t, form=S.FORM_SWEEP, accel=accel, accel_every=every)  # warm
            st, rep = ctx.solve(max_iter=20000, tol=t, form=S.FORM_SWEEP, accel=accel, accel_every=every)
            out[label] = dict(status=st, n_iter=rep.n_iter, accel_steps=rep.accel_steps, reverts=rep.accel_reverts,
                              ms=rep.ms_total,
                              T=ctx.temperature())
            ctx.close()
        T0, Tc = out["plain"]["T"] - p.T_ref, out["converged"]["T"] - p.T_ref
        for v in out.values():
            v["rel_l2_vs_plain"] = float(np.linalg.norm(v["T"] - p.T_ref - T0) / np.linalg.norm(T0))
            v["rel_l2_vs_converged"] = float(np.linalg.norm(v["T"] - p.T_ref - Tc) / np.linalg.norm(Tc))
            del v["T"]
        return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--problems", type=int, default=40)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--out", default=learned.WEIGHTS)
    ap.add_argument("--rounds", type=int, default=3)
    ap.add_argument("--val-problems", type=int, default=12)
    ap.add_argument("--report", default="")
    ap.add_argument("--no-eval", action="store_true", help="skip the square20k evaluation")
    args = ap.parse_args()
    t0 = time.time()
    specs = learned.training_problems(args.problems, args.seed)
    # round 0: the plain and Aitken-accelerated trajectories; then each round adds the
    # trajectories of the network just trained (it meets the states it creates)
    X, Y, info = learned.generate(specs, accel=0)
    Xa, Ya, info_a = learned.generate(specs, accel=2)
    X, Y = np.concatenate([X, Xa]), np.concatenate([Y, Ya])
    rng = np.random.default_rng(args.seed)
    p, rounds = None, []
    for r in range(args.rounds):
        val = rng.random(len(Y)) < 0.1
        Xt, Yt = learned.mirrored(X[~val], Y[~val])
        p, loss = learned.train(Xt, Yt, steps=args.steps, batch=args.batch, lr=args.lr, seed=args.seed + r, params=p)
        p, lam = learned.shrink(p, X[val], Y[val])
        rounds.append(dict(samples=int(len(Y)), loss_first=float(loss[:50].mean()), loss_last=float(loss[-50:].mean()),
                           shrink=lam))
        if r + 1 < args.rounds:
            Xl, Yl, info_l = learned.generate(specs, accel=1, params=p)
            rounds[-1]["learned_iters"] = int(sum(i["n_iter"] for i in info_l))
            X, Y = np.concatenate([X, Xl]), np.concatenate([Y, Yl])
    rounds[-1]["plain_iters"] = int(sum(i["n_iter"] for i in info))
    rounds[-1]["aitken_iters"] = int(sum(i["n_iter"] for i in info_a))
    # output scale chosen on held-out problems by the iterations it saves (0 = Aitken)
    p, totals = learned.select_scale(p, learned.training_problems(args.val_problems, args.seed + 1000))
    t2 = time.time()
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    np.save(args.out, p)
    ev = None if args.no_eval else evaluate(p)
    rep = dict(problems=info, train_s=t2 - t0, rounds=rounds, scale_selection=totals, eval=ev)
    print(json.dumps(rep))
    if args.report:
        json.dump(rep, open(args.report, "w"), indent=1)


if __name__ == "__main__":
    main()
