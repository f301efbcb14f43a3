"""Train the outer-iteration accelerator and write data/mlp_accel.npy.

    python -m staticbtesolver_gb300.train_accel [--problems 40] [--steps 4000] [--out path]

Training data are the solver's own temperature histories on seeded 2D
problems (learned.training_problems); the network is trained on the GPU by
the project's kernels (bte_mlp_train).  The held-out evaluation solves the
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


def evaluate(params, name="square20k", every=8):
    import staticbtesolver_gb300 as S

    with tempfile.TemporaryDirectory() as tmp:
        p = synth.make_problem(name, tmp)
        prob = S.Problem(p.geo, p.bc_file, p.band_file, p.DM, p.num_theta, p.num_phi, p.T_ref, p.L_x, p.L_y, p.L_z)
        out = {}
        for label, accel in (("plain", 0), ("learned", 1), ("aitken", 2)):
            ctx = S.Context(0).load(prob)
            if accel == 1:
                ctx.set_mlp(params)
            ctx.solve(max_iter=20000, tol=1e-5, form=S.FORM_SWEEP, accel=accel, accel_every=every)  # warm
            st, rep = ctx.solve(max_iter=20000, tol=1e-5, form=S.FORM_SWEEP, accel=accel, accel_every=every)
            out[label] = dict(status=st, n_iter=rep.n_iter, accel_steps=rep.accel_steps, ms=rep.ms_total,
                              T=ctx.temperature())
            ctx.close()
        T0 = out["plain"]["T"]
        for v in out.values():
            v["rel_l2_T_minus_Tref_vs_plain"] = float(np.linalg.norm(v["T"] - T0) / np.linalg.norm(T0 - 300.0))
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
    ap.add_argument("--report", default="")
    args = ap.parse_args()
    t0 = time.time()
    X, Y, info = learned.generate(learned.training_problems(args.problems, args.seed))
    t1 = time.time()
    p, loss = learned.train(X, Y, steps=args.steps, batch=args.batch, lr=args.lr, seed=args.seed)
    t2 = time.time()
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    np.save(args.out, p)
    ev = evaluate(p)
    rep = dict(samples=int(len(Y)), problems=info, generate_s=t1 - t0, train_s=t2 - t1,
               loss_first=float(loss[:50].mean()), loss_last=float(loss[-50:].mean()), eval=ev)
    print(json.dumps(rep))
    if args.report:
        json.dump(rep, open(args.report, "w"), indent=1)


if __name__ == "__main__":
    main()
