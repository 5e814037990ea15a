"""Training of the learned preconditioner on its block family, on the GPU.

The network is the polynomial graph-convolution preconditioner of the C ABI (astro_precond):
P r = (1/lambda) sum_k W_k T_k(xi(D^-1 A)) D^-1 r with one dpn x dpn weight per hop.  Its training
data are residual/error pairs of AStrO's own solves: for a block of the family, the plain FP64
Jacobi-GMRES iterates x_k after k Arnoldi steps give r_k = b - A x_k and e_k = x* - x_k with
A e_k = r_k, so the device loss ||r - A P r||^2 = ||A (P r - e)||^2 is the residual-space misfit
of the network's error prediction.  White-noise vectors are added so the whole spectrum of
D^-1 A is weighted (the GMRES residuals concentrate on its low end).  The weights are trained
block by block (a few conjugate-gradient steps with exact line search on each block's samples,
starting from the previous block's weights), then validated by the learned solve of a held-out
block: the trained weights are kept only if that solve needs fewer Krylov iterations than the
untrained (Chebyshev) network.

Command line (writes the network as JSON):
    python -m misc_gb300.learned --blocks 2000 --out trained.json

The per-node modulation (astro_precond_mlp) is the part of the network that sees the model: a
two-layer perceptron maps six features of every node of the assembled matrix (its stiffness
level, the contrast to its neighbours, connectivity, constraints, diagonal dominance) to a
scale of every Chebyshev hop at that node.  It is trained by Adam over a set of blocks of the
family, every step one device forward and backward pass (astro_precond_mlp_loss_grad) on one
block's samples:
    python -m misc_gb300.learned --mlp --blocks 48 --epochs 60 --out precond_mlp_cfg4.json
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import model as M
from .astro import (SOLVER_FGMRES_LEARNED, SOLVER_GMRES_JACOBI_FP64, AstroGPU, PrecondC, mlp_init, precond_init)


def block_system(m, fp32=False):
    """Context with the FP64 (and optionally FP32) stiffness assembled and the constraints scaled;
    returns (context, static right-hand side)."""
    g = AstroGPU(m)
    g.getElasticSolnLoad(1, export=False)
    if fp32:
        g.assemble_fp32()
    g.scaleElasticMPC()
    return g, g.static_rhs()


def gmres_residuals(g, b, steps=(10, 40, 160), restart=50):
    """r_k = b - A x_k for the plain FP64 Jacobi-GMRES iterate after k Arnoldi steps."""
    out = []
    for k in steps:
        m = min(k, restart)
        x, _ = g.solve_static(b, method=SOLVER_GMRES_JACOBI_FP64, rtol=1e-14, restart=m, max_iters=k,
                              allow_maxit=True)
        out.append(b - g.apply_operator(x, 64))
    return np.array(out)


def copy_precond(p):
    q = PrecondC()
    q.degree, q.dpn, q.ratio, q.lambda_scale = p.degree, p.dpn, p.ratio, p.lambda_scale
    for i in range(len(p.weights)):
        q.weights[i] = p.weights[i]
    return q


def to_json(p, meta=None):
    d = {"degree": int(p.degree), "dpn": int(p.dpn), "ratio": float(p.ratio), "lambda_scale": float(p.lambda_scale),
         "weights": [float(x) for x in p.weight_array().reshape(-1)]}
    if meta:
        d["meta"] = meta
    return d


def from_json(d):
    p = precond_init(d["degree"], d["ratio"], d["dpn"])
    p.lambda_scale = d["lambda_scale"]
    p.set_weights(np.array(d["weights"]))
    return p


def train_family(p0, seeds, nx=32, ny=16, nz=16, cg_steps=5, white=3, gmres_steps=(10, 40, 160), log=print):
    """Block-by-block training from p0 (not modified); returns (trained network, per-block log)."""
    p = copy_precond(p0)
    rng = np.random.default_rng(12345)
    hist = []
    for i, seed in enumerate(seeds):
        g, b = block_system(M.config4_block(nx, ny, nz, seed))
        parts = [gmres_residuals(g, b, gmres_steps)] if gmres_steps else []
        S = np.vstack(parts + [rng.standard_normal((white, g.n))])
        h = g.precond_train(p, S, iters=cg_steps)
        hist.append((int(seed), float(h[0]), float(h[-1])))
        if log and (i % 50 == 0 or i == len(seeds) - 1):
            log(f"block {i + 1}/{len(seeds)} seed {seed}: loss {h[0]:.4e} -> {h[-1]:.4e}")
        del g
    return p, hist


def validate(p_init, p_trained, m, rtol=1e-8):
    """Learned solves of a held-out block with both networks: (iterations initial, iterations
    trained, seconds initial, seconds trained)."""
    g, b = block_system(m, fp32=True)
    out = []
    for p in (p_init, p_trained):
        g.solve_static(b, method=SOLVER_FGMRES_LEARNED, rtol=rtol, precond=p, allow_maxit=True)
        _, st = g.solve_static(b, method=SOLVER_FGMRES_LEARNED, rtol=rtol, precond=p, allow_maxit=True)
        out.append((int(st.iterations) if st.status == 0 else 10 ** 9, float(st.seconds)))
    return out[0][0], out[1][0], out[0][1], out[1][1]


def mlp_to_json(p, mlp, meta=None):
    w1, b1, w2, b2 = mlp.params()
    d = {"network": to_json(p), "hidden": int(mlp.hidden), "outputs": int(mlp.outputs), "w1": w1.tolist(),
         "b1": b1.tolist(), "w2": w2.tolist(), "b2": b2.tolist()}
    if meta:
        d["meta"] = meta
    return d


def mlp_from_json(d):
    """(polynomial network, perceptron) of a file written by mlp_to_json."""
    p = from_json(d["network"])
    m = mlp_init(d["hidden"], d["outputs"])
    m.set_params(np.array(d["w1"]), np.array(d["b1"]), np.array(d["w2"]), np.array(d["b2"]))
    return p, m


def train_mlp(p, seeds, hidden=16, epochs=60, lr=3e-3, white=3, gmres_steps=(10, 40, 160), seed=0, log=print):
    """Adam over the blocks of seeds (32x16x16 of the config-4 family), one device forward and
    backward pass of the modulated network per block and step, the polynomial network p fixed.
    Returns (perceptron, mean loss over the blocks per epoch, mean loss of the unmodulated
    network)."""
    rng = np.random.default_rng(seed + 12345)
    sets = []
    for s in seeds:
        g, b = block_system(M.config4_block(32, 16, 16, s))
        parts = [gmres_residuals(g, b, gmres_steps)] if gmres_steps else []
        S = np.vstack(parts + [rng.standard_normal((white, g.n))])
        sets.append((g, S))
    mlp = mlp_init(hidden, p.degree + 1, seed=seed)
    x = mlp.vector()
    m1, m2 = np.zeros_like(x), np.zeros_like(x)
    base = float(np.mean([g.precond_loss_grad(p, S)[0] for g, S in sets]))
    hist, t = [], 0
    order = np.arange(len(sets))
    for ep in range(epochs):
        rng.shuffle(order)
        losses = []
        for i in order:
            g, S = sets[i]
            mlp.set_vector(x)
            L, _, gm = g.mlp_loss_grad(p, mlp, S)
            losses.append(L)
            gv = gm.vector()
            t += 1
            m1 = 0.9 * m1 + 0.1 * gv
            m2 = 0.999 * m2 + 0.001 * gv * gv
            x = x - lr * (m1 / (1 - 0.9 ** t)) / (np.sqrt(m2 / (1 - 0.999 ** t)) + 1e-12)
        hist.append(float(np.mean(losses)))
        if log and (ep % 10 == 0 or ep == epochs - 1):
            log(f"epoch {ep + 1}/{epochs}: mean loss {hist[-1]:.5e} (unmodulated {base:.5e})")
    mlp.set_vector(x)
    return mlp, hist, base


def validate_mlp(p, mlp, seeds, rtol=1e-8):
    """Learned solves of held-out blocks without and with the modulation: per block (iterations,
    seconds, status) of each, the second solve of each timed."""
    out = []
    for s in seeds:
        g, b = block_system(M.config4_block(32, 16, 16, s), fp32=True)
        r = {}
        for name, kw in (("chebyshev", {}), ("modulated", {"mlp": mlp})):
            for _ in range(2):
                _, st = g.solve_static(b, method=SOLVER_FGMRES_LEARNED, rtol=rtol, precond=p, allow_maxit=True, **kw)
            r[name] = (int(st.iterations), float(st.seconds), int(st.status))
        out.append({"seed": int(s), **r})
        del g
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--blocks", type=int, default=2000)
    ap.add_argument("--seed0", type=int, default=2000)
    ap.add_argument("--degree", type=int, default=24)
    ap.add_argument("--ratio", type=float, default=3000.0)
    ap.add_argument("--cg-steps", type=int, default=5)
    ap.add_argument("--out", required=True)
    ap.add_argument("--mlp", action="store_true", help="train the per-node modulation (perceptron)")
    ap.add_argument("--epochs", type=int, default=60)
    ap.add_argument("--hidden", type=int, default=16)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--white", type=int, default=3, help="white-noise samples per block")
    ap.add_argument("--gmres-steps", default="10,40,160",
                    help="GMRES residual samples per block: the step counts (empty: none)")
    a = ap.parse_args()
    t0 = time.time()
    if a.mlp:
        p = precond_init(a.degree, a.ratio, 3)
        seeds = list(range(a.seed0, a.seed0 + a.blocks))
        held = list(range(a.seed0 + a.blocks + 100, a.seed0 + a.blocks + 106))
        gsteps = tuple(int(x) for x in a.gmres_steps.split(",") if x.strip())
        mlp, hist, base = train_mlp(p, seeds, hidden=a.hidden, epochs=a.epochs, lr=a.lr, white=a.white,
                                    gmres_steps=gsteps)
        t1 = time.time()
        val = validate_mlp(p, mlp, held)
        meta = {"family": "config-4 32x16x16 brick blocks (model.config4_block)", "training_seeds": [seeds[0], seeds[-1]],
                "held_out_seeds": held,
                "samples_per_block": (f"GMRES residuals after {', '.join(map(str, gsteps))} steps + " if gsteps else "") +
                                     f"{a.white} white-noise vectors",
                "optimizer": f"Adam lr {a.lr}, {a.epochs} epochs", "hidden": a.hidden, "loss_unmodulated": base,
                "loss_per_epoch": hist, "train_seconds": t1 - t0, "validation": val}
        print(json.dumps({k: v for k, v in meta.items() if k != "loss_per_epoch"}))
        with open(a.out, "w") as f:
            json.dump(mlp_to_json(p, mlp, meta), f, indent=1)
        return
    p0 = precond_init(a.degree, a.ratio, 3)
    seeds = list(range(a.seed0, a.seed0 + a.blocks))
    p, hist = train_family(p0, seeds, cg_steps=a.cg_steps)
    t1 = time.time()
    it0, it1, s0, s1 = validate(p0, p, M.config4_block(32, 16, 16, a.seed0 + a.blocks + 7))
    keep = it1 < it0
    meta = {"blocks": a.blocks, "seeds": [seeds[0], seeds[-1]], "cg_steps_per_block": a.cg_steps,
            "samples_per_block": "GMRES residuals after 10, 40, 160 steps + 3 white-noise vectors",
            "train_seconds": t1 - t0, "loss_first_block": hist[0][1:], "loss_last_block": hist[-1][1:],
            "validation_iterations": {"initial": it0, "trained": it1}, "selected": "trained" if keep else "initial"}
    print(json.dumps(meta))
    with open(a.out, "w") as f:
        json.dump(to_json(p if keep else p0, meta), f, indent=1)


if __name__ == "__main__":
    main()
