"""Training loop of the learned accelerator: batches of (r, z) pairs from
data.PairSet, assembled on the GPU with torch, and forward, loss, backward and
Adam by the library's own kernels (doma_unet_*).

Usage on a GPU machine (writes the weights file):
    python -m doma_gb300.learned.train --problems 2000 --steps 6000 --out weights.npz
"""
from __future__ import annotations

import argparse
import math
import time

import numpy as np
import torch

from .. import problems as P
from . import data as D
from .net import IN_CHANNELS, UNet


def make_batch(ps: D.PairSet, gen: torch.Generator, batch: int):
    """x [B,n,n,n,16] bf16 and target [B,n,n,n] f32.  Each sample is a random
    (problem, group) with either one recorded iterate (random sign) or a
    Gaussian combination of all K recorded iterates."""
    Pn, K, G, N = ps.R.shape
    dev = ps.R.device
    p = torch.randint(0, Pn, (batch,), generator=gen, device="cpu").to(dev)
    g = torch.randint(0, G, (batch,), generator=gen, device="cpu").to(dev)
    coef = torch.randn((batch, K), generator=gen, device="cpu")
    onehot = torch.rand((batch,), generator=gen, device="cpu") < 0.5
    k = torch.randint(0, K, (batch,), generator=gen, device="cpu")
    sign = torch.where(torch.rand((batch,), generator=gen) < 0.5, -1.0, 1.0)
    oh = torch.zeros((batch, K))
    oh[torch.arange(batch), k] = sign
    coef = torch.where(onehot[:, None], oh, coef).to(dev)
    r = torch.einsum("bk,bkn->bn", coef, ps.R[p, :, g])
    z = torch.einsum("bk,bkn->bn", coef, ps.Z[p, :, g])
    s = r.pow(2).mean(dim=1, keepdim=True).sqrt().clamp_min(1e-30)
    n = ps.n
    x = torch.zeros((batch, N, IN_CHANNELS), dtype=torch.float32, device=dev)
    x[..., 0] = r / s
    x[..., 1] = ps.F[p, g, 0]
    x[..., 2] = ps.F[p, g, 1]
    x = x.to(torch.bfloat16).view(batch, n, n, n, IN_CHANNELS).contiguous()
    t = (z / s).view(batch, n, n, n).contiguous()
    return x, t


def sample_weights(t: torch.Tensor) -> torch.Tensor:
    """Per-sample loss weights that make each sample's squared error relative
    to its target's mean square (plus 1, so near-zero targets stay bounded),
    normalized to mean 1 over the batch."""
    w = 1.0 / (t.pow(2).flatten(1).mean(dim=1) + 1.0)
    return (w / w.mean()).float().contiguous()


def train(ps: D.PairSet, steps: int = 4000, batch: int = 16, lr: float = 1e-3,
          seed: int = 0, log_every: int = 200, log=print, init=None,
          weighted: bool = False) -> tuple[UNet, list]:
    """Adam with a short warm-up and cosine decay; `init` (a weights file)
    starts from trained weights instead of the seeded initialisation.  With
    `weighted`, every sample's squared error is divided by its target's mean
    square (sample_weights), so the few very large normalized targets do not
    dominate the loss."""
    torch.cuda.synchronize()
    net = UNet(seed=seed)
    if init is not None:
        net.load(init)
    gen = torch.Generator().manual_seed(seed)
    history = []
    t0 = time.perf_counter()
    for step in range(1, steps + 1):
        x, t = make_batch(ps, gen, batch)
        net.backward(x, t, sample_weights(t) if weighted else None)
        # cosine decay to 1% with a short warm-up
        warm = min(1.0, step / 200.0)
        rate = lr * warm * (0.01 + 0.99 * 0.5 * (1.0 + math.cos(math.pi * step / steps)))
        net.adam(rate)
        if step % log_every == 0 or step == steps:
            loss = net.loss()
            history.append((step, loss))
            log(f"  step {step}/{steps}  loss {loss:.4g}  lr {rate:.2e}  "
                f"{time.perf_counter() - t0:.1f} s")
    torch.cuda.synchronize()
    return net, history


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--problems", type=int, default=2000)
    ap.add_argument("--n", type=int, default=32)
    ap.add_argument("--groups", type=int, default=4)
    ap.add_argument("--steps", type=int, default=6000)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--random-rounds", type=int, default=16)
    ap.add_argument("--init", default=None, help="weights file to start from")
    ap.add_argument("--weighted", action="store_true",
                    help="relative per-sample loss (each sample's error over its target's size)")
    ap.add_argument("--out", default="accel_weights.npz")
    a = ap.parse_args()
    torch.cuda.set_device(0)
    probs = [P.learned_problem(a.seed * 1_000_003 + i, n=a.n, groups=a.groups)
             for i in range(a.problems)]
    ps = D.generate(probs)
    print(f"pairs from {ps.num_problems} problems in {ps.seconds:.1f} s; "
          f"iterations to converge {int(np.median(ps.iterations))} (median)")
    if a.random_rounds > 0:
        R, Z = D.generate_random([probs[i] for i in ps.kept], rounds=a.random_rounds, seed=a.seed)
        ps = D.PairSet(torch.cat([ps.R, R], dim=1), torch.cat([ps.Z, Z], dim=1), ps.F, ps.n,
                       ps.iterations, ps.seconds, ps.kept)
    net, _ = train(ps, steps=a.steps, batch=a.batch, lr=a.lr, seed=a.seed, init=a.init,
                   weighted=a.weighted)
    net.save(a.out)
    print(f"weights written to {a.out}")


if __name__ == "__main__":
    main()
