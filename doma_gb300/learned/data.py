"""Training pairs for the learned accelerator, generated by the GPU solver.

For each seeded problem the batched FP32 solver runs multigroup source
iterations from a zero flux, recording the increment delta_k and flux phi_k
after iterations k = 1..K, then continues to convergence (phi*).  With
e_k = phi* - phi_k and y = e_k + delta_k, the per-group pair is

    r_g = delta_g + kappa_g * y_{g-1}      (network input, before scaling)
    z_g = e_g     - kappa_g * y_{g-1}      (network target, before scaling)

kappa_g = S[g][g-1] / sigma_t,g.  This is the split the solver's correction
step uses (doma_gb300/csrc/accel.cuh): the network maps r_g / rms(r_g) and
the cell features to z_g / rms(r_g).  Pairs are linear in the increment, so
any linear combination of one problem's pairs is again a valid pair (used to
augment the training set).
"""
from __future__ import annotations

import time
from dataclasses import dataclass

import numpy as np
import torch

from .. import problems as P
from ..solver import Batch
from .net import IN_CHANNELS

# Feature scaling, identical to kFeatSigma / kFeatAbs* in csrc/accel.cuh.
FEAT_SIGMA = 0.8
FEAT_ABS_FLOOR = 1e-6
FEAT_ABS_SHIFT = -4.6
FEAT_ABS_SCALE = 1.5


def features(p: P.Problem) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """(f_sigma, f_abs, kappa), each [G][N] float32, per cell through its material."""
    m = p.cell_material
    st = p.total[m]                                  # [N][G]
    G = p.num_groups
    diag = p.scatter[m][:, np.arange(G), np.arange(G)]
    c = diag / st
    fsig = (np.log(st) / FEAT_SIGMA).T
    fabs_ = ((np.log(np.maximum(1.0 - c, FEAT_ABS_FLOOR)) - FEAT_ABS_SHIFT) / FEAT_ABS_SCALE).T
    kappa = np.zeros_like(st)
    for g in range(1, G):
        kappa[:, g] = p.scatter[m][:, g, g - 1] / st[:, g]
    return (fsig.astype(np.float32), fabs_.astype(np.float32), kappa.T.astype(np.float32).copy())


class _DeviceArray:
    """A device buffer owned by the library, seen by torch without a copy."""

    def __init__(self, ptr: int, count: int):
        self.__cuda_array_interface__ = {"shape": (count,), "typestr": "<f8",
                                         "data": (ptr, False), "version": 3}


def device_view(ptr: int, count: int) -> torch.Tensor:
    return torch.as_tensor(_DeviceArray(ptr, count), device="cuda")


def random_error_fields(gen: torch.Generator, count: int, n: int) -> torch.Tensor:
    """`count` random smooth fields on an n^3 periodic grid ([count][n^3]
    float64, on the GPU): a Gaussian random field of correlation length
    l ~ logU[1, 16] cells plus a mean offset m ~ U[-0.5, 2], times an
    amplitude a ~ U[0.1, 1], negative for a quarter of the fields.
    gen is a CUDA generator."""
    dev = torch.device("cuda")
    d = torch.arange(n, dtype=torch.float64, device=dev)
    d = torch.minimum(d, n - d)
    ell = torch.exp(torch.rand((count, 1), generator=gen, device=dev, dtype=torch.float64)
                    * np.log(16.0))
    k1 = torch.exp(-(d[None, :] ** 2) / (ell * ell))                      # [count][n]
    kern = k1[:, :, None, None] * k1[:, None, :, None] * k1[:, None, None, :]
    norm = torch.sqrt((kern * kern).sum(dim=(1, 2, 3)))
    w = torch.randn((count, n, n, n), generator=gen, device=dev, dtype=torch.float64)
    ax = (1, 2, 3)
    f = torch.fft.irfftn(torch.fft.rfftn(w, dim=ax) * torch.fft.rfftn(kern, dim=ax), s=(n, n, n),
                         dim=ax) / norm[:, None, None, None]
    m = torch.rand((count, 1, 1, 1), generator=gen, device=dev, dtype=torch.float64) * 2.5 - 0.5
    a = torch.rand((count, 1, 1, 1), generator=gen, device=dev, dtype=torch.float64) * 0.9 + 0.1
    sign = torch.where(torch.rand((count, 1, 1, 1), generator=gen, device=dev) < 0.75, 1.0, -1.0)
    return (sign * a * (m + f)).reshape(count, n ** 3)


def generate_random(problems: list[P.Problem], rounds: int = 16, seed: int = 0,
                    chunk: int = 256, log=print) -> tuple[torch.Tensor, torch.Tensor]:
    """Pairs from arbitrary error fields: for an iterate with error x, one
    source iteration gives the increment (I - K) x and leaves the error K x,
    so sweeping x itself (doma_batch_set_increment) yields the pair for any x.
    Returns R, Z [P][rounds][G][N] float32 in the same split as generate()
    (y = e + delta = x)."""
    t0 = time.perf_counter()
    n = problems[0].nx
    G = problems[0].num_groups
    N = n ** 3
    gen = torch.Generator(device="cuda").manual_seed(int(seed))
    stream = torch.cuda.Stream()
    Rs, Zs = [], []
    with torch.cuda.stream(stream):
        for c0 in range(0, len(problems), chunk):
            part = problems[c0:c0 + chunk]
            b = Batch(part, scheme="dd", precision="fp32", fs_tol=0.0, fs_max_it=1 << 30,
                      iteration="multigroup")
            b.set_stream(stream.cuda_stream)
            b.begin()
            kap = torch.stack([torch.from_numpy(features(p)[2]) for p in part]).cuda()  # [P][G][N]
            R = torch.empty((len(part), rounds, G, N), dtype=torch.float32, device="cuda")
            Z = torch.empty_like(R)
            for r in range(rounds):
                xs = random_error_fields(gen, len(part) * G, n).view(len(part), G, N)
                for i in range(len(part)):
                    b.set_increment(i, xs[i].data_ptr())
                b.iterate(1)
                for i in range(len(part)):
                    _, ip = b.state_pointers(i)
                    kx = device_view(ip, G * N).view(G, N)
                    x = xs[i]
                    xprev = torch.zeros_like(x)
                    xprev[1:] = x[:-1]
                    coup = kap[i].double() * xprev
                    R[i, r] = (x - kx + coup).float()
                    Z[i, r] = (kx - coup).float()
            b.close()
            Rs.append(R)
            Zs.append(Z)
            log(f"  random pairs {min(c0 + chunk, len(problems))}/{len(problems)} problems, "
                f"{time.perf_counter() - t0:.1f} s")
    stream.synchronize()
    return torch.cat(Rs), torch.cat(Zs)


@dataclass
class PairSet:
    """R, Z: [P][K][G][N] float32; F: [P][G][2][N] float32 (f_sigma, f_abs);
    all on the GPU.  n: mesh extent (n^3 cells)."""
    R: torch.Tensor
    Z: torch.Tensor
    F: torch.Tensor
    n: int
    iterations: list
    seconds: float
    kept: list = None    # indices (into the problem list) of the problems in the set

    @property
    def num_problems(self) -> int:
        return int(self.R.shape[0])


def generate(problems: list[P.Problem], k_max: int = 10, tol: float = 1e-6,
             max_it: int = 20000, chunk: int = 256, log=print) -> PairSet:
    """Solve every problem on the GPU (batched, FP32 multigroup DD) and return
    the pairs of the converged ones."""
    t0 = time.perf_counter()
    n = problems[0].nx
    G = problems[0].num_groups
    N = n ** 3
    stream = torch.cuda.Stream()
    Rs, Zs, Fs, iters, kept = [], [], [], [], []
    with torch.cuda.stream(stream):
        for c0 in range(0, len(problems), chunk):
            part = problems[c0:c0 + chunk]
            b = Batch(part, scheme="dd", precision="fp32", fs_tol=tol, fs_max_it=max_it,
                      iteration="multigroup")
            b.set_stream(stream.cuda_stream)
            b.begin()
            phis = torch.empty((len(part), k_max, G, N), dtype=torch.float32, device="cuda")
            deltas = torch.empty_like(phis)
            for k in range(k_max):
                b.iterate(1)
                for i in range(len(part)):
                    pp, dp = b.state_pointers(i)
                    phis[i, k] = device_view(pp, G * N).view(G, N).float()
                    deltas[i, k] = device_view(dp, G * N).view(G, N).float()
            b.iterate(max_it)
            reps = b.reports()
            for i, p in enumerate(part):
                if not reps[i].converged:
                    log(f"  {p.name}: not converged ({reps[i].mg_residual:.2e}), skipped")
                    continue
                pp, _ = b.state_pointers(i)
                star = device_view(pp, G * N).view(G, N).float()
                fsig, fab, kap = features(p)
                kappa = torch.from_numpy(kap).cuda()
                e = star[None] - phis[i]                  # [K][G][N]
                y = e + deltas[i]
                yprev = torch.zeros_like(y)
                yprev[:, 1:] = y[:, :-1]
                coup = kappa[None] * yprev
                Rs.append(deltas[i] + coup)
                Zs.append(e - coup)
                Fs.append(torch.from_numpy(np.stack([fsig, fab], axis=1)).cuda())
                iters.append(reps[i].mg_iterations)
                kept.append(c0 + i)
            b.close()
            torch.cuda.current_stream().synchronize()
            log(f"  generated {min(c0 + chunk, len(problems))}/{len(problems)} problems, "
                f"{time.perf_counter() - t0:.1f} s")
    stream.synchronize()
    return PairSet(torch.stack(Rs), torch.stack(Zs), torch.stack(Fs), n, iters,
                   time.perf_counter() - t0, kept)


def correction(net, delta: torch.Tensor, kappa: torch.Tensor, fsig: torch.Tensor,
               fabs_: torch.Tensor, n: int) -> torch.Tensor:
    """The solver's correction step (csrc/accel.cuh) in torch, batched over
    problems: delta [B][G][N] -> Delta [B][G][N] float32, with the y chain
    across groups.  kappa, fsig, fabs_: [B][G][N] float32 on the GPU."""
    B, G, N = delta.shape
    dev = delta.device
    y = torch.zeros((B, N), dtype=torch.float32, device=dev)
    out = torch.empty((B, n, n, n), dtype=torch.float32, device=dev)
    corr = torch.empty((B, G, N), dtype=torch.float32, device=dev)
    for g in range(G):
        kg = kappa[:, g]
        r = delta[:, g].float() + kg * y
        s = r.pow(2).mean(dim=1, keepdim=True).sqrt().clamp_min(1e-30)
        x = torch.zeros((B, N, IN_CHANNELS), dtype=torch.float32, device=dev)
        x[..., 0] = r / s
        x[..., 1] = fsig[:, g]
        x[..., 2] = fabs_[:, g]
        net.forward(x.to(torch.bfloat16).view(B, n, n, n, IN_CHANNELS).contiguous(), out)
        z = s * out.view(B, N)
        corr[:, g] = z + kg * y
        y = z + r
    return corr


def generate_guided(problems: list[P.Problem], net, first: int = 6, interval: int = 6,
                    corrections: int = 8, tol: float = 1e-6, max_it: int = 20000,
                    chunk: int = 32, log=print) -> PairSet:
    """Pairs from the states that the corrected iteration visits (DAgger):
    each problem is solved to convergence once for phi*, then iterated again
    from zero with a correction from `net` after `first` iterations and every
    `interval` iterations after that, without the guard.  A correction is
    applied the way the solver applies it: the next sweep takes delta + Delta,
    and the stored increment becomes the sweep's result minus Delta.  The
    states recorded are the one right after each correction and the one
    each later correction is computed from, 2 * corrections - 1 per problem."""
    t0 = time.perf_counter()
    n = problems[0].nx
    G = problems[0].num_groups
    N = n ** 3
    stream = torch.cuda.Stream()
    net.set_stream(stream.cuda_stream)
    Rs, Zs, Fs, iters, kept = [], [], [], [], []
    with torch.cuda.stream(stream):
        for c0 in range(0, len(problems), chunk):
            part = problems[c0:c0 + chunk]
            ref = Batch(part, scheme="dd", precision="fp32", fs_tol=tol, fs_max_it=max_it,
                        iteration="multigroup")
            ref.set_stream(stream.cuda_stream)
            ref.begin()
            ref.iterate(max_it)
            reps = ref.reports()
            stars = [device_view(ref.state_pointers(i)[0], G * N).view(G, N).float().clone()
                     for i in range(len(part))]
            ref.close()
            feats = [features(p) for p in part]
            fsig = torch.stack([torch.from_numpy(f[0]) for f in feats]).cuda()
            fab = torch.stack([torch.from_numpy(f[1]) for f in feats]).cuda()
            kap = torch.stack([torch.from_numpy(f[2]) for f in feats]).cuda()
            b = Batch(part, scheme="dd", precision="fp32", fs_tol=0.0, fs_max_it=1 << 30,
                      iteration="multigroup")
            b.set_stream(stream.cuda_stream)
            b.begin()

            def state():
                ph = torch.stack([device_view(b.state_pointers(i)[0], G * N).view(G, N)
                                  for i in range(len(part))]).float()
                de = torch.stack([device_view(b.state_pointers(i)[1], G * N).view(G, N)
                                  for i in range(len(part))])
                return ph, de

            rec_phi, rec_delta = [], []
            b.iterate(first)
            for c in range(corrections):
                phi, delta = state()
                if c > 0:
                    rec_phi.append(phi)
                    rec_delta.append(delta.float())
                corr = correction(net, delta, kap, fsig, fab, n).double()
                inc = delta + corr
                for i in range(len(part)):
                    b.set_increment(i, inc[i].data_ptr())
                b.iterate(1)
                phi, dout = state()
                fixed = (dout - corr).contiguous()
                for i in range(len(part)):
                    b.set_increment(i, fixed[i].data_ptr())
                rec_phi.append(phi)
                rec_delta.append(fixed.float())
                if c + 1 < corrections and interval > 1:
                    b.iterate(interval - 1)
            b.close()
            phis = torch.stack(rec_phi, dim=1)        # [P][K][G][N]
            deltas = torch.stack(rec_delta, dim=1)
            for i, p in enumerate(part):
                if not reps[i].converged:
                    log(f"  {p.name}: not converged ({reps[i].mg_residual:.2e}), skipped")
                    continue
                e = stars[i][None] - phis[i]
                y = e + deltas[i]
                yprev = torch.zeros_like(y)
                yprev[:, 1:] = y[:, :-1]
                coup = kap[i][None] * yprev
                Rs.append(deltas[i] + coup)
                Zs.append(e - coup)
                Fs.append(torch.stack([fsig[i], fab[i]], dim=1))
                iters.append(reps[i].mg_iterations)
                kept.append(c0 + i)
            torch.cuda.current_stream().synchronize()
            log(f"  guided pairs {min(c0 + chunk, len(problems))}/{len(problems)} problems, "
                f"{time.perf_counter() - t0:.1f} s")
    stream.synchronize()
    net.set_stream(None)
    return PairSet(torch.stack(Rs), torch.stack(Zs), torch.stack(Fs), n, iters,
                   time.perf_counter() - t0, kept)
