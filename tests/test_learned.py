"""Learned accelerator: workload generator, features, the solver's correction
plumbing (guard, reference stop) and training-pair generation."""
import numpy as np
import pytest

from doma_gb300 import problems as P
from doma_gb300.learned import data as D


def test_learned_problem_draws_the_documented_distribution():
    p = P.learned_problem(7, n=32, groups=4)
    assert p.num_cells == 32 ** 3 and p.num_materials == p.num_cells
    ls = np.log(p.total)
    assert abs(np.median(p.total) - 1.0) < 0.15
    assert 0.6 < ls.std() < 1.0
    G = p.num_groups
    c = p.scatter[:, np.arange(G), np.arange(G)] / p.total
    assert c.min() >= 0.9 and c.max() <= 0.999
    down = p.scatter[:, 1, 0] / p.total[:, 0]
    assert np.allclose(down, 0.5 * (1 - c[:, 0]))
    assert np.all(p.scatter[:, 0, 1] == 0.0)  # no upscatter
    again = P.learned_problem(7, n=32, groups=4)
    assert again.digest() == p.digest()
    # neighbouring cells are correlated (correlation length 4 cells)
    z = ls[:, 0].reshape(32, 32, 32)
    zc = (z - z.mean()) / z.std()
    assert (zc * np.roll(zc, 1, axis=2)).mean() > 0.8
    assert (zc * np.roll(zc, 16, axis=2)).mean() < 0.3


def test_features_follow_the_solver_formulas():
    p = P.learned_problem(3, n=16, groups=3)
    fsig, fab, kap = D.features(p)
    assert fsig.shape == (3, 16 ** 3) and kap.shape == (3, 16 ** 3)
    c = p.scatter[:, 1, 1] / p.total[:, 1]
    assert np.allclose(fab[1], (np.log(1 - c) + 4.6) / 1.5, rtol=1e-6)
    assert np.allclose(fsig[2], np.log(p.total[:, 2]) / 0.8, rtol=1e-6)
    assert np.all(kap[0] == 0.0)
    assert np.allclose(kap[2], p.scatter[:, 2, 1] / p.total[:, 2], rtol=1e-6)


@pytest.mark.gpu
def test_reference_stop_reports_the_true_error():
    from doma_gb300.learned import evaluate as E
    p = P.learned_problem(5, n=16, groups=2, np_=2, na=2)
    ref, info = E.reference_flux(p, tol=1e-11)
    r = E.time_to_error(p, ref, target=1e-3, warm=False)
    assert r["converged"]
    assert r["error"] <= 1e-3
    assert abs(r["error"] - r["reported_error"]) <= 1e-9 * r["error"]
    tighter = E.time_to_error(p, ref, target=1e-5, warm=False)
    assert tighter["iterations"] > r["iterations"]


@pytest.mark.gpu
def test_guarded_corrections_keep_the_plain_fixed_point():
    from doma_gb300.learned.net import UNet
    from doma_gb300.solver import Solver
    p = P.learned_problem(9, n=16, groups=3, np_=2, na=2)
    opts = P.make_options(scheme="dd", precision="fp32", fs_tol=1e-7, fs_max_it=20000,
                          iteration="multigroup")
    with Solver(p, opts) as s:
        plain = s.solve_fixed_source()
        want = s.scalar_flux()
    net = UNet(seed=1)  # untrained: its corrections are noise
    with Solver(p, opts) as s:
        s.set_accelerator(net, first=2, interval=2, max_corrections=10, guard=True)
        rep = s.solve_fixed_source()
        got = s.scalar_flux()
        st = s.accel_stats()
    net.close()
    assert plain.converged and rep.converged
    assert st["accepted"] + st["rejected"] == 10
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 2e-5


@pytest.mark.gpu
def test_captured_corrections_equal_eager_ones(monkeypatch):
    """From the second correction on, a correction's launches (per group:
    residual, input, U-Net forward, correction) replay as one captured graph;
    DOMA_ACCEL_GRAPH=0 launches them one by one.  Same kernels in the same
    order: the same bits, counts and guard decisions."""
    from pathlib import Path

    from doma_gb300.learned.net import UNet
    from doma_gb300.solver import Solver
    weights = Path(__file__).resolve().parents[1] / "doma_gb300" / "learned" / "weights" / "unet_c32.npz"
    p = P.learned_problem(900003, n=16, groups=3, np_=2, na=2)
    opts = P.make_options(scheme="dd", precision="fp32", fs_tol=1e-6, fs_max_it=20000,
                          iteration="multigroup")
    out = []
    with UNet(seed=0) as net:
        net.load(weights)
        for graph in ("1", "0"):
            monkeypatch.setenv("DOMA_ACCEL_GRAPH", graph)
            with Solver(p, opts) as s:
                s.set_accelerator(net, first=2, interval=3, max_corrections=6, guard=True)
                rep = s.solve_fixed_source()
                out.append((rep.si_iterations, s.accel_stats(), s.scalar_flux()))
    (i1, st1, phi1), (i0, st0, phi0) = out
    assert i1 == i0
    assert (st1["accepted"], st1["rejected"]) == (st0["accepted"], st0["rejected"])
    assert st1["accepted"] + st1["rejected"] >= 2   # the second one replays the graph
    assert np.array_equal(phi1, phi0)


@pytest.mark.gpu
def test_batch_stepping_equals_the_graph_solve():
    from doma_gb300.solver import Batch
    ps = [P.learned_problem(i, n=16, groups=2, np_=2, na=2) for i in range(3)]
    kw = dict(scheme="dd", precision="fp32", fs_tol=1e-6, fs_max_it=5000, iteration="multigroup")
    with Batch(ps, **kw) as b:
        a = b.solve()
        fa = [b.scalar_flux(i) for i in range(3)]
        b.begin()
        b.iterate(4)
        assert b.iterate(100000) == 0
        c = b.reports()
        fc = [b.scalar_flux(i) for i in range(3)]
    assert [r.mg_iterations for r in a] == [r.mg_iterations for r in c]
    assert all(np.array_equal(x, y) for x, y in zip(fa, fc))


@pytest.mark.gpu
def test_training_pairs_have_the_documented_structure():
    import torch
    ps = [P.learned_problem(20 + i, n=16, groups=3, np_=2, na=2) for i in range(2)]
    pairs = D.generate(ps, k_max=3, tol=1e-6, log=lambda *a: None)
    assert pairs.R.shape == (2, 3, 3, 16 ** 3) and pairs.F.shape == (2, 3, 2, 16 ** 3)
    # group 0 has no coupling: r = delta, and r + z = e + delta in every group
    # -> z_0 is the error itself, which shrinks along the iterations
    z0 = pairs.Z[:, :, 0].norm(dim=-1)
    assert torch.all(z0[:, 1:] < z0[:, :-1])
    assert torch.all(torch.isfinite(pairs.R)) and torch.all(torch.isfinite(pairs.Z))


@pytest.mark.gpu
def test_trained_network_cuts_the_iterations_to_tolerance():
    """What the trained network gains: on a held-out problem (a seed outside
    the training sets), plain FP32 multigroup iteration and the same
    iteration with guarded corrections from the committed weights both stop at
    1e-5 relative L2 error against an FP64 solution; the corrected one needs
    far fewer iterations."""
    from pathlib import Path

    from doma_gb300.learned import evaluate as E
    from doma_gb300.learned.net import UNet
    weights = Path(__file__).resolve().parents[1] / "doma_gb300" / "learned" / "weights" / "unet_c32.npz"
    p = P.learned_problem(900002, n=32, groups=4)
    ref, _ = E.reference_flux(p, tol=1e-9)
    plain = E.time_to_error(p, ref, 1e-5, max_it=20000, warm=False)
    with UNet(seed=0) as net:
        net.load(weights)
        lrn = E.time_to_error(p, ref, 1e-5, net=net, first=2, interval=2, max_corrections=64,
                              max_it=20000, warm=False)
    assert plain["converged"] and lrn["converged"]
    assert plain["error"] <= 1e-5 and lrn["error"] <= 1e-5
    assert lrn["accepted"] > 0
    assert lrn["iterations"] <= 0.5 * plain["iterations"], (plain["iterations"], lrn["iterations"])
