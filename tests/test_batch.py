"""Batched solves (doma_batch_*): many problems in one persistent sweep per
iteration must give exactly what each problem gives when solved alone."""
import numpy as np
import pytest

from doma_gb300 import problems as P


def test_batch_mix_draws_the_documented_distribution():
    ps = P.batch_mix(3, count=64)
    ns = {p.nx for p in ps}
    assert all(16 <= p.nx <= 96 and p.nx == p.ny == p.nz for p in ps)
    assert {p.num_groups for p in ps} <= {1, 2, 4, 8, 16}
    assert all(2 <= p.num_polar <= 6 and p.num_polar == p.num_azimuthal for p in ps)
    assert len(ns) > 10
    again = P.batch_mix(3, count=64)
    assert [p.digest() for p in ps] == [p.digest() for p in again]


def small_batch():
    return [
        P.checkerboard(1, n=12, groups=2, np_=2, na=2, block=4),
        P.checkerboard(2, n=17, groups=1, np_=3, na=3, block=8),
        P.checkerboard(3, n=9, groups=4, np_=5, na=5, block=4),
        P.random_problem(4, 3, 13, 7, 10, groups=3, np_=2, na=3, materials=3, fission=True),
        P.checkerboard(5, n=20, groups=2, np_=4, na=4, block=8),
    ]


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", ["dd", "tw_dd"])
def test_batch_equals_individual_solves(scheme):
    from doma_gb300.solver import Batch, Solver
    ps = small_batch()
    kw = dict(scheme=scheme, theta=0.8, precision="fp32", fs_tol=1e-6, fs_max_it=3000,
              iteration="multigroup")
    with Batch(ps, **kw) as b:
        reps = b.solve()
        got = [b.scalar_flux(i) for i in range(len(ps))]
    for p, rep, phi in zip(ps, reps, got):
        with Solver(p, P.make_options(**kw)) as s:
            r = s.solve_fixed_source()
            want = s.scalar_flux()
        assert rep.converged and r.converged
        assert rep.mg_iterations == r.mg_iterations
        assert np.array_equal(phi, want), (p.name, np.abs(phi - want).max())


@pytest.mark.gpu
def test_batch_tuner_keeps_results():
    from doma_gb300.solver import Batch
    ps = small_batch()[:3]
    kw = dict(scheme="dd", precision="fp32", fs_tol=1e-6, fs_max_it=3000, iteration="multigroup")
    with Batch(ps, **kw) as b:
        first = [r.mg_iterations for r in b.solve()]
        a = [b.scalar_flux(i) for i in range(len(ps))]
        tx = b.tune()
        assert tx in (8, 16, 32)
        tiles = b.tiles()
        assert len(tiles) == len(ps) and all(t in (8, 16, 32) for t in tiles)
        rep = b.tune_report()
        assert rep["classes"] >= 1 and min(rep["uniform_ms"].values()) > 0
        second = [r.mg_iterations for r in b.solve()]
        c = [b.scalar_flux(i) for i in range(len(ps))]
    assert first == second
    assert all(np.array_equal(x, y) for x, y in zip(a, c))


@pytest.mark.gpu
def test_batch_graph_loop_equals_host_loop(monkeypatch):
    """The captured WHILE loop and the host-driven loop run the same kernels."""
    from doma_gb300.solver import Batch
    ps = small_batch()
    kw = dict(scheme="tw_dd", theta=0.7, precision="fp32", fs_tol=1e-6, fs_max_it=3000,
              iteration="multigroup")
    with Batch(ps, **kw) as b:
        graph_reps = b.solve()
        graph_phi = [b.scalar_flux(i) for i in range(len(ps))]
    monkeypatch.setenv("DOMA_SOLVE_LOOP", "host")
    with Batch(ps, **kw) as b:
        host_reps = b.solve()
        host_phi = [b.scalar_flux(i) for i in range(len(ps))]
    assert [r.mg_iterations for r in graph_reps] == [r.mg_iterations for r in host_reps]
    assert graph_reps[0].kernel_launches == 4 * max(r.mg_iterations for r in graph_reps)
    assert all(np.array_equal(x, y) for x, y in zip(graph_phi, host_phi))


@pytest.mark.gpu
def test_batch_iteration_cap_reports_not_converged():
    from doma_gb300.solver import Batch
    ps = small_batch()[:2]
    with Batch(ps, scheme="dd", precision="fp32", fs_tol=1e-12, fs_max_it=5,
               iteration="multigroup") as b:
        reps = b.solve()
    assert all(not r.converged and r.mg_iterations == 5 for r in reps)
