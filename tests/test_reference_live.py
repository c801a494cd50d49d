"""Live comparison with DOMA itself where its sources were compiled here
(oracle/_ref/libdoma_ref.so).  Skipped where the DOMA tree is absent."""
import numpy as np
import pytest

import oracle_lib as ol
from doma_gb300 import problems as P

pytestmark = pytest.mark.skipif(not ol.ref_available(), reason="DOMA reference not built here")


@pytest.mark.parametrize("seed", [11, 12])
@pytest.mark.parametrize("scheme", ["dd", "tw_dd"])
@pytest.mark.parametrize("dims", [2, 3])
def test_oracle_vs_live_reference(seed, scheme, dims):
    p = P.random_problem(seed, dims, 6, 5, 4, groups=3, np_=2, na=1, materials=4,
                         fission=seed % 2 == 0)
    opts = P.make_options(scheme=scheme, fs_tol=1e-9, mg_tol=1e-9)
    r = ol.ref_solve(p, opts)
    o = ol.oracle_solve(p, opts)
    assert r[1] == o[1]
    assert list(r[2]) == list(o[2])
    assert np.array_equal(r[0], o[0])


def test_theta_parameter_reduces_to_reference_at_0_9():
    """DOMA's theta is constexpr 0.9; the restatement's parameter must agree there
    and differ elsewhere (checks the parameter is really used)."""
    p = P.small_cube(4, n=8)
    r = ol.ref_solve(p, P.make_options(scheme="tw_dd", theta=0.9))
    o9 = ol.oracle_solve(p, P.make_options(scheme="tw_dd", theta=0.9))
    o7 = ol.oracle_solve(p, P.make_options(scheme="tw_dd", theta=0.7))
    assert np.array_equal(r[0], o9[0])
    assert not np.array_equal(o9[0], o7[0])


@pytest.mark.parametrize("seed", [21, 22])
@pytest.mark.parametrize("scheme", ["dd", "tw_dd"])
@pytest.mark.parametrize("dims", [2, 3])
def test_oracle_eigenvalue_vs_live_reference(seed, scheme, dims):
    p = P.random_problem(seed, dims, 6, 5, 4, groups=2, np_=2, na=1, materials=3,
                         fission=True, fission_scale=8.0)
    opts = P.make_options(scheme=scheme, fs_tol=1e-9, mg_tol=1e-5, mg_max_it=300)
    phi_r, ok_r, si_r, pi_r, k_r, _ = ol.ref_solve_eigen(p, opts, 1e-7, precision=17)
    phi_o, k_o, ok_o, si_o, pi_o, _, _ = ol.oracle_solve_eigen(p, opts, 1e-7)
    assert ok_r == ok_o and pi_r == pi_o
    assert list(si_r) == list(si_o)
    if ok_r:  # DOMA prints the final k only when the power iteration converged
        assert k_r == k_o
    assert np.array_equal(phi_r, phi_o)
