"""The sweep entry point that allocates no memory (doma_sweep_noalloc).

It exists for callers that cannot call cudaMalloc, such as code running
inside another framework's memory pool or under a fixed device-memory
budget.  Its scratch is a static device array of DOMA_NOALLOC_SCRATCH_BYTES.
The test calls it through the C ABI twice in a row for each case (two
different problems follow each other, so a call must not see the previous
call's state) and compares each output with what the existing entry points
give: a solver's first source iteration from a zero flux
(doma_solver_source_iterations, then doma_solver_get_scalar_flux).  Both run
the same FP32 kernel on the same rounded inputs, so the outputs must be equal
bit for bit; the oracle's first source iteration (FP64) bounds both within
the FP32 tolerance.  Inputs and outputs are allocated by the test (torch),
never by the entry point.  This file is collected last.
"""
import ctypes

import numpy as np
import pytest

import oracle_lib as ol
from doma_gb300 import abi
from doma_gb300 import problems as P
from doma_gb300.solver import Solver

pytestmark = pytest.mark.gpu

FP32_RTOL = 1e-5   # relative L2, the tolerance of the FP32 parity tests


def group0_inputs(p, torch):
    """q and sigma_t of group 0 at the first source iteration (external source
    only), rounded to float as the solver's FP32 mode rounds them."""
    m = p.cell_material.astype(np.int64)
    src = p.source[m, 0] if p.source is not None else np.zeros(p.num_cells)
    scale = 0.25 if p.num_dims == 3 else 0.5
    q = ((scale * src) / np.pi).astype(np.float32)
    st = p.total[m, 0].astype(np.float32)
    dev = torch.device("cuda", 0)
    return torch.from_numpy(q).to(dev), torch.from_numpy(st).to(dev)


def noalloc_sweep(p, scheme, theta, torch):
    lib = abi.load_library()
    q, st = group0_inputs(p, torch)
    out = torch.zeros(p.num_cells, dtype=torch.float64, device="cuda:0")
    cp = p.to_c()
    status = lib.doma_sweep_noalloc(ctypes.byref(cp), scheme, theta, ctypes.c_void_p(q.data_ptr()),
                                    ctypes.c_void_p(st.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                    ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    abi.check(status, "doma_sweep_noalloc", lib)
    return out.cpu().numpy()


def solver_first_iteration(p, scheme, theta):
    opts = P.make_options(scheme={0: "dd", 1: "tw_dd"}[scheme], theta=theta, precision="fp32")
    with Solver(p, opts) as s:
        s.source_iterations(0, 1)
        return s.scalar_flux()[0]


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def oracle_first_iteration(p, scheme, theta):
    opts = P.make_options(scheme={0: "dd", 1: "tw_dd"}[scheme], theta=theta)
    phi, _ = ol.oracle_source_iterations(p, opts, 0, 1)
    return phi[0]


CASES = [
    ("checkerboard24_twdd", lambda: P.checkerboard(0, n=24, groups=2, np_=4, na=4, block=8),
     abi.DOMA_SCHEME_TW_DD, 0.7),
    ("random3d_dd", lambda: P.random_problem(8, 3, 13, 9, 7, groups=2, np_=3, na=3, materials=3),
     abi.DOMA_SCHEME_DD, 0.9),
    ("random2d_dd", lambda: P.random_problem(5, 2, 13, 9, 1, groups=2, np_=3, na=3, materials=3),
     abi.DOMA_SCHEME_DD, 0.9),
    ("random2d_twdd", lambda: P.random_problem(6, 2, 37, 19, 1, groups=1, np_=2, na=4,
                                               materials=3),
     abi.DOMA_SCHEME_TW_DD, 0.8),
]


def test_noalloc_sweep_matches_solver_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    torch.cuda.set_device(0)
    for name, make, scheme, theta in CASES:
        p = make()
        want = solver_first_iteration(p, scheme, theta)
        oracle = oracle_first_iteration(p, scheme, theta)
        assert np.abs(want).max() > 0
        for call in range(2):
            got = noalloc_sweep(p, scheme, theta, torch)
            assert np.isfinite(got).all()
            assert np.array_equal(got, want), (name, call, rel_l2(got, want))
            assert rel_l2(got, oracle) <= FP32_RTOL, (name, call, rel_l2(got, oracle))


def test_noalloc_sweep_rejects_problems_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    lib = abi.load_library()
    p = P.checkerboard(0, n=100, groups=1, np_=4, na=4, block=10)  # needs > 64 MiB
    cp = p.to_c()
    dummy = torch.zeros(1, device="cuda:0")
    status = lib.doma_sweep_noalloc(ctypes.byref(cp), 0, 0.9, ctypes.c_void_p(dummy.data_ptr()),
                                    ctypes.c_void_p(dummy.data_ptr()),
                                    ctypes.c_void_p(dummy.data_ptr()), None)
    assert status == abi.DOMA_BAD_INPUT
    assert "bytes of scratch" in abi.last_error(lib)
