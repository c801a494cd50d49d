"""C ABI checks that need no GPU: the library loads, exports every entry point
declared in include/doma_gb300.h, builds DOMA's quadrature bit for bit,
validates input, and fails loudly (DOMA_NO_DEVICE) rather than falling back
to a CPU path when no GPU is visible."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

from doma_gb300 import abi
from doma_gb300 import problems as P
from golden_cases import quadrature_sets

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "doma_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(doma_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    if not abi.LIB_PATH.exists():
        import __graft_entry__ as g
        g.build()
    return abi.load_library()


def test_header_declares_expected_entry_points():
    names = declared_functions()
    assert set(names) == set(abi.SIGNATURES), set(names) ^ set(abi.SIGNATURES)


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert lib.doma_abi_version() == abi.ABI_VERSION


def test_default_options(lib):
    o = abi.DomaOptions()
    lib.doma_default_options(ctypes.byref(o))
    assert o.scheme == abi.DOMA_SCHEME_DD and o.precision == abi.DOMA_PREC_FP64
    assert o.theta == 0.9 and o.fs_tol == 1e-8 and o.mg_tol == 1e-8


@pytest.mark.parametrize("dims,np_,na,mu,eta,xi,w,counts", quadrature_sets())
def test_library_quadrature_bitwise(lib, dims, np_, na, mu, eta, xi, w, counts):
    from doma_gb300.solver import quadrature
    m, e, x, ww, c = quadrature(np_, na, dims)
    assert np.array_equal(c, counts)
    for a, b in ((m, mu), (e, eta), (x, xi), (ww, w)):
        assert np.array_equal(a, b)


def _create(lib, p, o):
    cp = p.to_c()
    h = ctypes.c_void_p()
    st = lib.doma_solver_create(ctypes.byref(cp), ctypes.byref(o), ctypes.byref(h))
    if h.value:
        lib.doma_solver_destroy(h)
    return st


@pytest.mark.parametrize("mutate,msg", [
    (lambda p: p.cell_material.__setitem__(0, 7), "material"),
    (lambda p: p.dx.__setitem__(0, -1.0), "widths"),
    (lambda p: setattr(p, "num_polar", 0), "np"),
    (lambda p: setattr(p, "num_polar", 5000), "ordinates per octant"),
])
def test_bad_input_is_rejected(lib, mutate, msg):
    p = P.random_problem(0, 3, 3, 3, 3, groups=2)
    mutate(p)
    st = _create(lib, p, P.make_options())
    assert st == abi.DOMA_BAD_INPUT
    assert msg in abi.last_error(lib)


def test_bad_options_are_rejected(lib):
    p = P.random_problem(0, 3, 3, 3, 3, groups=2)
    assert _create(lib, p, P.make_options(theta=1.5)) == abi.DOMA_BAD_INPUT
    o = P.make_options()
    o.scheme = 9
    assert _create(lib, p, o) == abi.DOMA_BAD_INPUT


def test_no_cpu_fallback_without_gpu(lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    p = P.random_problem(0, 3, 3, 3, 3, groups=2)
    assert _create(lib, p, P.make_options()) == abi.DOMA_NO_DEVICE
    with pytest.raises(abi.DomaError):
        from doma_gb300.solver import Solver
        Solver(p, P.make_options())
