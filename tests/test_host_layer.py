"""The C++ drop-in layer: deck reader, mesh, text output and (on a GPU) the
TransportSolver3D/2D classes and the deck runner."""
import json
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle_lib as ol
from doma_gb300 import abi, build as nb
from doma_gb300 import problems as P
from doma_gb300.decks import read_deck_summary, write_deck

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "cpp" / "host_check.cpp"
EXE = ROOT / "tests" / "cpp" / "_build" / "host_check"
# DOMA's example decks, where its source tree is present ($DOMA_REFERENCE_TREE,
# else a directory named `reference` beside this repository)
REF_CASES = Path(os.environ.get("DOMA_REFERENCE_TREE", str(ROOT.parent / "reference"))) / "cases"


@pytest.fixture(scope="module")
def host_check():
    if not nb.HOST_LIB.exists() or not nb.LIB.exists():
        nb.build()
    if not EXE.exists() or EXE.stat().st_mtime < max(SRC.stat().st_mtime, nb.HOST_LIB.stat().st_mtime):
        EXE.parent.mkdir(parents=True, exist_ok=True)
        subprocess.run(["g++", "-O2", "-std=c++17", f"-I{nb.HOST / 'include'}", str(SRC), "-o", str(EXE),
                        f"-L{nb.OUT}", "-ldoma_gb300_host", "-ldoma_gb300",
                        f"-Wl,-rpath,{nb.OUT},-rpath,/usr/local/cuda/lib64"], check=True)
    return EXE


def run(exe, *args, check=True):
    r = subprocess.run([str(exe), *map(str, args)], capture_output=True, text=True)
    if check and r.returncode != 0:
        raise AssertionError(f"{args}: rc={r.returncode}\n{r.stdout}\n{r.stderr}")
    return r


@pytest.mark.parametrize("dims", [2, 3])
def test_generated_deck_round_trips(host_check, tmp_path, dims):
    p = P.random_problem(4, dims, 5, 4, 3, groups=3, np_=2, na=3, materials=4, fission=True)
    deck = write_deck(p, tmp_path / "d.xml", scheme="tw_dd", fs_tol=1e-9, theta=0.7,
                      precision="fp32")
    d = json.loads(run(host_check, "parse", deck).stdout)
    assert (d["groups"], d["np"], d["na"], d["dims"]) == (3, 2, 3, dims)
    assert d["scheme"] == 1 and d["fs_tol"] == 1e-9 and d["theta"] == 0.7 and d["precision"] == 1
    assert np.array_equal(d["dx"], p.dx) and d["blocks"] == list(map(int, p.cell_material))
    for m in range(p.num_materials):
        mat = d["materials"][str(m)]
        assert np.array_equal(mat["total"], p.total[m])
        assert np.array_equal(mat["scatter"], p.scatter[m].ravel())
        assert (len(mat["chi_p"]) > 0) == bool(p.has_fission[m])


@pytest.mark.parametrize("dims", [2, 3])
def test_transient_deck_round_trips(host_check, tmp_path, dims):
    """A transient deck carries t1 / t_steps, each block's delayed-neutron data
    (DOMA's [g * D_m + d] order) and the source steps of each kind."""
    p, tr = P.transient_problem(3, dims=dims, num_steps=5, t1=2.0)
    deck = write_deck(p, tmp_path / "t.xml", scheme="dd", transient=tr)
    d = json.loads(run(host_check, "parse", deck).stdout)
    assert d["mode"] == 2 and d["t0"] == 0.0 and d["t1"] == 2.0 and d["t_steps"] == 5
    assert d["ic"] == 0
    for m in range(p.num_materials):
        mat = d["materials"][str(m)]
        dm = int(tr.d_groups[m])
        assert mat["delayed_groups"] == dm
        assert np.array_equal(mat["inv_v"], tr.inv_v[m])
        assert np.array_equal(mat["chi_d"], tr.chi_d[m, :, :dm].ravel())
        assert np.array_equal(mat["beta"], tr.beta[m, :, :dm].ravel())
        assert np.array_equal(mat["lambda"], tr.lambda_[m, :dm])
    # DOMA's StepType values: Insert 0, Remove 1, Both 2
    kinds = {1: 2, 2: 0, 3: 1}
    steps = d["steps"]
    assert sorted(map(int, steps)) == [m for m in range(p.num_materials) if tr.step_type[m]]
    for k, v in steps.items():
        m = int(k)
        assert v["type"] == kinds[int(tr.step_type[m])]
        assert np.array_equal(v["source"], tr.step_source[m])
        if tr.step_type[m] in (1, 2):
            assert v["insert"] == tr.step_insert[m]
        if tr.step_type[m] in (1, 3):
            assert v["remove"] == tr.step_remove[m]


@pytest.mark.skipif(not REF_CASES.exists(), reason="DOMA's example decks are not present")
def test_reference_decks_parse(host_check):
    decks = sorted(REF_CASES.glob("[23]D_*.xml")) + sorted(REF_CASES.glob("*/[23]D_*.xml"))
    assert decks
    for deck in decks:
        d = json.loads(run(host_check, "parse", deck).stdout)
        s = read_deck_summary(deck)
        assert (d["np"], d["na"], d["dims"], d["refinement"]) == (s["np"], s["na"], s["dims"],
                                                                  s["refinement"]), deck
        assert d["blocks"] == s["blocks"], deck
        assert sorted(map(int, d["materials"])) == s["materials"], deck


@pytest.mark.parametrize("text,msg", [
    ("<doma_inp><angular_quad np='1' na='1'/></doma_inp>", "solver block"),
    ("<doma_inp><solver solve_type='steady' scheme='xx' num_groups='1'/></doma_inp>", "Unknown scheme"),
    ("<doma_inp><solver solve_type='steady'", "XML parse error"),
    ("<doma_inp><solver solve_type='steady' scheme='dd' num_groups='1' fs_tol='-1'/></doma_inp>",
     "valid param in fs_tol"),
])
def test_bad_decks_report_errors(host_check, tmp_path, text, msg):
    deck = tmp_path / "bad.xml"
    deck.write_text(text)
    r = run(host_check, "parse", deck, check=False)
    assert r.returncode == 1 and msg in r.stderr


@pytest.mark.skipif(not ol.ref_available(), reason="DOMA reference not built here")
@pytest.mark.parametrize("dims", [2, 3])
def test_text_output_identical_to_reference(host_check, tmp_path, dims):
    p = P.random_problem(6, dims, 6, 5, 4, groups=2, np_=1, na=2, materials=3)
    opts = P.make_options(scheme="dd")
    (tmp_path / "ref").mkdir()
    (tmp_path / "ours").mkdir()
    phi, ok, *_ = ol.ref_solve(p, opts, out_base=str(tmp_path / "ref" / "case"))
    assert ok
    deck = write_deck(p, tmp_path / "case.xml")
    phi.astype(np.float64).tofile(tmp_path / "phi.bin")
    run(host_check, "dump", deck, tmp_path / "phi.bin", tmp_path / "ours" / "case")
    ref_files = sorted(x.name for x in (tmp_path / "ref").iterdir())
    our_files = sorted(x.name for x in (tmp_path / "ours").iterdir())
    assert ref_files == our_files
    for f in ref_files:
        assert (tmp_path / "ref" / f).read_bytes() == (tmp_path / "ours" / f).read_bytes(), f


def test_flux_at_point(host_check, tmp_path):
    p = P.random_problem(8, 3, 4, 3, 2, groups=2)
    deck = write_deck(p, tmp_path / "d.xml")
    phi = np.arange(p.num_groups * p.num_cells, dtype=np.float64)
    phi.tofile(tmp_path / "phi.bin")
    x = p.dx[0] + 0.4 * p.dx[1]       # cell i = 1 (a point inside, away from faces)
    y = 0.5 * p.dy[0]                 # j = 0
    z = p.dz[0] + 0.5 * p.dz[1]       # k = 1
    d = json.loads(run(host_check, "point", deck, tmp_path / "phi.bin", x, y, z, 1).stdout)
    c = (1 * p.ny + 0) * p.nx + 1
    assert d["found"] and d["flux"] == phi[p.num_cells + c]
    d = json.loads(run(host_check, "point", deck, tmp_path / "phi.bin", -1, 0, 0, 0).stdout)
    assert not d["found"]


@pytest.mark.gpu
@pytest.mark.parametrize("dims,scheme", [(3, "dd"), (3, "tw_dd"), (2, "tw_dd")])
def test_dropin_solver_matches_oracle(host_check, tmp_path, dims, scheme):
    p = P.random_problem(12, dims, 7, 6, 5, groups=3, np_=2, na=2, materials=3, fission=True)
    deck = write_deck(p, tmp_path / "d.xml", scheme=scheme, fs_tol=1e-10, mg_tol=1e-10)
    d = json.loads(run(host_check, "solve", deck, tmp_path / "phi.bin").stdout.splitlines()[-1])
    phi = np.fromfile(tmp_path / "phi.bin").reshape(p.num_groups, p.num_cells)
    o_phi, ok, si, mg, _ = ol.oracle_solve(p, P.make_options(scheme=scheme, fs_tol=1e-10, mg_tol=1e-10))
    assert d["converged"] == ok and d["si_counts"] == list(map(int, si)) and d["mg"] == mg
    assert np.abs(phi - o_phi).max() <= 1e-12 * np.abs(o_phi).max()


@pytest.mark.gpu
def test_cli_writes_reference_layout(tmp_path):
    if not nb.CLI.exists():
        nb.build()
    p = P.small_cube(1, n=8)
    deck = write_deck(p, tmp_path / "cube.xml", scheme="dd")
    r = subprocess.run([str(nb.CLI), "-i", str(deck), "-n", "4"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "Fixed source solver finished executing." in r.stdout
    assert "SI converged after" in r.stdout and "Time elapsed:" in r.stdout
    dims = (tmp_path / "cube_dims.txt").read_text().split()
    assert dims == ["num_x:", "8", "num_y:", "8", "num_z:", "8", "num_g:", "2"]
    o_phi, *_ = ol.oracle_solve(p, P.make_options(scheme="dd"))
    for g in range(2):
        vals = np.array([float(x) for x in (tmp_path / f"cube_g{g}_flux.txt").read_text().split()])
        assert np.allclose(vals, o_phi[g], rtol=6e-6, atol=0)


@pytest.mark.gpu
@pytest.mark.parametrize("dims,scheme", [(3, "dd"), (2, "tw_dd")])
def test_dropin_eigenvalue_matches_oracle(host_check, tmp_path, dims, scheme):
    """TransportSolver3D/2D::solveEigenvalue on an eigenvalue deck (k_tol read
    from the deck) against the CPU restatement of DOMA's power iteration."""
    p = P.random_problem(13, dims, 7, 6, 5, groups=2, np_=2, na=2, materials=3, fission=True,
                         fission_scale=8.0)
    deck = write_deck(p, tmp_path / "e.xml", scheme=scheme, fs_tol=1e-10, mg_tol=1e-6,
                      mg_max_it=400, solve_type="eigen", k_tol=1e-7)
    d = json.loads(run(host_check, "solve", deck, tmp_path / "phi.bin").stdout.splitlines()[-1])
    phi = np.fromfile(tmp_path / "phi.bin").reshape(p.num_groups, p.num_cells)
    opts = P.make_options(scheme=scheme, fs_tol=1e-10, mg_tol=1e-6, mg_max_it=400)
    o_phi, k, ok, si, pi, _, _ = ol.oracle_solve_eigen(p, opts, 1e-7)
    assert d["converged"] == ok and d["mg"] == pi and d["si_counts"] == list(map(int, si))
    assert abs(d["k"] - k) <= 1e-12 * k
    assert np.abs(phi - o_phi).max() <= 1e-12 * np.abs(o_phi).max()


@pytest.mark.gpu
def test_cli_runs_eigenvalue_decks(tmp_path):
    if not nb.CLI.exists():
        nb.build()
    p = P.random_problem(14, 3, 6, 6, 6, groups=2, np_=1, na=2, materials=3, fission=True,
                         fission_scale=8.0)
    deck = write_deck(p, tmp_path / "core.xml", scheme="dd", mg_tol=1e-5, mg_max_it=400,
                      solve_type="eigen", k_tol=1e-6)
    r = subprocess.run([str(nb.CLI), "-i", str(deck)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "Eigenvalue solver finished executing." in r.stdout
    assert "Converged value of k = " in r.stdout and "Time elapsed:" in r.stdout
    _, k, ok, *_ = ol.oracle_solve_eigen(p, P.make_options(scheme="dd", mg_tol=1e-5, mg_max_it=400),
                                         1e-6)
    assert ok
    assert f"Converged value of k = {k:g}" in r.stdout
    assert (tmp_path / "core_g1_flux.txt").exists()


def _read_column(path):
    return np.array([float(x) for x in Path(path).read_text().split()])


@pytest.mark.gpu
@pytest.mark.parametrize("dims,scheme", [(3, "dd"), (2, "tw_dd")])
def test_dropin_transient_matches_oracle(host_check, tmp_path, dims, scheme):
    """TransportSolver3D/2D::solveTransient on a transient deck: the flux it
    ends with, the SI counts and DOMA's per-step text files (initial
    condition, _t<step>_g<g>_flux.txt, _t<step>_d<d>_dnps.txt, where a cell
    whose material has fewer delayed groups than the most prints 0) against
    the CPU restatement of DOMA's transient."""
    p, tr = P.transient_problem(15, dims=dims, nx=6, ny=5, nz=4, np_=2, na=2, num_steps=3,
                                t1=0.6)
    kw = dict(scheme=scheme, fs_tol=1e-10, mg_tol=1e-10)
    deck = write_deck(p, tmp_path / "tr.xml", transient=tr, **kw)
    base = tmp_path / "out" / "tr"
    base.parent.mkdir()
    d = json.loads(run(host_check, "solve", deck, tmp_path / "phi.bin", "quiet", base)
                   .stdout.splitlines()[-1])
    phi = np.fromfile(tmp_path / "phi.bin").reshape(p.num_groups, p.num_cells)
    o_phis, o_dnps, ok, done, si = ol.oracle_solve_transient(p, tr, P.make_options(**kw))
    assert d["converged"] == ok and done == 3 and d["si_counts"] == list(map(int, si))
    assert np.abs(phi - o_phis[-1]).max() <= 1e-12 * np.abs(o_phis[-1]).max()
    assert (base.parent / "tr_dims.txt").exists()
    assert not _read_column(base.parent / "tr_g0_flux.txt").any()   # the zero start
    D = tr.num_d_groups
    full = np.array([tr.d_groups[m] == D for m in p.cell_material])
    for step in range(3):
        for g in range(p.num_groups):
            vals = _read_column(base.parent / f"tr_t{step}_g{g}_flux.txt")
            assert np.allclose(vals, o_phis[step, g], rtol=6e-6, atol=0)
        assert not (base.parent / f"tr_t{step}_dims.txt").exists()
    for dd in range(D):
        vals = _read_column(base.parent / f"tr_t2_d{dd}_dnps.txt")
        assert np.allclose(vals, np.where(full, o_dnps[dd], 0.0), rtol=6e-6, atol=0)
    assert not (base.parent / f"tr_t2_d{D}_dnps.txt").exists()


@pytest.mark.gpu
def test_cli_runs_transient_decks(tmp_path):
    if not nb.CLI.exists():
        nb.build()
    p, tr = P.transient_problem(16, dims=3, nx=6, ny=6, nz=6, np_=1, na=2, num_steps=2, t1=0.5)
    deck = write_deck(p, tmp_path / "pulse.xml", scheme="dd", mg_tol=1e-8, transient=tr)
    r = subprocess.run([str(nb.CLI), "-i", str(deck)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = r.stdout
    assert out.startswith("Setting up initial conditions...\nSolving timestep 0...\n")
    assert "Solving timestep 1..." in out and "Transient solver finished executing." in out
    assert "Time elapsed:" in out
    for f in ("pulse_dims.txt", "pulse_t0_g0_flux.txt", "pulse_t1_g2_flux.txt",
              "pulse_t1_d0_dnps.txt"):
        assert (tmp_path / f).exists(), f
    steady = write_deck(p, tmp_path / "steady_ic.xml", scheme="dd", transient=tr)
    steady.write_text(steady.read_text().replace('ics="zero"', 'ics="steady"'))
    r = subprocess.run([str(nb.CLI), "-i", str(steady)], capture_output=True, text=True)
    assert r.returncode == 1 and "zero initial conditions" in r.stderr
