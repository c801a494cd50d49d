"""Golden fixtures from DOMA's own example decks, made by running DOMA.

Run from the repository root where DOMA's source tree is present (the tree
is $DOMA_REFERENCE_TREE, or a directory named `reference` beside the
repository):

    make -C oracle ref REF=<DOMA tree>        # DOMA compiled from its sources
    python -m doma_gb300.build                # the deck reader used below
    python tests/golden/make_deck_golden.py [--jobs 4] [--only NAME,...]

For each deck it
  * copies the deck to tests/golden/decks/<name>.xml (input data for the GPU
    tests, which run where DOMA's tree is absent), unchanged except for the
    variants in VARIANTS, which say what they change in a comment;
  * reads it with the project's deck reader (DOMA's own needs pugixml, which
    is absent) into the fields of DOMA's InputParameters;
  * runs DOMA single-threaded (its bit-reproducible summation order) through
    oracle/ref_harness.cpp: DOMA's BrickMesh3D/2D expands the intervals, its
    solver solves and its dumpToTextFile writes the text output;
  * stores tests/golden/decks/<name>.npz: DOMA's stdout, return value and
    source-iteration counts, the SHA-256 of its scalar flux (all cells and
    groups, as float64 bytes in [G][N] order) with a strided sample of the
    flux, the whole flux where it is small, and the SHA-256 of every text
    file it wrote.
"""
from __future__ import annotations

import argparse
import ctypes
import hashlib
import json
import multiprocessing as mp
import os
import re
import shutil
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
HERE = Path(__file__).resolve().parent
DECKS = HERE / "decks"
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

# DOMA's fixed-source example decks (cases/), 2D and 3D
DECK_NAMES = ["2D_test", "2D_watanabe", "2D_assembly_fs", "3D_kobayashi_1", "3D_kobayashi_3",
              "3D_assembly_fs_mg1"]
# Decks changed from DOMA's: name -> (DOMA deck, solver attributes to set).
# 3D_assembly_fs converges in about 20 Gauss-Seidel passes of roughly 400
# sweeps of 109 M updates each: half a day for DOMA on one thread.  Its
# variant stops after the first pass (mg_max_it = 1), so every group's source
# iteration runs to the deck's own tolerance and the solve ends on DOMA's
# failed-MGI path.
VARIANTS = {"3D_assembly_fs_mg1": ("3D_assembly_fs", {"mg_max_it": "1"})}
FULL_FLUX_MAX = 50_000      # store the whole flux up to this many values
SAMPLE_COUNT = 20_000       # otherwise a strided sample of about this many


def reference_tree() -> Path:
    env = os.environ.get("DOMA_REFERENCE_TREE")
    for cand in ([Path(env)] if env else []) + [ROOT.parent / "reference"]:
        if (cand / "cases").is_dir():
            return cand
    raise SystemExit("DOMA's source tree not found (set DOMA_REFERENCE_TREE)")


_u32p = ctypes.POINTER(ctypes.c_uint32)
_dp = ctypes.POINTER(ctypes.c_double)
_u8p = ctypes.POINTER(ctypes.c_uint8)


class RefDeck(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint32) for n in ("dims", "num_groups", "num_polar", "num_azimuthal",
                                               "scheme", "mode")] + \
               [("fs_tol", ctypes.c_double), ("mg_tol", ctypes.c_double),
                ("k_tol", ctypes.c_double), ("fs_max_it", ctypes.c_uint32),
                ("mg_max_it", ctypes.c_uint32), ("nxi", ctypes.c_uint32),
                ("nyi", ctypes.c_uint32), ("nzi", ctypes.c_uint32),
                ("dx", _dp), ("dy", _dp), ("dz", _dp), ("ix", _u32p), ("iy", _u32p),
                ("iz", _u32p), ("blocks", _u32p), ("num_mats", ctypes.c_uint32),
                ("mat_ids", _u32p), ("total", _dp), ("scatter", _dp), ("has_source", _u8p),
                ("source", _dp), ("has_fission", _u8p), ("chi_p", _dp), ("prod", _dp)]


def parse_deck(path: Path) -> dict:
    from doma_gb300 import build as nb
    exe = ROOT / "tests" / "cpp" / "_build" / "host_check"
    src = ROOT / "tests" / "cpp" / "host_check.cpp"
    if not exe.exists() or exe.stat().st_mtime < src.stat().st_mtime:
        exe.parent.mkdir(parents=True, exist_ok=True)
        subprocess.run(["g++", "-O2", "-std=c++17", f"-I{nb.HOST / 'include'}", str(src), "-o",
                        str(exe), f"-L{nb.OUT}", "-ldoma_gb300_host", "-ldoma_gb300",
                        f"-Wl,-rpath,{nb.OUT},-rpath,/usr/local/cuda/lib64"], check=True)
    r = subprocess.run([str(exe), "parse", str(path)], capture_output=True, text=True, check=True)
    return json.loads(r.stdout)


def deck_struct(d: dict, keep: list) -> RefDeck:
    G = d["groups"]
    mats = sorted(d["materials"].items(), key=lambda kv: int(kv[0]))

    def arr(v, dt):
        a = np.ascontiguousarray(np.asarray(v, dtype=dt))
        keep.append(a)
        return a.ctypes.data_as({np.float64: _dp, np.uint32: _u32p, np.uint8: _u8p}[dt])

    def per_mat(key, width):
        out = np.zeros((len(mats), width))
        for m, (_, mp_) in enumerate(mats):
            v = mp_[key]
            if len(v):
                out[m] = v
        return out

    dims = d["dims"]
    s = RefDeck(dims=dims, num_groups=G, num_polar=d["np"], num_azimuthal=d["na"],
                scheme=d["scheme"], mode=d["mode"], fs_tol=d["fs_tol"], mg_tol=d["mg_tol"],
                k_tol=d["k_tol"], fs_max_it=d["fs_max_it"], mg_max_it=d["mg_max_it"],
                nxi=len(d["ix"]), nyi=len(d["iy"]), nzi=len(d["iz"]) if dims == 3 else 1)
    s.dx, s.dy = arr(d["dx"], np.float64), arr(d["dy"], np.float64)
    s.dz = arr(d["dz"] if dims == 3 else [1.0], np.float64)
    s.ix, s.iy = arr(d["ix"], np.uint32), arr(d["iy"], np.uint32)
    s.iz = arr(d["iz"] if dims == 3 else [1], np.uint32)
    s.blocks = arr(d["blocks"], np.uint32)
    s.num_mats = len(mats)
    s.mat_ids = arr([int(k) for k, _ in mats], np.uint32)
    s.total = arr(per_mat("total", G), np.float64)
    s.scatter = arr(per_mat("scatter", G * G), np.float64)
    s.has_source = arr([1 if len(m["source"]) else 0 for _, m in mats], np.uint8)
    s.source = arr(per_mat("source", G), np.float64)
    s.has_fission = arr([1 if len(m["prod"]) else 0 for _, m in mats], np.uint8)
    s.chi_p = arr(per_mat("chi_p", G), np.float64)
    s.prod = arr(per_mat("prod", G), np.float64)
    return s


_SI_RE = re.compile(r"SI (?:converged|failed to converge) after (\d+) iterations")
_MG_RE = re.compile(r"MGI (?:converged|failed to converge) after (\d+) iterations")


def run_deck(name: str) -> str:
    import oracle_lib as ol
    deck = DECKS / f"{name}.xml"
    d = parse_deck(deck)
    lib = ctypes.CDLL(str(ol.REF_LIB))
    lib.ref_solve_deck.restype = ctypes.c_int
    lib.ref_solve_deck.argtypes = [ctypes.POINTER(RefDeck), ctypes.c_uint32, _dp, ctypes.c_size_t,
                                   ctypes.POINTER(ctypes.c_size_t), _dp, ctypes.c_char_p,
                                   ctypes.c_size_t, ctypes.c_char_p, ctypes.c_int]
    keep: list = []
    s = deck_struct(d, keep)
    G = d["groups"]
    n_cells = int(np.prod([sum(d["ix"]), sum(d["iy"])] + ([sum(d["iz"])] if d["dims"] == 3 else [])))
    phi = np.zeros(G * n_cells)
    log = ctypes.create_string_buffer(1 << 24)
    n_out = ctypes.c_size_t(0)
    k = ctypes.c_double(0)
    with tempfile.TemporaryDirectory() as tmp:
        base = str(Path(tmp) / name)
        t0 = time.time()
        rc = lib.ref_solve_deck(ctypes.byref(s), 1, phi.ctypes.data_as(_dp), phi.size,
                                ctypes.byref(n_out), ctypes.byref(k), log, len(log),
                                base.encode(), 0)
        dt = time.time() - t0
        if rc < 0 or n_out.value != n_cells:
            raise RuntimeError(f"{name}: rc={rc}, cells {n_out.value} != {n_cells}")
        files = {}
        for f in sorted(Path(tmp).iterdir()):
            files[f.name[len(name):]] = hashlib.sha256(f.read_bytes()).hexdigest()
    text = log.value.decode()
    si = [int(x) for x in _SI_RE.findall(text)]
    mg = [int(x) for x in _MG_RE.findall(text)]
    phi = phi.reshape(G, n_cells)
    flat = phi.reshape(-1)
    stride = max(1, flat.size // SAMPLE_COUNT)
    out = {
        "deck_sha256": hashlib.sha256(deck.read_bytes()).hexdigest(),
        "converged": bool(rc), "si_counts": np.array(si, dtype=np.uint32),
        "mg_iterations": mg[-1] if mg else -1, "log": text,
        "groups": G, "num_cells": n_cells,
        "phi_sha256": hashlib.sha256(np.ascontiguousarray(phi, dtype="<f8").tobytes()).hexdigest(),
        "sample_stride": stride, "phi_sample": flat[::stride].copy(),
        "output_files": json.dumps(files), "doma_seconds": dt,
    }
    if flat.size <= FULL_FLUX_MAX:
        out["phi"] = phi
    np.savez_compressed(DECKS / f"{name}.npz", **out)
    return f"{name}: converged={bool(rc)} SI={si} MGI={mg[-1] if mg else None} {dt:.1f} s"


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=4)
    ap.add_argument("--only", default="")
    a = ap.parse_args()
    names = [n for n in a.only.split(",") if n] or DECK_NAMES
    DECKS.mkdir(exist_ok=True)
    cases = reference_tree() / "cases"
    for n in names:
        if n in VARIANTS:
            src, attrs = VARIANTS[n]
            text = (cases / f"{src}.xml").read_text()
            for k, v in attrs.items():
                text, count = re.subn(rf'({k}=")[^"]*(")', rf"\g<1>{v}\g<2>", text, count=1)
                assert count == 1, (n, k)
            changed = ", ".join(f"{k}={v}" for k, v in attrs.items())
            text = f"<!-- DOMA's cases/{src}.xml with {changed} -->\n" + text
            (DECKS / f"{n}.xml").write_text(text)
        else:
            shutil.copyfile(cases / f"{n}.xml", DECKS / f"{n}.xml")
    ctx = mp.get_context("spawn")
    with ctx.Pool(min(a.jobs, len(names))) as pool:
        for line in pool.imap_unordered(run_deck, names):
            print(line, flush=True)


if __name__ == "__main__":
    main()
