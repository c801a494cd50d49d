"""DOMA's own example decks, solved on the GPU and compared with DOMA.

The fixtures under tests/golden/decks/ were made by running DOMA itself
(compiled from its sources, single-threaded) on copies of its cases/ decks
(tests/golden/make_deck_golden.py).  Each deck is solved twice here, in the
FP64 drop-in mode the decks select:
  * through the C++ drop-in classes (tests/cpp/host_check.cpp): DOMA's
    progress lines on stdout, its return value and source-iteration counts,
    the scalar flux bit for bit (SHA-256 of all values; a strided sample
    within 1e-12 relative L-infinity), and the text output files byte for
    byte;
  * through the deck runner (`doma_gb300 -i <deck>`): the same stdout,
    followed by DOMA's closing lines, and the same text output files.
"""
import hashlib
import json
import re
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from doma_gb300 import build as nb

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
DECKS = ROOT / "tests" / "golden" / "decks"
SRC = ROOT / "tests" / "cpp" / "host_check.cpp"
EXE = ROOT / "tests" / "cpp" / "_build" / "host_check"
FP64_RTOL = 1e-12


def deck_names():
    return sorted(p.stem for p in DECKS.glob("*.npz"))


def load(name):
    z = np.load(DECKS / f"{name}.npz", allow_pickle=False)
    d = {k: z[k] for k in z.files}
    d["log"] = str(d["log"])
    d["output_files"] = json.loads(str(d["output_files"]))
    return d


@pytest.fixture(scope="module")
def host_check():
    if not nb.HOST_LIB.exists() or not nb.LIB.exists():
        nb.build()
    if not EXE.exists() or EXE.stat().st_mtime < max(SRC.stat().st_mtime,
                                                      nb.HOST_LIB.stat().st_mtime):
        EXE.parent.mkdir(parents=True, exist_ok=True)
        subprocess.run(["g++", "-O2", "-std=c++17", f"-I{nb.HOST / 'include'}", str(SRC), "-o",
                        str(EXE), f"-L{nb.OUT}", "-ldoma_gb300_host", "-ldoma_gb300",
                        f"-Wl,-rpath,{nb.OUT},-rpath,/usr/local/cuda/lib64"], check=True)
    return EXE


def output_digests(directory: Path, stem: str) -> dict:
    return {f.name[len(stem):]: hashlib.sha256(f.read_bytes()).hexdigest()
            for f in sorted(directory.iterdir()) if f.name.startswith(stem + "_")}


@pytest.mark.parametrize("name", deck_names())
def test_deck_drop_in_matches_doma(name, host_check, tmp_path):
    exp = load(name)
    deck = tmp_path / f"{name}.xml"
    shutil.copyfile(DECKS / f"{name}.xml", deck)
    assert hashlib.sha256(deck.read_bytes()).hexdigest() == str(exp["deck_sha256"])
    flux = tmp_path / "phi.bin"
    r = subprocess.run([str(host_check), "solve", str(deck), str(flux), "quiet",
                        str(tmp_path / name)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.splitlines(keepends=True)
    res = json.loads(lines[-1])
    assert "".join(lines[:-1]) == exp["log"]
    assert res["converged"] == bool(exp["converged"])
    assert res["si_counts"] == [int(x) for x in exp["si_counts"]]
    phi = np.fromfile(flux, dtype="<f8").reshape(int(exp["groups"]), int(exp["num_cells"]))
    sample = phi.reshape(-1)[::int(exp["sample_stride"])]
    want = exp["phi_sample"]
    assert float(np.abs(sample - want).max() / np.abs(want).max()) <= FP64_RTOL
    if "phi" in exp:
        assert float(np.abs(phi - exp["phi"]).max() / np.abs(exp["phi"]).max()) <= FP64_RTOL
    assert hashlib.sha256(phi.tobytes()).hexdigest() == str(exp["phi_sha256"]), \
        "flux within tolerance but not bit-equal to DOMA's"
    assert output_digests(tmp_path, name) == exp["output_files"]


@pytest.mark.parametrize("name", deck_names())
def test_deck_runner_matches_doma(name, tmp_path):
    exp = load(name)
    if not nb.CLI.exists():
        nb.build()
    deck = tmp_path / f"{name}.xml"
    shutil.copyfile(DECKS / f"{name}.xml", deck)
    r = subprocess.run([str(nb.CLI), "-i", str(deck)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = r.stdout
    assert out.startswith(exp["log"])
    tail = out[len(exp["log"]):]
    if exp["converged"]:
        assert re.fullmatch(r"Fixed source solver finished executing\.\nTime elapsed: \d+ \(s\)\.\n",
                            tail), tail
    else:
        assert tail == ""
    assert output_digests(tmp_path, name) == exp["output_files"]
