"""Loading of the committed golden fixtures (tests/golden/*.npz)."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

from doma_gb300 import problems as P

GOLDEN = Path(__file__).resolve().parent / "golden"


def case_names():
    """The fixed-source fixtures."""
    return sorted(p.stem for p in GOLDEN.glob("*.npz")
                  if p.stem != "quadrature" and not p.stem.startswith(("eigen", "transient")))


def eigen_case_names():
    """The k-eigenvalue fixtures."""
    return sorted(p.stem for p in GOLDEN.glob("eigen*.npz"))


def load_eigen_case(name: str):
    """-> (problem, options, k_tol, expected dict)"""
    z = np.load(GOLDEN / f"{name}.npz")
    meta = json.loads(str(z["meta"]))
    p = getattr(P, meta["generator"])(**meta["kwargs"])
    if p.digest() != meta["digest"]:
        raise AssertionError(f"{name}: regenerated inputs differ from the fixture's")
    opts = P.make_options(**meta["options"])
    exp = {"phi": z["phi"], "si_counts": z["si_counts"], "converged": meta["converged"],
           "pi_iterations": meta["pi_iterations"], "k": meta["k"],
           "k_is_final": meta["k_is_final"], "log": meta["log"],
           "log_verbose": meta.get("log_verbose")}
    return p, opts, meta["k_tol"], exp


def transient_case_names():
    """The transient (zero initial condition) fixtures."""
    return sorted(p.stem for p in GOLDEN.glob("transient*.npz"))


def load_transient_case(name: str):
    """-> (problem, transient, options, expected dict).  phi_steps holds DOMA's
    flux after each completed step and, when a step failed, the partial flux it
    stopped with; dnps the precursors after the last completed step."""
    z = np.load(GOLDEN / f"{name}.npz")
    meta = json.loads(str(z["meta"]))
    p, tr = P.transient_problem(**meta["kwargs"])
    if p.digest() != meta["digest"] or tr.digest() != meta["transient_digest"]:
        raise AssertionError(f"{name}: regenerated inputs differ from the fixture's")
    opts = P.make_options(**meta["options"])
    exp = {"phi_steps": z["phi_steps"], "dnps": z["dnps"], "si_counts": z["si_counts"],
           "converged": meta["converged"], "steps_done": meta["steps_done"],
           "times": meta["times"], "log": meta["log"], "log_verbose": meta.get("log_verbose")}
    return p, tr, opts, exp


def load_case(name: str):
    """-> (problem, options, expected dict)"""
    z = np.load(GOLDEN / f"{name}.npz")
    meta = json.loads(str(z["meta"]))
    p = getattr(P, meta["generator"])(**meta["kwargs"])
    if p.digest() != meta["digest"]:
        raise AssertionError(f"{name}: regenerated inputs differ from the fixture's")
    opts = P.make_options(**meta["options"])
    exp = {"phi": z["phi"], "si_counts": z["si_counts"], "converged": meta["converged"],
           "mg_iterations": meta["mg_iterations"], "meta": meta, "log": meta.get("log"),
           "log_verbose": meta.get("log_verbose")}
    return p, opts, exp


def quadrature_sets():
    z = np.load(GOLDEN / "quadrature.npz")
    keys = sorted({k.rsplit("_", 1)[0] for k in z.files})
    out = []
    for k in keys:
        d, n_p, n_a = k.split("_")
        out.append((int(d[1:]), int(n_p[2:]), int(n_a[2:]), z[k + "_mu"], z[k + "_eta"],
                    z[k + "_xi"], z[k + "_w"], z[k + "_counts"]))
    return out
