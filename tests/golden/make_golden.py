"""Generate the golden fixtures by running DOMA's own code.

Run from the repository root where the DOMA source tree is present:

    make -C oracle ref        # builds oracle/_ref/libdoma_ref.so from DOMA's sources
    python tests/golden/make_golden.py            # every fixture
    python tests/golden/make_golden.py --eigen    # the k-eigenvalue fixtures only
    python tests/golden/make_golden.py --transient  # the transient fixtures only
    python tests/golden/make_golden.py --only NAME[,NAME...]  # the named fixed-source fixtures

Each case is a seeded synthetic problem (doma_gb300.problems) solved by DOMA
(single thread, the bit-reproducible order).  A fixture stores the generator
call, the SHA-256 digest of the regenerated inputs, the options, DOMA's scalar
flux, its return value and the source-iteration counts it printed.  The
quadrature file stores DOMA's direction cosines and weights.
"""
from __future__ import annotations

import json
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import oracle_lib as ol  # noqa: E402
from doma_gb300 import problems as P  # noqa: E402

HERE = Path(__file__).resolve().parent

# name -> (generator, kwargs, options kwargs)
CASES = {
    "small_cube_dd": ("small_cube", {"seed": 0, "n": 20}, {"scheme": "dd"}),
    "small_cube_twdd": ("small_cube", {"seed": 0, "n": 20}, {"scheme": "tw_dd", "theta": 0.9}),
    "random3d_fission_dd": ("random_problem",
                            {"seed": 3, "dims": 3, "nx": 7, "ny": 6, "nz": 5, "groups": 3,
                             "np_": 2, "na": 2, "materials": 4, "fission": True},
                            {"scheme": "dd", "fs_tol": 1e-10, "mg_tol": 1e-10}),
    "random3d_fission_twdd": ("random_problem",
                              {"seed": 3, "dims": 3, "nx": 7, "ny": 6, "nz": 5, "groups": 3,
                               "np_": 2, "na": 2, "materials": 4, "fission": True},
                              {"scheme": "tw_dd", "theta": 0.9, "fs_tol": 1e-10,
                               "mg_tol": 1e-10}),
    "random2d_dd": ("random_problem",
                    {"seed": 5, "dims": 2, "nx": 9, "ny": 7, "groups": 3, "np_": 2, "na": 3,
                     "materials": 3, "fission": True},
                    {"scheme": "dd", "fs_tol": 1e-10, "mg_tol": 1e-10}),
    "random2d_twdd": ("random_problem",
                      {"seed": 5, "dims": 2, "nx": 9, "ny": 7, "groups": 3, "np_": 2, "na": 3,
                       "materials": 3, "fission": True},
                      {"scheme": "tw_dd", "theta": 0.9, "fs_tol": 1e-10, "mg_tol": 1e-10}),
    "square2d_dd": ("square_2d", {"seed": 1, "n": 24, "groups": 2}, {"scheme": "dd"}),
    "square2d_twdd": ("square_2d", {"seed": 1, "n": 24, "groups": 2},
                      {"scheme": "tw_dd", "theta": 0.9}),
    "checkerboard_n16_twdd": ("checkerboard",
                              {"seed": 0, "n": 16, "groups": 8, "np_": 4, "na": 4, "block": 4},
                              {"scheme": "tw_dd", "theta": 0.9, "fs_tol": 1e-6,
                               "mg_tol": 1e-6}),
    "checkerboard_n16_dd": ("checkerboard",
                            {"seed": 0, "n": 16, "groups": 8, "np_": 4, "na": 4, "block": 4},
                            {"scheme": "dd", "fs_tol": 1e-6, "mg_tol": 1e-6}),
    "streaming_n24_dd": ("streaming_duct",
                         {"seed": 0, "n": 24, "np_": 3, "na": 3, "width": 4, "src": 4},
                         {"scheme": "dd", "fs_tol": 1e-8, "mg_tol": 1e-8}),
    "capped_si_twdd": ("small_cube", {"seed": 2, "n": 12},
                       {"scheme": "tw_dd", "theta": 0.9, "fs_max_it": 3}),
    "capped_mg_dd": ("random_problem",
                     {"seed": 7, "dims": 3, "nx": 6, "ny": 5, "nz": 4, "groups": 4, "np_": 1,
                      "na": 2, "materials": 3},
                     {"scheme": "dd", "fs_tol": 1e-9, "mg_tol": 1e-12, "mg_max_it": 2}),
    # more ordinates per octant than one GPU task holds (16): 36 = 16 + 16 + 4, 25 = 16 + 9
    "random3d_np6_dd": ("random_problem",
                        {"seed": 8, "dims": 3, "nx": 6, "ny": 5, "nz": 4, "groups": 2, "np_": 6,
                         "na": 6, "materials": 3},
                        {"scheme": "dd", "fs_tol": 1e-10, "mg_tol": 1e-10}),
    "random3d_np5_twdd": ("random_problem",
                          {"seed": 9, "dims": 3, "nx": 5, "ny": 6, "nz": 7, "groups": 2,
                           "np_": 5, "na": 5, "materials": 3},
                          {"scheme": "tw_dd", "theta": 0.9, "fs_tol": 1e-10, "mg_tol": 1e-10}),
    "random2d_np6_twdd": ("random_problem",
                          {"seed": 10, "dims": 2, "nx": 11, "ny": 8, "groups": 2, "np_": 6,
                           "na": 6, "materials": 3},
                          {"scheme": "tw_dd", "theta": 0.9, "fs_tol": 1e-10, "mg_tol": 1e-10}),
    # one cell thick along x (3D) and along y (2D)
    "slab3d_thin_twdd": ("random_problem",
                         {"seed": 12, "dims": 3, "nx": 1, "ny": 9, "nz": 2, "groups": 2,
                          "np_": 2, "na": 2, "materials": 3},
                         {"scheme": "tw_dd", "theta": 0.9, "fs_tol": 1e-10, "mg_tol": 1e-10}),
    "line2d_thin_dd": ("random_problem",
                       {"seed": 13, "dims": 2, "nx": 17, "ny": 1, "groups": 3, "np_": 3,
                        "na": 2, "materials": 3},
                       {"scheme": "dd", "fs_tol": 1e-10, "mg_tol": 1e-10}),
}

# k-eigenvalue cases: name -> (generator, kwargs, options kwargs, k_tol).  DOMA's
# solveEigenvalue is run twice: with the stream's default precision (the log a
# user sees) and with 17 digits (the exact k it prints).
_FIS3 = {"seed": 11, "dims": 3, "nx": 7, "ny": 6, "nz": 5, "groups": 3, "np_": 2, "na": 2,
         "materials": 4, "fission": True, "fission_scale": 10.0}
_FIS2 = {"seed": 12, "dims": 2, "nx": 9, "ny": 7, "groups": 3, "np_": 2, "na": 3,
         "materials": 3, "fission": True, "fission_scale": 10.0}
EIGEN_CASES = {
    "eigen3d_dd": ("random_problem", _FIS3,
                   {"scheme": "dd", "fs_tol": 1e-9, "mg_tol": 1e-7, "mg_max_it": 400}, 1e-8),
    "eigen3d_twdd": ("random_problem", _FIS3,
                     {"scheme": "tw_dd", "theta": 0.9, "fs_tol": 1e-9, "mg_tol": 1e-7,
                      "mg_max_it": 400}, 1e-8),
    "eigen2d_dd": ("random_problem", _FIS2,
                   {"scheme": "dd", "fs_tol": 1e-9, "mg_tol": 1e-7, "mg_max_it": 400}, 1e-8),
    "eigen2d_twdd": ("random_problem", _FIS2,
                     {"scheme": "tw_dd", "theta": 0.9, "fs_tol": 1e-9, "mg_tol": 1e-7,
                      "mg_max_it": 400}, 1e-8),
    "eigen_capped_dd": ("random_problem", _FIS3,
                        {"scheme": "dd", "fs_tol": 1e-9, "mg_tol": 1e-7, "mg_max_it": 4}, 1e-8),
}

# transient cases (zero initial condition): name -> (transient_problem kwargs, options kwargs).
# Every step's flux is DOMA's: step k comes from a run of k steps with t1 = k dt, which
# reproduces the first k steps exactly because (k dt) / k == dt for these dt.
TRANSIENT_CASES = {
    "transient3d_dd": ({"seed": 1, "dims": 3, "num_steps": 4, "delayed": 3},
                       {"scheme": "dd", "fs_tol": 1e-9, "mg_tol": 1e-9}),
    "transient3d_twdd": ({"seed": 1, "dims": 3, "num_steps": 4, "delayed": 3},
                         {"scheme": "tw_dd", "theta": 0.9, "fs_tol": 1e-9, "mg_tol": 1e-9}),
    "transient2d_dd": ({"seed": 1, "dims": 2, "num_steps": 4, "delayed": 3},
                       {"scheme": "dd", "fs_tol": 1e-9, "mg_tol": 1e-9}),
    "transient2d_twdd": ({"seed": 1, "dims": 2, "num_steps": 4, "delayed": 3},
                         {"scheme": "tw_dd", "theta": 0.9, "fs_tol": 1e-9, "mg_tol": 1e-9}),
    "transient3d_g1_nodelay_twdd": ({"seed": 4, "dims": 3, "groups": 1, "num_steps": 3,
                                     "delayed": 0},
                                    {"scheme": "tw_dd", "theta": 0.9, "fs_tol": 1e-9,
                                     "mg_tol": 1e-9}),
    "transient2d_thirds_twdd": ({"seed": 7, "dims": 2, "num_steps": 3, "t1": 1.0},
                                {"scheme": "tw_dd", "theta": 0.9, "fs_tol": 1e-9,
                                 "mg_tol": 1e-9}),
    "transient3d_capped_mid_dd": ({"seed": 9, "dims": 3, "num_steps": 4},
                                  {"scheme": "dd", "fs_tol": 1e-9, "mg_tol": 1e-10,
                                   "mg_max_it": 11}),
    "transient2d_capped_si_dd": ({"seed": 6, "dims": 2, "num_steps": 4, "t1": 3.0},
                                 {"scheme": "dd", "fs_tol": 1e-12, "fs_max_it": 12}),
}

# cases whose --verbose output (every SI residual) is also recorded
VERBOSE_LOGS = {"capped_mg_dd", "capped_si_twdd", "random2d_dd", "eigen_capped_dd",
                "transient2d_dd"}

QUAD_SETS = [(dims, np_, na) for dims in (2, 3)
             for (np_, na) in [(1, 1), (2, 2), (3, 3), (4, 4), (6, 6), (2, 5), (5, 2)]]


def make_problem(gen: str, kwargs: dict) -> P.Problem:
    return getattr(P, gen)(**kwargs)


def make_eigen() -> None:
    for name, (gen, kw, okw, k_tol) in EIGEN_CASES.items():
        p = make_problem(gen, kw)
        opts = P.make_options(**okw)
        t0 = time.time()
        phi, ok, si, pi, _, log = ol.ref_solve_eigen(p, opts, k_tol, threads=1)
        dt = time.time() - t0
        phi17, _, _, _, k17, log17 = ol.ref_solve_eigen(p, opts, k_tol, threads=1, precision=17)
        assert np.array_equal(phi, phi17)
        if k17 is None:  # not converged: the last k printed is the one before the last pass
            k17 = float(log17.rsplit("k = ", 1)[-1].split()[0]) if "k = " in log17 else None
        meta = {"generator": gen, "kwargs": kw, "options": okw, "k_tol": k_tol,
                "digest": p.digest(), "converged": ok, "pi_iterations": pi, "k": k17,
                "k_is_final": bool(ok), "reference_seconds": round(dt, 3), "log": log}
        if name in VERBOSE_LOGS:
            vopts = P.make_options(**okw, verbose=2)
            meta["log_verbose"] = ol.ref_solve_eigen(p, vopts, k_tol, threads=1)[5]
        np.savez_compressed(HERE / f"{name}.npz", phi=phi, si_counts=si,
                            meta=np.array(json.dumps(meta)))
        print(f"{name:28s} converged={ok} pi={pi} k={k17} {dt:.2f}s")


def make_transient() -> None:
    import dataclasses
    for name, (kw, okw) in TRANSIENT_CASES.items():
        p, tr = P.transient_problem(**kw)
        opts = P.make_options(**okw)
        t0 = time.time()
        phi, dnps, ok, si, log = ol.ref_solve_transient(p, tr, opts, threads=1)
        dt = time.time() - t0
        done = log.count("Solving timestep") - (0 if ok else 1)
        steps = []
        for k in range(1, done + 1):
            if k == tr.num_steps:
                steps.append(phi)
                continue
            t1k = k * tr.dt
            assert t1k / k == tr.dt, (name, k)
            trk = dataclasses.replace(tr, t1=t1k, num_steps=k)
            phik, _, okk, _, _ = ol.ref_solve_transient(p, trk, opts, threads=1)
            assert okk
            steps.append(phik)
        if not ok:
            steps.append(phi)  # the partial flux the failing step stopped with
        meta = {"generator": "transient_problem", "kwargs": kw, "options": okw,
                "digest": p.digest(), "transient_digest": tr.digest(), "converged": ok,
                "steps_done": done, "times": tr.times()[: len(steps)],
                "reference_seconds": round(dt, 3), "log": log}
        if name in VERBOSE_LOGS:
            vopts = P.make_options(**okw, verbose=2)
            meta["log_verbose"] = ol.ref_solve_transient(p, tr, vopts, threads=1)[4]
        np.savez_compressed(HERE / f"{name}.npz", phi_steps=np.array(steps), dnps=dnps,
                            si_counts=si, meta=np.array(json.dumps(meta)))
        print(f"{name:28s} converged={ok} steps={done} si={len(si)} {dt:.2f}s")


def main() -> None:
    if not ol.ref_available():
        raise SystemExit("oracle/_ref/libdoma_ref.so is missing: run `make -C oracle ref` first")
    if "--eigen" in sys.argv:
        make_eigen()
        return
    if "--transient" in sys.argv:
        make_transient()
        return
    only = None
    if "--only" in sys.argv:
        only = set(sys.argv[sys.argv.index("--only") + 1].split(","))
        unknown = only - set(CASES)
        if unknown:
            raise SystemExit(f"unknown fixtures: {sorted(unknown)}")
    if only is None:
        quad = {}
        for dims, np_, na in QUAD_SETS:
            mu, eta, xi, w, counts = ol.ref_quadrature(np_, na, dims)
            key = f"d{dims}_np{np_}_na{na}"
            quad[key + "_mu"], quad[key + "_eta"], quad[key + "_xi"] = mu, eta, xi
            quad[key + "_w"], quad[key + "_counts"] = w, counts
        np.savez_compressed(HERE / "quadrature.npz", **quad)
        print("quadrature.npz", len(QUAD_SETS), "sets")

    for name, (gen, kw, okw) in CASES.items():
        if only is not None and name not in only:
            continue
        p = make_problem(gen, kw)
        opts = P.make_options(**okw)
        t0 = time.time()
        phi, ok, si, mg, log = ol.ref_solve(p, opts, threads=1)
        dt = time.time() - t0
        meta = {"generator": gen, "kwargs": kw, "options": okw, "digest": p.digest(),
                "converged": ok, "mg_iterations": mg, "reference_seconds": round(dt, 3),
                "log": log}
        if name in VERBOSE_LOGS:
            vopts = P.make_options(**okw, verbose=2)
            meta["log_verbose"] = ol.ref_solve(p, vopts, threads=1)[4]
        np.savez_compressed(HERE / f"{name}.npz", phi=phi, si_counts=si,
                            meta=np.array(json.dumps(meta)))
        print(f"{name:28s} converged={ok} mg={mg} si={list(map(int, si))[:8]}... "
              f"{dt:.2f}s")
    if only is None:
        make_eigen()
        make_transient()


if __name__ == "__main__":
    main()
