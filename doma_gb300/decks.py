"""Write a Problem as a DOMA <doma_inp> deck (and read simple decks back).

The deck uses one mesh interval per cell along each axis, block id =
material index, and the reaction names of DOMA's schema
(src/InputParameters.cpp:270-416), so DOMA itself, the C++ drop-in layer
and the CLI all read it as the same problem.
"""
from __future__ import annotations

import xml.etree.ElementTree as ET
from pathlib import Path

import numpy as np

from .problems import Problem, Transient


def _fmt(v) -> str:
    return ", ".join(repr(float(x)) for x in np.ravel(v))


def _fmt_u(v) -> str:
    return ", ".join(str(int(x)) for x in np.ravel(v))


def deck_text(p: Problem, scheme: str = "dd", fs_tol: float = 1e-8, fs_max_it: int = 1000,
              mg_tol: float = 1e-8, mg_max_it: int = 100, theta: float | None = None,
              precision: str | None = None, solve_type: str = "steady",
              k_tol: float | None = None, transient: Transient | None = None) -> str:
    """A deck for p.  With `transient` the deck is a transient one (t0 = 0,
    t1, t_steps, zero initial condition): every material gets delayed_groups
    and inv_vel (plus chi_d, beta, lambda_d where it has delayed groups), and
    the source steps become <transients>/<source_step> blocks."""
    G = p.num_groups
    extra = ""
    tr = transient
    if tr is not None:
        solve_type = "transient"
        extra += f' t0="0.0" t1="{float(tr.t1)!r}" t_steps="{tr.num_steps}" ics="zero"'
    if k_tol is not None:
        extra += f' k_tol="{k_tol!r}"'
    if theta is not None:
        extra += f' theta="{theta!r}"'
    if precision is not None:
        extra += f' precision="{precision}"'
    lines = ["<doma_inp>",
             f'  <solver solve_type="{solve_type}" scheme="{scheme}" num_groups="{G}" fs_tol="{fs_tol!r}"'
             f' mg_tol="{mg_tol!r}" fs_max_it="{fs_max_it}" mg_max_it="{mg_max_it}"{extra}/>',
             f'  <angular_quad type="gc" np="{p.num_polar}" na="{p.num_azimuthal}"/>',
             f'  <mesh dims="{p.num_dims}" refinement="0">',
             f'    <dx vals="{_fmt(p.dx)}"/>',
             f'    <dy vals="{_fmt(p.dy)}"/>']
    if p.num_dims == 3:
        lines.append(f'    <dz vals="{_fmt(p.dz)}"/>')
    lines.append(f'    <ix vals="{_fmt_u(np.ones(p.nx))}"/>')
    lines.append(f'    <iy vals="{_fmt_u(np.ones(p.ny))}"/>')
    if p.num_dims == 3:
        lines.append(f'    <iz vals="{_fmt_u(np.ones(p.nz))}"/>')
    lines.append(f'    <blocks vals="{_fmt_u(p.cell_material)}"/>')
    lines.append("  </mesh>")
    lines.append("  <materials>")
    for m in range(p.num_materials):
        dm = 0 if tr is None or tr.d_groups is None else int(tr.d_groups[m])
        lines.append(f'    <mat block="{m}"' + ("" if tr is None else f' delayed_groups="{dm}"') + ">")
        lines.append(f'      <reaction type="total" mgxs="{_fmt(p.total[m])}"/>')
        lines.append(f'      <reaction type="scatter" mgxs="{_fmt(p.scatter[m])}"/>')
        if p.source is not None and np.any(p.source[m] != 0.0):
            lines.append(f'      <reaction type="source" mgxs="{_fmt(p.source[m])}"/>')
        if p.has_fission is not None and p.has_fission[m]:
            lines.append(f'      <reaction type="chi_p" mgxs="{_fmt(p.chi_p[m])}"/>')
            lines.append(f'      <reaction type="nu_sigma_f" mgxs="{_fmt(p.nu_sigma_f[m])}"/>')
        if tr is not None:
            lines.append(f'      <reaction type="inv_vel" mgxs="{_fmt(tr.inv_v[m])}"/>')
            if dm:
                lines.append(f'      <reaction type="chi_d" mgxs="{_fmt(tr.chi_d[m, :, :dm])}"/>')
                lines.append(f'      <reaction type="beta" mgxs="{_fmt(tr.beta[m, :, :dm])}"/>')
                lines.append(f'      <reaction type="lambda_d" mgxs="{_fmt(tr.lambda_[m, :dm])}"/>')
        lines.append("    </mat>")
    lines.append("  </materials>")
    if tr is not None and tr.step_type is not None and np.any(tr.step_type != 0):
        lines.append("  <transients>")
        for m in range(p.num_materials):
            st = int(tr.step_type[m])
            if st == 0:
                continue
            at = ""
            if st in (1, 2):
                at += f' insert_at="{float(tr.step_insert[m])!r}"'
            if st in (1, 3):
                at += f' remove_at="{float(tr.step_remove[m])!r}"'
            lines.append(f'    <source_step block="{m}"{at} mgxs="{_fmt(tr.step_source[m])}"/>')
        lines.append("  </transients>")
    lines.append("</doma_inp>")
    return "\n".join(lines) + "\n"


def write_deck(p: Problem, path: str | Path, **kw) -> Path:
    path = Path(path)
    path.write_text(deck_text(p, **kw))
    return path


def read_deck_summary(path: str | Path) -> dict:
    """Independent (ElementTree) reading of the attributes the solver uses."""
    root = ET.parse(str(path)).getroot()
    s = root.find("solver").attrib
    aq = root.find("angular_quad").attrib
    m = root.find("mesh")
    return {"solver": dict(s), "np": int(aq["np"]), "na": int(aq["na"]),
            "dims": int(m.attrib["dims"]), "refinement": int(m.attrib["refinement"]),
            "blocks": [int(x) for x in m.find("blocks").attrib["vals"].replace("\n", "").split(",")],
            "materials": sorted(int(x.attrib["block"]) for x in root.find("materials"))}
