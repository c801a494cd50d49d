"""Fixed-source problems: the container passed across the C ABI and the seeded
synthetic workloads used by tests and benchmarks.

A :class:`Problem` is a tensor-product Cartesian mesh (per-axis cell widths,
cells numbered x fastest as in DOMA's ``BrickMesh3D``, src/BrickMesh3D.cpp:83-102),
a material index per cell, and per-material multigroup data laid out like
DOMA's ``MaterialProps`` (include/InputParameters.h:24-48): ``total[M][G]``,
``scatter[M][G][G]`` indexed ``[to][from]``, ``source[M][G]`` and optional
prompt fission (``chi_p``, ``nu_sigma_f``).

The generators are deterministic functions of a seed.  Random numbers come
from a counter-based SplitMix64 stream (Steele, Lea and Flood, "Fast
splittable pseudorandom number generators", OOPSLA 2014): value k of a stream
is mix(key + (k + 1) * 0x9E3779B97F4A7C15); uniforms use the top 53 bits.
Every transform uses only correctly rounded basic arithmetic (no libm or
SIMD transcendental functions, whose last bits differ between x86-64 and
aarch64 builds): normals are Irwin-Hall sums of twelve uniforms and
exponentials come from a scaled Taylor series, so inputs are bit-identical on
every machine.
"""
from __future__ import annotations

import ctypes
import hashlib
from dataclasses import dataclass, field, replace

import numpy as np

from . import abi

_GOLDEN = 0x9E3779B97F4A7C15
_M1 = 0xBF58476D1CE4E5B9
_M2 = 0x94D049BB133111EB
_MASK = (1 << 64) - 1


def _mix_int(z: int) -> int:
    z &= _MASK
    z = ((z ^ (z >> 30)) * _M1) & _MASK
    z = ((z ^ (z >> 27)) * _M2) & _MASK
    return z ^ (z >> 31)


def _mix_arr(z: np.ndarray) -> np.ndarray:
    z = z.astype(np.uint64, copy=True)
    z ^= z >> np.uint64(30)
    z *= np.uint64(_M1)
    z ^= z >> np.uint64(27)
    z *= np.uint64(_M2)
    z ^= z >> np.uint64(31)
    return z


class Rng:
    """Counter-based SplitMix64 stream keyed by (seed, tag)."""

    def __init__(self, seed: int, tag: str = ""):
        key = _mix_int(int(seed) & _MASK)
        for b in tag.encode():
            key = _mix_int(key ^ b)
        self.key = key
        self.counter = 0

    def child(self, tag: str) -> "Rng":
        r = Rng(0)
        key = self.key
        for b in tag.encode():
            key = _mix_int(key ^ b)
        r.key = key
        return r

    def bits(self, n: int) -> np.ndarray:
        idx = np.arange(self.counter + 1, self.counter + 1 + n, dtype=np.uint64)
        self.counter += n
        z = np.uint64(self.key) + idx * np.uint64(_GOLDEN)
        return _mix_arr(z)

    def uniform(self, n: int, lo: float = 0.0, hi: float = 1.0) -> np.ndarray:
        u = (self.bits(n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
        return lo + (hi - lo) * u

    def normal(self, n: int) -> np.ndarray:
        """Approximately standard normal: sum of 12 uniforms minus 6 (Irwin-Hall)."""
        u = self.uniform(12 * n).reshape(n, 12)
        acc = np.zeros(n)
        for k in range(12):  # fixed summation order
            acc = acc + u[:, k]
        return acc - 6.0

    def integers(self, n: int, lo: int, hi: int) -> np.ndarray:
        """Integers in [lo, hi)."""
        return lo + np.minimum((self.uniform(n) * (hi - lo)).astype(np.int64), hi - lo - 1)

    def permutation(self, n: int) -> np.ndarray:
        return np.argsort(self.uniform(n), kind="stable")


def portable_exp(x) -> np.ndarray:
    """exp(x) from basic arithmetic only: exp(x) = (exp(x / 256))^256, the inner
    factor by a 14-term Taylor series in Horner form, then 8 squarings.
    Relative error about 1e-13 for |x| < 10; bit-identical on every platform."""
    x = np.asarray(x, dtype=np.float64) / 256.0
    acc = np.ones_like(x)
    for k in range(14, 0, -1):
        acc = 1.0 + (x / float(k)) * acc
    for _ in range(8):
        acc = acc * acc
    return acc


@dataclass
class Problem:
    """A 2D or 3D fixed-source problem (see module docstring for the layout)."""

    num_dims: int
    dx: np.ndarray
    dy: np.ndarray
    dz: np.ndarray
    cell_material: np.ndarray
    total: np.ndarray
    scatter: np.ndarray
    source: np.ndarray | None
    num_polar: int
    num_azimuthal: int
    has_fission: np.ndarray | None = None
    chi_p: np.ndarray | None = None
    nu_sigma_f: np.ndarray | None = None
    name: str = "problem"
    meta: dict = field(default_factory=dict)

    def __post_init__(self):
        self.dx = np.ascontiguousarray(self.dx, dtype=np.float64)
        self.dy = np.ascontiguousarray(self.dy, dtype=np.float64)
        self.dz = np.ascontiguousarray(self.dz if self.num_dims == 3 else [1.0], dtype=np.float64)
        self.cell_material = np.ascontiguousarray(self.cell_material, dtype=np.uint32).reshape(-1)
        self.total = np.ascontiguousarray(self.total, dtype=np.float64)
        M, G = self.total.shape
        self.scatter = np.ascontiguousarray(self.scatter, dtype=np.float64).reshape(M, G, G)
        if self.source is not None:
            self.source = np.ascontiguousarray(self.source, dtype=np.float64).reshape(M, G)
        if self.has_fission is not None:
            self.has_fission = np.ascontiguousarray(self.has_fission, dtype=np.uint8).reshape(M)
            self.chi_p = np.ascontiguousarray(self.chi_p, dtype=np.float64).reshape(M, G)
            self.nu_sigma_f = np.ascontiguousarray(self.nu_sigma_f, dtype=np.float64).reshape(M, G)

    # -- shape ------------------------------------------------------------
    @property
    def nx(self) -> int:
        return int(self.dx.size)

    @property
    def ny(self) -> int:
        return int(self.dy.size)

    @property
    def nz(self) -> int:
        return int(self.dz.size) if self.num_dims == 3 else 1

    @property
    def num_cells(self) -> int:
        return self.nx * self.ny * self.nz

    @property
    def num_groups(self) -> int:
        return int(self.total.shape[1])

    @property
    def num_materials(self) -> int:
        return int(self.total.shape[0])

    @property
    def num_directions(self) -> int:
        return (8 if self.num_dims == 3 else 4) * self.num_polar * self.num_azimuthal

    @property
    def directions_per_octant(self) -> int:
        return self.num_polar * self.num_azimuthal

    def updates_per_sweep(self) -> int:
        """Cell * direction updates of one sweep of one group."""
        return self.num_cells * self.num_directions

    def cell_volumes(self) -> np.ndarray:
        if self.num_dims == 3:
            v = (self.dx[None, None, :] * self.dy[None, :, None]) * self.dz[:, None, None]
        else:
            v = self.dx[None, :] * self.dy[:, None]
        return v.reshape(-1)

    def digest(self) -> str:
        """SHA-256 over every array, to check that a regenerated input is identical."""
        h = hashlib.sha256()
        h.update(np.array([self.num_dims, self.num_polar, self.num_azimuthal], dtype=np.int64).tobytes())
        for a in (self.dx, self.dy, self.dz, self.cell_material, self.total, self.scatter,
                  self.source, self.has_fission, self.chi_p, self.nu_sigma_f):
            h.update(b"|" if a is None else np.ascontiguousarray(a).tobytes())
        return h.hexdigest()

    def with_(self, **kw) -> "Problem":
        return replace(self, **kw)

    # -- C ABI ------------------------------------------------------------
    def to_c(self) -> abi.DomaProblem:
        """A doma_problem pointing at this object's arrays (keep self alive)."""
        dp = ctypes.POINTER(ctypes.c_double)

        def ptr(a, t=dp):
            return None if a is None else a.ctypes.data_as(t)

        return abi.DomaProblem(
            num_dims=self.num_dims, nx=self.nx, ny=self.ny, nz=self.nz,
            dx=ptr(self.dx), dy=ptr(self.dy), dz=ptr(self.dz),
            num_groups=self.num_groups, num_materials=self.num_materials,
            cell_material=ptr(self.cell_material, ctypes.POINTER(ctypes.c_uint32)),
            total=ptr(self.total), scatter=ptr(self.scatter), source=ptr(self.source),
            has_fission=ptr(self.has_fission, ctypes.POINTER(ctypes.c_uint8)),
            chi_p=ptr(self.chi_p), nu_sigma_f=ptr(self.nu_sigma_f),
            num_polar=self.num_polar, num_azimuthal=self.num_azimuthal,
        )


@dataclass
class Transient:
    """Time-dependent data of a transient solve, per material (the layout of
    doma_transient).  Delayed-group arrays are padded to D = num_d_groups;
    material m uses the first d_groups[m].  t1 is the end time handed to a
    DOMA deck (t0 = 0); dt = t1 / num_steps."""

    t1: float
    num_steps: int
    inv_v: np.ndarray
    d_groups: np.ndarray | None = None
    chi_d: np.ndarray | None = None
    beta: np.ndarray | None = None
    lambda_: np.ndarray | None = None
    step_type: np.ndarray | None = None
    step_insert: np.ndarray | None = None
    step_remove: np.ndarray | None = None
    step_source: np.ndarray | None = None

    def __post_init__(self):
        self.inv_v = np.ascontiguousarray(self.inv_v, dtype=np.float64)
        M, G = self.inv_v.shape
        if self.d_groups is not None:
            self.d_groups = np.ascontiguousarray(self.d_groups, dtype=np.uint32).reshape(M)
            D = int(self.d_groups.max()) if M else 0
            self.chi_d = np.ascontiguousarray(self.chi_d, dtype=np.float64).reshape(M, G, D)
            self.beta = np.ascontiguousarray(self.beta, dtype=np.float64).reshape(M, G, D)
            self.lambda_ = np.ascontiguousarray(self.lambda_, dtype=np.float64).reshape(M, D)
        if self.step_type is not None:
            self.step_type = np.ascontiguousarray(self.step_type, dtype=np.uint32).reshape(M)
            self.step_insert = np.ascontiguousarray(self.step_insert, dtype=np.float64).reshape(M)
            self.step_remove = np.ascontiguousarray(self.step_remove, dtype=np.float64).reshape(M)
            self.step_source = np.ascontiguousarray(self.step_source, dtype=np.float64).reshape(M, G)

    @property
    def dt(self) -> float:
        return (self.t1 - 0.0) / float(self.num_steps)

    @property
    def num_d_groups(self) -> int:
        return 0 if self.d_groups is None else int(self.chi_d.shape[2])

    def times(self) -> list[float]:
        """The times of the steps, accumulated as t += dt."""
        t, out = 0.0, []
        for _ in range(self.num_steps):
            out.append(t)
            t += self.dt
        return out

    def digest(self) -> str:
        h = hashlib.sha256()
        h.update(np.array([self.t1, float(self.num_steps)]).tobytes())
        for a in (self.inv_v, self.d_groups, self.chi_d, self.beta, self.lambda_, self.step_type,
                  self.step_insert, self.step_remove, self.step_source):
            h.update(b"|" if a is None else np.ascontiguousarray(a).tobytes())
        return h.hexdigest()

    def to_c(self) -> abi.DomaTransient:
        """A doma_transient pointing at this object's arrays (keep self alive)."""
        dp = ctypes.POINTER(ctypes.c_double)
        up = ctypes.POINTER(ctypes.c_uint32)

        def ptr(a, t=dp):
            return None if a is None else a.ctypes.data_as(t)

        return abi.DomaTransient(
            dt=self.dt, num_steps=self.num_steps, num_d_groups=self.num_d_groups,
            inv_v=ptr(self.inv_v), d_groups=ptr(self.d_groups, up), chi_d=ptr(self.chi_d),
            beta=ptr(self.beta), lambda_=ptr(self.lambda_), step_type=ptr(self.step_type, up),
            step_insert=ptr(self.step_insert), step_remove=ptr(self.step_remove),
            step_source=ptr(self.step_source))


def make_options(scheme: str = "dd", theta: float = 0.9, precision: str = "fp64",
                 fs_tol: float = 1e-8, fs_max_it: int = 1000, mg_tol: float = 1e-8,
                 mg_max_it: int = 200, verbose: int = 0, tile=(0, 0, 0),
                 iteration: str = "gauss_seidel") -> abi.DomaOptions:
    schemes = {"dd": abi.DOMA_SCHEME_DD, "tw_dd": abi.DOMA_SCHEME_TW_DD}
    precs = {"fp64": abi.DOMA_PREC_FP64, "fp32": abi.DOMA_PREC_FP32}
    iters = {"gauss_seidel": abi.DOMA_ITER_GAUSS_SEIDEL, "multigroup": abi.DOMA_ITER_MULTIGROUP}
    return abi.DomaOptions(
        scheme=schemes[scheme], theta=theta, precision=precs[precision],
        fs_tol=fs_tol, fs_max_it=fs_max_it, mg_tol=mg_tol, mg_max_it=mg_max_it,
        verbose=verbose, tile_x=tile[0], tile_y=tile[1], tile_z=tile[2],
        iteration=iters[iteration],
    )


# ---------------------------------------------------------------------------
# Scattering matrices

def _scatter_split(G: int, c: np.ndarray, sig: np.ndarray) -> np.ndarray:
    """[to][from] matrix with total out-scatter c*sigma_t per source group.

    Source group g keeps 60% in-group and sends 30% to g+1 and 10% to g+2;
    the next-to-last group keeps 70% and sends 30% down; the last group keeps
    80% and sends 20% up to the group above it (upscatter between the last two
    groups).  One group keeps everything; two groups: 70/30 down, 80/20 up.
    """
    S = np.zeros((G, G))
    cs = c * sig
    for g in range(G):
        if G == 1:
            S[0, 0] = cs[0]
        elif g == G - 1:
            S[g, g] = 0.8 * cs[g]
            S[g - 1, g] = 0.2 * cs[g]
        elif g == G - 2:
            S[g, g] = 0.7 * cs[g]
            S[g + 1, g] = 0.3 * cs[g]
        else:
            S[g, g] = 0.6 * cs[g]
            S[g + 1, g] = 0.3 * cs[g]
            S[g + 2, g] = 0.1 * cs[g]
    return S


# ---------------------------------------------------------------------------
# Workloads

def small_cube(seed: int = 0, n: int = 20, length: float = 10.0, scheme: str = "dd") -> Problem:
    """Plain method, small: 10 cm cube as an n^3 grid, 2 groups, 4x8 = 32
    directions (np = na = 2).  Each cell is material 0 or 1 with probability
    1/2; per material and group sigma_t ~ U[0.5, 2] /cm and scattering ratio
    c ~ U[0.3, 0.7]; downscatter only, group 0 sends 30% of its scattering to
    group 1.  Unit isotropic group-0 source in the central 5^3 cells (indices
    7..11 at n = 20), vacuum boundaries."""
    r = Rng(seed, "small_cube")
    N = n ** 3
    mat = (r.uniform(N) < 0.5).astype(np.uint32)
    G = 2
    sig = r.uniform(2 * G, 0.5, 2.0).reshape(2, G)
    c = r.uniform(2 * G, 0.3, 0.7).reshape(2, G)
    S = np.zeros((4, G, G))
    for m in range(2):
        S[m, 0, 0] = 0.7 * c[m, 0] * sig[m, 0]
        S[m, 1, 0] = 0.3 * c[m, 0] * sig[m, 0]
        S[m, 1, 1] = c[m, 1] * sig[m, 1]
    S[2:] = S[:2]
    total = np.concatenate([sig, sig])
    src = np.zeros((4, G))
    src[2:, 0] = 1.0
    lo = max(0, (n - 5) // 2)  # 7 at n = 20
    idx = np.arange(n)
    inside = (idx >= lo) & (idx < lo + 5)
    box = inside[:, None, None] & inside[None, :, None] & inside[None, None, :]
    mat = mat.reshape(n, n, n)
    mat[box] += 2
    w = np.full(n, length / n)
    return Problem(3, w, w.copy(), w.copy(), mat.reshape(-1), total, S, src, 2, 2,
                   name=f"small_cube_n{n}_s{seed}", meta={"scheme": scheme, "theta": 0.5})


def checkerboard(seed: int = 0, n: int = 64, groups: int = 8, np_: int = 4, na: int = 4,
                 block: int = 8, cell: float = 1.0) -> Problem:
    """Plain method at scale: n^3 mesh of `cell`-cm cells, `groups` groups,
    8np x 4na directions.  Four materials in a seeded checkerboard of block^3
    cell blocks (material = perm[(bi + bj + bk) mod 4]); per material and
    group sigma_t = exp(0.5 Z) (lognormal, median 1 /cm) and c ~ U[0.5, 0.95];
    scattering as in _scatter_split (lower-triangular plus upscatter between
    the last two groups).  Unit group-0 source in one seeded block^3 block,
    vacuum boundaries."""
    r = Rng(seed, "checkerboard")
    G = groups
    perm = r.permutation(4)
    sig = portable_exp(0.5 * r.normal(4 * G)).reshape(4, G)
    c = r.uniform(4 * G, 0.5, 0.95).reshape(4, G)
    S = np.stack([_scatter_split(G, c[m], sig[m]) for m in range(4)])
    idx = np.arange(n) // block
    nb = int(idx[-1]) + 1
    bsum = idx[:, None, None] + idx[None, :, None] + idx[None, None, :]
    mat = perm[bsum % 4].astype(np.uint32)
    sb = r.integers(3, 0, nb)  # source block (bk, bj, bi)
    in_src = ((idx[:, None, None] == sb[0]) & (idx[None, :, None] == sb[1])
              & (idx[None, None, :] == sb[2]))
    mat[in_src] += 4
    total = np.concatenate([sig, sig])
    S = np.concatenate([S, S])
    src = np.zeros((8, G))
    src[4:, 0] = 1.0
    w = np.full(n, cell)
    return Problem(3, w, w.copy(), w.copy(), mat.reshape(-1), total, S, src, np_, na,
                   name=f"checkerboard_n{n}_g{G}_s{seed}",
                   meta={"source_block": sb.tolist()})


def streaming_duct(seed: int = 0, n: int = 100, np_: int = 6, na: int = 6, width: int = 10,
                   src: int = 10, cell: float = 1.0) -> Problem:
    """Streaming/shielding shape: one group on an n^3 mesh of `cell`-cm cells.
    A src^3 unit source sits in the (0,0,0) corner (absorber cross sections).
    A width-cell-wide near-void duct (sigma_t = 1e-4 /cm, c = 0.5) follows a
    seeded 3-segment axis-aligned path away from the source; each segment runs
    along an axis different from the previous one, for U{3n/10 .. 6n/10} cells.
    The absorber has sigma_t = 0.1 /cm, c = 0.5.  Vacuum boundaries."""
    r = Rng(seed, "streaming_duct")
    mat = np.zeros((n, n, n), dtype=np.uint32)  # [k][j][i]
    cur = [0, 0, 0]  # lower corner (x, y, z) of the cursor cube
    prev_axis = -1
    lo_len, hi_len = max(1, (3 * n) // 10), max(2, (6 * n) // 10 + 1)
    for seg in range(3):
        choices = [a for a in range(3) if a != prev_axis]
        axis = choices[int(r.integers(1, 0, len(choices))[0])]
        length = int(r.integers(1, lo_len, hi_len)[0])
        lo = [cur[0], cur[1], cur[2]]
        hi = [cur[0] + width, cur[1] + width, cur[2] + width]
        lo[axis] = cur[axis] + src
        hi[axis] = cur[axis] + src + length
        lo = [min(max(v, 0), n) for v in lo]
        hi = [min(max(v, 0), n) for v in hi]
        mat[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]] = 1
        cur[axis] = min(cur[axis] + length, n - width)
        prev_axis = axis
    mat[:src, :src, :src] = 2
    total = np.array([[0.1], [1e-4], [0.1]])
    S = (0.5 * total).reshape(3, 1, 1)
    source = np.array([[0.0], [0.0], [1.0]])
    w = np.full(n, cell)
    return Problem(3, w, w.copy(), w.copy(), mat.reshape(-1), total, S, source, np_, na,
                   name=f"streaming_duct_n{n}_s{seed}")


def random_problem(seed: int = 0, dims: int = 3, nx: int = 5, ny: int = 4, nz: int = 3,
                   groups: int = 3, np_: int = 1, na: int = 1, materials: int = 3,
                   fission: bool = False, upscatter: bool = True,
                   fission_scale: float = 1.0) -> Problem:
    """Small irregular problem for unit tests: non-uniform widths in
    U[0.3, 1.5] cm, random materials, dense scattering (upscatter included
    when asked) with c ~ U[0.1, 0.9], a source in every other material and,
    optionally, prompt fission in material 0 (nu sigma_f ~ U[0.01, 0.1] times
    fission_scale)."""
    r = Rng(seed, f"random_problem_{dims}")
    G, M = groups, materials
    if dims == 2:
        nz = 1
    N = nx * ny * nz
    dx = r.uniform(nx, 0.3, 1.5)
    dy = r.uniform(ny, 0.3, 1.5)
    dz = r.uniform(nz, 0.3, 1.5) if dims == 3 else np.ones(1)
    mat = r.integers(N, 0, M).astype(np.uint32)
    sig = r.uniform(M * G, 0.2, 2.0).reshape(M, G)
    c = r.uniform(M * G, 0.1, 0.9).reshape(M, G)
    S = np.zeros((M, G, G))
    for m in range(M):
        frac = r.uniform(G * G, 0.0, 1.0).reshape(G, G)  # [to][from]
        if not upscatter:
            frac = np.tril(frac)
        frac[np.arange(G), np.arange(G)] += 1.0
        frac /= frac.sum(axis=0, keepdims=True)
        S[m] = frac * (c[m] * sig[m])[None, :]
    src = np.zeros((M, G))
    for m in range(0, M, 2):
        src[m] = r.uniform(G, 0.0, 2.0)
    hf = chi = nsf = None
    if fission:
        hf = np.zeros(M, dtype=np.uint8)
        hf[0] = 1
        chi = np.zeros((M, G))
        chi[0] = r.uniform(G, 0.0, 1.0)
        chi[0] /= chi[0].sum()
        nsf = np.zeros((M, G))
        nsf[0] = r.uniform(G, 0.01, 0.1) * fission_scale
    return Problem(dims, dx, dy, dz, mat, sig, S, src, np_, na, has_fission=hf, chi_p=chi,
                   nu_sigma_f=nsf, name=f"random{dims}d_{nx}x{ny}x{nz}_g{G}_s{seed}")


def transient_problem(seed: int = 0, dims: int = 3, nx: int = 6, ny: int = 5, nz: int = 4,
                      groups: int = 3, np_: int = 1, na: int = 2, materials: int = 4,
                      num_steps: int = 4, t1: float = 1.0, delayed: int = 3,
                      steps: bool = True) -> tuple[Problem, Transient]:
    """A random_problem with fission in materials 0 and 1 and the data of a
    transient: inverse velocities U[0.5, 5]; `delayed` precursor groups in
    material 0 and one fewer in material 1 (materials without fission have
    none), beta ~ U[0.001, 0.01], lambda ~ U[0.05, 2], normalised chi_d; and,
    with `steps`, a source step of each kind: material 1 on between t1/4 and
    t1/2 (both ends), material 2 inserted at 0.3 t1, material 3 removed at
    t1/2 (a removal time equal to a step time is still on)."""
    if materials < 4:
        raise ValueError("transient_problem needs at least 4 materials")
    p = random_problem(seed, dims, nx, ny, nz, groups, np_, na, materials, fission=True)
    r = Rng(seed, f"transient_{dims}")
    G, M = groups, materials
    hf = p.has_fission.copy()
    chi, nsf = p.chi_p.copy(), p.nu_sigma_f.copy()
    hf[1] = 1
    chi[1] = r.uniform(G, 0.0, 1.0)
    chi[1] /= chi[1].sum()
    nsf[1] = r.uniform(G, 0.01, 0.1)
    p = p.with_(has_fission=hf, chi_p=chi, nu_sigma_f=nsf, name=p.name + "_transient")
    inv_v = r.uniform(M * G, 0.5, 5.0).reshape(M, G)
    tr = Transient(t1=t1, num_steps=num_steps, inv_v=inv_v)
    if delayed > 0:
        D = delayed
        dg = np.zeros(M, dtype=np.uint32)
        dg[0], dg[1] = D, max(D - 1, 0)
        chi_d = np.zeros((M, G, D))
        beta = np.zeros((M, G, D))
        lam = np.zeros((M, D))
        for m in (0, 1):
            d = int(dg[m])
            if d == 0:
                continue
            cd = r.uniform(G * d, 0.0, 1.0).reshape(G, d)
            chi_d[m, :, :d] = cd / cd.sum(axis=0, keepdims=True)
            beta[m, :, :d] = r.uniform(G * d, 0.001, 0.01).reshape(G, d)
            lam[m, :d] = r.uniform(d, 0.05, 2.0)
        tr.d_groups, tr.chi_d, tr.beta, tr.lambda_ = dg, chi_d, beta, lam
    if steps:
        st = np.zeros(M, dtype=np.uint32)
        ins = np.zeros(M)
        rem = np.zeros(M)
        ssrc = np.zeros((M, G))
        st[1], ins[1], rem[1] = abi.DOMA_STEP_BOTH, 0.25 * t1, 0.5 * t1
        st[2], ins[2] = abi.DOMA_STEP_INSERT, 0.3 * t1
        st[3], rem[3] = abi.DOMA_STEP_REMOVE, 0.5 * t1
        for m in range(M):
            if st[m]:
                ssrc[m] = r.uniform(G, 0.5, 3.0)
        tr.step_type, tr.step_insert, tr.step_remove, tr.step_source = st, ins, rem, ssrc
    tr.__post_init__()
    return p, tr


def square_2d(seed: int = 0, n: int = 32, groups: int = 2, np_: int = 2, na: int = 2,
              cell: float = 0.5) -> Problem:
    """2D analogue of small_cube: n^2 cells, random two-material mix, central
    source block of n/4 cells on a side."""
    r = Rng(seed, "square_2d")
    G = groups
    mat = (r.uniform(n * n) < 0.5).astype(np.uint32).reshape(n, n)
    sig = r.uniform(2 * G, 0.5, 2.0).reshape(2, G)
    c = r.uniform(2 * G, 0.3, 0.8).reshape(2, G)
    S = np.stack([_scatter_split(G, c[m], sig[m]) for m in range(2)])
    b = max(1, n // 4)
    lo = (n - b) // 2
    mat[lo:lo + b, lo:lo + b] += 2
    total = np.concatenate([sig, sig])
    S = np.concatenate([S, S])
    src = np.zeros((4, G))
    src[2:, 0] = 1.0
    w = np.full(n, cell)
    return Problem(2, w, w.copy(), np.ones(1), mat.reshape(-1), total, S, src, np_, na,
                   name=f"square2d_n{n}_g{G}_s{seed}")


def batch_mix(seed: int = 0, count: int = 256, n_range=(16, 96), groups=(1, 2, 4, 8, 16),
              k_range=(2, 6)) -> list[Problem]:
    """Batched-solve workload: `count` independent checkerboard problems, each
    drawing its mesh n^3 with n ~ U{n_range}, its group count from `groups` and
    its quadrature (2k polar x 4k azimuthal, np = na = k) with k ~ U{k_range};
    materials, scattering and source drawn as in `checkerboard`."""
    r = Rng(seed, "batch_mix")
    ns = r.integers(count, n_range[0], n_range[1] + 1)
    gs = r.integers(count, 0, len(groups))
    ks = r.integers(count, k_range[0], k_range[1] + 1)
    return [checkerboard(seed * 100003 + i, n=int(ns[i]), groups=int(groups[gs[i]]),
                         np_=int(ks[i]), na=int(ks[i]), block=8) for i in range(count)]


# ---------------------------------------------------------------------------
# Learned-accelerator workload

def gaussian_field(rng: np.random.Generator, n: int, corr: float = 4.0) -> np.ndarray:
    """Unit-variance periodic Gaussian random field on an n^3 grid: white
    normal noise convolved (by FFT) with exp(-d^2 / corr^2), d the periodic
    distance in cells, so the field's covariance is exp(-d^2 / (2 corr^2))."""
    d = np.minimum(np.arange(n), n - np.arange(n)).astype(np.float64)
    k1 = np.exp(-(d * d) / (corr * corr))
    kern = k1[:, None, None] * k1[None, :, None] * k1[None, None, :]
    w = rng.standard_normal((n, n, n))
    ax = (0, 1, 2)
    f = np.fft.irfftn(np.fft.rfftn(w, axes=ax) * np.fft.rfftn(kern, axes=ax), s=(n, n, n), axes=ax)
    return f / np.sqrt(np.sum(kern * kern))


def learned_problem(seed: int = 0, n: int = 32, groups: int = 4, np_: int = 3, na: int = 3,
                    log_sigma: float = 0.8, corr: float = 4.0, c_range=(0.9, 0.999),
                    downscatter: float = 0.5, max_blocks: int = 3) -> Problem:
    """High-scattering heterogeneous problem of the learned accelerator.

    n^3 cells of 1 cm.  Per cell and group, sigma_t = exp(log_sigma * Z) with Z
    a unit-variance Gaussian random field of correlation length `corr` cells
    (median 1 cm^-1), and a scattering ratio c ~ U[c_range] drawn per cell.
    Group g keeps c * sigma_t in-group and sends downscatter * (1 - c) *
    sigma_t to group g+1 (the last group keeps only its in-group part), so
    the problem is subcritical and dominated by in-group scattering.  Sources:
    1..max_blocks unit blocks of (n/8)^3 cells at seeded positions, each in a
    seeded group.  Every cell is its own material.  Inputs come from numpy's
    PCG64 generator: deterministic for a seed, meant for training and
    evaluation data, not for bitwise fixtures."""
    rng = np.random.default_rng([int(seed), 0x6C65_6172])
    N, G = n ** 3, groups
    total = np.empty((N, G))
    c = rng.uniform(c_range[0], c_range[1], (N, G))
    for g in range(G):
        total[:, g] = np.exp(log_sigma * gaussian_field(rng, n, corr)).reshape(-1)
    scatter = np.zeros((N, G, G))
    for g in range(G):
        scatter[:, g, g] = c[:, g] * total[:, g]
        if g + 1 < G:
            scatter[:, g + 1, g] = downscatter * (1.0 - c[:, g]) * total[:, g]
    source = np.zeros((n, n, n, G))
    b = max(2, n // 8)
    for _ in range(int(rng.integers(1, max_blocks + 1))):
        z, y, x = (int(v) for v in rng.integers(0, n - b + 1, 3))
        source[z:z + b, y:y + b, x:x + b, int(rng.integers(0, G))] = 1.0
    return Problem(
        num_dims=3, dx=np.ones(n), dy=np.ones(n), dz=np.ones(n),
        cell_material=np.arange(N, dtype=np.uint32), total=total, scatter=scatter,
        source=source.reshape(N, G), num_polar=np_, num_azimuthal=na,
        name=f"learned_s{seed}_n{n}_g{G}", meta={"seed": seed, "c_range": c_range},
    )
