"""Case generation: `.grid` / `.data` inputs for MPH-I runs.

Two generators live here.

* ``boid_to_particles`` follows the reference pre-processor
  (generator/generator.cpp:170-193): every cuboid is filled with a
  cell-centred lattice whose spacing is the cuboid width divided by the
  rounded cell count, in x-major / z-minor order.
* ``dam_case`` builds the synthetic benchmark geometries: a block of fluid
  resting in the lower corner of a closed box of wall particles (three layers
  thick), with a seeded uniform jitter on the fluid positions.  Domain = wall
  box plus a margin, so the periodic wrap of the solver
  (source/main.cpp:4741-4752) never couples opposite walls.

The text formats are those of the reference: `.grid` is read by
source/main.cpp:565-669, `.data` by source/main.cpp:523-563.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

FLUID_TYPES = (0, 1)
WALL_TYPES = (2, 3)


@dataclasses.dataclass
class Params:
    """Keyword parameters of a `.data` file (source/main.cpp:536-555)."""
    dt: float = 1.0e-4
    output_interval: float = 1.0
    vtk_output_interval: float = 1.0
    end_time: float = 1.0
    radius_ratio_a: float = 3.5
    radius_ratio_p: float = 1.7
    radius_ratio_v: float = 3.5
    density: Tuple[float, float, float, float] = (1000.0, 1000.0, 1000.0, 1000.0)
    bulk_modulus: Tuple[float, float, float, float] = (1.0e6, 1.0e6, 1.0e6, 1.0e6)
    bulk_viscosity: Tuple[float, float, float, float] = (1.0e5, 1.0e5, 1.0e5, 1.0e5)
    shear_viscosity: Tuple[float, float, float, float] = (0.1, 0.1, 0.1, 0.1)
    surface_tension: Tuple[float, float, float, float] = (0.0, 0.0, 0.0, 0.0)
    interaction_ratio: Tuple[Tuple[float, ...], ...] = ((1.0,) * 4,) * 4
    gravity: Tuple[float, float, float] = (0.0, -9.8, 0.0)
    wall2: Tuple[float, ...] = (0.0,) * 9   # center xyz, velocity xyz, omega xyz
    wall3: Tuple[float, ...] = (0.0,) * 9

    def to_text(self) -> str:
        def row(vals):
            return "  ".join(repr(float(v)) for v in vals)
        lines = [
            "# MPH-I parameter file",
            f"Dt  {self.dt!r}",
            f"OutputInterval  {self.output_interval!r}",
            f"VtkOutputInterval  {self.vtk_output_interval!r}",
            f"EndTime  {self.end_time!r}",
            f"RadiusRatioA  {self.radius_ratio_a!r}",
            f"RadiusRatioP  {self.radius_ratio_p!r}",
            f"RadiusRatioV  {self.radius_ratio_v!r}",
            f"Density  {row(self.density)}",
            f"BulkModulus  {row(self.bulk_modulus)}",
            f"BulkViscosity  {row(self.bulk_viscosity)}",
            f"ShearViscosity  {row(self.shear_viscosity)}",
            f"SurfaceTension  {row(self.surface_tension)}",
        ]
        for t in range(4):
            lines.append(f"InteractionRatio(Type{t})  {row(self.interaction_ratio[t])}")
        lines.append(f"Gravity  {row(self.gravity)}")
        w2, w3 = self.wall2, self.wall3
        lines.append("Wall2  Center {} {} {} Velocity {} {} {} Omega {} {} {}".format(*[repr(float(v)) for v in w2]))
        lines.append("Wall3  Center {} {} {} Velocity {} {} {} Omega {} {} {}".format(*[repr(float(v)) for v in w3]))
        return "\n".join(lines) + "\n"


@dataclasses.dataclass
class Particles:
    """Particle set of a `.grid` file (source/main.cpp:565-669)."""
    time: float
    spacing: float
    domain_min: np.ndarray   # (3,)
    domain_max: np.ndarray   # (3,)
    types: np.ndarray        # (N,) int32
    pos: np.ndarray          # (N, 3) float64
    vel: np.ndarray          # (N, 3) float64

    @property
    def count(self) -> int:
        return int(self.types.shape[0])

    def to_text(self, fmt: str = "%.17e") -> str:
        head = f"{self.time:.17e}\n" if fmt != "%e" else f"{self.time:f}\n"
        dm, dM = self.domain_min, self.domain_max
        head += ("%d " + fmt + "  " + " ".join([fmt] * 6) + "\n") % (
            self.count, self.spacing, dm[0], dM[0], dm[1], dM[1], dm[2], dM[2])
        body = np.empty((self.count, 7), dtype=object)
        lines = [head]
        rowfmt = "%d   " + " ".join([fmt] * 3) + "    " + " ".join([fmt] * 3) + "\n"
        for i in range(self.count):
            lines.append(rowfmt % (int(self.types[i]), *self.pos[i], *self.vel[i]))
        del body
        return "".join(lines)


def generator_text(parts: "Particles") -> str:
    """`.grid` text exactly as the reference pre-processor prints it
    (generator/generator.cpp:199-217)."""
    dm, dM = parts.domain_min, parts.domain_max
    lines = ["%f\n" % 0.0,
             "%d %e  %e %e %e  %e %e %e\n" % (parts.count, parts.spacing, dm[0], dM[0], dm[1], dM[1], dm[2], dM[2])]
    for i in range(parts.count):
        lines.append("%d   %e %e %e    %e %e %e\n" % (int(parts.types[i]), *parts.pos[i], *parts.vel[i]))
    return "".join(lines)


def write_case(prefix: str, params: Params, parts: Particles) -> Tuple[str, str]:
    data_path, grid_path = prefix + ".data", prefix + ".grid"
    with open(data_path, "w") as f:
        f.write(params.to_text())
    with open(grid_path, "w") as f:
        f.write(parts.to_text())
    return data_path, grid_path


def _lattice(lower: Sequence[float], upper: Sequence[float], space: float, dims: int) -> np.ndarray:
    """Cell-centred lattice filling [lower, upper) as in generator.cpp:173-191."""
    lo = np.asarray(lower, dtype=np.float64)
    hi = np.asarray(upper, dtype=np.float64)
    width = hi - lo
    axes = []
    for d in range(3):
        if d >= dims:
            axes.append(np.array([0.5 * (lo[d] + hi[d])]) if width[d] != 0 else np.array([lo[d]]))
            continue
        n = int(round(width[d] / space))
        sp = width[d] / n
        # generator.cpp increments px by spacing; reproduce the accumulated sum
        vals = []
        p = lo[d] + 0.5 * sp
        while p < hi[d] - 0.49 * sp:
            vals.append(p)
            p += sp
        axes.append(np.array(vals))
    gx, gy, gz = np.meshgrid(axes[0], axes[1], axes[2], indexing="ij")
    return np.stack([gx.ravel(), gy.ravel(), gz.ravel()], axis=1)


def boid_to_particles(spacing: float, lower_domain, upper_domain, cuboids: List[Dict]) -> Particles:
    """Fill cuboids (dicts with space, type, lower, upper, velocity) with particles,
    in the reference generator's order (generator/generator.cpp:170-193)."""
    types, pos, vel = [], [], []
    for c in cuboids:
        pts = _lattice(c["lower"], c["upper"], c["space"], 3)
        types.append(np.full(len(pts), int(c["type"]), dtype=np.int32))
        pos.append(pts)
        vel.append(np.tile(np.asarray(c["velocity"], dtype=np.float64), (len(pts), 1)))
    return Particles(0.0, float(spacing), np.asarray(lower_domain, float), np.asarray(upper_domain, float),
                     np.concatenate(types), np.concatenate(pos), np.concatenate(vel))


def dam_case(dim: int, fluid: Sequence[int], interior: Sequence[int], l0: float,
             wall_layers: int = 3, margin: int = 4, jitter: float = 0.01, seed: int = 0,
             fluid_types: Optional[np.ndarray] = None, wall_type_fn=None) -> Particles:
    """Fluid block `fluid` (cells) in the lower corner of a closed box whose
    interior is `interior` cells, surrounded by `wall_layers` layers of type-2
    wall particles.  Fluid positions get a uniform +-jitter*l0 perturbation in
    the active axes (seeded)."""
    assert dim in (2, 3)
    nf = list(fluid) + [1] * (3 - len(fluid))
    ni = list(interior) + [1] * (3 - len(interior))
    # fluid lattice (cell centred)
    idx = [np.arange(nf[d]) if d < dim else np.array([0]) for d in range(3)]
    g = np.meshgrid(*idx, indexing="ij")
    fpos = np.stack([(gi.ravel() + 0.5) * l0 for gi in g], axis=1)
    if dim == 2:
        fpos[:, 2] = 0.0
    rng = np.random.default_rng(seed)
    if jitter:
        jit = rng.uniform(-jitter * l0, jitter * l0, size=(fpos.shape[0], dim))
        fpos[:, :dim] += jit
    ftype = np.zeros(fpos.shape[0], dtype=np.int32) if fluid_types is None else np.asarray(fluid_types, np.int32)
    # wall lattice: cells of [-L, n+L) minus the interior [0, n)
    widx = [np.arange(-wall_layers, ni[d] + wall_layers) if d < dim else np.array([0]) for d in range(3)]
    w = np.meshgrid(*widx, indexing="ij")
    wc = np.stack([wi.ravel() for wi in w], axis=1)
    inside = np.ones(wc.shape[0], dtype=bool)
    for d in range(dim):
        inside &= (wc[:, d] >= 0) & (wc[:, d] < ni[d])
    wc = wc[~inside]
    wpos = (wc + 0.5) * l0
    if dim == 2:
        wpos[:, 2] = 0.0
    if wall_type_fn is None:
        wtype = np.full(wpos.shape[0], 2, dtype=np.int32)
    else:
        wtype = np.asarray(wall_type_fn(wc), dtype=np.int32)
    lo = np.array([-(wall_layers + margin) * l0] * 3)
    hi = np.array([(ni[d] + wall_layers + margin) * l0 for d in range(3)])
    if dim == 2:
        lo[2], hi[2] = -0.5 * l0, 0.5 * l0
    types = np.concatenate([ftype, wtype])
    pos = np.concatenate([fpos, wpos])
    vel = np.zeros_like(pos)
    return Particles(0.0, float(l0), lo, hi, types, pos, vel)


def baseline_params(dim: int, l0: float, dt: float, rho: float = 1000.0, mu: float = 0.1,
                    kappa: float = 1.0e6, gravity_axis: Optional[int] = None) -> Params:
    """Material constants of the benchmark cases: lambda chosen so that
    lambda*dt/(rho*l0^2) = 100, RA=RV=3.5, RP=1.7, sigma=0."""
    lam = 100.0 * rho * l0 * l0 / dt
    g = [0.0, 0.0, 0.0]
    g[gravity_axis if gravity_axis is not None else (1 if dim == 2 else 2)] = -9.8
    return Params(dt=dt, end_time=1.0e9, output_interval=1.0e9, vtk_output_interval=1.0e9,
                  density=(rho,) * 4, bulk_modulus=(kappa,) * 4, bulk_viscosity=(lam,) * 4,
                  shear_viscosity=(mu,) * 4, gravity=tuple(g))


# Named benchmark / test geometries ------------------------------------------------
def square_drop_2d(scale: float = 1.0, seed: int = 0) -> Tuple[Params, Particles]:
    """2D dam case: fluid 100x100 (l0=0.01) in a 3-layer wall box around a
    200x150 interior; dt=1e-4.  `scale` shrinks both blocks for small tests."""
    nf = max(2, int(round(100 * scale)))
    ni = (max(nf + 2, int(round(200 * scale))), max(nf + 2, int(round(150 * scale))))
    parts = dam_case(2, (nf, nf), ni, 0.01, seed=seed)
    return baseline_params(2, 0.01, 1.0e-4), parts


def cube_collapse_3d(n: int = 100, seed: int = 0) -> Tuple[Params, Particles]:
    """3D dam case: fluid n^3 (l0=0.005) in a 3-layer wall tank around a
    1.6n x 1.1n x 1.1n interior; gravity -9.8 in z; dt=5e-5."""
    ni = (int(round(1.6 * n)), int(round(1.1 * n)), int(round(1.1 * n)))
    parts = dam_case(3, (n, n, n), ni, 0.005, seed=seed)
    return baseline_params(3, 0.005, 5.0e-5), parts


# Batched and served workloads ----------------------------------------------------
def ensemble_case_2d(n: int, m: int, mu: float, gravity_deg: float, two_fluids: bool,
                     seed: int) -> Tuple[Params, Particles]:
    """One 2D case of the batched ensemble: an n x m fluid block (l0 = 0.01)
    in a 3-layer wall box around a 2n x 1.5m interior (the proportions of the
    2D dam case), shear viscosity mu, gravity 9.8 m/s^2 tilted by
    gravity_deg from -y, and with two_fluids the upper half of the block of
    type 1 with density 1.2x type 0; dt = 1e-4."""
    types = None
    if two_fluids:
        iy = np.tile(np.arange(m), n)           # lattice order: ix major, iy minor
        types = (iy >= m // 2).astype(np.int32)
    parts = dam_case(2, (n, m), (2 * n, int(round(1.5 * m)) + 2), 0.01, seed=seed, fluid_types=types)
    p = baseline_params(2, 0.01, 1.0e-4, mu=mu)
    a = np.deg2rad(gravity_deg)
    p = dataclasses.replace(p, gravity=(9.8 * float(np.sin(a)), -9.8 * float(np.cos(a)), 0.0))
    if two_fluids:
        p = dataclasses.replace(p, density=(1000.0, 1200.0, 1000.0, 1000.0))
    return p, parts


def ensemble_2d(count: int = 512, seed: int = 1, nmin: int = 40, nmax: int = 250):
    """The batched 2D ensemble: `count` cases with n, m ~ U[nmin, nmax], shear
    viscosity log-uniform in [0.01, 1] Pa s, gravity angle ~ U[0, 30] deg, two
    fluid types in every other case (seeded)."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        n, m = (int(v) for v in rng.integers(nmin, nmax + 1, size=2))
        mu = float(10.0 ** rng.uniform(-2.0, 0.0))
        ang = float(rng.uniform(0.0, 30.0))
        out.append(ensemble_case_2d(n, m, mu, ang, k % 2 == 1, seed=seed * 1000003 + k))
    return out


def serving_requests(count: int, seed: int = 2, rate: float = 20.0, nmin: float = 1.0e4, nmax: float = 5.0e5,
                     smin: int = 50, smax: int = 400, step_scale: float = 1.0):
    """Poisson arrivals (mean `rate` per second) of 2D and 3D cases whose
    total particle count is log-uniform in [nmin, nmax], each running a
    number of steps ~ U[smin, smax] (times step_scale, at least 1).  2D cases
    are ensemble cases; 3D cases are the cube-collapse geometry and constants
    with the fluid cube sized to the count.  Returns dicts with the arrival
    time t, dim, params, parts and steps (seeded)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for k in range(count):
        t += float(rng.exponential(1.0 / rate))
        total = float(np.exp(rng.uniform(np.log(nmin), np.log(nmax))))
        steps = max(1, int(round(int(rng.integers(smin, smax + 1)) * step_scale)))
        if rng.random() < 0.5:
            aspect = float(rng.uniform(0.5, 2.0))
            nm = 0.85 * total
            n = max(8, int(round(np.sqrt(nm * aspect))))
            m = max(8, int(round(nm / n)))
            mu = float(10.0 ** rng.uniform(-2.0, 0.0))
            ang = float(rng.uniform(0.0, 30.0))
            p, parts = ensemble_case_2d(n, m, mu, ang, bool(rng.random() < 0.5), seed=seed * 1000003 + k)
            dim = 2
        else:
            n = max(6, int(round((0.77 * total) ** (1.0 / 3.0))))
            p, parts = cube_collapse_3d(n, seed=seed * 1000003 + k)
            dim = 3
        out.append({"t": t, "dim": dim, "params": p, "parts": parts, "steps": steps})
    return out
