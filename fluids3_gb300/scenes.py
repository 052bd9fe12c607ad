"""Seeded synthetic scenes for the SPH step.

The reference seeds particles with ``rand()`` jitter on a lattice
(SetupAddVolume, fluids4.0/fluid_system.cpp:292-334: y layers outermost,
then x fastest within each xz layer, stopping at the point budget). These
generators keep that fill order and replace ``rand()`` with a counter-based
splitmix64 stream, so a (scene, seed) pair gives bit-identical float32
positions on any machine (numpy float32 arithmetic is IEEE, no FMA).

Workloads:
  dam_break      32,768 points, 32^3 lattice, box (-30,0,-30)..(30,60,30)
  dam_break_scaled  the dam break at n points with box and block scaled to
                 keep its density (65,536: the differentiated rollout)
  wave_tank      4,000,000 points filling the low-x 40% of a ~330-unit box,
                 X- wall forcing at frequency 0.2, amplitude 0.3
  fit_scenes     64 scenes of 8,192..32,768 points with a hidden viscosity
                 each (the batched parameter fit)
  batch_scenes   256 independent scenes, 2,048..65,536 points each
                 (log-uniform), each a block filling 20..60% of its own box,
                 with its own viscosity (0.1..0.5) and rest density (500..700)
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .params import FlParams
from .system import default_params, derive_params

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(counter: np.ndarray) -> np.ndarray:
    """splitmix64 of a uint64 counter array (Steele, Lea, Flood 2014)."""
    with np.errstate(over="ignore"):
        z = counter.astype(np.uint64) * _GOLDEN + _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform01(seed: int, stream: int, n: int) -> np.ndarray:
    """n float32 values in [0, 1) with 24 random bits each."""
    base = (np.uint64(seed) << np.uint64(40)) ^ (np.uint64(stream) << np.uint64(56))
    bits = splitmix64(base + np.arange(n, dtype=np.uint64)) >> np.uint64(40)
    return bits.astype(np.float32) * np.float32(2.0 ** -24)


@dataclass
class Scene:
    name: str
    params: FlParams
    pos: np.ndarray                  # (N, 3) float32
    vel: np.ndarray = field(default=None)
    veval: np.ndarray = field(default=None)
    clr: np.ndarray = field(default=None)
    steps: int = 100

    @property
    def n(self) -> int:
        return int(self.pos.shape[0])


# Parameters shared by the workloads (dam-break set: h = 0.01 m, cell = 2h).
SPH_PARAMS = dict(
    sim_scale=0.004, psmoothradius=0.01, pmass=0.00020543, prest_dens=600.0, pvisc=0.35,
    pintstiff=1.0, bound_stiff=10000.0, bound_damp=256.0, AL=200.0, VL=3.0,
    grav_dir=(0.0, -9.8, 0.0), grav_amt=1.0, dt=0.003, pradius=0.015,
    bound_slope=0.0, bound_friction=0.0, bound_wall_force=0.0, bound_wall_freq=0.0,
    grid_density=0.75,   # cell = 1.5 h / 0.75 = 2 h
)


def make_params(bound_min, bound_max, derive=None, **overrides) -> FlParams:
    """The dam-break parameter set in the given box. `derive` (FlParams ->
    FlParams) replaces the library's derivation; with it the inputs start
    from zero instead of SetupDefaultParams (every input is set here)."""
    p = default_params() if derive is None else FlParams()
    p.set(**SPH_PARAMS)
    p.set(bound_min=tuple(bound_min), bound_max=tuple(bound_max))
    p.set(**overrides)
    return derive_params(p) if derive is None else derive(p)


def lattice_spacing() -> np.float32:
    """0.0059 m rest distance over sim_scale 0.004, in world units (float32)."""
    return np.float32(0.0059) / np.float32(0.004)


def lattice_block(n: int, origin, cnt_x: int, cnt_z: int, spacing: np.float32, seed: int,
                  jitter_frac: float = 0.05) -> np.ndarray:
    """n points on a cnt_x x cnt_z lattice per y layer, layers stacked upward,
    each jittered by U(-jitter_frac, +jitter_frac) * spacing per axis."""
    k = np.arange(n, dtype=np.int64)
    per_layer = cnt_x * cnt_z
    iy = k // per_layer
    xz = k % per_layer
    ix = xz % cnt_x
    iz = xz // cnt_x
    o = np.asarray(origin, dtype=np.float32)
    s = np.float32(spacing)
    amp = np.float32(2.0 * jitter_frac) * s
    pos = np.empty((n, 3), dtype=np.float32)
    for axis, idx in enumerate((ix, iy, iz)):
        u = uniform01(seed, axis, n)
        jit = (u - np.float32(0.5)) * amp
        pos[:, axis] = (o[axis] + idx.astype(np.float32) * s) + jit
    return pos


def colours(pos: np.ndarray, lo, hi) -> np.ndarray:
    """RGBA8 by x/z position (the reference's COLORA gradient, cpp:324-328)."""
    lo = np.asarray(lo, np.float32)
    hi = np.asarray(hi, np.float32)
    t = np.clip((pos - lo) / np.maximum(hi - lo, 1e-6), 0, 1) * 0.8 + 0.2
    r = (t[:, 0] * 255).astype(np.uint32)
    b = (t[:, 2] * 255).astype(np.uint32)
    return r | (b << np.uint32(16)) | (np.uint32(255) << np.uint32(24))


def _finish(name, params, pos, steps, lo, hi) -> Scene:
    n = pos.shape[0]
    z = np.zeros((n, 3), np.float32)
    return Scene(name=name, params=params, pos=pos, vel=z.copy(), veval=z.copy(),
                 clr=colours(pos, lo, hi), steps=steps)


def dam_break(n: int = 32768, seed: int = 1, steps: int = 100) -> Scene:
    """Plain SPH dam break: a 32^3 jittered block in the low-x half of the box
    (-30,0,-30)..(30,60,30); the block starts 4 units inside the walls and, at
    32 points of 1.475 units, reaches x = 21.2."""
    bmin, bmax = (-30.0, 0.0, -30.0), (30.0, 60.0, 30.0)
    params = make_params(bmin, bmax)
    side = 32
    origin = (bmin[0] + 4.0, bmin[1] + 4.0, bmin[2] + 4.0)
    pos = lattice_block(n, origin, side, side, lattice_spacing(), seed)
    return _finish("dam_break_32k" if n == 32768 else f"dam_break_{n}", params, pos, steps, bmin, bmax)


def dam_break_scaled(n: int = 65536, seed: int = 4, steps: int = 200) -> Scene:
    """The dam break scaled to n points at the 32,768-point scene's density:
    box and block edges grow by k = (n / 32768)^(1/3), the lattice keeps its
    spacing (round(32 k) points per row, layers stacked to n). At 65,536
    points: k = 1.26, box (-37.8, 0, -37.8)..(37.8, 75.6, 37.8), 40 x 40
    points per layer, 41 layers (the last one partial)."""
    k = (n / 32768.0) ** (1.0 / 3.0)
    half, height = round(30.0 * k, 1), round(60.0 * k, 1)
    bmin, bmax = (-half, 0.0, -half), (half, height, half)
    params = make_params(bmin, bmax)
    side = int(round(32 * k))
    origin = (bmin[0] + 4.0 * k, bmin[1] + 4.0 * k, bmin[2] + 4.0 * k)
    pos = lattice_block(n, origin, side, side, lattice_spacing(), seed)
    name = "dam_break_65k" if n == 65536 else f"dam_break_scaled_{n}"
    return _finish(name, params, pos, steps, bmin, bmax)


def shifted_target(sc: Scene, frac: float = 0.3, seed: int = 5) -> np.ndarray:
    """A seeded target cloud: the scene's lattice block re-jittered with
    another seed and shifted `frac` box widths in +x (world units)."""
    lo, hi = np.asarray(sc.params.bound_min, np.float64), np.asarray(sc.params.bound_max, np.float64)
    s = lattice_spacing()
    rng_jit = (uniform01(seed, 7, sc.n) - np.float32(0.5)) * np.float32(0.1) * s
    out = sc.pos.astype(np.float64).copy()
    out[:, 0] += frac * (hi[0] - lo[0])
    out[:, 1] += rng_jit.astype(np.float64)
    return out


def wave_tank(n: int = 4_000_000, seed: int = 2, steps: int = 1000,
              wall_force: float = 0.3, wall_freq: float = 0.2, derive=None) -> Scene:
    """4M-point dam break with X- wall forcing: the block fills the low-x 40%
    of a box scaled to hold it (86 x 216 lattice per layer, ~216 layers).
    `derive`: see make_params."""
    s = lattice_spacing()
    cnt_x, cnt_z = 86, 216
    layers = -(-n // (cnt_x * cnt_z))
    margin = 4.0
    block_x = float(cnt_x * s)
    lx = (block_x + 2 * margin) / 0.4
    lz = float(cnt_z * s) + 2 * margin
    ly = max(float(layers * s) + 2 * margin, lz)
    bmin, bmax = (0.0, 0.0, 0.0), (round(lx, 1), round(ly, 1), round(lz, 1))
    params = make_params(bmin, bmax, derive=derive, bound_wall_force=wall_force, bound_wall_freq=wall_freq)
    pos = lattice_block(n, (margin, margin, margin), cnt_x, cnt_z, s, seed)
    return _finish("wave_tank_4m" if n == 4_000_000 else f"wave_tank_{n}", params, pos, steps, bmin, bmax)


def _draws(seed: int, stream: int, n: int) -> np.ndarray:
    return uniform01(seed, 100 + stream, n).astype(np.float64)


def block_scene(n: int, fill: float, seed: int, name: str, steps: int = 100, **overrides) -> Scene:
    """A dam-break block of n points filling the low-x fraction `fill` of a
    cubic box scaled to hold it (block spans the box's full y and z)."""
    s = lattice_spacing()
    margin = 4.0
    edge = float(s) * (n / fill) ** (1.0 / 3.0)
    cnt_z = max(1, int((edge - 2 * margin) / float(s)))
    cnt_x = max(1, int(round(fill * edge / float(s))))
    layers = -(-n // (cnt_x * cnt_z))
    lx = (cnt_x * float(s) + 2 * margin) / fill
    lz = cnt_z * float(s) + 2 * margin
    ly = max(layers * float(s) + 2 * margin, lz)
    bmin, bmax = (0.0, 0.0, 0.0), (round(lx, 1), round(ly, 1), round(lz, 1))
    params = make_params(bmin, bmax, **overrides)
    pos = lattice_block(n, (margin, margin, margin), cnt_x, cnt_z, s, seed)
    return _finish(name, params, pos, steps, bmin, bmax)


def batch_scenes(nscenes: int = 256, seed: int = 3, nmin: int = 2048, nmax: int = 65536,
                 steps: int = 500) -> list[Scene]:
    """Scenes of uneven sizes: point counts log-uniform in [nmin, nmax], fill
    fraction U[0.2, 0.6], viscosity U[0.1, 0.5], rest density U[500, 700];
    the other parameters are the dam-break set."""
    u = [_draws(seed, k, nscenes) for k in range(4)]
    out = []
    for k in range(nscenes):
        n = int(round(np.exp(np.log(nmin) + u[0][k] * (np.log(nmax) - np.log(nmin)))))
        fill = 0.2 + 0.4 * u[1][k]
        visc = float(np.float32(0.1 + 0.4 * u[2][k]))
        rest = float(np.float32(500.0 + 200.0 * u[3][k]))
        out.append(block_scene(n, fill, seed * 1000 + k, f"scene_{k}", steps, pvisc=visc, prest_dens=rest))
    return out


def fit_scenes(nscenes: int = 64, seed: int = 6, nmin: int = 8192, nmax: int = 32768,
               steps: int = 100) -> list[Scene]:
    """Scenes for the batched parameter fit: point counts log-uniform in
    [nmin, nmax], fill fraction U[0.2, 0.6], and a hidden viscosity
    U[0.1, 0.5] (in params.pvisc); every other parameter is the dam-break set."""
    u = [_draws(seed, k, nscenes) for k in range(3)]
    out = []
    for k in range(nscenes):
        n = int(round(np.exp(np.log(nmin) + u[0][k] * (np.log(nmax) - np.log(nmin)))))
        fill = 0.2 + 0.4 * u[1][k]
        visc = float(np.float32(0.1 + 0.4 * u[2][k]))
        out.append(block_scene(n, fill, seed * 1000 + k, f"fit_{k}", steps, pvisc=visc))
    return out


def concat(scenes: list) -> dict:
    """The scenes' arrays concatenated in scene order (the batched layout)."""
    return {k: np.concatenate([getattr(sc, k) for sc in scenes]) for k in ("pos", "vel", "veval", "clr")}
