"""TEST INFRASTRUCTURE ONLY: Python access to the CPU oracle.

Two host libraries, both built from C/C++ in this directory:
  _build/libfluids_oracle.so  -- fluids_oracle.c, the C restatement (FP32 in
                                  the reference's operation order + FP64)
  _ref/libfluids_ref.so       -- the reference's own fluids4.0/fluid_kernels.cu
                                  compiled for the host (only where the
                                  reference tree was present at build time)

Only tests/, bench.py's CPU arm and __graft_entry__.smoke() import this
module, and only to check or time the CUDA path -- never as the product.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from dataclasses import dataclass
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "_build" / "libfluids_oracle.so"
REF_LIB = HERE / "_ref" / "libfluids_ref.so"

_orc = None
_ref = None


def build(ref: bool = True) -> None:
    subprocess.run(["bash", str(HERE / "build_oracle.sh")], check=True)
    if ref:
        subprocess.run(["bash", str(HERE / "build_ref.sh")], check=True)


def params_from_bytes(raw) -> "FlParams":
    """FlParams from its exact bytes (as stored in the golden fixtures)."""
    from fluids3_gb300.params import FlParams
    raw = bytes(bytearray(raw))
    p = FlParams()
    if len(raw) != C.sizeof(FlParams):
        raise ValueError(f"params blob is {len(raw)} bytes, FlParams is {C.sizeof(FlParams)}")
    C.memmove(C.byref(p), raw, len(raw))
    return p


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def orc():
    global _orc
    if _orc is None:
        if not ORACLE_LIB.exists():
            build(ref=False)
        _orc = C.CDLL(str(ORACLE_LIB))
        vp, i, f = C.c_void_p, C.c_int, C.c_float
        _orc.orc_insert.argtypes = [vp, i, vp, vp, vp, vp]
        _orc.orc_prefix_sum.argtypes = [i, vp, vp]
        _orc.orc_counting_sort.argtypes = [vp, i, vp] + [vp] * 16
        _orc.orc_density.argtypes = [vp, i, vp, vp, vp, vp, vp, i]
        _orc.orc_force.argtypes = [vp, i, vp, vp, vp, vp, vp, vp, vp, i]
        _orc.orc_advance.argtypes = [vp, i, f, f, f, vp, vp, vp, vp, vp, i]
        _orc.orc_density_f64.argtypes = [vp, i, vp, vp, vp, vp, vp, i]
        _orc.orc_force_f64.argtypes = [vp, i, vp, vp, vp, vp, vp, vp, vp, vp, i]
        _orc.orc_run.argtypes = [vp, i, i, C.POINTER(f), i] + [vp] * 18
        _orc.orc_density_at.argtypes = [vp, i, vp, vp, vp, vp, vp, vp, i]
        _orc.orc_force_at.argtypes = [vp, i, vp, vp, vp, vp, vp, vp, vp, vp, i]
        _orc.orc_density_f64_at.argtypes = [vp, i, vp, vp, vp, vp, vp, vp, i]
        _orc.orc_force_f64_at.argtypes = [vp, i, vp, vp, vp, vp, vp, vp, vp, vp, vp, i]
    return _orc


def ref_available() -> bool:
    return REF_LIB.exists()


def ref():
    global _ref
    if _ref is None:
        if not REF_LIB.exists():
            raise FileNotFoundError("oracle/_ref/libfluids_ref.so is not built (reference tree absent)")
        _ref = C.CDLL(str(REF_LIB))
        vp, i, f = C.c_void_p, C.c_int, C.c_float
        _ref.ref_set_params.argtypes = [vp]
        _ref.ref_set_params.restype = i
        _ref.ref_bind.argtypes = [i, vp]
        _ref.ref_insert.argtypes = [i]
        _ref.ref_prefix_sum.argtypes = [i]
        _ref.ref_counting_sort.argtypes = [i]
        _ref.ref_compute_pressure.argtypes = [i, i]
        _ref.ref_compute_force.argtypes = [i, i]
        _ref.ref_advance.argtypes = [f, f, f, i, i]
        _ref.ref_run.argtypes = [i, i, C.POINTER(f), f, i]
    return _ref


# ---------------------------------------------------------------------------
@dataclass
class State:
    """Host SPH state in fluid.h layout."""
    pos: np.ndarray
    vel: np.ndarray
    veval: np.ndarray
    force: np.ndarray
    press: np.ndarray
    clr: np.ndarray
    gcell: np.ndarray
    gndx: np.ndarray
    cnt: np.ndarray      # C + 1 (entry C: out-of-range bin)
    off: np.ndarray      # C + 1

    @staticmethod
    def new(params, pos, vel=None, veval=None, clr=None) -> "State":
        n = pos.shape[0]
        c = params.gridTotal + 1
        z3 = lambda a: np.zeros((n, 3), np.float32) if a is None else np.array(a, np.float32).reshape(n, 3)
        return State(pos=np.array(pos, np.float32).reshape(n, 3), vel=z3(vel), veval=z3(veval),
                     force=np.zeros((n, 3), np.float32), press=np.zeros(n, np.float32),
                     clr=np.zeros(n, np.uint32) if clr is None else np.array(clr, np.uint32),
                     gcell=np.zeros(n, np.uint32), gndx=np.zeros(n, np.uint32),
                     cnt=np.zeros(c, np.uint32), off=np.zeros(c, np.uint32))

    def copy(self) -> "State":
        return State(**{k: v.copy() for k, v in self.__dict__.items()})

    @property
    def n(self) -> int:
        return self.pos.shape[0]


def insert(params, st: State) -> None:
    orc().orc_insert(C.byref(params), st.n, _p(st.pos), _p(st.gcell), _p(st.gndx), _p(st.cnt))


def prefix_sum(params, st: State) -> None:
    orc().orc_prefix_sum(params.gridTotal + 1, _p(st.cnt), _p(st.off))


def counting_sort(params, st: State) -> None:
    out = State.new(params, st.pos)
    orc().orc_counting_sort(C.byref(params), st.n, _p(st.off),
                            *[_p(a) for a in (st.pos, st.vel, st.veval, st.force, st.press, st.clr, st.gcell, st.gndx)],
                            *[_p(a) for a in (out.pos, out.vel, out.veval, out.force, out.press, out.clr, out.gcell, out.gndx)])
    for k in ("pos", "vel", "veval", "force", "press", "clr", "gcell", "gndx"):
        setattr(st, k, getattr(out, k))


def density(params, st: State, threads: int = 1) -> None:
    orc().orc_density(C.byref(params), st.n, _p(st.pos), _p(st.gcell), _p(st.off), _p(st.cnt),
                      _p(st.press), threads)


def force(params, st: State, threads: int = 1) -> None:
    orc().orc_force(C.byref(params), st.n, _p(st.pos), _p(st.veval), _p(st.press), _p(st.gcell),
                    _p(st.off), _p(st.cnt), _p(st.force), threads)


def advance(params, st: State, time: float, dt: float, ss: float, threads: int = 1) -> None:
    orc().orc_advance(C.byref(params), st.n, C.c_float(time), C.c_float(dt), C.c_float(ss),
                      _p(st.gcell), _p(st.force), _p(st.pos), _p(st.vel), _p(st.veval), threads)


def density_f64(params, pos, gcell, off, cnt, threads: int = 1) -> np.ndarray:
    out = np.zeros(pos.shape[0], np.float64)
    orc().orc_density_f64(C.byref(params), pos.shape[0], _p(pos), _p(gcell), _p(off), _p(cnt),
                          _p(out), threads)
    return out


def force_f64(params, pos, veval, press, gcell, off, cnt, threads: int = 1):
    """(force, scale): FP64 force and, per point, the sum of its pair-term magnitudes."""
    out = np.zeros((pos.shape[0], 3), np.float64)
    scale = np.zeros(pos.shape[0], np.float64)
    orc().orc_force_f64(C.byref(params), pos.shape[0], _p(pos), _p(veval), _p(press), _p(gcell),
                        _p(off), _p(cnt), _p(out), _p(scale), threads)
    return out, scale


def _idx(idx):
    return np.ascontiguousarray(idx, np.uint32)


def density_at(params, st: State, idx, threads: int = 1) -> np.ndarray:
    """FP32 densities of the sorted slots `idx` of a sorted state (every slot
    is still a neighbour): a sample of a state too large to evaluate whole."""
    idx = _idx(idx)
    out = np.zeros(idx.size, np.float32)
    orc().orc_density_at(C.byref(params), idx.size, _p(idx), _p(st.pos), _p(st.gcell), _p(st.off), _p(st.cnt),
                         _p(out), threads)
    return out


def force_at(params, pos, veval, press, gcell, off, cnt, idx, threads: int = 1) -> np.ndarray:
    """FP32 forces of the sorted slots `idx` from the given densities."""
    idx = _idx(idx)
    out = np.zeros((idx.size, 3), np.float32)
    orc().orc_force_at(C.byref(params), idx.size, _p(idx), _p(pos), _p(veval), _p(press), _p(gcell), _p(off),
                       _p(cnt), _p(out), threads)
    return out


def density_f64_at(params, pos, gcell, off, cnt, idx, threads: int = 1) -> np.ndarray:
    idx = _idx(idx)
    out = np.zeros(idx.size, np.float64)
    orc().orc_density_f64_at(C.byref(params), idx.size, _p(idx), _p(pos), _p(gcell), _p(off), _p(cnt), _p(out),
                             threads)
    return out


def force_f64_at(params, pos, veval, press, gcell, off, cnt, idx, threads: int = 1):
    """(force, scale) in FP64 at the sorted slots `idx`, from the given densities."""
    idx = _idx(idx)
    out = np.zeros((idx.size, 3), np.float64)
    scale = np.zeros(idx.size, np.float64)
    orc().orc_force_f64_at(C.byref(params), idx.size, _p(idx), _p(pos), _p(veval), _p(press), _p(gcell),
                           _p(off), _p(cnt), _p(out), _p(scale), threads)
    return out, scale


def step(params, st: State, time: float, threads: int = 1) -> float:
    """One Run step (RUN_GPU_FULL order); returns the new time."""
    insert(params, st)
    prefix_sum(params, st)
    counting_sort(params, st)
    density(params, st, threads)
    force(params, st, threads)
    advance(params, st, time, params.dt, params.sim_scale, threads)
    return float(np.float32(np.float32(time) + np.float32(params.dt)))


def run(params, st: State, steps: int, time: float, threads: int = 1) -> float:
    """`steps` steps in C (no Python per phase); returns the new time."""
    t = C.c_float(time)
    s2 = State.new(params, st.pos)
    orc().orc_run(C.byref(params), st.n, steps, C.byref(t), threads,
                  *[_p(a) for a in (st.pos, st.vel, st.veval, st.force, st.press, st.clr, st.gcell, st.gndx)],
                  *[_p(a) for a in (s2.pos, s2.vel, s2.veval, s2.force, s2.press, s2.clr, s2.gcell, s2.gndx)],
                  _p(st.cnt), _p(st.off))
    return float(t.value)


# ---------------------------------------------------------------------------
class RefKernels:
    """The reference kernels run on the host (tier 1). Buffers are numpy
    arrays in fluid.h layout bound into the kernels' fbuf table."""

    IDS = dict(pos=0, vel=1, veval=2, force=3, press=4, clr=5, gcell=6, gndx=7,
               grid=12, gridcnt=13, gridoff=14)

    def __init__(self, params, pos, vel=None, veval=None, clr=None):
        self.lib = ref()
        self.params = params
        if self.lib.ref_set_params(C.byref(params)) != 0:
            raise ValueError("reference FParams holds at most 64 adjacency entries")
        n = pos.shape[0]
        self.n = n
        z3 = lambda a: np.zeros((n, 3), np.float32) if a is None else np.array(a, np.float32).reshape(n, 3)
        self.buf = dict(pos=np.array(pos, np.float32).reshape(n, 3), vel=z3(vel), veval=z3(veval),
                        force=np.zeros((n, 3), np.float32), press=np.zeros(n, np.float32),
                        clr=np.zeros(n, np.uint32) if clr is None else np.array(clr, np.uint32),
                        gcell=np.zeros(n, np.uint32), gndx=np.zeros(n, np.uint32),
                        grid=np.zeros(n, np.uint32),
                        gridcnt=np.zeros(params.gridTotal, np.uint32),
                        gridoff=np.zeros(params.gridTotal, np.uint32))
        for k, a in self.buf.items():
            self.lib.ref_bind(self.IDS[k], _p(a))

    def rebind(self):
        self.lib.ref_set_params(C.byref(self.params))
        for k, a in self.buf.items():
            self.lib.ref_bind(self.IDS[k], _p(a))

    def insert(self):
        self.rebind()
        self.lib.ref_insert(self.n)

    def prefix_sum(self, zero_offsets=1):
        self.rebind()
        self.lib.ref_prefix_sum(zero_offsets)

    def counting_sort(self):
        self.rebind()
        self.lib.ref_counting_sort(self.n)

    def pressure(self, threads=1):
        self.rebind()
        self.lib.ref_compute_pressure(self.n, threads)

    def force(self, threads=1):
        self.rebind()
        self.lib.ref_compute_force(self.n, threads)

    def advance(self, time, dt, ss, threads=1):
        self.rebind()
        self.lib.ref_advance(C.c_float(time), C.c_float(dt), C.c_float(ss), self.n, threads)

    def sample(self, res, bmin, bmax, scalar):
        """sampleParticles over the current sorted state; (z, y, x) array."""
        self.rebind()
        if not getattr(self.lib, "_sample_ready", False):
            self.lib.ref_sample_particles.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p,
                                                      C.c_void_p, C.c_int, C.c_float]
            self.lib._sample_ready = True
        out = np.zeros((res[2], res[1], res[0]), np.float32)
        self.lib.ref_sample_particles(_p(out), res[0], res[1], res[2], _p(np.array(bmin, np.float32)),
                                      _p(np.array(bmax, np.float32)), self.n, C.c_float(scalar))
        return out

    def run(self, steps, time, threads=1) -> float:
        self.rebind()
        t = C.c_float(time)
        self.lib.ref_run(self.n, steps, C.byref(t), C.c_float(self.params.dt), threads)
        return float(t.value)


# ---------------------------------------------------------------------------
# FP64 adjoint model (adjoint64.c): the step with its integer structure
# frozen, evaluated in double, and its hand-written reverse pass.

@dataclass
class Frozen:
    """The integer structure of `steps` FP32 oracle steps: per step the sort
    permutation (slot -> pre-sort index), the in-range flags and the pairs
    (CSR over sorted slots), the time, and the state before the step."""
    n: int
    steps: int
    perm: np.ndarray     # (T, n) uint32
    inr: np.ndarray      # (T, n) uint8
    poff: np.ndarray     # (T, n + 1) uint32
    pnbr: np.ndarray     # concatenated uint32
    pbase: np.ndarray    # (T + 1,) uint64 offsets of each step's pairs in pnbr
    time: np.ndarray     # (T,) float64
    states: np.ndarray   # (T, 3, n, 3) float64: x, v, e before each step


def _adj_lib():
    lib = orc()
    if not getattr(lib, "_adj_ready", False):
        vp, i = C.c_void_p, C.c_int
        lib.orc_pairs.argtypes = [vp, i, vp, vp, vp, vp, vp, vp]
        lib.adj64_forward.argtypes = [vp, vp, i, i] + [vp] * 10 + [i]
        lib.adj64_backward.argtypes = [vp, vp, i, i] + [vp] * 14
        lib._adj_ready = True
    return lib


def frozen_run(params, st: State, steps: int, time: float, states=None, times=None) -> Frozen:
    """Run `steps` FP32 oracle steps on `st` (in place) and record their structure.
    With `states` (per step a (pos, vel, veval) float32 triple, e.g. read back
    from another implementation) each step starts from the given state, and
    `times` (per step) replaces the oracle's own clock."""
    lib = _adj_lib()
    n = st.n
    perm = np.zeros((steps, n), np.uint32)
    inr = np.zeros((steps, n), np.uint8)
    poff = np.zeros((steps, n + 1), np.uint32)
    nbrs, times_out = [], np.zeros(steps, np.float64)
    C_ = params.gridTotal
    given = states
    states = np.zeros((steps, 3, n, 3), np.float64)
    for t in range(steps):
        if given is not None:
            st.pos, st.vel, st.veval = (np.array(a, np.float32).reshape(n, 3) for a in given[t])
        if times is not None:
            time = float(times[t])
        states[t, 0], states[t, 1], states[t, 2] = st.pos, st.vel, st.veval
        times_out[t] = time
        insert(params, st)
        prefix_sum(params, st)
        cell = np.where(st.gcell == 0xFFFFFFFF, C_, st.gcell).astype(np.int64)
        slot = st.off[cell].astype(np.int64) + st.gndx
        perm[t, slot] = np.arange(n, dtype=np.uint32)
        counting_sort(params, st)
        inr[t] = (st.gcell != 0xFFFFFFFF)
        lib.orc_pairs(C.byref(params), n, _p(st.pos), _p(st.gcell), _p(st.off), _p(st.cnt),
                      _p(poff[t]), None)
        nbr = np.zeros(int(poff[t, n]), np.uint32)
        lib.orc_pairs(C.byref(params), n, _p(st.pos), _p(st.gcell), _p(st.off), _p(st.cnt),
                      _p(poff[t]), _p(nbr))
        nbrs.append(nbr)
        density(params, st)
        force(params, st)
        advance(params, st, time, params.dt, params.sim_scale)
        time = float(np.float32(np.float32(time) + np.float32(params.dt)))
    pbase = np.zeros(steps + 1, np.uint64)
    pbase[1:] = np.cumsum([a.size for a in nbrs])
    pnbr = np.concatenate(nbrs) if nbrs else np.zeros(0, np.uint32)
    return Frozen(n=n, steps=steps, perm=perm, inr=inr, poff=poff, pnbr=pnbr, pbase=pbase,
                  time=times_out, states=states)


def _theta(theta):
    return None if theta is None else np.ascontiguousarray(theta, np.float64)


def adj64_forward(params, fz: Frozen, x0, v0, e0, theta=None, masks=None, mask_mode: int = 0):
    """The FP64 frozen-structure forward from (x0, v0, e0): the final (x, v, e).
    theta = (visc, rest density, IntStiff) overrides the parameter block.
    masks ((T, n) uint8) with mask_mode 1 records the wall and clamp decisions
    of every step, with mask_mode 2 reuses them (decisions frozen too)."""
    x, v, e = (np.array(a, np.float64).reshape(fz.n, 3) for a in (x0, v0, e0))
    th = _theta(theta)
    if masks is not None:
        assert masks.dtype == np.uint8 and masks.shape == (fz.steps, fz.n) and masks.flags.c_contiguous
    _adj_lib().adj64_forward(C.byref(params), _p(th), fz.n, fz.steps, _p(fz.perm), _p(fz.inr),
                             _p(fz.poff), _p(fz.pnbr), _p(fz.pbase), _p(fz.time), _p(x), _p(v), _p(e),
                             _p(masks), int(mask_mode if masks is not None else 0))
    return x, v, e


def adj64_backward(params, fz: Frozen, xb, vb, eb, x0=None, v0=None, e0=None, theta=None,
                   use_states: bool = True):
    """dL/d(x0, v0, e0) and dL/d(visc, rest density, IntStiff) from dL/d(final
    x, v, e). With use_states the model is linearised around the recorded
    (FP32) states; else around its own FP64 forward from (x0, v0, e0)."""
    n = fz.n
    xb, vb, eb = (np.array(a, np.float64).reshape(n, 3) for a in (xb, vb, eb))
    g = np.zeros(3, np.float64)
    th = _theta(theta)
    if use_states:
        st = np.ascontiguousarray(fz.states)
        z = fz.states[0] if fz.steps else np.zeros((3, n, 3))
        x0, v0, e0 = z[0], z[1], z[2]
    else:
        st = None
    x0, v0, e0 = (np.ascontiguousarray(a, np.float64).reshape(n, 3) for a in (x0, v0, e0))
    _adj_lib().adj64_backward(C.byref(params), _p(th), n, fz.steps, _p(fz.perm), _p(fz.inr), _p(fz.poff),
                              _p(fz.pnbr), _p(fz.pbase), _p(fz.time), _p(st), _p(x0), _p(v0), _p(e0),
                              _p(xb), _p(vb), _p(eb), _p(g))
    return xb, vb, eb, g


def sample_volume(params, pos, off, cnt, res, bmin, bmax, scalar):
    """sampleParticles on a sorted state (pos in slot order, off/cnt per
    cell); returns a (res_z, res_y, res_x) float32 array."""
    lib = orc()
    if not getattr(lib, "_sample_ready", False):
        vp = C.c_void_p
        lib.orc_sample_volume.argtypes = [vp] * 7 + [C.c_float, C.c_float, C.c_float, vp]
        lib._sample_ready = True
    sr = np.float32(params.psmoothradius)
    gk = np.float32(1.0) / np.float32(_libm_powf(np.float32(3.141592) * np.float32(2.0) * sr * sr, 1.5))
    h2 = np.float32(2.0 * float(np.float32(params.r2)) / 8.0)
    r = np.array(res, np.int32)
    out = np.zeros((res[2], res[1], res[0]), np.float32)
    pos = np.ascontiguousarray(pos, np.float32)
    off = np.ascontiguousarray(off, np.uint32)
    cnt = np.ascontiguousarray(cnt, np.uint32)
    lib.orc_sample_volume(C.byref(params), _p(pos), _p(off), _p(cnt), _p(r), _p(np.array(bmin, np.float32)),
                          _p(np.array(bmax, np.float32)), C.c_float(scalar), C.c_float(gk), C.c_float(h2), _p(out))
    return out


def _libm_powf(x, y):
    libm = C.CDLL("libm.so.6")
    libm.powf.restype = C.c_float
    libm.powf.argtypes = [C.c_float, C.c_float]
    return np.float32(libm.powf(C.c_float(x), C.c_float(y)))
