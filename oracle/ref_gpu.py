"""TEST AND BASELINE INFRASTRUCTURE ONLY: the reference's own GPU kernels,
driven headless.

build_ref.sh compiles the reference's kernel module fluids4.0/fluid_kernels.cu
for sm_103a with the code-generation flags of the reference's own build
(fluids4.0/CMakeLists.txt:91: -O3 --use_fast_math --maxrregcount=32) into
_ref/fluid_kernels_sm103a.fatbin. RefGpu loads that module through the CUDA
driver API and drives it the way FluidSystem does
(fluids4.0/fluid_system.cpp):

  module, kernels, __constant__ blocks    cpp:83-118   (LoadKernel)
  launch shapes, 512 threads per block    cpp:2193-2287 (computeNumBlocks,
                                                        FluidSetupCUDA)
  buffers: fbuf + ftemp copies, grid,     cpp:181-270  (AllocateBuffer,
    scan auxiliaries                                    AllocateParticles,
                                                        AllocateGrid)
  Run, RUN_GPU_FULL                       cpp:506-524, with
    InsertParticlesCUDA 2334-2350, PrefixSumCellsCUDA 2354-2424 (the GPU
    branch), CountingSortFullCUDA 2455-2479, ComputePressureCUDA 2515-2519,
    ComputeForceCUDA 2521-2525, AdvanceCUDA 2527-2531, then
    cuCtxSynchronize; AdvanceTime adds dt to a float time.

All launches, memsets and copies go to the legacy default stream, as the
reference's do. The GL interop buffers become plain device allocations.
The FParams / FBufs blocks are restated field by field below
(fluids4.0/fluid.h:79-131, 155-192); the module's own symbol sizes are
checked against them at load, and a CPU test checks every field offset
against the reference header.

Only tests/ (GPU results of the reference vs the product) and bench.py's
baseline leg (the reference's GPU step timed on the same GPU) use this.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
FATBIN = HERE / "_ref" / "fluid_kernels_sm103a.fatbin"

F3 = C.c_float * 3
I3 = C.c_int * 3
MAX_BUF = 23
# buffer ids of fluid.h:45-67
FPOS, FVEL, FVEVAL, FFORCE, FPRESS, FCLR, FGCELL, FGNDX = range(8)
FGRID, FGRIDCNT, FGRIDOFF, FGRIDACT = 12, 13, 14, 15
FAUXARRAY1, FAUXSCAN1, FAUXARRAY2, FAUXSCAN2 = 19, 20, 21, 22
POINT_BYTES = {FPOS: 12, FVEL: 12, FVEVAL: 12, FFORCE: 12, FPRESS: 4, FCLR: 4, FGCELL: 4, FGNDX: 4}
SCAN_BLOCKSIZE = 512        # fluid_kernels.cu:20, fluid_system.cpp:22
THREADS_PER_BLOCK = 512     # FluidSetupCUDA, cpp:2272


class RefFParams(C.Structure):
    """FParams (fluid.h:155-192) with f3 = float3 and i3 = int3."""
    _fields_ = [
        ("mode", C.c_int), ("example", C.c_int), ("sim_scale", C.c_float), ("capture", C.c_bool),
        ("numThreads", C.c_int), ("numBlocks", C.c_int), ("gridThreads", C.c_int), ("gridBlocks", C.c_int),
        ("szPnts", C.c_int), ("szHash", C.c_int), ("szGrid", C.c_int),
        ("stride", C.c_int), ("pnum", C.c_int), ("chk", C.c_int),
        ("pdist", C.c_float), ("pmass", C.c_float), ("prest_dens", C.c_float), ("pintstiff", C.c_float),
        ("pradius", C.c_float), ("psmoothradius", C.c_float), ("pspacing", C.c_float), ("r2", C.c_float),
        ("pvisc", C.c_float),
        ("AL", C.c_float), ("AL2", C.c_float), ("VL", C.c_float), ("VL2", C.c_float),
        ("d2", C.c_float), ("rd2", C.c_float), ("vterm", C.c_float),
        ("poly6kern", C.c_float), ("spikykern", C.c_float), ("lapkern", C.c_float), ("gausskern", C.c_float),
        ("grid_size", C.c_float), ("grid_density", C.c_float),
        ("gridSize", F3), ("gridDelta", F3), ("gridMin", F3), ("gridMax", F3),
        ("gridRes", I3), ("gridScanMax", I3),
        ("gridSrch", C.c_int), ("gridTotal", C.c_int), ("gridAdjCnt", C.c_int), ("gridActive", C.c_int),
        ("gridAdj", C.c_int * 64),
        ("bound_slope", C.c_float), ("bound_stiff", C.c_float), ("bound_friction", C.c_float),
        ("bound_damp", C.c_float), ("bound_wall_force", C.c_float), ("bound_wall_freq", C.c_float),
        ("bound_min", F3), ("bound_max", F3), ("init_min", F3), ("init_max", F3),
        ("grav_dir", F3), ("grav_pos", F3), ("gravity", F3), ("grav_amt", C.c_float),
        ("emit_rate", F3), ("emit_pos", F3), ("emit_ang", F3), ("emit_dang", F3), ("emit_spread", F3),
        ("brickRes", I3), ("pemit", C.c_int), ("pmem", C.c_int),
    ]


class RefFBufs(C.Structure):
    """FBufs as the kernels see it (fluid.h:79-131, CUDA_KERNEL branch)."""
    _fields_ = [("mcpu", C.c_void_p * MAX_BUF), ("mgpu", C.c_uint64 * MAX_BUF),
                ("mgrsc", C.c_void_p * MAX_BUF), ("mglid", C.c_int * MAX_BUF)]


def available() -> bool:
    return FATBIN.exists()


def num_blocks(count: int, min_threads: int) -> tuple[int, int]:
    """computeNumBlocks (cpp:2193-2197): (threads, blocks)."""
    threads = min(min_threads, count)
    blocks = 1 if threads == 0 else -(-count // threads)
    return threads, blocks


def fparams_from(p, n: int) -> RefFParams:
    """The reference's parameter block for derived FlParams `p` and n points:
    the fields its kernels read (the mapping of the host build's
    ref_set_params) plus what FluidSetupCUDA records (cpp:2249-2287)."""
    f = RefFParams()
    for k in ("sim_scale", "pmass", "prest_dens", "pintstiff", "pradius", "psmoothradius", "r2", "pvisc",
              "AL", "AL2", "VL", "VL2", "d2", "rd2", "vterm", "poly6kern", "spikykern", "lapkern",
              "grid_size", "grid_density", "gridSrch", "gridTotal", "gridAdjCnt", "pdist",
              "bound_slope", "bound_stiff", "bound_friction", "bound_damp", "bound_wall_force",
              "bound_wall_freq", "grav_amt"):
        setattr(f, k, getattr(p, k))
    for k in ("gridSize", "gridDelta", "gridMin", "gridMax", "gridRes", "gridScanMax",
              "bound_min", "bound_max", "gravity", "grav_dir"):
        src, dst = getattr(p, k), getattr(f, k)
        for i in range(3):
            dst[i] = src[i]
    if p.gridAdjCnt > 64:
        raise ValueError("the reference's FParams holds at most 64 adjacency entries")
    for c in range(p.gridAdjCnt):
        f.gridAdj[c] = p.gridAdj[c]
    f.pnum = n
    f.numThreads, f.numBlocks = num_blocks(n, THREADS_PER_BLOCK)
    f.gridThreads, f.gridBlocks = num_blocks(p.gridTotal, THREADS_PER_BLOCK)
    f.szPnts = f.numBlocks * f.numThreads
    f.szGrid = f.gridBlocks * f.gridThreads
    f.mode = 5   # RUN_GPU_FULL (fluid_system.h:34)
    return f


_cu = None


def cu():
    """libcuda (driver API) with the argument types of the calls used here."""
    global _cu
    if _cu is None:
        lib = C.CDLL("libcuda.so.1")
        vp, u64, sz = C.c_void_p, C.c_uint64, C.c_size_t
        lib.cuGetErrorString.argtypes = [C.c_int, C.POINTER(C.c_char_p)]
        lib.cuModuleLoad.argtypes = [C.POINTER(vp), C.c_char_p]
        lib.cuModuleUnload.argtypes = [vp]
        lib.cuModuleGetFunction.argtypes = [C.POINTER(vp), vp, C.c_char_p]
        lib.cuModuleGetGlobal_v2.argtypes = [C.POINTER(u64), C.POINTER(sz), vp, C.c_char_p]
        lib.cuMemcpyHtoD_v2.argtypes = [u64, vp, sz]
        lib.cuMemcpyDtoH_v2.argtypes = [vp, u64, sz]
        lib.cuMemcpyDtoD_v2.argtypes = [u64, u64, sz]
        lib.cuMemsetD8_v2.argtypes = [u64, C.c_ubyte, sz]
        lib.cuLaunchKernel.argtypes = [vp, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                       C.c_uint, vp, C.POINTER(vp), C.POINTER(vp)]
        lib.cuCtxSynchronize.argtypes = []
        _cu = lib
    return _cu


def check(what: str, r: int) -> None:
    if r != 0:
        s = C.c_char_p()
        cu().cuGetErrorString(r, C.byref(s))
        raise RuntimeError(f"{what}: CUDA driver error {r} ({s.value.decode() if s.value else 'unknown'})")


class RefGpu:
    """One FluidSystem's GPU state and phases, over n points."""

    KERNELS = ("insertParticles", "prefixSum", "prefixFixup", "countingSortFull", "computePressure",
               "computeForce", "advanceParticles")

    def __init__(self, params, n: int):
        import torch
        if not FATBIN.exists():
            raise FileNotFoundError(f"{FATBIN.name} is not built (the reference tree was absent at build time)")
        if n <= 0:
            raise ValueError("RefGpu needs at least one point")
        torch.zeros(1, device="cuda")   # the primary context, current on this thread
        torch.cuda.synchronize()
        self.torch = torch
        self.n = n
        self.params = params
        self.dt = float(params.dt)
        self.ss = float(params.sim_scale)
        lib = cu()
        self.mod = C.c_void_p()
        check("cuModuleLoad", lib.cuModuleLoad(C.byref(self.mod), str(FATBIN).encode()))
        self.fn = {}
        for name in self.KERNELS:
            f = C.c_void_p()
            check(f"cuModuleGetFunction {name}", lib.cuModuleGetFunction(C.byref(f), self.mod, name.encode()))
            self.fn[name] = f
        self.sym = {}
        for name, want in (("fparam", C.sizeof(RefFParams)), ("fbuf", C.sizeof(RefFBufs)),
                           ("ftemp", C.sizeof(RefFBufs))):
            d, size = C.c_uint64(), C.c_size_t()
            check(f"cuModuleGetGlobal {name}", lib.cuModuleGetGlobal_v2(C.byref(d), C.byref(size), self.mod,
                                                                        name.encode()))
            if size.value != want:
                raise RuntimeError(f"module symbol {name} is {size.value} bytes, the restated block {want}")
            self.sym[name] = d.value

        self.fp = fparams_from(params, n)
        self.threads, self.blocks = self.fp.numThreads, self.fp.numBlocks
        gt = params.gridTotal
        self.gt = gt
        bs = SCAN_BLOCKSIZE << 1
        self.ne1 = gt
        self.ne2 = gt // bs + 1
        self.ne3 = self.ne2 // bs + 1
        if self.ne1 > SCAN_BLOCKSIZE ** 3:
            raise ValueError("grid exceeds the reference scan's three levels")

        self.mem = {}
        fb, ft = RefFBufs(), RefFBufs()

        def alloc(key, nbytes):
            t = torch.zeros(max(int(nbytes), 16), dtype=torch.uint8, device="cuda")
            self.mem[key] = t
            return t.data_ptr()

        for b, e in POINT_BYTES.items():
            fb.mgpu[b] = alloc(b, e * n)
            ft.mgpu[b] = alloc(("temp", b), e * n)
        for b, count in ((FGRID, self.fp.szPnts), (FGRIDCNT, self.fp.szGrid), (FGRIDOFF, self.fp.szGrid),
                         (FGRIDACT, self.fp.szGrid), (FAUXARRAY1, self.ne2), (FAUXSCAN1, self.ne2),
                         (FAUXARRAY2, self.ne3), (FAUXSCAN2, self.ne3)):
            fb.mgpu[b] = alloc(b, 4 * count)
        self.fb, self.ft = fb, ft
        torch.cuda.synchronize()
        check("cuMemcpyHtoD fbuf", lib.cuMemcpyHtoD_v2(self.sym["fbuf"], C.addressof(fb), C.sizeof(fb)))
        check("cuMemcpyHtoD ftemp", lib.cuMemcpyHtoD_v2(self.sym["ftemp"], C.addressof(ft), C.sizeof(ft)))
        check("cuMemcpyHtoD fparam", lib.cuMemcpyHtoD_v2(self.sym["fparam"], C.addressof(self.fp),
                                                         C.sizeof(self.fp)))

    # -- buffers ---------------------------------------------------------------
    def ptr(self, b) -> int:
        return self.mem[b].data_ptr()

    def set_state(self, pos, vel=None, veval=None, clr=None) -> None:
        """TransferToCUDA (cpp:2312-2321): the point fields from host arrays;
        force and density start at zero."""
        n = self.n
        lib = cu()
        for b, a, dt in ((FPOS, pos, np.float32), (FVEL, vel, np.float32), (FVEVAL, veval, np.float32),
                         (FCLR, clr, np.uint32)):
            if a is None:
                self.mem[b].zero_()
                continue
            h = np.ascontiguousarray(a, dtype=dt).reshape(n, -1)
            if h.nbytes != POINT_BYTES[b] * n:
                raise ValueError(f"buffer {b}: {h.nbytes} bytes for {n} points")
            self.torch.cuda.synchronize()
            check("cuMemcpyHtoD", lib.cuMemcpyHtoD_v2(self.ptr(b), h.ctypes.data, h.nbytes))
        self.mem[FFORCE].zero_()
        self.mem[FPRESS].zero_()
        self.torch.cuda.synchronize()

    def put(self, b, a) -> None:
        """Overwrite point buffer b (slot order) from a host array."""
        h = np.ascontiguousarray(a, dtype=np.float32 if b in (FPOS, FVEL, FVEVAL, FFORCE, FPRESS) else np.uint32)
        if h.nbytes != POINT_BYTES[b] * self.n:
            raise ValueError(f"buffer {b}: {h.nbytes} bytes for {self.n} points")
        self.torch.cuda.synchronize()
        check("cuMemcpyHtoD", cu().cuMemcpyHtoD_v2(self.ptr(b), h.ctypes.data, h.nbytes))

    def get(self, b) -> np.ndarray:
        """A buffer's current contents (point fields n long, grid fields
        gridTotal long)."""
        if b in POINT_BYTES:
            shape, dt = ((self.n, 3), np.float32) if POINT_BYTES[b] == 12 else \
                ((self.n,), np.float32 if b == FPRESS else np.uint32)
        elif b in (FGRIDCNT, FGRIDOFF):
            shape, dt = (self.gt,), np.uint32
        elif b == FGRID:
            shape, dt = (self.n,), np.uint32
        else:
            raise ValueError(f"buffer {b}")
        out = np.empty(shape, dt)
        self.torch.cuda.synchronize()
        check("cuMemcpyDtoH", cu().cuMemcpyDtoH_v2(out.ctypes.data, self.ptr(b), out.nbytes))
        return out

    # -- phases ----------------------------------------------------------------
    def _launch(self, name, grid, block, *args):
        argv = (C.c_void_p * len(args))(*[C.addressof(a) for a in args])
        check(name, cu().cuLaunchKernel(self.fn[name], grid, 1, 1, block, 1, 1, 0, None, argv, None))

    def insert(self) -> None:
        lib = cu()
        check("cuMemsetD8 gridcnt", lib.cuMemsetD8_v2(self.ptr(FGRIDCNT), 0, self.gt * 4))
        check("cuMemsetD8 gridoff", lib.cuMemsetD8_v2(self.ptr(FGRIDOFF), 0, self.gt * 4))
        self._launch("insertParticles", self.blocks, self.threads, C.c_int(self.n))

    def prefix_sum(self, zero_offsets: int = 1) -> None:
        u = C.c_uint64
        a1, s1 = u(self.ptr(FGRIDCNT)), u(self.ptr(FGRIDOFF))
        a2, s2 = u(self.ptr(FAUXARRAY1)), u(self.ptr(FAUXSCAN1))
        a3, s3 = u(self.ptr(FAUXARRAY2)), u(self.ptr(FAUXSCAN2))
        n1, n2, n3 = C.c_int(self.ne1), C.c_int(self.ne2), C.c_int(self.ne3)
        zon = C.c_int(1)
        self._launch("prefixSum", self.ne2, SCAN_BLOCKSIZE, a1, s1, a2, n1, C.c_int(zero_offsets))
        self._launch("prefixSum", self.ne3, SCAN_BLOCKSIZE, a2, s2, a3, n2, zon)
        if self.ne3 > 1:
            self._launch("prefixSum", 1, SCAN_BLOCKSIZE, a3, s3, u(0), n3, zon)
            self._launch("prefixFixup", self.ne3, SCAN_BLOCKSIZE, s2, s3, n2)
        self._launch("prefixFixup", self.ne2, SCAN_BLOCKSIZE, s1, s2, n1)

    def counting_sort(self) -> None:
        lib = cu()
        for b, e in POINT_BYTES.items():
            check("cuMemcpyDtoD", lib.cuMemcpyDtoD_v2(self.ptr(("temp", b)), self.ptr(b), e * self.n))
        self._launch("countingSortFull", self.blocks, self.threads, C.c_int(self.n))

    def pressure(self) -> None:
        self._launch("computePressure", self.blocks, self.threads, C.c_int(self.n))

    def force(self) -> None:
        self._launch("computeForce", self.blocks, self.threads, C.c_int(self.n))

    def advance(self, time: float) -> None:
        self._launch("advanceParticles", self.blocks, self.threads, C.c_float(time), C.c_float(self.dt),
                     C.c_float(self.ss), C.c_int(self.n))

    def run(self, time: float) -> float:
        """One Run (RUN_GPU_FULL) at `time`; returns time + dt in float."""
        self.insert()
        self.prefix_sum(1)
        self.counting_sort()
        self.pressure()
        self.force()
        self.advance(time)
        check("cuCtxSynchronize", cu().cuCtxSynchronize())
        return float(np.float32(time) + np.float32(self.dt))

    def close(self) -> None:
        if self.mod:
            self.torch.cuda.synchronize()
            cu().cuModuleUnload(self.mod)
            self.mod = None
        self.mem.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
