#!/usr/bin/env python3
"""Throughput of the SPH time step on GB300: Mparticle-steps/s.

Workload (N=1): the 4,000,000-point wave tank -- a jittered lattice filling
the low-x 40% of a ~330-unit box, dam-break parameters (h = 0.01 m, cell 2h,
gridSrch 2), X- wall forcing at frequency 0.2 and amplitude 0.3. One step
is one full Run: insert, scan, index scatter, canonical cell sort (and the
crowded-cell sort), gather, density, force + advance (eight kernels; the
neighbour passes per --passes, by default switching from the per-point to
the cell-task passes once a cell crowds past 512 points).

  value   device-timed throughput, state resident in HBM, graph replay of
          exactly K steps between CUDA events on the system stream, run as
          segments of at most --segment (50) steps that each restart from the
          post-warm-up state (device checkpoint restore inside the timed
          interval). With these parameters the fluid clumps: by step 300 the
          median point shares its cell with ~3,000 others (max ~18,000), and
          the reference's O(points x cell occupancy) search degenerates for
          any implementation; segments keep every timed step in the
          configured regime.
  e2e     the same metric through the public C ABI with host buffers: per
          step one fl_run_from_host call -- the step's inputs uploaded from
          pinned host memory (all but the positions on a copy engine during
          the step's first kernels), the step, and the new positions written
          into pinned host memory by the force pass itself
  roofline  the dominant kernel's algorithmic bytes per launch / its mean
          launch time (per-phase CUDA events over a second K-step region)
  cpu_baseline  the reference's CPU path (the reference kernels built for the
          host where available, else the oracle port) on a bounded sample
  reference_gpu  the reference's own GPU kernels (its kernel module built for
          sm_103a with its build's flags, driven as its Run drives them) on
          the same workload, state and segment protocol as value

  long_continuous  --long-steps continuous steps from the warm state, timed
          per --long-chunk-step run, with the largest cell after each
  batched  256 scenes stepped as one batched system vs one at a time
  adjoint  adjoint/forward time per step: the differentiated 65,536-point
          rollout (checkpointed and every-step tapes, their device memory)
          and the 4M wave tank
  fit     the 64-scene batched parameter fit: viscosity recovery error,
          device memory of a 100-step tape with and without checkpointing

--impl reference prints the reference arm instead (CPU, all host threads).
Multi-GPU (torchrun): every rank steps its own replica (no exchange), the
slowest rank's time sets the aggregate.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mparticle-steps/s"
# Algorithmic bytes per point per phase of the step: each input read once,
# each output written once (the per-unit figures of the step's functions;
# grid terms per cell are added separately): 256 B per point in all.
ALGO_BYTES = {
    "insert": 20,          # R pos 12, W cell + rank 8
    "scan": 0,             # per cell: R 4, W 4 (+ clear 4) -> 12 B/cell
    "sort": 92,            # R pos, vel, veval, clr, gcell, gndx; W pos, vel, veval, clr, gcell
    "density": 16,         # R pos 12, W density 4
    "force_advance": 128,  # force 40 (R pos, veval, density; W F) + advance 88
}
# Bytes per point this implementation moves beyond those: the index scatter
# between the counting atomics and the cell sort (R cell + rank, W index).
IMPL_BYTES = {"scatter": 12}
KERNELS_PER_STEP = 8   # insert, scan, scatter, cell sort, crowded-cell sort, gather, density, force+advance


def parse():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=4_000_000, help="points in the wave tank")
    ap.add_argument("--segment", type=int, default=50,
                    help="timed steps run as rollouts of at most this many steps from the warm state")
    ap.add_argument("--long-steps", type=int, default=300,
                    help="also time this many continuous steps from the warm state, per --long-chunk-step run")
    ap.add_argument("--long-chunk", type=int, default=100, help="steps per timed run of --long-steps")
    ap.add_argument("--e2e-steps", type=int, default=None, help="steps in the e2e region (default: min(K, 20))")
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="CPU baseline sample budget")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ref-gpu", action="store_true",
                    help="skip timing the reference's own GPU kernels on the same workload")
    ap.add_argument("--batch-scenes", type=int, default=256,
                    help="scenes in the batched-vs-one-at-a-time comparison (0 skips it)")
    ap.add_argument("--batch-passes", choices=["cells", "points", "pairs", "auto"], default="auto",
                    help="neighbour passes of both arms of the batched comparison")
    ap.add_argument("--batch-steps", type=int, default=500,
                    help="continuous steps of the batched comparison")
    ap.add_argument("--adjoint-steps", type=int, default=200,
                    help="steps of the differentiated 65,536-point rollout (0 skips the adjoint section)")
    ap.add_argument("--adjoint-every", type=int, default=20, help="checkpoint interval of that rollout")
    ap.add_argument("--no-autotune", action="store_true", help="keep the compiled block shapes")
    ap.add_argument("--profile", action="store_true",
                    help="profiling run for ncu: the wave tank of --n points, --warmup eager steps, then "
                         "--steps eager steps (one launch per kernel per step), no timing, no JSON line")
    ap.add_argument("--profile-tape", type=int, default=0,
                    help="with --profile: then record this many steps on a tape (checkpoints every "
                         "--adjoint-every) and run one reverse pass")
    ap.add_argument("--passes", choices=["cells", "points", "pairs", "auto"], default="auto",
                    help="neighbour passes of the fused step (bit-identical results)")
    ap.add_argument("--fit-iters", type=int, default=40,
                    help="iterations of the 64-scene batched parameter fit (0 skips it)")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def allmax(dist, x: float) -> float:
    """The largest x over all ranks (the slowest rank's time sets the job's)."""
    if not dist:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(world: int, points_per_rank: int, steps: int, ms_slowest: float) -> float:
    """Whole-job Mparticle-steps/s: every rank steps its own replica of
    points_per_rank points; the slowest rank's time is the job's."""
    return world * points_per_rank * steps / (ms_slowest / 1e3) / 1e6


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 100 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.samples = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "100",
                 "-i", str(self.gpu)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return self
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append((time.perf_counter(), [x.strip() for x in line.split(",")]))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)

    def summary(self, t0: float, t1: float) -> dict:
        rows = [r for t, r in self.samples if t0 - 0.15 <= t <= t1 + 0.15 and len(r) >= 9]
        if not rows:
            rows = [r for _, r in self.samples if len(r) >= 9][-3:]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": num(rows[0][2]), "reasons": reasons, "samples": len(rows),
                "power_w_max": max((num(r[3]) or 0.0) for r in rows)}


def measured_peak():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        try:
            d = json.loads(f.read_text())
            return float(d["hbm_gbs"]), "measured"
        except (ValueError, KeyError):
            pass
    return 6800.0, "fallback"


def ncu_record(kernel: str) -> dict:
    """The committed ncu figures for `kernel` (DRAM bytes per launch, observed
    bound, issue activity), if any."""
    f = ROOT / "profiles" / "traffic.json"
    if not f.exists():
        return {}
    try:
        return json.loads(f.read_text()).get(kernel, {})
    except ValueError:
        return {}


# ---------------------------------------------------------------------------
def cpu_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_reference_rate(scene, budget_s: float, threads: int):
    """Particle-steps/s of the reference's CPU path on a sample of `scene`:
    the first points of the scene in fill order (its bottom layers, same box
    and grid), sized so the sample runs about `budget_s` seconds."""
    from oracle import oracle as O

    kind = "reference" if O.ref_available() else "port"
    p = scene.params

    def run(n, steps):
        pos, vel, veval, clr = scene.pos[:n], scene.vel[:n], scene.veval[:n], scene.clr[:n]
        if kind == "reference":
            R = O.RefKernels(p, pos, vel, veval, clr)
            t0 = time.perf_counter()
            R.run(steps, 0.0, threads=threads)
        else:
            st = O.State.new(p, pos, vel, veval, clr)
            t0 = time.perf_counter()
            O.run(p, st, steps, 0.0, threads=threads)
        return time.perf_counter() - t0

    n = min(scene.n, 250_000)
    dt1 = run(n, 1)
    per_point = max(dt1 / n, 1e-9)
    steps = 2
    n = int(min(scene.n, max(10_000, budget_s / (steps * per_point))))
    el = run(n, steps)
    return {"value": n * steps / el / 1e6, "unit": METRIC, "cores": threads, "kind": kind,
            "sample": f"{steps} full steps over the first {n:,} of the {scene.n:,} points (same box, grid "
                      f"and parameters), {el:.1f} s, {threads} host threads"}, el


def continuous_profile(s, steps: int, chunk: int = 100) -> dict:
    """Device time of `steps` continuous steps from the current state, per
    run of `chunk` steps (graph replay, CUDA events), with the largest cell
    at the end of each run: how the step cost grows as the fluid clumps."""
    import fluids3_gb300 as F
    rows, done, total = [], 0, 0.0
    while done < steps:
        k = min(chunk, steps - done)
        ms = s.TimeSteps(k, graph=True)
        done += k
        total += ms
        rows.append({"steps": done, "ms_per_step": ms / k, "largest_cell": int(s.GetBuffer(F.FGRIDCNT).max())})
    return {"steps": steps, "ms_total": total, "value": s.NumPoints() * steps / (total / 1e3) / 1e6,
            "unit": METRIC, "runs": rows}


def reference_gpu_rate(scene, warm: dict, t_start: float, steps: int, segment: int, value: float,
                       value_continuous: float | None = None) -> dict:
    """The reference's own GPU step on this GPU: fluids4.0/fluid_kernels.cu
    built for sm_103a with its build's flags, driven as FluidSystem::Run
    drives it (phase by phase on the default stream, cuCtxSynchronize at the
    end of every step). Same workload and protocol as `value`: the
    post-warm-up state, K steps run as segments of at most `segment` steps
    that each restart from it (the restart upload is not timed)."""
    from oracle import ref_gpu as R

    if not R.available():
        return {"unavailable": "the reference's GPU module was not built (reference tree absent at build time)"}
    import torch

    n = scene.n
    with R.RefGpu(scene.params, n) as ref:
        ref.set_state(warm["pos"], warm["vel"], warm["veval"], warm["clr"])
        t = t_start
        for _ in range(3):   # module's first launches
            t = ref.run(t)
        total_ms, left, n_in = 0.0, steps, []
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        while left > 0:
            chunk = min(left, segment) if segment > 0 else left
            ref.set_state(warm["pos"], warm["vel"], warm["veval"], warm["clr"])
            t = t_start
            ev0.record()
            for _ in range(chunk):
                t = ref.run(t)
            ev1.record()
            torch.cuda.synchronize()
            total_ms += ev0.elapsed_time(ev1)
            n_in.append(int(ref.get(R.FGRIDCNT).sum(dtype=np.int64)))
            left -= chunk
        # the same steps as one continuous trajectory from the warm state
        ref.set_state(warm["pos"], warm["vel"], warm["veval"], warm["clr"])
        t = t_start
        ev0.record()
        for _ in range(steps):
            t = ref.run(t)
        ev1.record()
        torch.cuda.synchronize()
        cont_ms = ev0.elapsed_time(ev1)
        # per-phase device times over one segment from the same state: events
        # between the phases of each Run (a separate, untimed pass)
        names = ("insert", "prefix_sum", "counting_sort", "pressure", "force", "advance")
        acc = dict.fromkeys(names, 0.0)
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(len(names) + 1)]
        ref.set_state(warm["pos"], warm["vel"], warm["veval"], warm["clr"])
        t = t_start
        k = min(steps, segment) if segment > 0 else steps
        for _ in range(k):
            evs[0].record()
            for a, phase in enumerate((ref.insert, lambda: ref.prefix_sum(1), ref.counting_sort, ref.pressure,
                                       ref.force, lambda: ref.advance(t))):
                phase()
                evs[a + 1].record()
            torch.cuda.synchronize()
            t = float(np.float32(t) + np.float32(ref.dt))
            for a, name in enumerate(names):
                acc[name] += evs[a].elapsed_time(evs[a + 1])
    rate = n * steps / (total_ms / 1e3) / 1e6
    rate_cont = n * steps / (cont_ms / 1e3) / 1e6
    return {"value": rate, "unit": METRIC, "ms_per_step": total_ms / steps, "steps": steps,
            "value_continuous": rate_cont, "ms_per_step_continuous": cont_ms / steps,
            "value_continuous_over_reference": (value_continuous / rate_cont) if value_continuous else None,
            "kind": "reference kernels on this GPU",
            "build": "fluids4.0/fluid_kernels.cu, nvcc -gencode arch=compute_103a,code=sm_103a -O3 "
                     "--use_fast_math --maxrregcount=32 (the reference build's flags)",
            "driver": "RUN_GPU_FULL phase sequence through the CUDA driver API, 512 threads per block, "
                      "default stream, cuCtxSynchronize per step (fluid_system.cpp:506-524)",
            "timing": "CUDA events on the default stream around each segment",
            "points_in_range_at_segment_ends": n_in,
            "phases_ms": {name: round(v / k, 5) for name, v in acc.items()}, "phase_steps": k,
            "value_over_reference": value / rate}


def reference_gpu_rollout_ms(sc, steps: int):
    """Milliseconds per step of the reference's own GPU kernels over the same
    rollout from the same start (its Run per step, cuCtxSynchronize included;
    CUDA events on the default stream); None where the module is absent."""
    from oracle import ref_gpu as R

    if not R.available() or steps <= 0:
        return None
    import torch
    with R.RefGpu(sc.params, sc.n) as ref:
        ref.set_state(sc.pos, sc.vel, sc.veval, sc.clr)
        ref.run(0.0)                                   # the module's first launches
        ref.set_state(sc.pos, sc.vel, sc.veval, sc.clr)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t = 0.0
        e0.record()
        for _ in range(steps):
            t = ref.run(t)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps


def reference_arm(args, rank, world):
    """The reference's CPU implementation of the step on this machine's host cores.
    A step is one full step over a bounded sample of the workload -- its first
    points in fill order, same box, grid and parameters -- sized so that the
    W + K steps take about two minutes."""
    if rank != 0:
        return
    from fluids3_gb300 import scenes
    from oracle import oracle as O
    from oracle import params_oracle as PO

    # parameters from the oracle's own restatement of the reference's
    # derivation: nothing of the product library is loaded in this arm
    scene = scenes.wave_tank(n=args.n, derive=PO.derive_flparams)
    p = scene.params
    threads = cpu_threads()
    kind = "reference" if O.ref_available() else "port"

    def make(n):
        a = (scene.pos[:n], scene.vel[:n], scene.veval[:n], scene.clr[:n])
        return O.RefKernels(p, *a) if kind == "reference" else O.State.new(p, *a)

    def steps(obj, k, t):
        return obj.run(k, t, threads=threads) if kind == "reference" else O.run(p, obj, k, t, threads=threads)

    calib_n = min(scene.n, 100_000)
    obj = make(calib_n)
    c0 = time.perf_counter()
    steps(obj, 1, 0.0)
    per_point = max((time.perf_counter() - c0) / calib_n, 1e-9)
    total = args.steps + max(args.warmup, 0)
    n = int(min(scene.n, max(10_000, 120.0 / (max(total, 1) * per_point))))
    obj = make(n)
    t = steps(obj, max(args.warmup, 0), 0.0)
    t0 = time.perf_counter()
    steps(obj, args.steps, t)
    el = time.perf_counter() - t0
    value = n * args.steps / el / 1e6
    info = {"value": value, "unit": METRIC, "cores": threads, "kind": kind,
            "sample": f"each step: one full step over the first {n:,} of the {scene.n:,} points (same box, "
                      f"grid, parameters); {args.steps} timed steps in {el:.1f} s on {threads} host threads"}
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / max(args.steps, 1) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": config_of(scene, args), "cpu_baseline": info,
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def batched_comparison(args):
    """The batched multi-scene workload: `args.batch_scenes` scenes of
    2,048..65,536 points (log-uniform), each with its own box, grid,
    viscosity and rest density, stepped (a) together as one batched system
    and (b) one at a time, each as its own plain system. Both start from the
    state after the warm-up steps and run `args.batch_steps` continuous steps
    (graph replay, no restarts) with the same launch shapes: the batch's
    autotuned shapes, pinned on every plain system. Every scene's final state
    (positions, velocities, evaluated velocities, cells) is compared bit for
    bit between (a) and (b)."""
    import fluids3_gb300 as F
    from fluids3_gb300 import scenes

    scs = scenes.batch_scenes(args.batch_scenes)
    total = sum(sc.n for sc in scs)
    k = args.batch_steps
    warm = max(args.warmup, 3)
    cat = scenes.concat(scs)
    b = F.FluidSystem.batch([sc.params for sc in scs], [sc.n for sc in scs])
    b.SetParticles(cat["pos"], cat["vel"], cat["veval"], clr=cat["clr"])
    b.SetNeighbourPasses(args.batch_passes)
    b.RunSteps(warm)
    if not args.no_autotune:
        b.Autotune(3)
    shapes = b.LaunchShapes()
    b.SaveCheckpoint(0)
    b.RunSteps(2)                       # capture the graph for the tuned shapes
    b.RestoreCheckpoint(0)
    ms_b = b.TimeSteps(k, graph=True)
    b.Sync()
    st_b = {f: b.GetBuffer(getattr(F, "F" + f.upper())) for f in ("pos", "vel", "veval", "gcell")}
    infos = [b.SceneInfo(q) for q in range(len(scs))]
    largest_cell = int(b.GetBuffer(F.FGRIDCNT).max())
    b.close()
    ms_seq = 0.0
    same = 0
    for q, sc in enumerate(scs):
        s = F.FluidSystem(sc.params, sc.n)
        s.SetParticles(sc.pos, sc.vel, sc.veval, clr=sc.clr)
        s.SetNeighbourPasses(args.batch_passes)
        s.RunSteps(warm)
        s.SetLaunchShapes(**shapes)
        s.SaveCheckpoint(0)
        s.RunSteps(2)
        s.RestoreCheckpoint(0)
        ms_seq += s.TimeSteps(k, graph=True)
        s.Sync()
        a, n = infos[q]["point_base"], infos[q]["n"]
        ok = True
        for f in st_b:
            got = st_b[f][a:a + n].copy()
            if f == "gcell":   # batched cells index the concatenated grid
                got[got != 0xFFFFFFFF] -= np.uint32(infos[q]["cell_base"])
            ok = ok and np.array_equal(s.GetBuffer(getattr(F, "F" + f.upper())).view(np.uint32),
                                       got.view(np.uint32))
        same += int(ok)
        s.close()
    vb = total * k / (ms_b / 1e3) / 1e6
    vs = total * k / (ms_seq / 1e3) / 1e6
    return {"scenes": len(scs), "points": total, "steps": k, "warmup_steps": warm, "value": vb, "unit": METRIC,
            "one_at_a_time_value": vs, "speedup": vb / vs, "ms_per_step": ms_b / k,
            "one_at_a_time_ms_per_step": ms_seq / k, "scenes_bit_identical": same,
            "launch_shapes_both": shapes, "largest_cell_at_end": largest_cell,
            "neighbour_passes": args.batch_passes,
            "protocol": f"{k} continuous graph-replayed steps after {warm} warm-up steps, both arms with the "
                        "batch's autotuned launch shapes; final pos/vel/veval/gcell compared per scene",
            "workload": "scenes log-uniform 2,048..65,536 points, fill U[0.2,0.6] of own box, "
                        "visc U[0.1,0.5], rest density U[500,700], dam-break parameters otherwise"}


def _finite(v):
    """JSON-safe: non-finite floats become None."""
    if isinstance(v, list):
        return [_finite(x) for x in v]
    return v if np.isfinite(v) else None


def _device_free():
    try:
        import torch
        return int(torch.cuda.mem_get_info()[0])
    except Exception:
        return None


def _time_backward(s, dpos, scaled: bool = False):
    """Wall time of one fl_backward (or fl_backward_scaled) with the
    cotangent and the gradients in device memory (the call returns after its
    stream is done). Returns (ms, parameter gradients, state gradients,
    per-scene binary exponents of the state gradients (zeros unscaled))."""
    import torch
    from fluids3_gb300 import _lib
    d = torch.from_numpy(np.ascontiguousarray(dpos, np.float32)).cuda()
    outs = [torch.empty_like(d) for _ in range(3)]
    gp = np.zeros((s.NumScenes(), 3), np.float64)
    ex = np.zeros(s.NumScenes(), np.int32)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    if scaled:
        _lib.check("fl_backward_scaled", _lib.lib().fl_backward_scaled(
            s.handle, d.data_ptr(), None, None, outs[0].data_ptr(), outs[1].data_ptr(), outs[2].data_ptr(),
            gp.ctypes.data_as(ctypes.c_void_p), ex.ctypes.data_as(ctypes.c_void_p)))
    else:
        _lib.check("fl_backward", _lib.lib().fl_backward(s.handle, d.data_ptr(), None, None, outs[0].data_ptr(),
                                                       outs[1].data_ptr(), outs[2].data_ptr(),
                                                       gp.ctypes.data_as(ctypes.c_void_p)))
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    return (t1 - t0) * 1e3, gp, outs, ex


def _rms_scaled(mantissa, exponent: int) -> float:
    """RMS of mantissa * 2^exponent, formed in float64."""
    m = mantissa.double()
    return float(m.pow(2).mean().sqrt()) * 2.0 ** int(exponent)


def adjoint_measurements(args):
    """Adjoint cost against the forward (adjoint/forward time per step).

    rollout_65k: the differentiated rollout -- the 65,536-point scaled dam
    break for --adjoint-steps steps, loss = mean squared distance of the
    final positions to the seeded target cloud (the initial block shifted
    0.3 box widths in +x), gradients for viscosity, rest density, IntStiff
    and the initial velocities; with checkpoints every --adjoint-every steps
    and with every step kept (device memory of both tapes).
    wave_tank_4m: the bench workload after the warm-up, 10 recorded steps,
    every = 1 and 5, each also with the recorded / replayed steps keeping
    their pair lists (FL_TAPE_KEEP_LISTS).
    forward = graph-replayed steps without a tape; taped = the recorded
    steps; backward = fl_backward with device buffers, per recorded step."""
    import fluids3_gb300 as F
    from fluids3_gb300 import scenes
    from fluids3_gb300.rollout import position_loss

    out = {}
    sc = scenes.dam_break_scaled(65536)
    target = scenes.shifted_target(sc)
    T = args.adjoint_steps
    free_before = _device_free()
    s = F.FluidSystem(sc.params, sc.n)
    s.SetParticles(sc.pos, sc.vel, sc.veval, clr=sc.clr)
    s.SaveCheckpoint(0)
    free_sys = _device_free()
    s.RunSteps(2)                                  # graph capture
    s.RestoreCheckpoint(0)
    ms_fwd = s.TimeSteps(T, graph=True) / T
    runs = {}
    every_k = max(1, min(args.adjoint_every, T))
    variants = [(every_k, False), (every_k, True)] + ([(1, False)] if every_k != 1 else [])
    for every, keep in variants:
        s.RestoreCheckpoint(0)
        f0 = _device_free()
        s.TapeBegin(T, every, keep)
        f1 = _device_free()
        s.Sync()
        t0 = time.perf_counter()
        s.RunSteps(T)
        s.Sync()
        t1 = time.perf_counter()
        loss, dpos, counted = position_loss(s, target)
        ms_b, gp, outs, ex = _time_backward(s, dpos, scaled=True)
        s.TapeEnd()
        gv = _rms_scaled(outs[1], ex[0])
        runs[(every, keep)] = {"every": every, "keep_lists": keep, "tape_bytes": (f0 - f1) if f0 is not None else None,
                       "taped_forward_ms_per_step": (t1 - t0) * 1e3 / T,
                       "backward_ms_per_step": ms_b / T, "ratio": ms_b / T / ms_fwd,
                       "loss": loss, "points_in_loss": counted,
                       "grad_finite": bool(np.isfinite(gp).all() and np.isfinite(gv)),
                       "grad_params": dict(zip(("pvisc", "prest_dens", "pintstiff"), _finite(gp[0].tolist()))),
                       "grad_vel_rms": _finite(gv), "grad_state_exponent": int(ex[0])}
    # the exact gradient grows ~1.3-1.5x per step (trajectories diverge):
    # its size against the horizon, each from the same start
    growth = []
    for h in (5, 10, 20, 40, 80):
        if h > T:
            break
        s.RestoreCheckpoint(0)
        s.TapeBegin(h, 1)
        s.RunSteps(h)
        loss, dpos, _ = position_loss(s, target)
        _, gp, outs, ex = _time_backward(s, dpos, scaled=True)
        s.TapeEnd()
        growth.append({"steps": h, "grad_vel_rms": _finite(_rms_scaled(outs[1], ex[0])),
                       "grad_pvisc": _finite(float(gp[0, 0]))})
    s.close()
    out["rollout_65k"] = {
        "workload": f"{sc.name}: 65,536-point dam break, box scaled x1.26 (same density as the 32,768-point "
                    f"scene), {T} steps; loss vs the initial block shifted 0.3 box widths in +x",
        "steps": T, "forward_ms_per_step": ms_fwd,
        "reference_gpu_forward_ms_per_step": None if args.no_ref_gpu else reference_gpu_rollout_ms(sc, T),
        "system_bytes": (free_before - free_sys) if free_before is not None else None,
        "checkpointed": runs[(every_k, False)], "checkpointed_kept_lists": runs[(every_k, True)],
        "every_step": runs[(1, False)] if (1, False) in runs else runs[(every_k, False)],
        "adjoint_forward_ratio": runs[(every_k, False)]["ratio"],
        "adjoint_forward_ratio_kept_lists": runs[(every_k, True)]["ratio"],
        "gradient_vs_horizon": growth,
        "note": "exact gradients (FP64-checked over 8 and 300 steps); they grow ~1.4x per step because "
                "trajectories diverge, so the state gradients come back as FP32 mantissas with a per-scene "
                "binary exponent (fl_backward_scaled); RMS values here are formed in float64"}

    scene = scenes.wave_tank(n=args.n)
    s = F.FluidSystem(scene.params, scene.n)
    s.SetParticles(scene.pos, scene.vel, scene.veval, clr=scene.clr)
    s.RunSteps(max(args.warmup, 3))
    s.SaveCheckpoint(0)
    T4 = 10
    ms_fwd = s.TimeSteps(T4, graph=True) / T4
    rows = []
    w = np.random.default_rng(1).standard_normal((scene.n, 3)).astype(np.float32)
    for every, keep in ((1, False), (1, True), (5, False), (5, True)):
        s.RestoreCheckpoint(0)
        s.TapeBegin(T4, every, keep)
        s.Sync()
        t0 = time.perf_counter()
        s.RunSteps(T4)
        s.Sync()
        t1 = time.perf_counter()
        _time_backward(s, w)                       # first call: staging buffers
        ms_b, _, _, _ = _time_backward(s, w)
        s.TapeEnd()
        rows.append({"every": every, "keep_lists": keep, "taped_forward_ms_per_step": (t1 - t0) * 1e3 / T4,
                     "backward_ms_per_step": ms_b / T4, "ratio": ms_b / T4 / ms_fwd})
    s.close()
    out["wave_tank_4m"] = {"steps": T4, "forward_ms_per_step": ms_fwd, "runs": rows}
    return out


def fit_measurement(args):
    """The batched parameter fit: 64 scenes of 8,192..32,768 points
    (log-uniform), each with a hidden viscosity U[0.1, 0.5] generating its
    100-step target trajectory; per-scene viscosity and IntStiff fitted from
    0.3 / 1.0 by Adam on adjoint gradients, each iteration ten 10-step
    windows along the target trajectory (checkpoints every 10 steps). Device
    memory of one 100-step tape of the whole batch with and without
    checkpointing."""
    import fluids3_gb300 as F
    from fluids3_gb300 import scenes
    from fluids3_gb300.fit import batched_fit

    scs = scenes.fit_scenes()
    total = sum(sc.n for sc in scs)
    cat = scenes.concat(scs)
    mem = {}
    with F.FluidSystem.batch([sc.params for sc in scs], [sc.n for sc in scs]) as b:
        b.SetParticles(cat["pos"], cat["vel"], cat["veval"], clr=cat["clr"])
        for every in (10, 1):
            f0 = _device_free()
            b.TapeBegin(100, every)
            f1 = _device_free()
            b.TapeEnd()
            mem[every] = (f0 - f1) if f0 is not None else None
    t0 = time.perf_counter()
    res = batched_fit(scs, steps=100, window=10, every=10, iters=args.fit_iters, lr=0.05)
    el = time.perf_counter() - t0
    err = res.visc_rel_err
    start_err = np.abs(0.3 - res.hidden_visc) / res.hidden_visc
    return {"scenes": len(scs), "points": total, "steps": 100, "window": 10, "every": 10,
            "iterations": args.fit_iters, "seconds": el,
            "loss_first": res.losses[0], "loss_last": res.losses[-1],
            "visc_rel_err": {"median": float(np.median(err)), "p90": float(np.percentile(err, 90)),
                             "max": float(err.max()), "start_median": float(np.median(start_err))},
            "intstiff": {"hidden": 1.0, "median": float(np.median(res.stiff)),
                         "min": float(res.stiff.min()), "max": float(res.stiff.max())},
            "tape_bytes_100_steps": {"every_10": mem[10], "every_1": mem[1]}}


def config_of(scene, args):
    p = scene.params
    return {"workload": f"{scene.name}: {scene.n:,}-point SPH wave tank (dam break with X- wall forcing, "
                        f"freq {p.bound_wall_freq:g}, amplitude {p.bound_wall_force:g}), cell 2h, gridSrch {p.gridSrch}",
            "n_points": scene.n, "cells": p.gridTotal, "grid": list(p.gridRes),
            "l2": "inputs larger than L2 (state ~1 GB in HBM), no flush needed",
            "segment_steps": args.segment,
            "neighbour_passes": getattr(args, "passes", "points"),
            "step": "insert, scan, index scatter, canonical sort+gather, density, force+advance"}


# ---------------------------------------------------------------------------
def our_arm(args, rank, world, local_rank):
    import ctypes as C

    import fluids3_gb300 as F
    from fluids3_gb300 import scenes

    dist = None
    if world > 1:
        import torch
        import torch.distributed as tdist
        torch.cuda.set_device(local_rank)
        tdist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        dist = tdist
    else:
        try:
            import torch
            if torch.cuda.is_available():
                torch.cuda.set_device(local_rank)
        except ImportError:
            pass

    def barrier():
        if dist:
            dist.barrier()


    scene = scenes.wave_tank(n=args.n)
    p = scene.params
    s = F.FluidSystem(p, scene.n)
    s.SetParticles(scene.pos, scene.vel, scene.veval, clr=scene.clr)
    s.SetNeighbourPasses(args.passes)

    # warm-up (untimed): graph capture + W steps; keep the state so the
    # per-kernel region below replays exactly the timed steps
    s.RunSteps(max(args.warmup, 3))
    s.Sync()
    tuned = s.Autotune(3) if not args.no_autotune else None
    s.SaveCheckpoint(0)
    s.RunSteps(2)                       # capture the graph for the tuned shapes
    s.RestoreCheckpoint(0)
    warm = None
    if rank == 0 and not args.no_ref_gpu:   # start state of the timed segments, for the reference's GPU leg
        warm = {"pos": s.GetBuffer(F.FPOS), "vel": s.GetBuffer(F.FVEL), "veval": s.GetBuffer(F.FVEVAL),
                "clr": s.GetBuffer(F.FCLR), "time": s.time}

    # -- timed region: exactly K steps, graph replay ---------------------------
    clocks = ClockSampler(local_rank).start()
    time.sleep(0.3)
    barrier()
    s.Sync()
    t0 = time.perf_counter()
    ms = s.TimeSteps(args.steps, graph=True, restart_every=args.segment, restart_slot=0)
    t1 = time.perf_counter()
    s.Sync()
    barrier()
    time.sleep(0.25)
    clocks.stop()
    ms = allmax(dist, ms)
    status = s.DeviceStatus()
    # the same K steps as one continuous trajectory from the warm state (no
    # restarts; beside `value`, which restarts every --segment steps)
    s.RestoreCheckpoint(0)
    barrier()
    ms_cont = allmax(dist, s.TimeSteps(args.steps, graph=True))
    long_run = None
    if args.long_steps > 0:
        s.RestoreCheckpoint(0)
        long_run = continuous_profile(s, args.long_steps, args.long_chunk)

    # -- per-kernel times: the same K steps again from the saved state, eager,
    #    each launch bracketed by CUDA events
    s.SetTiming(True)
    left = min(args.steps, 4096)
    while left > 0:
        s.RestoreCheckpoint(0)
        chunk = min(left, args.segment) if args.segment > 0 else left
        s.RunSteps(chunk)
        left -= chunk
    phases, nsteps_timed = s.PhaseTimes()
    s.SetTiming(False)
    n_in = int(s.GetBuffer(F.FGRIDCNT).sum(dtype=np.int64))

    # -- conservation drift over one segment (FP64 sums on the device)
    s.RestoreCheckpoint(0)
    c0 = s.Conservation()[0]
    seg_steps = args.segment if args.segment > 0 else args.steps
    s.RunSteps(seg_steps)
    c1 = s.Conservation()[0]
    e0, e1 = c0[5] + c0[6], c1[5] + c1[6]
    conservation = {"steps": seg_steps, "points": [int(c0[0]), int(c1[0])],
                    "mass_rel_drift": float(c1[1] / c0[1] - 1.0),
                    "energy_start_J": float(e0), "energy_end_J": float(e1),
                    "energy_rel_change": float((e1 - e0) / abs(e0)),
                    "kinetic_end_J": float(c1[5]), "momentum_end": [float(v) for v in c1[2:5]],
                    "centre_of_mass_shift": [float(a / c1[0] - b / c0[0]) for a, b in zip(c1[7:10], c0[7:10])],
                    "note": "kinetic + gravitational potential energy; walls, viscosity and the limits "
                            "dissipate it, the moving X- wall feeds it"}

    # -- e2e: host buffers through the C ABI ------------------------------------
    # inputs of every e2e step: the timed segments' start state advanced half
    # a segment (the mean regime of the timed steps; the fluid clumps as a
    # segment goes on)
    e2e_steps = args.e2e_steps or min(args.steps, 20)
    s.RestoreCheckpoint(0)
    s.RunSteps(max(1, seg_steps // 2))
    s.Sync()
    n = scene.n
    pin_pos = F.PinnedArray((n, 3), np.float32)
    pin_vel = F.PinnedArray((n, 3), np.float32)
    pin_vev = F.PinnedArray((n, 3), np.float32)
    pin_clr = F.PinnedArray((n,), np.uint32)
    pin_out = F.PinnedArray((n, 3), np.float32)
    pin_pos.array[:] = s.GetBuffer(F.FPOS)
    pin_vel.array[:] = s.GetBuffer(F.FVEL)
    pin_vev.array[:] = s.GetBuffer(F.FVEVAL)
    pin_clr.array[:] = s.GetBuffer(F.FCLR)
    lib = F.lib()
    vp = lambda a: a.ctypes.data_as(C.c_void_p)
    h2d = n * (12 * 3 + 4)
    d2h = n * 12

    def e2e_step():
        F._lib.check("fl_run_from_host", lib.fl_run_from_host(
            s.handle, n, vp(pin_pos.array), vp(pin_vel.array), vp(pin_vev.array), vp(pin_clr.array),
            vp(pin_out.array)))

    e2e_step()   # untimed warm-up: first uploads, the captured step graph released
    barrier()
    s.Sync()
    te0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    te1 = time.perf_counter()
    barrier()
    e2e_s = allmax(dist, te1 - te0)
    for a in (pin_pos, pin_vel, pin_vev, pin_clr, pin_out):
        a.free()
    s.close()

    if rank != 0:
        return

    batched = batched_comparison(args) if args.batch_scenes > 0 else None
    adjoint = adjoint_measurements(args) if args.adjoint_steps > 0 else None
    fit = fit_measurement(args) if args.fit_iters > 0 else None
    value = job_value(world, scene.n, args.steps, ms)
    dominant = max((k for k in phases if k in ALGO_BYTES and k != "scan"), key=lambda k: phases[k])
    dur_ms = phases[dominant]
    algo = ALGO_BYTES[dominant] * n_in
    achieved = algo / (dur_ms / 1e3) / 1e9
    peak, peak_kind = measured_peak()
    rec = ncu_record(dominant)
    roofline = {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": f"of {peak_kind}",
                "traffic": rec.get("dram_bytes_per_launch"),
                "algorithmic_bytes_per_launch": algo, "mean_launch_ms": dur_ms,
                "bound_observed": rec.get("bound_observed"),
                "issue_active_pct_ncu": rec.get("issue_active_pct"),
                "issue_roofline_frac_ncu": rec.get("issue_roofline_frac"),
                "fp32_fma_pipe_pct_ncu": rec.get("fp32_fma_pipe_pct"),
                "issue_roofline_note": "warp instructions / (time x 152 SMs x 4 schedulers x SM clock), "
                                       "from the committed ncu capture: the roof this kernel meets",
                "profile": "profiles/ncu_step_wave_tank.md"}
    step_bytes = sum(ALGO_BYTES.values()) * n_in + 12 * (p.gridTotal + 1)
    cpu = None
    if not args.no_cpu_baseline:
        cpu, _ = cpu_reference_rate(scene, args.cpu_seconds, cpu_threads())
    ref_gpu = None
    if warm is not None:
        try:
            ref_gpu = reference_gpu_rate(scene, warm, warm["time"], args.steps, args.segment, value,
                                         job_value(world, scene.n, args.steps, ms_cont))
        except (OSError, RuntimeError, ValueError) as e:
            ref_gpu = {"unavailable": f"{type(e).__name__}: {e}"}
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded jittered lattice (splitmix64), no dataset",
        "config": config_of(scene, args),
        "value_continuous": job_value(world, scene.n, args.steps, ms_cont),
        "ms_per_step_continuous": ms_cont / args.steps,
        "long_continuous": long_run,
        "roofline": roofline,
        "step_roofline": {"algorithmic_bytes_per_step": step_bytes,
                          "bytes_per_point": sum(ALGO_BYTES.values()),
                          "implementation_bytes_per_point_not_counted": IMPL_BYTES,
                          "achieved_gbs": step_bytes / (ms / args.steps / 1e3) / 1e9,
                          "frac": step_bytes / (ms / args.steps / 1e3) / 1e9 / peak},
        "phases_ms": {k: round(v, 5) for k, v in phases.items()}, "phase_steps": nsteps_timed,
        "cpu_baseline": cpu,
        "reference_gpu": ref_gpu,
        "e2e": {"value": world * n * e2e_steps / e2e_s / 1e6, "unit": METRIC, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "steps": e2e_steps,
                "inputs": f"every step uploads the state {max(1, seg_steps // 2)} steps into a timed segment "
                          "(its mean regime) from page-locked host memory and reads the positions back"},
        "autotuned_block_shapes": tuned,
        "conservation": conservation,
        "batched": batched,
        "adjoint": adjoint,
        "fit": fit,
        "clocks": clocks.summary(t0, t1),
        "gpu_launches": KERNELS_PER_STEP * args.steps,
        "device_status": status,
        "points_in_range": n_in,
    }
    print(json.dumps(line), flush=True)


def profile_run(args):
    """Launches for a profiler: every step eager, so kernel k of step j is
    launch j of that kernel (skip --warmup of them with ncu -s)."""
    import fluids3_gb300 as F
    from fluids3_gb300 import scenes
    scene = scenes.wave_tank(n=args.n)
    with F.FluidSystem(scene.params, scene.n) as s:
        s.SetParticles(scene.pos, scene.vel, scene.veval, clr=scene.clr)
        s.SetNeighbourPasses(args.passes)
        for _ in range(args.warmup + args.steps):
            s.Run()
        s.Sync()
        tape = ""
        if args.profile_tape > 0:   # then one reverse pass over a recorded rollout
            T = args.profile_tape
            every = max(1, min(args.adjoint_every, T))
            s.TapeBegin(T, every)
            s.RunSteps(T)
            w = np.random.default_rng(1).standard_normal((scene.n, 3)).astype(np.float32)
            s.Backward(w)
            s.Sync()
            tape = f", then a {T}-step tape (checkpoints every {every}) and one fl_backward"
        print(f"profile run: {scene.n:,} points, {args.warmup} + {args.steps} eager steps ({args.passes} passes)"
              f"{tape}, device status {s.DeviceStatus()}", flush=True)


def main():
    args = parse()
    rank, world, local_rank = dist_env()
    if args.profile:
        profile_run(args)
        return
    if args.impl == "reference":
        reference_arm(args, rank, world)
        return
    our_arm(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
