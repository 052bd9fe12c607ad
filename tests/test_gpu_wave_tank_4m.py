"""The 4,000,000-point wave tank over a continuous 400-step trajectory.

The reference's headline size (fluids4.0/main.cpp:157): one system steps
without a restart (graph replay in 100-step runs). Every 100 steps -- at
steps 0, 100, ..., 400 -- the GPU's state is fed to the oracle, which
inserts, scans and sorts it, and the GPU takes its next step from the same
state. This is the check the reference itself makes in ValidateCUDA
(fluids4.0/fluid_system.cpp:363-464), at every checkpoint:

* integers, bit-exact over all 4M points: each point's cell (FGCELL), its
  rank in the cell (FGNDX), the cell counts (FGRIDCNT) and offsets
  (FGRIDOFF), and the sorted permutation (the colour field carried through
  the sort, FCLR);
* floats on a seeded sample of 100,000 in-range slots (the fluid clumps into
  cells of thousands of points, where a full CPU pass would take minutes):
  density and force bit-exact against the oracle's FP32 evaluation in the
  reference's order; at the steps after 0, 100 and 200 also density within
  1e-5 and force within 1e-4 of the FP64 oracle.

The moving X- wall only enters the advance, which this test does not
compare (CUDA's sinf and the host's differ by an ulp).

Why 400 and not 1,000 steps: with these parameters the fluid collapses
(each point sums only over the 2x2x2 block c-1..c, fluid_kernels.cu:120,
so the pair forces are not antisymmetric). Measured on one GB300 along
this trajectory: 2.2, 6.8, 70 and 777 ms per step over steps 0-100,
100-200, 200-300 and 300-400, the largest cell growing from 800 to 289,000
points; the search is O(points x cell occupancy) for any implementation of
the reference's step, so the next hundreds of steps cost seconds each.
"""
from __future__ import annotations

import os
import time

import numpy as np
import pytest

import fluids3_gb300 as F
from fluids3_gb300 import scenes
from oracle import oracle as O

from helpers import assert_bit_equal, density_normwise_err, density_rel_err, force_rel_err

pytestmark = pytest.mark.gpu
UNDEF = 0xFFFFFFFF
SAMPLE = 100_000
FP64_AT = (0, 100, 200)
LAST = 400


def _threads() -> int:
    try:
        return max(1, len(os.sched_getaffinity(0)))
    except AttributeError:
        return os.cpu_count() or 1


def test_wave_tank_4m_continuous_400_steps():
    sc = scenes.wave_tank()
    p = sc.params
    assert sc.n == 4_000_000
    th = _threads()
    rng = np.random.default_rng(11)
    log = []
    with F.FluidSystem(p, sc.n) as s:
        s.SetParticles(sc.pos, sc.vel, sc.veval, clr=sc.clr)
        done = 0
        for k in range(0, LAST + 1, 100):
            t0 = time.perf_counter()
            if k > done:
                s.RunSteps(k - done)
                done = k
            s.Sync()
            t1 = time.perf_counter()
            st0 = s.state()
            ref = O.State.new(p, st0["pos"], st0["vel"], st0["veval"], st0["clr"])
            O.insert(p, ref)
            O.prefix_sum(p, ref)
            O.counting_sort(p, ref)
            s.Run()
            done += 1
            s.Sync()
            st = s.state()
            for f in ("gcell", "gndx", "clr"):
                assert_bit_equal(st[f], getattr(ref, f), f"step {k}: {f}")
            assert_bit_equal(st["gridcnt"], ref.cnt[:-1], f"step {k}: gridcnt")
            assert_bit_equal(st["gridoff"], ref.off[:-1], f"step {k}: gridoff")

            inr = np.flatnonzero(ref.gcell != UNDEF)
            idx = np.sort(rng.choice(inr, min(SAMPLE, inr.size), replace=False)).astype(np.uint32)
            assert_bit_equal(st["press"][idx], O.density_at(p, ref, idx, threads=th), f"step {k}: density")
            fargs = (ref.pos, ref.veval, st["press"], ref.gcell, ref.off, ref.cnt)
            assert_bit_equal(st["force"][idx], O.force_at(p, *fargs, idx, threads=th), f"step {k}: force")
            if k in FP64_AT:
                m = np.ones(idx.size, bool)
                d64 = O.density_f64_at(p, ref.pos, ref.gcell, ref.off, ref.cnt, idx, threads=th)
                assert density_rel_err(st["press"][idx], d64, m, p.prest_dens) <= 1e-5, f"step {k}"
                assert density_normwise_err(st["press"][idx], d64, m) <= 1e-6, f"step {k}"
                f64, scale = O.force_f64_at(p, *fargs, idx, threads=th)
                assert force_rel_err(st["force"][idx], f64, scale, m) <= 1e-4, f"step {k}"
            cnt = st["gridcnt"]
            log.append((k, round(t1 - t0, 2), round(time.perf_counter() - t1, 2), int(inr.size),
                        int(cnt.max()), int(np.median(cnt[st["gcell"][inr]]))))
    print("\nstep, gpu s, check s, points in range, largest cell, median point's cell")
    for row in log:
        print(*row)
    assert len(log) == LAST // 100 + 1
