"""Regenerates the golden fixtures in this directory from the reference's own
kernel source (fluids4.0/fluid_kernels.cu built for the host by
oracle/build_ref.sh into oracle/_ref/). Needs the reference tree; run once
in a container that has it:

    python tests/golden/make_golden.py

Fixtures:
  kat_insert_64.npz     64 hand-placed points in an 8 x 8 x 8-cell grid:
                        insert/scan/sort outputs (known-answer test)
  dam_break_2000.npz    2,000-point dam break (ragged size): inputs, every
                        phase output of step 1, and the state after 20 steps
  digests.json          sha256 of the full state after selected steps of the
                        32,768-point dam break and a 60,000-point wave tank
                        (all points in range throughout)
  params.json           derived parameter blocks of the workloads
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from fluids3_gb300 import scenes  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent
FIELDS = ("pos", "vel", "veval", "force", "press", "clr", "gcell", "gndx")


def pbytes(p) -> np.ndarray:
    """The exact FlParams block, so tests replay it without re-deriving (the
    powf-derived kernel constants may differ by an ulp between libm builds)."""
    return np.frombuffer(bytes(p), dtype=np.uint8).copy()


def digest(buf: dict) -> str:
    h = hashlib.sha256()
    for k in FIELDS:
        h.update(np.ascontiguousarray(buf[k]).tobytes())
    return h.hexdigest()


def kat_scene():
    """8 x 8 x 8-cell grid (cell = 5 world units), 64 points placed by hand:
    clusters in a few cells so counts, offsets and the within-cell order are
    easy to check by eye."""
    p = scenes.make_params((0.0, 0.0, 0.0), (30.0, 30.0, 30.0))
    rng_free = []
    cells = [(2, 2, 2), (2, 2, 3), (3, 2, 2), (4, 4, 4), (5, 3, 2), (2, 5, 5)]
    k = 0
    for idx in range(64):
        cx, cy, cz = cells[idx % len(cells)]
        sub = idx // len(cells)
        # inside the cell, offset by a deterministic sub-position
        x = p.gridMin[0] + (cx + 0.1 + 0.07 * (sub % 4)) * 5.0
        y = p.gridMin[1] + (cy + 0.1 + 0.07 * ((sub // 4) % 4)) * 5.0
        z = p.gridMin[2] + (cz + 0.2 + 0.05 * (sub % 3)) * 5.0
        rng_free.append((x, y, z))
        k += 1
    pos = np.array(rng_free, np.float32)
    return p, pos


def main():
    if not O.ref_available():
        O.build(ref=True)
    assert O.ref_available(), "reference tree needed to regenerate fixtures"

    # --- known-answer insert/scan/sort ---------------------------------------
    p, pos = kat_scene()
    R = O.RefKernels(p, pos)
    R.insert()
    kat = dict(params=pbytes(p), pos=pos, gcell=R.buf["gcell"].copy(), gndx=R.buf["gndx"].copy(),
               gridcnt=R.buf["gridcnt"].copy())
    R.prefix_sum(1)
    kat["gridoff"] = R.buf["gridoff"].copy()
    R.counting_sort()
    kat["sorted_pos"] = R.buf["pos"].copy()
    kat["sorted_gcell"] = R.buf["gcell"].copy()
    kat["sorted_gndx"] = R.buf["gndx"].copy()
    np.savez_compressed(OUT / "kat_insert_64.npz", **kat)

    # --- 2,000-point dam break: every phase of step 1, then 20 steps ---------
    sc = scenes.dam_break(n=2000, seed=7)
    p = sc.params
    R = O.RefKernels(p, sc.pos, sc.vel, sc.veval, sc.clr)
    d = {f"in_{k}": R.buf[k].copy() for k in ("pos", "vel", "veval", "clr")}
    d["params"] = pbytes(p)
    R.insert()
    d.update(ins_gcell=R.buf["gcell"].copy(), ins_gndx=R.buf["gndx"].copy(),
             ins_gridcnt=R.buf["gridcnt"].copy())
    R.prefix_sum(1)
    d["gridoff"] = R.buf["gridoff"].copy()
    R.counting_sort()
    for k in ("pos", "vel", "veval", "clr", "gcell", "gndx"):
        d[f"sort_{k}"] = R.buf[k].copy()
    R.pressure()
    d["press"] = R.buf["press"].copy()
    R.force()
    d["force"] = R.buf["force"].copy()
    R.advance(0.0, p.dt, p.sim_scale)
    for k in ("pos", "vel", "veval"):
        d[f"adv_{k}"] = R.buf[k].copy()
    t = float(np.float32(p.dt))
    t = R.run(19, t)
    assert int((R.buf["gcell"] == 0xFFFFFFFF).sum()) == 0
    for k in FIELDS:
        d[f"s20_{k}"] = R.buf[k].copy()
    d["s20_time"] = np.float32(t)
    np.savez_compressed(OUT / "dam_break_2000.npz", **d)

    # --- digests of larger rollouts ------------------------------------------
    digests = {}
    for sc, marks in ((scenes.dam_break(), (1, 10, 30, 60)), (scenes.wave_tank(n=60000), (1, 10, 50))):
        p = sc.params
        R = O.RefKernels(p, sc.pos, sc.vel, sc.veval, sc.clr)
        t, done = 0.0, 0
        rec = {"params": bytes(p).hex(), "n": sc.n,
               "inputs": hashlib.sha256(sc.pos.tobytes() + sc.clr.tobytes()).hexdigest()}
        for m in marks:
            t = R.run(m - done, t, threads=8)
            done = m
            assert int((R.buf["gcell"] == 0xFFFFFFFF).sum()) == 0, (sc.name, m)
            rec[f"step_{m}"] = digest(R.buf)
        digests[sc.name] = rec
    (OUT / "digests.json").write_text(json.dumps(digests, indent=1) + "\n")

    # --- derived parameters ---------------------------------------------------
    params = {}
    for name, sc in (("dam_break_32k", scenes.dam_break(n=8)), ("wave_tank_4m", scenes.wave_tank(n=8)),
                     ("kat", None)):
        pp = kat_scene()[0] if sc is None else sc.params
        params[name] = pp.as_dict()
    (OUT / "params.json").write_text(json.dumps(params, indent=1) + "\n")
    print("golden fixtures written to", OUT)


if __name__ == "__main__":
    main()
