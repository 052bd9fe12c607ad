"""Batched multi-scene step (fl_batch_create): every scene of a batch must
evolve bit-identically to the same scene stepped alone on the plain path,
through the fused step, graph replay and the phase API."""
from __future__ import annotations

import numpy as np
import pytest

import fluids3_gb300 as F
from fluids3_gb300 import scenes
from oracle import oracle as O

from helpers import FIELDS, assert_bit_equal

pytestmark = pytest.mark.gpu
UNDEF = 0xFFFFFFFF


def small_batch(k=9, seed=7):
    return scenes.batch_scenes(nscenes=k, seed=seed, nmin=300, nmax=6000)


def per_scene(state: dict, info: dict) -> dict:
    """One scene's slice of a batched readback, with its cell ids made local."""
    a, n = info["point_base"], info["n"]
    out = {k: state[k][a:a + n].copy() for k in FIELDS}
    g = out["gcell"]
    g[g != UNDEF] -= np.uint32(info["cell_base"])
    return out


def plain_state(sc, steps, graph):
    with F.FluidSystem(sc.params, sc.n) as s:
        s.SetParticles(sc.pos, sc.vel, sc.veval, clr=sc.clr)
        if graph:
            s.RunSteps(steps)
        else:
            for _ in range(steps):
                s.Run()
        s.Sync()
        return s.state()


@pytest.mark.parametrize("graph", [False, True])
def test_batch_matches_each_scene_alone(graph):
    scs = small_batch()
    cat = scenes.concat(scs)
    with F.FluidSystem.batch([sc.params for sc in scs], [sc.n for sc in scs]) as b:
        assert b.NumScenes() == len(scs)
        b.SetParticles(cat["pos"], cat["vel"], cat["veval"], clr=cat["clr"])
        if graph:
            b.RunSteps(6)
        else:
            for _ in range(6):
                b.Run()
        b.Sync()
        st = b.state()
        assert b.IntegrityCheck() == 0
        infos = [b.SceneInfo(k) for k in range(len(scs))]
    for k, sc in enumerate(scs):
        want = plain_state(sc, 6, graph)
        got = per_scene(st, infos[k])
        for f in FIELDS:
            assert_bit_equal(got[f], want[f], f"scene {k} {f}")
        # grid: the scene's cells, offsets shifted by its first point
        c0, nc = infos[k]["cell_base"], infos[k]["ncells"]
        assert_bit_equal(st["gridcnt"][c0:c0 + nc], want["gridcnt"], f"scene {k} gridcnt")
        assert_bit_equal(st["gridoff"][c0:c0 + nc] - np.uint32(infos[k]["point_base"]), want["gridoff"],
                         f"scene {k} gridoff")


def test_batch_phase_api_matches_oracle():
    scs = small_batch(k=5, seed=11)
    cat = scenes.concat(scs)
    with F.FluidSystem.batch([sc.params for sc in scs], [sc.n for sc in scs]) as b:
        b.SetParticles(cat["pos"], cat["vel"], cat["veval"], clr=cat["clr"])
        b.InsertParticlesCUDA()
        b.PrefixSumCellsCUDA(1)
        b.CountingSortFullCUDA()
        b.ComputePressureCUDA()
        b.ComputeForceCUDA()
        b.AdvanceCUDA(0.0, scs[0].params.dt, scs[0].params.sim_scale)
        b.Sync()
        st = b.state()
        infos = [b.SceneInfo(k) for k in range(len(scs))]
    for k, sc in enumerate(scs):
        ref = O.State.new(sc.params, sc.pos, sc.vel, sc.veval, sc.clr)
        O.insert(sc.params, ref); O.prefix_sum(sc.params, ref); O.counting_sort(sc.params, ref)
        O.density(sc.params, ref); O.force(sc.params, ref)
        O.advance(sc.params, ref, 0.0, sc.params.dt, sc.params.sim_scale)
        got = per_scene(st, infos[k])
        for f in FIELDS:
            assert_bit_equal(got[f], getattr(ref, f), f"scene {k} {f}")


def test_batch_with_escapes_and_empty_scene():
    scs = small_batch(k=4, seed=13)
    scs[1].pos[:3] = [(-500.0, 1.0, 1.0), (1.0, -300.0, 1.0), (np.nan, 0.0, 0.0)]
    empty = scenes.block_scene(1, 0.3, 5, "one_point")
    empty.pos = empty.pos[:0]; empty.vel = empty.vel[:0]; empty.veval = empty.veval[:0]; empty.clr = empty.clr[:0]
    scs.insert(2, empty)
    cat = scenes.concat(scs)
    with F.FluidSystem.batch([sc.params for sc in scs], [sc.n for sc in scs]) as b:
        b.SetParticles(cat["pos"], cat["vel"], cat["veval"], clr=cat["clr"])
        b.RunSteps(3)
        b.Sync()
        st = b.state()
        infos = [b.SceneInfo(k) for k in range(len(scs))]
    for k, sc in enumerate(scs):
        ref = O.State.new(sc.params, sc.pos, sc.vel, sc.veval, sc.clr)
        O.run(sc.params, ref, 3, 0.0)
        got = per_scene(st, infos[k])
        for f in FIELDS:
            assert_bit_equal(got[f], getattr(ref, f), f"scene {k} {f}")


def test_batch_rejects_mixed_dt_and_wrong_count():
    scs = small_batch(k=2)
    p1 = scs[1].params.copy()
    p1.dt = 0.002
    with pytest.raises(F.FluidsError) as e:
        F.FluidSystem.batch([scs[0].params, p1], [scs[0].n, scs[1].n])
    assert e.value.code == -3
    with F.FluidSystem.batch([sc.params for sc in scs], [sc.n for sc in scs]) as b:
        with pytest.raises(F.FluidsError):
            b.SetParticles(scs[0].pos)
