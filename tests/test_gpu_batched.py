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


def test_batch_with_crowded_cells_matches_each_scene_alone():
    """Crowded cells (above 128 points, sorted by a block each) in two of the
    scenes: the batch still steps each scene as it steps alone."""
    scs = small_batch()
    for k in (0, 2):
        sc = scs[k]
        m = min(600, sc.n // 2)
        c = sc.pos[sc.n // 3].copy()
        sc.pos[:m] = c + np.random.default_rng(60 + k).uniform(-1.5, 1.5, (m, 3)).astype(np.float32)
    cat = scenes.concat(scs)
    with F.FluidSystem.batch([sc.params for sc in scs], [sc.n for sc in scs]) as b:
        b.SetParticles(cat["pos"], cat["vel"], cat["veval"], clr=cat["clr"])
        b.RunSteps(4)
        b.Sync()
        st = b.state()
        assert st["gridcnt"].max() > 128
        infos = [b.SceneInfo(k) for k in range(len(scs))]
    for k, sc in enumerate(scs):
        want = plain_state(sc, 4, True)
        got = per_scene(st, infos[k])
        for f in FIELDS:
            assert_bit_equal(got[f], want[f], f"scene {k} {f}")


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


def test_batch_set_params_equals_a_scene_created_with_them():
    """fl_batch_set_params: a scene whose viscosity and IntStiff are replaced
    steps exactly like a system created with them; a block that changes the
    scene's grid is rejected."""
    from fluids3_gb300.fit import set_scene_physics
    scs = scenes.batch_scenes(nscenes=3, nmin=1500, nmax=3000, seed=31)
    cat = scenes.concat(scs)
    with F.FluidSystem.batch([sc.params for sc in scs], [sc.n for sc in scs]) as b:
        b.SetParticles(cat["pos"], cat["vel"], cat["veval"], clr=cat["clr"])
        for k in (0, 2):
            set_scene_physics(b, k, 0.123, 1.7)
        b.RunSteps(6)
        got = b.GetBuffer(F.FPOS)
        bad = scenes.make_params((0.0, 0.0, 0.0), (10.0, 10.0, 10.0))
        with pytest.raises(F.FluidsError) as e:
            b.SetSceneParams(1, bad)
        assert e.value.code == -3
    base = 0
    for k, sc in enumerate(scs):
        p = sc.params.copy()
        if k != 1:
            p.pvisc, p.pintstiff = 0.123, 1.7
        p = F.derive_params(p)
        with F.FluidSystem(p, sc.n) as s:
            s.SetParticles(sc.pos, sc.vel, sc.veval, clr=sc.clr)
            s.RunSteps(6)
            assert_bit_equal(got[base:base + sc.n], s.GetBuffer(F.FPOS), f"scene {k}")
        base += sc.n


def test_batched_fit_recovers_viscosity_on_a_small_batch():
    """A small version of the batched parameter fit: 4 scenes, 40 steps,
    checkpoints every 10. The loss falls and the viscosity error shrinks."""
    from fluids3_gb300.fit import batched_fit
    scs = scenes.fit_scenes(nscenes=4, nmin=2000, nmax=4000, seed=32)
    res = batched_fit(scs, steps=40, every=10, iters=25, lr=0.05)
    start_err = np.abs(0.3 - res.hidden_visc) / res.hidden_visc
    assert res.losses[-1] < 0.5 * res.losses[0], res.losses
    assert np.median(res.visc_rel_err) < 0.5 * np.median(start_err), (res.visc, res.hidden_visc)


def test_batched_autotune_changes_no_result():
    scs = scenes.batch_scenes(nscenes=6, nmin=1500, nmax=6000, seed=41)
    cat = scenes.concat(scs)
    outs = []
    for tune in (False, True):
        with F.FluidSystem.batch([sc.params for sc in scs], [sc.n for sc in scs]) as b:
            b.SetParticles(cat["pos"], cat["vel"], cat["veval"], clr=cat["clr"])
            b.RunSteps(3)
            if tune:
                b.Autotune(2)
            b.RunSteps(5)
            outs.append(b.GetBuffer(F.FPOS))
    assert_bit_equal(outs[1], outs[0], "autotuned batch")


def test_batch_of_32_scenes_over_100_steps_matches_each_scene_alone():
    """The batched workload's shape at test size: 32 scenes of 2,048..65,536
    points (log-uniform, own box, grid, viscosity and rest density) stepped
    100 times as one batch (graph replay) and one at a time, both with the
    same pinned non-default launch shapes; every scene's final state is
    bit-identical."""
    scs = scenes.batch_scenes(nscenes=32, seed=17)
    cat = scenes.concat(scs)
    shapes = {"density": 384, "force": 96, "sort": 128, "sort_cells": 2}
    with F.FluidSystem.batch([sc.params for sc in scs], [sc.n for sc in scs]) as b:
        b.SetParticles(cat["pos"], cat["vel"], cat["veval"], clr=cat["clr"])
        b.SetLaunchShapes(**shapes)
        assert b.LaunchShapes() == shapes
        b.RunSteps(100)
        b.Sync()
        st = b.state()
        assert b.IntegrityCheck() == 0
        infos = [b.SceneInfo(k) for k in range(len(scs))]
    for k, sc in enumerate(scs):
        with F.FluidSystem(sc.params, sc.n) as s:
            s.SetParticles(sc.pos, sc.vel, sc.veval, clr=sc.clr)
            s.SetLaunchShapes(**shapes)
            s.RunSteps(100)
            s.Sync()
            want = s.state()
        got = per_scene(st, infos[k])
        for f in FIELDS:
            assert_bit_equal(got[f], want[f], f"scene {k} {f}")
