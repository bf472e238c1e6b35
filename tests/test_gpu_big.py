"""Worlds larger than the resolver's shared-memory slot (more than 64
bodies) go through k_resolve_big: bodies and contacts in global memory,
per-body contact lists for the per-iteration update, 32 lanes per world or
16 (two worlds per warp in lockstep).  Same bar as the small worlds:
bit-identical with the oracle in both forms, alone and mixed with small
worlds in one batch."""
import numpy as np
import pytest

from cubez_gb300 import scenes
from oracle.oracle import FP32 as ORC_FP32
from oracle.oracle import FP64 as ORC_FP64
from oracle.oracle import OracleBatch

from tests.test_gpu_parity import STATE, assert_bodies_equal, assert_contacts_equal

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0


def _run(scene, form, frames, settle=0, lanes=32):
    from cubez_gb300.batch import WorldBatch
    ref = OracleBatch(scene, form=ORC_FP64 if form == 0 else ORC_FP32)
    if settle:
        ref.step(settle, DT)
        st = ref.bodies()
        scene = scene.copy()
        for k in STATE:
            setattr(scene, k, st[k])
        ref = OracleBatch(scene, form=ORC_FP64 if form == 0 else ORC_FP32)
    gpu = WorldBatch.from_scene(scene, form=form)
    gpu.set_tuning(large_world_lanes=lanes)
    assert gpu.get_tuning()["large_world_lanes"] == lanes
    gpu.step(frames, DT)
    ref.step(frames, DT)
    return gpu, ref, scene


@pytest.mark.parametrize("lanes", [16, 32])
@pytest.mark.parametrize("form", [0, 1])
def test_pile_worlds_bit_exact(form, lanes, cuda_lib):
    # 80 cubes per world on a 5 x 4 x 4 lattice, dropped onto the plane; with
    # 16 lanes the third world shares its warp with an empty group
    scene = scenes.piles(num_worlds=3, seed=51, nx=5, nz=4, ny=4)
    assert scene.counts.min() > 64
    gpu, ref, _ = _run(scene, form, frames=45, lanes=lanes)
    g, r = gpu.download(), ref.bodies()
    assert_bodies_equal(g, r)
    gs, rs = gpu.stats(), ref.stats()
    assert rs["contacts"].min() > 100           # the piles are resting on the plane and on each other
    assert rs["vel_iterations"].min() > 50
    np.testing.assert_array_equal(gpu.contact_counts(), rs["contacts"])
    for k in ("pos_iterations", "vel_iterations"):
        np.testing.assert_array_equal(gs[k], rs[k])
    assert (gs["status"] == 0).all()
    assert_contacts_equal(gpu, ref, scene.num_worlds)


@pytest.mark.parametrize("lanes", [16, 32])
@pytest.mark.parametrize("form", [0, 1])
def test_small_and_big_worlds_in_one_batch(form, lanes, cuda_lib):
    scene = scenes.mixed(num_worlds=10, seed=52, min_bodies=30, max_bodies=110)
    assert (scene.counts > 64).any() and (scene.counts <= 64).any()
    gpu, ref, _ = _run(scene, form, frames=20, settle=100, lanes=lanes)
    assert_bodies_equal(gpu.download(), ref.bodies())
    gs, rs = gpu.stats(), ref.stats()
    assert rs["vel_iterations"].sum() > 100
    np.testing.assert_array_equal(gpu.contact_counts(), rs["contacts"])
    for k in ("pos_iterations", "vel_iterations"):
        np.testing.assert_array_equal(gs[k], rs[k])


def test_big_world_launch_accounting(cuda_lib):
    from cubez_gb300 import _lib
    from cubez_gb300.batch import FORM_FP32, WorldBatch
    scene = scenes.piles(num_worlds=2, seed=53, nx=5, nz=4, ny=4)
    b = WorldBatch.from_scene(scene, form=FORM_FP32)
    b.step(1, DT)
    n0 = _lib.kernel_launches()
    b.step(5, DT)
    assert _lib.kernel_launches() - n0 == 5 * 3  # integrate, narrowphase, k_resolve_big
