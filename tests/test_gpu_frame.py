"""The fused frame (cz_tuning.fused_frame): each frame one launch, in which
a warp takes a world from the device queue, integrates its bodies, runs its
narrowphase and resolves its contacts, then takes the next.  Same bits as the
three-launch frame and as the oracle, in both forms; it is taken only where
the batch runs one world per warp with the plain resolver."""
import numpy as np
import pytest

from cubez_gb300 import scenes
from oracle.oracle import OracleBatch

from tests.test_gpu_parity import STATE, assert_bodies_equal, assert_contacts_equal

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0


def _fused(scene, form):
    from cubez_gb300.batch import WorldBatch
    b = WorldBatch.from_scene(scene, form=form)
    b.set_tuning(resolver_lanes=32, fused_frame=1)
    assert b.get_tuning()["fused_frame"] == 1
    return b


@pytest.mark.parametrize("form", [0, 1])
def test_fused_frame_bit_exact(form, cuda_lib):
    scene = scenes.mixed(num_worlds=48, seed=42, min_bodies=8, max_bodies=64)
    gpu, ref = _fused(scene, form), OracleBatch(scene, form=form)
    for frames in (1, 59, 90):
        gpu.step(frames, DT)
        ref.step(frames, DT)
        assert_bodies_equal(gpu.download(), ref.bodies())
        assert_contacts_equal(gpu, ref, scene.num_worlds)
        gs, rs = gpu.stats(), ref.stats()
        np.testing.assert_array_equal(gs["pos_iterations"], rs["pos_iterations"])
        np.testing.assert_array_equal(gs["vel_iterations"], rs["vel_iterations"])
    assert ref.stats()["vel_iterations"].sum() > 0


@pytest.mark.parametrize("form", [0, 1])
def test_fused_frame_sleep_offsets_and_timed(form, cuda_lib):
    """Sleeping bodies, collider Offsets, and the timed rollout (its time is
    reported as the resolve phase)."""
    sleepy = scenes.mixed(num_worlds=16, seed=27, min_bodies=8, max_bodies=40)
    sleepy.can_sleep[:] = 1
    for scene in (sleepy, scenes.offsets(num_worlds=8, bodies=24, seed=9)):
        gpu, ref = _fused(scene, form), OracleBatch(scene, form=form)
        if scene is sleepy:  # bodies settle and fall asleep from about frame 300
            gpu.step(360, DT)
            ref.step(360, DT)
        gpu.prepare_rollout(120, DT)
        tot, ph = gpu.step_timed(120, DT)
        ref.step(120, DT)
        g = gpu.download()
        assert_bodies_equal(g, ref.bodies(), STATE + ("motion", "is_awake"))
        assert ph[0] == 0.0 and ph[1] == 0.0 and ph[2] > 0.0
        if scene is sleepy:
            assert (g["is_awake"] == 0).sum() > 100  # bodies went to sleep


def test_fused_frame_launches_and_fallbacks(cuda_lib):
    from cubez_gb300 import _lib
    from cubez_gb300.batch import WorldBatch
    from cubez_gb300.learned import BLOB, OFF_IS, OFF_OS, set_warm_start
    scene = scenes.mixed(num_worlds=64, seed=33)
    b = _fused(scene, 1)
    b.prepare_rollout(10, DT)
    before = _lib.kernel_launches()
    b.step(10, DT)
    assert _lib.kernel_launches() - before == 10 * 2  # the frame, the queue reorder
    # two worlds per warp: the three-launch frame
    b.set_tuning(resolver_lanes=16)
    b.prepare_rollout(10, DT)
    before = _lib.kernel_launches()
    b.step(10, DT)
    assert _lib.kernel_launches() - before == 10 * 4
    # the learned warm start: the three-launch frame with the features kernel
    w = WorldBatch.from_scene(scene, form=1)
    w.set_tuning(resolver_lanes=32, fused_frame=1)
    blob = np.zeros(BLOB, np.float32)
    blob[OFF_IS:OFF_IS + 18] = 1.0
    blob[OFF_OS:OFF_OS + 3] = 1.0
    set_warm_start(w, blob)
    w.prepare_rollout(10, DT)
    before = _lib.kernel_launches()
    w.step(10, DT)
    assert _lib.kernel_launches() - before == 10 * 5
    # a world above 64 bodies: the three-launch frame and the large-world resolver
    big = _fused(scenes.piles(num_worlds=2, seed=51, nx=5, nz=4, ny=4), 1)
    big.prepare_rollout(5, DT)
    before = _lib.kernel_launches()
    big.step(5, DT)
    assert _lib.kernel_launches() - before == 5 * 3
