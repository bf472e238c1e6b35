"""GPU parity, through the C ABI, for collider Offsets (colliders.go:44,62,
173-176, 302-304) and static infinite-mass bodies (the backboard of
examples/ballistic.go:183-187): bit-identical to the oracle in both forms."""
import numpy as np
import pytest

from cubez_gb300 import scenes
from oracle.oracle import FP32 as ORC_FP32
from oracle.oracle import FP64 as ORC_FP64
from oracle.oracle import OracleBatch
from tests.test_gpu_parity import assert_bodies_equal, assert_contacts_equal

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0


def _pair(scene, form, **kw):
    from cubez_gb300.batch import WorldBatch
    return (WorldBatch.from_scene(scene, form=form, **kw),
            OracleBatch(scene, form=ORC_FP64 if form == 0 else ORC_FP32))


@pytest.mark.parametrize("form", [0, 1])
def test_offsets_bit_exact(form, cuda_lib):
    """Rigid and scaled Offsets, small worlds and two 72-body worlds (the
    large-world resolver) in one batch, stepped through the captured graphs."""
    sc = scenes.Scene.concat([scenes.offsets(num_worlds=16, bodies=24, seed=41, nonrigid=0.25),
                              scenes.offsets(num_worlds=2, bodies=72, seed=42, nonrigid=0.25)])
    gpu, ref = _pair(sc, form)
    for steps in (1, 59, 60):
        gpu.step(steps, DT)
        ref.step(steps, DT)
        assert_bodies_equal(gpu.download(), ref.bodies())
    # the narrowphase right after an integrate, as in the frame loop (the
    # oracle's collider transforms are those of the last Integrate)
    gpu.integrate(DT)
    ref.integrate(DT)
    gpu.narrowphase()
    ref.narrowphase()
    assert_contacts_equal(gpu, ref, sc.num_worlds)
    assert gpu.contact_counts().sum() > 0
    gpu.close()


def test_offset_known_answers(cuda_lib):
    """The oracle's known answers (a sphere moved down by its Offset touches
    the plane; a long cube turned on end by its Offset has 4 contacts 1 m
    deep) on the GPU."""
    from tests.test_offsets import _single
    down = np.array([1.0, 0, 0, 0, 1.0, 0, 0, 0, 1.0, 0, -0.6, 0])
    turn = np.array([0.0, 1.0, 0, -1.0, 0.0, 0, 0, 0, 1.0, 0, 0, 0])
    for sc, n in ((_single(scenes.SPHERE, radius=0.5, y=1.0, offset=down), 1),
                  (_single(scenes.CUBE, half=(2.0, 0.5, 0.5), y=1.0, offset=turn), 4)):
        gpu, ref = _pair(sc, 0)
        gpu.narrowphase()
        ref.narrowphase()
        assert_contacts_equal(gpu, ref, 1)
        assert gpu.contact_counts()[0] == n
        gpu.close()


@pytest.mark.parametrize("form", [0, 1])
def test_offset_download(form, cuda_lib):
    from cubez_gb300.batch import WorldBatch
    sc = scenes.offsets(num_worlds=3, bodies=7, seed=43)
    b = WorldBatch.from_scene(sc, form=form)
    got = b.download(fields=("collider_offset",))["collider_offset"]
    expect = sc.collider_offset if form == 0 else sc.collider_offset.astype(np.float32).astype(np.float64)
    assert np.array_equal(got, expect)
    plain = sc.copy()
    plain.collider_offset = None
    b.upload(plain)
    got = b.download(fields=("collider_offset",))["collider_offset"]
    assert np.array_equal(got, np.tile(scenes.IDENTITY_OFFSET, (sc.num_bodies, 1)))
    b.close()


def test_offset_upload_switch(cuda_lib):
    """Uploading without Offsets after a rollout with them (and back) takes
    effect in the next captured rollout."""
    from cubez_gb300.batch import WorldBatch
    sc = scenes.offsets(num_worlds=8, bodies=20, seed=44)
    plain = sc.copy()
    plain.collider_offset = None
    b = WorldBatch.from_scene(sc, form=0)
    b.step(20, DT)
    b.upload(plain)
    b.step(20, DT)
    fresh = WorldBatch.from_scene(plain, form=0)
    fresh.step(20, DT)
    assert_bodies_equal(b.download(), fresh.download())
    b.upload(sc)
    b.step(20, DT)
    ref = OracleBatch(sc)
    ref.step(20, DT)
    assert_bodies_equal(b.download(), ref.bodies())
    b.close()
    fresh.close()


@pytest.mark.parametrize("form", [0, 1])
def test_ballistic_loop_bit_exact(form, cuda_lib):
    """examples/ballistic.go's frame through the batch API: integrate, the
    example's test order through cz_collide, ResolveContacts with
    len(contacts) * 8; the static backboard never moves."""
    sc = scenes.ballistic(num_worlds=12, bullets=8, seed=45)
    gpu, ref = _pair(sc, form, iteration_multiplier=8)
    units = scenes.ballistic_units(int(sc.counts[0]))
    boards = [sc.world_slice(w).start + 1 for w in range(sc.num_worlds)]
    start = gpu.download()
    total = 0
    for fr in range(150):
        gpu.integrate(DT)
        ref.integrate(DT)
        for w in range(sc.num_worlds):
            gpu.collide(w, units)
            ref.collide(w, units)
        total += int(gpu.contact_counts().sum())
        gpu.resolve(DT)
        ref.resolve(DT, iter_mult=8)
        if fr % 10 == 9:
            g = gpu.download()
            assert_bodies_equal(g, ref.bodies())
            for k in ("position", "orientation"):
                assert np.array_equal(g[k][boards], start[k][boards]), k
    assert total > 100
    gpu.close()
