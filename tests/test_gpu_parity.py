"""Parity of the CUDA path (through the C ABI) with the oracle.

Plain form (float64): bit-identical contact lists (count, body pair, order,
point, normal, penetration) and bit-identical body state after 1, 60 and 240
steps.  The acceptance tolerance for body state is 1e-9 relative; the tests
assert bit equality, which is stronger.

Precision form (float32 with float64 islands): bit-identical to the oracle's
precision-form instantiation, which evaluates the same operations in the same
types.
"""
import numpy as np
import pytest

from cubez_gb300 import scenes
from oracle.oracle import FP32 as ORC_FP32
from oracle.oracle import FP64 as ORC_FP64
from oracle.oracle import OracleBatch

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0
STATE = ("position", "orientation", "velocity", "rotation")


def _pair(scene, form, cuda_lib):
    from cubez_gb300.batch import WorldBatch
    gpu = WorldBatch.from_scene(scene, form=form)
    ref = OracleBatch(scene, form=ORC_FP64 if form == 0 else ORC_FP32)
    return gpu, ref


def assert_bodies_equal(g, r, fields=STATE):
    for k in fields:
        a, b = g[k], r[k]
        if not np.array_equal(a, b):
            bad = np.argwhere(~((a == b) | (np.isnan(a) & np.isnan(b))))
            i = bad[0][0]
            raise AssertionError("%s differs at body %d: gpu=%r oracle=%r (%d entries differ)" %
                                 (k, i, a[i], b[i], len(bad)))


def assert_contacts_equal(gpu, ref, num_worlds):
    counts = gpu.contact_counts()
    for w in range(num_worlds):
        gc = gpu.contacts(w)
        rc = ref.contacts(w)
        assert counts[w] == len(rc["penetration"]), "world %d: count %d vs %d" % (w, counts[w], len(rc["penetration"]))
        assert np.array_equal(gc["bodies"], rc["bodies"]), "world %d: body pairs/order differ" % w
        for k in ("point", "normal", "penetration"):
            assert np.array_equal(gc[k], rc[k]), "world %d: contact %s differs" % (w, k)
        assert np.all(gc["friction"] == 0.9 if gpu.form == 0 else gc["friction"] == np.float32(0.9))


@pytest.mark.parametrize("form", [0, 1])
def test_integrate_bit_exact(form, cuda_lib):
    scene = scenes.mixed(num_worlds=16, seed=21)
    gpu, ref = _pair(scene, form, cuda_lib)
    for _ in range(3):
        gpu.integrate(DT)
        ref.integrate(DT)
    g = gpu.download()
    r = ref.bodies()
    assert_bodies_equal(g, r, STATE + ("iit_world",) if False else STATE)
    assert np.array_equal(g["inverse_inertia_world"], r["iit_world"])


@pytest.mark.parametrize("form", [0, 1])
def test_narrowphase_bit_exact(form, cuda_lib):
    scene = scenes.mixed(num_worlds=24, seed=22)
    gpu, ref = _pair(scene, form, cuda_lib)
    # let bodies fall into contact first, with the oracle alone
    ref.step(90, DT)
    st = ref.bodies()
    moved = scene.copy()
    for k in ("position", "orientation", "velocity", "rotation"):
        setattr(moved, k, st[k])
    gpu, ref = _pair(moved, form, cuda_lib)
    gpu.integrate(DT)
    ref.integrate(DT)
    gpu.narrowphase()
    ref.narrowphase()
    assert sum(len(ref.contacts(w)["penetration"]) for w in range(moved.num_worlds)) > 50
    assert_contacts_equal(gpu, ref, moved.num_worlds)


@pytest.mark.parametrize("form", [0, 1])
def test_one_step_bit_exact(form, cuda_lib):
    scene = scenes.mixed(num_worlds=32, seed=23)
    gpu, ref = _pair(scene, form, cuda_lib)
    gpu.step(1, DT)
    ref.step(1, DT)
    assert_contacts_equal(gpu, ref, scene.num_worlds)
    assert_bodies_equal(gpu.download(), ref.bodies())
    gs, rs = gpu.stats(), ref.stats()
    assert np.array_equal(gs["pos_iterations"], rs["pos_iterations"])
    assert np.array_equal(gs["vel_iterations"], rs["vel_iterations"])


@pytest.mark.parametrize("form", [0, 1])
def test_sixty_steps_bit_exact(form, cuda_lib):
    scene = scenes.mixed(num_worlds=48, seed=24)
    gpu, ref = _pair(scene, form, cuda_lib)
    gpu.step(60, DT)
    ref.step(60, DT)
    assert_bodies_equal(gpu.download(), ref.bodies())
    assert_contacts_equal(gpu, ref, scene.num_worlds)
    gs, rs = gpu.stats(), ref.stats()
    assert np.array_equal(gs["vel_iterations"], rs["vel_iterations"])


def test_cubedrop_240_steps_fp64(cuda_lib):
    scene = scenes.cubedrop()
    gpu, ref = _pair(scene, 0, cuda_lib)
    for chunk in range(4):
        gpu.step(60, DT)
        ref.step(60, DT)
        assert_bodies_equal(gpu.download(), ref.bodies())
    assert_contacts_equal(gpu, ref, 1)
    assert ref.stats()["contacts"][0] > 40  # the pile is resting on the plane


def test_precision_scene_fp64_step(cuda_lib):
    scene = scenes.precision(num_worlds=64, seed=25)
    gpu, ref = _pair(scene, 0, cuda_lib)
    gpu.step(120, DT)
    ref.step(120, DT, threads=8)
    assert_bodies_equal(gpu.download(), ref.bodies())
    assert_contacts_equal(gpu, ref, scene.num_worlds)


@pytest.mark.parametrize("form", [0, 1])
@pytest.mark.parametrize("lanes", [4, 8, 16, 32])
def test_resolver_lanes_per_world_bit_exact(form, lanes, cuda_lib):
    """Every lanes-per-world setting of the resolver gives the oracle's bits;
    a small shared-memory contact tile forces some worlds onto the global
    working rows as well."""
    scene = scenes.mixed(num_worlds=40, seed=26)
    ref = OracleBatch(scene, form=ORC_FP64 if form == 0 else ORC_FP32)
    ref.step(150, DT)  # settle: piles with many contacts
    st = ref.bodies()
    moved = scene.copy()
    for k in ("position", "orientation", "velocity", "rotation"):
        setattr(moved, k, st[k])
    gpu, ref = _pair(moved, form, cuda_lib)
    gpu.set_tuning(resolver_lanes=lanes, resolver_contacts=32)
    assert gpu.get_tuning()["resolver_lanes"] == lanes
    gpu.step(30, DT)
    ref.step(30, DT)
    assert_bodies_equal(gpu.download(), ref.bodies())
    gs, rs = gpu.stats(), ref.stats()
    assert np.array_equal(gs["pos_iterations"], rs["pos_iterations"])
    assert np.array_equal(gs["vel_iterations"], rs["vel_iterations"])
    assert rs["contacts"].max() > 32  # some worlds exceed the shared-memory tile


@pytest.mark.parametrize("form", [0, 1])
def test_sleeping_bodies_bit_exact(form, cuda_lib):
    """CanSleep on (rigidbody.go:248-258): motion average, SetAwake(false)
    zeroing the velocities, matchAwakeState waking a partner and the asleep
    body's CalculateDerivedData inside applyPositionChange (contact.go:185-202,
    380-382).  The configurations disable sleeping; this exercises the path."""
    scene = scenes.mixed(num_worlds=24, seed=27, min_bodies=8, max_bodies=40)
    scene.can_sleep[:] = 1
    gpu, ref = _pair(scene, form, cuda_lib)
    for chunk in range(8):
        gpu.step(60, DT)
        ref.step(60, DT)
        g, r = gpu.download(), ref.bodies()
        assert_bodies_equal(g, r, STATE + ("motion", "is_awake"))
    assert (g["is_awake"] == 0).sum() > 100  # bodies went to sleep (326 of 585 in the oracle)
