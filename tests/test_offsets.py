"""Collider Offsets and static (infinite-mass) bodies on the oracle, CPU only.

The reference's colliders carry an Offset (colliders.go:44,62) multiplied into
their transform (colliders.go:173-176, 302-304); its ballistic example keeps a
backboard of infinite mass that it never integrates (examples/ballistic.go:
183-187).  These tests pin the oracle's handling of both, which the GPU
parity tests then compare against.
"""
import numpy as np
import pytest

from cubez_gb300 import scenes
from oracle.oracle import FP32, FP64, OracleBatch

DT = 1.0 / 60.0
STATE = ("position", "orientation", "velocity", "rotation")


def _single(shape, half=(0.5, 0.5, 0.5), radius=0.5, y=1.0, offset=None):
    """One body (the ballistic cube's mass properties) at (0, y, 0), at rest."""
    sc = scenes.ballistic(num_worlds=1, bullets=0)
    one = {k: np.array(getattr(sc, k)[:1]) for k in sc.FIELDS}
    one["shape"][:] = shape
    one["half_size"][:] = half
    one["radius"][:] = radius
    one["position"][:] = (0.0, y, 0.0)
    if offset is not None:
        one["collider_offset"] = np.asarray(offset, np.float64).reshape(1, 12)
    return scenes.Scene([1], sc.plane, **one)


@pytest.mark.parametrize("form", [FP64, FP32])
def test_identity_offset_equals_none(form, oracle_lib):
    plain = scenes.mixed(num_worlds=6, seed=31, min_bodies=10, max_bodies=20)
    ident = plain.copy()
    ident.collider_offset = np.tile(scenes.IDENTITY_OFFSET, (plain.num_bodies, 1))
    a, b = OracleBatch(plain, form=form), OracleBatch(ident, form=form)
    a.step(60, DT)
    b.step(60, DT)
    ra, rb = a.bodies(), b.bodies()
    for k in STATE:
        assert np.array_equal(ra[k], rb[k]), k
    assert np.array_equal(a.stats()["contacts"], b.stats()["contacts"])


def test_offset_known_answers(oracle_lib):
    """A sphere whose Offset moves it 0.6 m down touches the plane: the
    half-space test (colliders.go:180-207) sees the collider centre, not the
    body's.  A 2 x 0.5 x 0.5 cube whose Offset turns it 90 degrees about z
    stands on end: 4 vertices 1 m under the plane instead of none."""
    down = np.array([1.0, 0, 0, 0, 1.0, 0, 0, 0, 1.0, 0, -0.6, 0])
    o = OracleBatch(_single(scenes.SPHERE, radius=0.5, y=1.0, offset=down))
    o.narrowphase()
    c = o.contacts(0)
    assert len(c["penetration"]) == 1
    centre_y = 1.0 + -0.6
    d = centre_y - 0.5
    assert c["penetration"][0] == -d
    assert np.array_equal(c["point"][0], [0.0, (d - 0.5) + centre_y, 0.0])
    o = OracleBatch(_single(scenes.SPHERE, radius=0.5, y=1.0))
    o.narrowphase()
    assert len(o.contacts(0)["penetration"]) == 0

    turn = np.array([0.0, 1.0, 0, -1.0, 0.0, 0, 0, 0, 1.0, 0, 0, 0])  # x axis -> y, y axis -> -x
    o = OracleBatch(_single(scenes.CUBE, half=(2.0, 0.5, 0.5), y=1.0, offset=turn))
    o.narrowphase()
    c = o.contacts(0)
    assert len(c["penetration"]) == 4
    assert np.all(c["penetration"] == 1.0)
    o = OracleBatch(_single(scenes.CUBE, half=(2.0, 0.5, 0.5), y=1.0))
    o.narrowphase()
    assert len(o.contacts(0)["penetration"]) == 0


@pytest.mark.parametrize("form", [FP64, FP32])
def test_offsets_change_the_run(form, oracle_lib):
    sc = scenes.offsets(num_worlds=4, bodies=16, seed=32)
    plain = sc.copy()
    plain.collider_offset = None
    a, b = OracleBatch(sc, form=form), OracleBatch(plain, form=form)
    a.step(90, DT)
    b.step(90, DT)
    assert not np.array_equal(a.bodies()["position"], b.bodies()["position"])
    assert a.stats()["contacts"].sum() > 0


@pytest.mark.parametrize("form", [FP64, FP32])
def test_static_backboard_stays_put(form, oracle_lib):
    """ballistic(): integrating the static backboard every frame leaves its
    state bit for bit as set up, while the bullets hit it."""
    sc = scenes.ballistic(num_worlds=3, bullets=6, seed=33)
    o = OracleBatch(sc, form=form)
    units = scenes.ballistic_units(int(sc.counts[0]))
    start = o.bodies()
    boards = [sc.world_slice(w).start + 1 for w in range(sc.num_worlds)]
    touched = 0
    for _ in range(150):
        o.integrate(DT)
        for w in range(sc.num_worlds):
            o.collide(w, units)
            c = o.contacts(w)
            touched += int(np.any(c["bodies"] == 1))
        o.resolve(DT, iter_mult=8)
        now = o.bodies()
        for k in ("position", "orientation"):
            assert np.array_equal(now[k][boards], start[k][boards]), k
        assert not np.any(now["velocity"][boards]) and not np.any(now["rotation"][boards])
    assert touched > 0  # something reached the backboard


def test_ballistic_units_order():
    u = scenes.ballistic_units(4)
    assert u.tolist() == [[0, -1], [0, 1], [2, -1], [0, 2], [1, 2], [3, 2], [3, -1], [0, 3], [1, 3], [2, 3]]


def test_scene_offsets_survive_copy_concat_subset():
    a = scenes.offsets(num_worlds=2, bodies=5, seed=34)
    b = scenes.mixed(num_worlds=2, seed=35, min_bodies=3, max_bodies=4)
    c = scenes.Scene.concat([a, b])
    assert c.collider_offset.shape == (c.num_bodies, 12)
    assert np.array_equal(c.collider_offset[:a.num_bodies], a.collider_offset)
    assert np.array_equal(c.collider_offset[a.num_bodies:], np.tile(scenes.IDENTITY_OFFSET, (b.num_bodies, 1)))
    s = c.subset([1, 2])
    assert np.array_equal(s.collider_offset[:5], a.collider_offset[5:])
    assert a.copy().collider_offset is not a.collider_offset
    assert scenes.Scene.concat([b, b]).collider_offset is None
