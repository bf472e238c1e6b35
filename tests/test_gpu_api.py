"""The single-world ResolveContacts entry point and the error paths of the C
ABI, on the GPU.  Errors are status codes read on the host; no test makes the
device fault."""
import numpy as np
import pytest

from cubez_gb300 import scenes
from oracle.oracle import OracleBatch
from tests import cases

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0
_DT = {"is_awake": np.uint8, "can_sleep": np.uint8, "shape": np.int32}


def frame_state(scene, frames, form=0):
    """The oracle `frames` frames into `scene`'s loop and then Integrate'd once
    more: the body state ResolveContacts meets in the next frame of
    examples/cubedrop.go:69-75, so the resolver has work.  Returns the oracle
    batch (its last-frame accelerations and world inertia are the frame's) and
    the moved scene."""
    ref = OracleBatch(scene, form=form)
    ref.step(frames, DT)
    ref.integrate(DT)
    st = ref.bodies()
    moved = scene.copy()
    for k in ("position", "orientation", "velocity", "rotation", "motion", "is_awake"):
        setattr(moved, k, np.array(st[k], dtype=_DT.get(k, np.float64), copy=True))
    return ref, moved, st


def scene_with_contacts(seed=31, bodies=24, frames=150, form=0):
    """A mixed world mid-rollout and the contacts the narrowphase gives for it,
    with the colliders' friction 0.9 and restitution 0.1."""
    sc = scenes.mixed(num_worlds=1, seed=seed, min_bodies=bodies, max_bodies=bodies)
    _, moved, _ = frame_state(sc, frames, form)
    ref = OracleBatch(moved, form=form)
    ref.narrowphase()
    c = ref.contacts(0)
    c["friction"] = np.full(len(c["penetration"]), 0.9)
    c["restitution"] = np.full(len(c["penetration"]), 0.1)
    return moved, c


def host_arrays(scene):
    """Fresh copies of the scene's body arrays: the entry points write their
    results back in place, and the oracle must start from the untouched scene."""
    return {k: np.array(getattr(scene, k), dtype=_DT.get(k, np.float64), copy=True) for k in scene.FIELDS}


def cz_contacts(c):
    from cubez_gb300 import _lib
    n = len(c["penetration"])
    arr = (_lib.Contact * n)()
    for i in range(n):
        arr[i].body[0], arr[i].body[1] = int(c["bodies"][i][0]), int(c["bodies"][i][1])
        arr[i].friction, arr[i].restitution = float(c["friction"][i]), float(c["restitution"][i])
        for k in range(3):
            arr[i].point[k] = float(c["point"][i][k])
            arr[i].normal[k] = float(c["normal"][i][k])
        arr[i].penetration = float(c["penetration"][i])
    return arr


def resolve_both(scene, c, max_iterations, form=0, ref=None, extra=None):
    """cz_resolve_contacts on copies of the scene's arrays, and the oracle's
    ResolveContacts on the same contacts.  `ref` is an oracle batch holding the
    same state (default: a fresh one built from the scene, whose last-frame
    accelerations are zero, as a NULL last_frame_acceleration is); `extra`
    adds optional body arrays (last_frame_acceleration, inverse_inertia_world)."""
    import ctypes as C

    from cubez_gb300.batch import WorldBatch, bodies_struct
    gpu = WorldBatch(scene.counts, form=form, plane=scene.plane)
    arrays = host_arrays(scene)
    arrays["inverse_inertia_world"] = None
    for k, v in (extra or {}).items():
        arrays[k] = np.array(v, dtype=np.float64, copy=True)
    s = bodies_struct(arrays)
    arr = cz_contacts(c)
    st = gpu.L.cz_resolve_contacts(gpu.h, max_iterations, C.cast(arr, C.c_void_p), len(arr), DT, C.byref(s))
    gpu.close()
    if ref is None:
        ref = OracleBatch(scene, form=form)
    ref.set_contacts(0, c)
    assert ref.resolve_fixed(max_iterations, DT) == 0
    return st, arrays, arr, ref


def assert_matches_oracle(arrays, arr, ref, fields=("position", "orientation", "velocity", "rotation")):
    r = ref.bodies()
    for k in fields:
        np.testing.assert_array_equal(arrays[k], r[k], err_msg=k)
    rc = ref.resolved_contacts(0)
    n = len(arr)
    np.testing.assert_array_equal(np.array([arr[i].penetration for i in range(n)]), rc["penetration"])
    np.testing.assert_array_equal(np.array([list(arr[i].normal) for i in range(n)]), rc["normal"])
    np.testing.assert_array_equal(np.array([list(arr[i].body) for i in range(n)]), rc["bodies"])


@pytest.mark.parametrize("form", [0, 1])
@pytest.mark.parametrize("seed,bodies,frames", [(31, 24, 150), (41, 64, 150)])
def test_resolve_contacts_matches_oracle(form, seed, bodies, frames, cuda_lib):
    scene, c = scene_with_contacts(seed, bodies, frames, form)
    n = len(c["penetration"])
    assert n > 20
    st, arrays, arr, ref = resolve_both(scene, c, 4 * n, form)
    assert st == 0, cuda_lib.cz_last_error()
    s = ref.stats()
    assert s["pos_iterations"][0] > 0 and s["vel_iterations"][0] > 0   # the resolver had work
    assert_matches_oracle(arrays, arr, ref)


def frame_inputs(form, seed=32):
    """A world mid-rollout with the optional inputs a frame loop passes after
    Integrate: lastFrameAccelleration = Acceleration + forceAccum * inverseMass
    (rigidbody.go:222-223), here gravity plus a horizontal push so that its
    tangential part reaches the contact velocities (contact.go:172-180), and
    the world inverse inertia.  Returns the scene, the contacts, the optional
    arrays and an oracle batch holding the same state."""
    sc = scenes.mixed(num_worlds=1, seed=seed, min_bodies=24, max_bodies=24)
    _, moved, st = frame_state(sc, 150, form)
    rng = np.random.default_rng(5)
    n = moved.num_bodies
    lfa = moved.acceleration + np.stack([rng.uniform(-3, 3, n), np.zeros(n), rng.uniform(-3, 3, n)], axis=1)
    ref = OracleBatch(moved, form=form, last_frame_acceleration=lfa)
    ref.narrowphase()
    c = ref.contacts(0)
    c["friction"] = np.full(len(c["penetration"]), 0.9)
    c["restitution"] = np.full(len(c["penetration"]), 0.1)
    extra = {"last_frame_acceleration": lfa, "inverse_inertia_world": st["iit_world"]}
    return moved, c, extra, ref


@pytest.mark.parametrize("form", [0, 1])
def test_resolve_contacts_with_frame_inputs(form, cuda_lib):
    """last_frame_acceleration (the restitution and local-velocity terms of
    contact.go:87-112,159-182) and an explicit world inverse inertia against
    the oracle given the same values."""
    moved, c, extra, ref = frame_inputs(form)
    n = len(c["penetration"])
    st, arrays, arr, ref = resolve_both(moved, c, 4 * n, form, ref=ref, extra=extra)
    assert st == 0, cuda_lib.cz_last_error()
    assert ref.stats()["vel_iterations"][0] > 0
    assert_matches_oracle(arrays, arr, ref)
    # the accelerations matter: without them the result differs
    st0, arrays0, _, _ = resolve_both(moved, c, 4 * n, form)
    assert st0 == 0
    assert not np.array_equal(arrays0["velocity"], arrays["velocity"])


def test_resolve_contacts_swaps_nil_first_body(cuda_lib):
    scene = cases.cube_resting()
    c = {"bodies": np.array([[-1, 0]], np.int32), "point": np.array([[0.5, -0.02, 0.5]]),
         "normal": np.array([[0.0, -1.0, 0.0]]), "penetration": np.array([0.02]),
         "friction": np.array([0.9]), "restitution": np.array([0.1])}
    st, arrays, arr, ref = resolve_both(scene, c, 4, 0)
    assert st == 0
    assert list(arr[0].body) == [0, -1]          # calculateInternals, contact.go:61-65
    assert list(arr[0].normal) == [0.0, 1.0, 0.0]
    assert ref.stats()["pos_iterations"][0] > 0
    assert_matches_oracle(arrays, arr, ref)


def test_resolve_contacts_zero_iterations_and_guards(cuda_lib):
    scene, c = scene_with_contacts(seed=32)
    n = len(c["penetration"])
    # the same contacts need iterations when allowed some
    ref = OracleBatch(scene)
    ref.set_contacts(0, c)
    ref.resolve_fixed(4 * n, DT)
    assert ref.stats()["pos_iterations"][0] > 0
    st, arrays, arr, ref = resolve_both(scene, c, 0, 0)
    assert st == 0
    # no iteration: no body moves (prepareContacts alone mutates no body)
    for k in ("position", "orientation", "velocity", "rotation"):
        np.testing.assert_array_equal(arrays[k], getattr(scene, k))
    assert_matches_oracle(arrays, arr, ref)


def test_capacity_overflow_is_reported(cuda_lib):
    from cubez_gb300 import CubezError
    from cubez_gb300.batch import WorldBatch
    scene = cases.cube_resting()
    b = WorldBatch(scene.counts, plane=scene.plane, contact_capacity=2)
    b.upload(scene)
    with pytest.raises(CubezError) as e:
        b.narrowphase()
    assert e.value.status == 5  # CZ_ERR_CAPACITY
    assert b.contact_counts()[0] == 4
    assert b.stats()["status"][0] & 4


def test_nonfinite_box_state_is_reported(cuda_lib):
    from cubez_gb300 import CubezError
    from cubez_gb300.batch import WorldBatch
    scene = cases.cube_on_cube()
    scene.orientation = scene.orientation.copy()
    scene.orientation[1] = [np.nan, 0.0, 0.0, 0.0]
    b = WorldBatch(scene.counts, plane=scene.plane)
    b.upload(scene)
    with pytest.raises(CubezError) as e:
        b.narrowphase()
    assert e.value.status == 4  # CZ_ERR_NONFINITE: the reference would panic here
    # the batch stays usable: a finite state steps again
    b.upload(cases.cube_on_cube())
    b.step(2, DT)


def test_bad_arguments_on_a_live_batch(cuda_lib):
    import ctypes as C

    from cubez_gb300 import _lib
    from cubez_gb300.batch import WorldBatch
    scene = cases.sphere_pair()
    b = WorldBatch(scene.counts, plane=scene.plane)
    b.upload(scene)
    assert b.L.cz_download_contacts(b.h, 5, None, 0, None) == 1
    t = _lib.Tuning(48, 0, 0, 0, 0)
    assert b.L.cz_set_tuning(b.h, C.byref(t)) == 1  # not a multiple of 32
    t = _lib.Tuning(0, 0, 0, 0, 6)
    assert b.L.cz_set_tuning(b.h, C.byref(t)) == 1  # lanes per world must be 4, 8, 16 or 32
    t = _lib.Tuning(0, 0, 0, 0, 0, 0, 8)
    assert b.L.cz_set_tuning(b.h, C.byref(t)) == 1  # large-world lanes must be 16 or 32
    bad = {"bodies": np.array([[0, 7]], np.int32), "point": np.zeros((1, 3)), "normal": np.array([[1.0, 0, 0]]),
           "penetration": np.array([0.1]), "friction": np.array([0.9]), "restitution": np.array([0.1])}
    arr = cz_contacts(bad)
    from cubez_gb300.batch import bodies_struct
    s = bodies_struct({k: getattr(scene, k) for k in scene.FIELDS})
    assert b.L.cz_resolve_contacts(b.h, 4, C.cast(arr, C.c_void_p), 1, DT, C.byref(s)) == 1


def test_batches_with_different_tiles_coexist(cuda_lib):
    """A kernel's shared-memory limit is process-wide: a batch with a small
    tile created later must not stop an earlier batch with a large tile."""
    from cubez_gb300.batch import WorldBatch
    scene = scenes.mixed(num_worlds=16, seed=34)
    big = WorldBatch.from_scene(scene)
    big.set_tuning(resolver_lanes=8, resolver_contacts=256)
    small = WorldBatch.from_scene(scene)
    small.set_tuning(resolver_lanes=8, resolver_contacts=32)
    big.step(5, DT)
    small.step(5, DT)
    a, b = big.download(), small.download()
    np.testing.assert_array_equal(a["position"], b["position"])


def test_kernel_launch_accounting(cuda_lib):
    from cubez_gb300 import _lib
    from cubez_gb300.batch import WorldBatch
    scene = scenes.mixed(num_worlds=64, seed=33)
    b = WorldBatch.from_scene(scene)
    b.prepare_rollout(10, DT)
    before = _lib.kernel_launches()
    b.step(10, DT)
    assert _lib.kernel_launches() - before == 10 * 4  # integrate, narrowphase, resolve, queue reorder


@pytest.mark.parametrize("form", [0, 1])
def test_bounded_wait_gives_up_and_the_batch_steps_on(form, cuda_lib):
    """The narrowphase's one device wait (bulk copies of each world's bodies
    completing on an mbarrier) runs out: the test hook makes it expect 16
    bytes more than it copies, so every real copy lands and nothing is in
    flight when it gives up after 64 polls.  The call reports CZ_ERR_TIMEOUT;
    with the hook off the batch steps on, bit for bit with the oracle."""
    from cubez_gb300 import CubezError
    from cubez_gb300.batch import WorldBatch
    sc = scenes.mixed(num_worlds=8, seed=35)
    b = WorldBatch.from_scene(sc, form=form)
    ref = OracleBatch(sc, form=form)
    b.step(3, DT)
    ref.step(3, DT)
    assert b.L.cz_set_wait_test(b.h, 16, 64) == 0
    with pytest.raises(CubezError) as e:
        b.narrowphase()
    assert e.value.status == 6  # CZ_ERR_TIMEOUT
    assert np.any(b.stats()["status"] & 8)  # the worlds whose wait gave up are flagged
    assert b.L.cz_set_wait_test(b.h, 0, 0) == 0
    assert b.L.cz_set_wait_test(b.h, -1, 0) == 1
    b.step(3, DT)
    ref.step(3, DT)
    g, r = b.download(), ref.bodies()
    for k in ("position", "orientation", "velocity", "rotation"):
        np.testing.assert_array_equal(g[k], r[k], err_msg=k)
