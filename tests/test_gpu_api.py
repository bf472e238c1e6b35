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


def _scene_with_contacts(seed=31):
    """A settled mixed world and the contacts the narrowphase gives for it."""
    sc = scenes.mixed(num_worlds=1, seed=seed, min_bodies=24, max_bodies=24)
    ref = OracleBatch(sc)
    ref.step(150, DT)
    st = ref.bodies()
    moved = sc.copy()
    for k in ("position", "orientation", "velocity", "rotation"):
        setattr(moved, k, st[k])
    ref = OracleBatch(moved)
    ref.narrowphase()
    c = ref.contacts(0)
    c["friction"] = np.full(len(c["penetration"]), 0.9)
    c["restitution"] = np.full(len(c["penetration"]), 0.1)
    return moved, c


def _cz_contacts(c):
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


def _resolve_both(scene, c, max_iterations, form=0):
    import ctypes as C

    from cubez_gb300 import _lib
    from cubez_gb300.batch import WorldBatch, bodies_struct
    gpu = WorldBatch(scene.counts, form=form, plane=scene.plane)
    n = scene.num_bodies
    arrays = {k: np.ascontiguousarray(getattr(scene, k), dtype={"is_awake": np.uint8, "can_sleep": np.uint8,
                                                              "shape": np.int32}.get(k, np.float64))
              for k in scene.FIELDS}
    arrays["inverse_inertia_world"] = None
    s = bodies_struct(arrays)
    arr = _cz_contacts(c)
    st = gpu.L.cz_resolve_contacts(gpu.h, max_iterations, C.cast(arr, C.c_void_p), len(arr), DT, C.byref(s))
    ref = OracleBatch(scene, form=form)
    ref.set_contacts(0, c)
    ref.resolve_fixed(max_iterations, DT)
    return st, arrays, arr, ref, n


@pytest.mark.parametrize("form", [0, 1])
def test_resolve_contacts_matches_oracle(form, cuda_lib):
    scene, c = _scene_with_contacts()
    assert len(c["penetration"]) > 20
    st, arrays, arr, ref, n = _resolve_both(scene, c, 4 * len(c["penetration"]), form)
    assert st == 0
    r = ref.bodies()
    for k in ("position", "orientation", "velocity", "rotation"):
        np.testing.assert_array_equal(arrays[k], r[k])
    rc = ref.resolved_contacts(0)
    pen = np.array([arr[i].penetration for i in range(len(arr))])
    np.testing.assert_array_equal(pen, rc["penetration"])


def test_resolve_contacts_swaps_nil_first_body(cuda_lib):
    scene = cases.cube_resting()
    c = {"bodies": np.array([[-1, 0]], np.int32), "point": np.array([[0.5, -0.02, 0.5]]),
         "normal": np.array([[0.0, -1.0, 0.0]]), "penetration": np.array([0.01]),
         "friction": np.array([0.9]), "restitution": np.array([0.1])}
    st, arrays, arr, ref, n = _resolve_both(scene, c, 4, 0)
    assert st == 0
    assert list(arr[0].body) == [0, -1]          # calculateInternals, contact.go:61-65
    assert list(arr[0].normal) == [0.0, 1.0, 0.0]
    r = ref.bodies()
    np.testing.assert_array_equal(arrays["position"], r["position"])
    np.testing.assert_array_equal(arrays["velocity"], r["velocity"])


def test_resolve_contacts_zero_iterations_and_guards(cuda_lib):
    scene, c = _scene_with_contacts(seed=32)
    st, arrays, arr, ref, n = _resolve_both(scene, c, 0, 0)
    assert st == 0
    # no iteration: positions unchanged (prepareContacts alone mutates no body)
    np.testing.assert_array_equal(arrays["position"], scene.position)


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
    arr = _cz_contacts(bad)
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
