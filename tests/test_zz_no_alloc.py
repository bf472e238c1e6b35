"""cz_resolve_contacts_static: ResolveContacts for one world with no memory
allocation, for callers that cannot call cudaMalloc (a frame loop that must
not allocate, or a host that only lends the library device memory it already
owns).  Here torch plays that caller: it owns every device buffer, and the
library's scratch is its statically reserved array.

Checked against the allocating entry point cz_resolve_contacts on the same
inputs, bit for bit (the tolerance of every parity test in this suite), on two
calls in a row so that the second call starts from the scratch contents the
first one left behind.  Last, both entry points with per-contact friction and
restitution against the oracle."""
import ctypes as C

import numpy as np
import pytest

from cubez_gb300 import scenes

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0
_DT = {"is_awake": np.uint8, "can_sleep": np.uint8, "shape": np.int32}


def _settled_world(seed, bodies):
    from oracle.oracle import OracleBatch
    sc = scenes.mixed(num_worlds=1, seed=seed, min_bodies=bodies, max_bodies=bodies)
    ref = OracleBatch(sc)
    ref.step(150, DT)
    st = ref.bodies()
    moved = sc.copy()
    for k in ("position", "orientation", "velocity", "rotation"):
        setattr(moved, k, st[k])
    ref = OracleBatch(moved)
    ref.narrowphase()
    c = ref.contacts(0)
    n = len(c["penetration"])
    return moved, c, n


def _contact_array(c):
    from cubez_gb300 import _lib
    n = len(c["penetration"])
    arr = (_lib.Contact * n)()
    for i in range(n):
        arr[i].body[0], arr[i].body[1] = int(c["bodies"][i][0]), int(c["bodies"][i][1])
        arr[i].friction, arr[i].restitution = 0.9, 0.1
        for k in range(3):
            arr[i].point[k] = float(c["point"][i][k])
            arr[i].normal[k] = float(c["normal"][i][k])
        arr[i].penetration = float(c["penetration"][i])
    return arr


def _contacts_np(arr):
    raw = np.frombuffer(arr, dtype=np.dtype([("body", "<i4", 2), ("friction", "<f8"), ("restitution", "<f8"),
                                             ("point", "<f8", 3), ("normal", "<f8", 3), ("penetration", "<f8")]))
    return raw.copy()


def _host_arrays(scene):
    """Fresh copies: both entry points write their results back in place."""
    return {k: np.array(getattr(scene, k), dtype=_DT.get(k, np.float64), copy=True) for k in scene.FIELDS}


def _with_existing_entry_point(scene, arr, form):
    """The allocating entry point, on host arrays."""
    from cubez_gb300.batch import WorldBatch, bodies_struct
    b = WorldBatch(scene.counts, form=form, plane=scene.plane)
    host = _host_arrays(scene)
    s = bodies_struct(host)
    st = b.L.cz_resolve_contacts(b.h, 4 * len(arr), C.cast(arr, C.c_void_p), len(arr), DT, C.byref(s))
    b.close()
    return st, host


def _with_static_entry_point(lib, scene, arr, form):
    """The allocation-free entry point, on device buffers the caller owns."""
    import torch
    from cubez_gb300 import _lib
    host = _host_arrays(scene)
    dev = {k: torch.from_numpy(v.copy()).cuda() for k, v in host.items()}
    raw = _contacts_np(arr)
    dcontacts = torch.from_numpy(raw.view(np.uint8).copy()).cuda()
    s = _lib.Bodies()
    for name in ("position", "orientation", "velocity", "rotation", "acceleration", "inverse_inertia",
                 "inverse_mass", "motion", "is_awake"):
        setattr(s, name, C.c_void_p(dev[name].data_ptr()))
    torch.cuda.synchronize()
    st = lib.cz_resolve_contacts_static(form, 4 * len(arr), C.c_void_p(dcontacts.data_ptr()), len(arr), DT,
                                        C.byref(s), scene.num_bodies, None)
    out = {k: v.cpu().numpy() for k, v in dev.items()}
    out_contacts = dcontacts.cpu().numpy().view(raw.dtype)
    return st, out, out_contacts


def _compare(host, arr_after, out, out_contacts):
    for k in ("position", "orientation", "velocity", "rotation", "motion", "is_awake"):
        np.testing.assert_array_equal(out[k], host[k], err_msg=k)
    ref = _contacts_np(arr_after)
    np.testing.assert_array_equal(out_contacts["penetration"], ref["penetration"])
    np.testing.assert_array_equal(out_contacts["normal"], ref["normal"])
    np.testing.assert_array_equal(out_contacts["body"], ref["body"])


@pytest.mark.parametrize("form", [0, 1])
def test_static_scratch_matches_existing_entry_point_twice(form, cuda_lib):
    # first call: a large world whose contacts exceed the shared-memory tile
    # (they use the working rows in the static scratch); second call: a small
    # world, starting from the scratch the first call left behind
    for seed, bodies in ((41, 64), (42, 20)):
        scene, c, n = _settled_world(seed, bodies)
        assert n > 0
        if bodies == 64:
            assert n > 128
        arr_a = _contact_array(c)
        arr_b = _contact_array(c)
        st_a, host = _with_existing_entry_point(scene, arr_a, form)
        st_b, out, out_contacts = _with_static_entry_point(cuda_lib, scene, arr_b, form)
        assert st_a == 0
        assert st_b == 0, cuda_lib.cz_last_error()
        _compare(host, arr_a, out, out_contacts)


def test_static_scratch_rejects_sizes_beyond_its_maximum(cuda_lib):
    from cubez_gb300 import _lib
    s = _lib.Bodies()
    assert cuda_lib.cz_resolve_contacts_static(0, 4, None, 1, DT, C.byref(s), 65, None) == 1
    assert cuda_lib.cz_resolve_contacts_static(0, 4, None, 8193, DT, C.byref(s), 8, None) == 1


@pytest.mark.parametrize("form", [0, 1])
def test_resolve_contacts_with_contact_materials(form, cuda_lib):
    """Per-contact friction and restitution, the exported Contact fields the
    resolver reads (the colliders write 0.9 and 0.1): every two-body contact
    frictionless (calculateFrictionlessImpulse, contact.go:496-531, with its
    inverted nil test), the single-body ones with friction in [0.2, 1], and
    restitution in [0, 0.6].  The allocating entry point against the oracle,
    and the allocation-free one against it, bit for bit."""
    from oracle.oracle import OracleBatch
    from tests.test_gpu_api import _resolve_both
    # a 3 x 3 x 2 pile one second after the drop: 50 contacts, 24 between cubes
    scene = scenes.piles(num_worlds=1, seed=76, nx=3, nz=3, ny=2, spacing=1.1)
    ref = OracleBatch(scene)
    ref.step(60, DT)
    st = ref.bodies()
    scene = scene.copy()
    for k in ("position", "orientation", "velocity", "rotation"):
        setattr(scene, k, st[k])
    ref = OracleBatch(scene)
    ref.narrowphase()
    c = ref.contacts(0)
    n = len(c["penetration"])
    rng = np.random.default_rng(9)
    two = c["bodies"][:, 1] >= 0
    c["friction"] = np.where(two, 0.0, rng.uniform(0.2, 1.0, n))
    c["restitution"] = rng.uniform(0.0, 0.6, n)
    assert two.sum() > 10 and (~two).sum() > 10
    st, arrays, arr, ref, _ = _resolve_both(scene, c, 4 * n, form)
    assert st == 0, cuda_lib.cz_last_error()
    assert ref.stats()["vel_iterations"][0] > 20
    r = ref.bodies()
    for k in ("position", "orientation", "velocity", "rotation"):
        np.testing.assert_array_equal(arrays[k], r[k], err_msg=k)
    rc = ref.resolved_contacts(0)
    np.testing.assert_array_equal(np.array([arr[i].penetration for i in range(n)]), rc["penetration"])
    # the allocation-free entry point on the same materials
    from tests.test_gpu_api import _cz_contacts
    arr_s = _cz_contacts(c)
    st_s, out, out_contacts = _with_static_entry_point(cuda_lib, scene, arr_s, form)
    assert st_s == 0, cuda_lib.cz_last_error()
    for k in ("position", "orientation", "velocity", "rotation"):
        np.testing.assert_array_equal(out[k], arrays[k], err_msg=k)
