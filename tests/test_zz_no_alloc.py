"""cz_resolve_contacts_static: ResolveContacts for one world with no memory
allocation, for callers that cannot call cudaMalloc (a frame loop that must
not allocate, or a host that only lends the library device memory it already
owns).  Here torch plays that caller: it owns every device buffer, and the
library's scratch is its statically reserved array.

Checked against the allocating entry point cz_resolve_contacts on the same
inputs, bit for bit (the tolerance of every parity test in this suite), on two
calls in a row so that the second call starts from the scratch contents the
first one left behind, and against the oracle directly.  Every world here is
taken mid-rollout, after an Integrate, so the resolver iterates.  Last, both
entry points with per-contact friction and restitution against the oracle."""
import ctypes as C

import numpy as np
import pytest

from cubez_gb300 import scenes
from tests.test_gpu_api import (assert_matches_oracle, cz_contacts, frame_inputs, host_arrays, resolve_both,
                                scene_with_contacts)

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0
_OPTIONAL = ("last_frame_acceleration", "inverse_inertia_world")


def _contacts_np(arr):
    raw = np.frombuffer(arr, dtype=np.dtype([("body", "<i4", 2), ("friction", "<f8"), ("restitution", "<f8"),
                                             ("point", "<f8", 3), ("normal", "<f8", 3), ("penetration", "<f8")]))
    return raw.copy()


def _with_static_entry_point(lib, scene, arr, form, extra=None):
    """The allocation-free entry point, on device buffers the caller owns."""
    import torch
    from cubez_gb300 import _lib
    host = host_arrays(scene)
    for k, v in (extra or {}).items():
        host[k] = np.array(v, dtype=np.float64, copy=True)
    dev = {k: torch.from_numpy(v.copy()).cuda() for k, v in host.items()}
    raw = _contacts_np(arr)
    dcontacts = torch.from_numpy(raw.view(np.uint8).copy()).cuda()
    s = _lib.Bodies()
    for name in ("position", "orientation", "velocity", "rotation", "acceleration", "inverse_inertia",
                 "inverse_mass", "motion", "is_awake") + tuple(k for k in _OPTIONAL if k in dev):
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


def _static_against_oracle(out, out_contacts, ref):
    r = ref.bodies()
    for k in ("position", "orientation", "velocity", "rotation"):
        np.testing.assert_array_equal(out[k], r[k], err_msg=k)
    rc = ref.resolved_contacts(0)
    np.testing.assert_array_equal(out_contacts["penetration"], rc["penetration"])
    np.testing.assert_array_equal(out_contacts["normal"], rc["normal"])
    np.testing.assert_array_equal(out_contacts["body"], rc["bodies"])


@pytest.mark.parametrize("form", [0, 1])
def test_static_scratch_matches_existing_entry_point_twice(form, cuda_lib):
    # first call: a 64-body world whose contacts exceed the shared-memory tile
    # (they use the working rows in the static scratch); second call: a small
    # world, starting from the scratch the first call left behind
    for seed, bodies in ((41, 64), (42, 20)):
        scene, c = scene_with_contacts(seed, bodies, 150, form)
        n = len(c["penetration"])
        if bodies == 64:
            assert n > 128
        st_a, host, arr_a, ref = resolve_both(scene, c, 4 * n, form)
        assert st_a == 0, cuda_lib.cz_last_error()
        assert ref.stats()["pos_iterations"][0] > 0 and ref.stats()["vel_iterations"][0] > 0
        assert_matches_oracle(host, arr_a, ref)
        st_b, out, out_contacts = _with_static_entry_point(cuda_lib, scene, cz_contacts(c), form)
        assert st_b == 0, cuda_lib.cz_last_error()
        _compare(host, arr_a, out, out_contacts)
        _static_against_oracle(out, out_contacts, ref)


@pytest.mark.parametrize("form", [0, 1])
def test_static_scratch_with_frame_inputs(form, cuda_lib):
    """The optional inputs a frame loop passes after Integrate: last-frame
    accelerations and the world inverse inertia, against the oracle given the
    same values and against the allocating entry point."""
    moved, c, extra, ref = frame_inputs(form)
    n = len(c["penetration"])
    st_a, host, arr_a, ref = resolve_both(moved, c, 4 * n, form, ref=ref, extra=extra)
    assert st_a == 0, cuda_lib.cz_last_error()
    assert ref.stats()["vel_iterations"][0] > 0
    st_b, out, out_contacts = _with_static_entry_point(cuda_lib, moved, cz_contacts(c), form, extra)
    assert st_b == 0, cuda_lib.cz_last_error()
    _compare(host, arr_a, out, out_contacts)
    _static_against_oracle(out, out_contacts, ref)


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
    # a 3 x 3 x 2 pile one second after the drop: 50 contacts, 24 between cubes
    scene = scenes.piles(num_worlds=1, seed=76, nx=3, nz=3, ny=2, spacing=1.1)
    ref = OracleBatch(scene, form=form)
    ref.step(60, DT)
    st = ref.bodies()
    scene = scene.copy()
    for k in ("position", "orientation", "velocity", "rotation"):
        setattr(scene, k, np.array(st[k], copy=True))
    ref = OracleBatch(scene, form=form)
    ref.narrowphase()
    c = ref.contacts(0)
    n = len(c["penetration"])
    rng = np.random.default_rng(9)
    two = c["bodies"][:, 1] >= 0
    c["friction"] = np.where(two, 0.0, rng.uniform(0.2, 1.0, n))
    c["restitution"] = rng.uniform(0.0, 0.6, n)
    assert two.sum() > 10 and (~two).sum() > 10
    st, arrays, arr, ref = resolve_both(scene, c, 4 * n, form)
    assert st == 0, cuda_lib.cz_last_error()
    assert ref.stats()["vel_iterations"][0] > 20
    assert_matches_oracle(arrays, arr, ref)
    # the allocation-free entry point on the same materials
    st_s, out, out_contacts = _with_static_entry_point(cuda_lib, scene, cz_contacts(c), form)
    assert st_s == 0, cuda_lib.cz_last_error()
    _static_against_oracle(out, out_contacts, ref)
