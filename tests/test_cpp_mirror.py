"""The C++ mirror of the cubez API (include/cubez.hpp): the frame loops of
examples/cubedrop.go and examples/ballistic.go written one body and one pair
at a time, as the Go examples call the package, must reproduce the oracle
(the reference's float64 path) bit for bit, frame by frame."""
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

from cubez_gb300 import scenes
from oracle.oracle import OracleBatch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "cubez_gb300", "_build")
SRC = os.path.join(ROOT, "tests", "cpp", "mirror_loops.cpp")
DT = 1.0 / 60.0


def _compile(out_dir):
    gxx = shutil.which("g++")
    if gxx is None or not os.path.exists(os.path.join(LIBDIR, "libcubez_gb300.so")):
        pytest.skip("g++ or the built library is missing")
    exe = os.path.join(str(out_dir), "mirror_loops")
    cmd = [gxx, "-std=c++17", "-O2", "-ffp-contract=off", "-Wall", "-I", os.path.join(ROOT, "include"), SRC,
           "-L", LIBDIR, "-lcubez_gb300", "-Wl,-rpath," + LIBDIR, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _write_input(scene, path):
    n = scene.num_bodies
    is_cube = scene.shape == scenes.CUBE
    half, radius = scene.half_size, scene.radius
    mass = np.where(is_cube, ((8.0 * half[:, 0]) * half[:, 1]) * half[:, 2],
                    (((4.0 / 3.0) * math.pi) * radius * radius) * radius)
    if not np.array_equal(1.0 / mass, scene.inverse_mass):  # masses not from density 1
        inv = scene.inverse_mass
        mass = np.where(inv > 0, 1.0 / np.where(inv > 0, inv, 1.0), 0.0)
    # SetMass(mass) (or SetInfiniteMass for 0) gives the scene's inverse mass
    assert np.array_equal(np.where(mass > 0, 1.0 / np.where(mass > 0, mass, 1.0), 0.0), scene.inverse_mass)
    rows = np.zeros((n, 49))
    rows[:, 0] = scene.shape
    rows[:, 1] = mass
    rows[:, 2:5] = half
    rows[:, 5] = radius
    rows[:, 6:9] = scene.position
    rows[:, 9:13] = scene.orientation
    rows[:, 13:16] = scene.velocity
    rows[:, 16:19] = scene.rotation
    rows[:, 19:22] = scene.acceleration
    rows[:, 22:31] = scene.inverse_inertia.reshape(n, 9)
    rows[:, 31] = scene.linear_damping
    rows[:, 32] = scene.angular_damping
    rows[:, 33] = scene.can_sleep
    rows[:, 37:49] = scene.collider_offset if scene.collider_offset is not None else scenes.IDENTITY_OFFSET
    data = np.concatenate([np.asarray(scene.plane, np.float64), [float(n)], rows.ravel()])
    data.astype(np.float64).tofile(path)


def test_cpp_mirror_compiles(tmp_path):
    _compile(tmp_path)


def _run_mirror(exe, loop, scene, frames, tmp_path):
    inp, out = os.path.join(str(tmp_path), "in.bin"), os.path.join(str(tmp_path), "out.bin")
    _write_input(scene, inp)
    r = subprocess.run([exe, loop, inp, out, str(frames)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return np.fromfile(out, np.float64).reshape(frames, 1 + 13 * scene.num_bodies)


@pytest.mark.gpu
@pytest.mark.parametrize("which", ["cubedrop", "mixed", "offsets"])
def test_cpp_mirror_cubedrop_loop_matches_oracle(which, tmp_path, cuda_lib):
    if which == "cubedrop":
        scene, frames = scenes.cubedrop(seed=1), 150
    elif which == "mixed":
        scene, frames = scenes.mixed(num_worlds=1, seed=71, min_bodies=14, max_bodies=14), 150
    else:  # colliders with Offsets, some of them not rigid
        scene, frames = scenes.offsets(num_worlds=1, bodies=14, seed=73, nonrigid=0.3), 150
    exe = _compile(tmp_path)
    got = _run_mirror(exe, "cubedrop", scene, frames, tmp_path)
    n = scene.num_bodies
    ref = OracleBatch(scene)
    total = 0
    for fr in range(frames):
        ref.step(1, DT)
        st = ref.bodies()
        count = int(ref.stats()["contacts"][0])
        total += count
        assert int(got[fr, 0]) == count, "frame %d: %d contacts vs %d" % (fr, got[fr, 0], count)
        g = got[fr, 1:].reshape(n, 13)
        for name, sl in (("position", slice(0, 3)), ("orientation", slice(3, 7)), ("velocity", slice(7, 10)),
                         ("rotation", slice(10, 13))):
            assert np.array_equal(g[:, sl], st[name]), "frame %d: %s differs" % (fr, name)
    assert total > 100  # the bodies landed and touched


@pytest.mark.gpu
def test_cpp_mirror_ballistic_loop_matches_oracle(tmp_path, cuda_lib):
    """examples/ballistic.go's loop: the backboard (SetInfiniteMass) is never
    integrated, the tests run in the example's order and ResolveContacts gets
    len(contacts) * 8.  The oracle integrates every body (the backboard is
    static, so that changes nothing), runs the same unit list and resolves."""
    scene, frames = scenes.ballistic(num_worlds=1, bullets=6, seed=74), 120
    exe = _compile(tmp_path)
    got = _run_mirror(exe, "ballistic", scene, frames, tmp_path)
    n = scene.num_bodies
    units = scenes.ballistic_units(n)
    ref = OracleBatch(scene)
    total = 0
    for fr in range(frames):
        ref.integrate(DT)
        ref.collide(0, units)
        ref.resolve(DT, iter_mult=8)
        st = ref.bodies()
        count = int(ref.stats()["contacts"][0])
        total += count
        assert int(got[fr, 0]) == count, "frame %d: %d contacts vs %d" % (fr, got[fr, 0], count)
        g = got[fr, 1:].reshape(n, 13)
        for name, sl in (("position", slice(0, 3)), ("orientation", slice(3, 7)), ("velocity", slice(7, 10)),
                         ("rotation", slice(10, 13))):
            assert np.array_equal(g[:, sl], st[name]), "frame %d: %s differs" % (fr, name)
    assert total > 50
    assert np.array_equal(got[-1, 1:].reshape(n, 13)[1, :3], scene.position[1])  # the backboard stayed


@pytest.mark.gpu
def test_collide_unit_lists(cuda_lib):
    """cz_collide: the units of generateContacts in its order reproduce the
    narrowphase; any other order gives the same per-unit contacts in that
    order; a caller's plane replaces the batch's."""
    from cubez_gb300.batch import FORM_FP64, WorldBatch
    scene = scenes.mixed(num_worlds=3, seed=72, min_bodies=10, max_bodies=16)
    ref = OracleBatch(scene)
    ref.step(110, DT)
    st = ref.bodies()
    moved = scene.copy()
    for k in ("position", "orientation", "velocity", "rotation"):
        setattr(moved, k, st[k])
    b = WorldBatch.from_scene(moved, form=FORM_FP64)
    b.narrowphase()
    for w in range(scene.num_worlds):
        n = int(scene.counts[w])
        full = b.contacts(w)
        units = []
        for i in range(n):
            units.append((i, -1))
            units.extend((i, j) for j in range(n) if j != i)
        b.collide(w, units)
        got = b.contacts(w)
        for k in full:
            assert np.array_equal(got[k], full[k]), k
        assert len(full["penetration"]) > 0
        # per-unit contact lists, then the units in reverse order
        per = []
        for u in units:
            b.collide(w, [u])
            per.append(b.contacts(w))
        b.collide(w, units[::-1])
        rev = b.contacts(w)
        for k in full:
            expect = np.concatenate([p[k] for p in per[::-1]]) if per else full[k]
            assert np.array_equal(rev[k], expect), k
    # the plane of the call, not the batch's: lift the ground by 100 m
    b.collide(0, [(i, -1) for i in range(int(scene.counts[0]))], plane=(0.0, 1.0, 0.0, 100.0))
    assert len(b.contacts(0)["penetration"]) >= int(scene.counts[0])  # every body is below y = 100
