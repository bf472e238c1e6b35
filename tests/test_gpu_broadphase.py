"""The narrowphase's grid broadphase (the reference's roadmap item,
README.md:98-99; its all-pairs loop is marked O(n^2) at
examples/cubedrop.go:54).  The grid drops only pairs the float32 culls
already reject and lists each body's remaining units in the reference's
order, so the contact lists are bit-identical with the all-pairs path and
with the oracle: checked on cube piles (where the grid is on by default),
on mixed worlds with the grid forced on small worlds, and on worlds where
it falls back to all pairs (a body far away; non-rigid collider Offsets,
whose culls are off)."""
import numpy as np
import pytest

from cubez_gb300 import scenes
from oracle.oracle import OracleBatch

from tests.test_gpu_parity import assert_bodies_equal, assert_contacts_equal

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0


def _pair(scene, form, grid):
    from cubez_gb300.batch import WorldBatch
    gpu = WorldBatch.from_scene(scene, form=form)
    gpu.set_tuning(broadphase_min_bodies=grid)
    assert gpu.get_tuning()["broadphase_min_bodies"] == grid
    return gpu, OracleBatch(scene, form=form)


@pytest.mark.parametrize("form", [0, 1])
def test_piles_with_the_grid_bit_exact(form, cuda_lib):
    # 150 cubes per world on a 5 x 5 x 6 lattice: the grid is on by default (>= 128 bodies)
    scene = scenes.piles(num_worlds=3, seed=52, nx=5, nz=5, ny=6)
    gpu, ref = _pair(scene, form, 128)
    off, _ = _pair(scene, form, -1)
    for frames in (1, 29):
        gpu.step(frames, DT)
        off.step(frames, DT)
        ref.step(frames, DT)
        assert_bodies_equal(gpu.download(), ref.bodies())
        assert_contacts_equal(gpu, ref, scene.num_worlds)
        np.testing.assert_array_equal(gpu.contact_counts(), off.contact_counts())
    assert ref.stats()["contacts"].min() > 100
    gs, rs = gpu.stats(), ref.stats()
    np.testing.assert_array_equal(gs["vel_iterations"], rs["vel_iterations"])


@pytest.mark.parametrize("form", [0, 1])
def test_grid_forced_on_mixed_worlds(form, cuda_lib):
    """Spheres and cubes of both sizes, falling and landed, with the grid on
    for every world of at least 8 bodies."""
    scene = scenes.mixed(num_worlds=24, seed=37, min_bodies=8, max_bodies=64)
    gpu, ref = _pair(scene, form, 8)
    gpu.narrowphase()
    ref.narrowphase()
    assert_contacts_equal(gpu, ref, scene.num_worlds)
    for frames in (60, 90):
        gpu.step(frames, DT)
        ref.step(frames, DT)
        assert_bodies_equal(gpu.download(), ref.bodies())
        assert_contacts_equal(gpu, ref, scene.num_worlds)


@pytest.mark.parametrize("form", [0, 1])
def test_grid_falls_back_to_all_pairs(form, cuda_lib):
    """A body a kilometre away would need too many cells, and non-rigid
    collider Offsets have no cull radius: both worlds take the all-pairs path,
    with the same contacts as the oracle."""
    far = scenes.piles(num_worlds=1, seed=53, nx=3, nz=3, ny=2)
    far.position = far.position.copy()
    far.position[0] = [1000.0, 3.0, -1000.0]
    offs = scenes.offsets(num_worlds=2, bodies=24, seed=9, nonrigid=0.5)
    for scene in (far, offs):
        gpu, ref = _pair(scene, form, 8)
        for frames in (1, 20):
            gpu.step(frames, DT)
            ref.step(frames, DT)
            assert_bodies_equal(gpu.download(), ref.bodies())
            assert_contacts_equal(gpu, ref, scene.num_worlds)


def test_broadphase_threshold_argument_checks(cuda_lib):
    from cubez_gb300 import CubezError
    from cubez_gb300.batch import WorldBatch
    b = WorldBatch.from_scene(scenes.mixed(num_worlds=2, seed=38))
    with pytest.raises(CubezError):
        b.set_tuning(broadphase_min_bodies=-2)
    b.set_tuning(broadphase_min_bodies=-1)
    assert b.get_tuning()["broadphase_min_bodies"] == -1
