"""Parity at the benchmark's full sizes.  The small-scene tests pin every
branch; these check that nothing changes at scale (queue order, tiles that
spill to global rows, many CTAs): the 16384 x 32 precision workload and the
256 x 1024 piles, bit-identical to the oracle over frames taken from a
settled state.  The oracle runs on all host cores."""
import numpy as np
import pytest

from cubez_gb300 import scenes
from oracle.oracle import FP32 as ORC_FP32
from oracle.oracle import FP64 as ORC_FP64
from oracle.oracle import OracleBatch, hardware_threads

from tests.test_gpu_parity import STATE, assert_bodies_equal

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0


def _settled_pair(scene, form, settle, tuning=None):
    from cubez_gb300.batch import WorldBatch
    gpu = WorldBatch.from_scene(scene, form=form)
    if tuning:
        gpu.set_tuning(**tuning)
    gpu.step(settle, DT)
    st = gpu.download(STATE + ("motion", "is_awake"))
    moved = scene.copy()
    for k, v in st.items():
        setattr(moved, k, v)
    ref = OracleBatch(moved, form=ORC_FP64 if form == 0 else ORC_FP32)
    gpu = WorldBatch.from_scene(moved, form=form)
    if tuning:
        gpu.set_tuning(**tuning)
    return gpu, ref, moved


@pytest.mark.parametrize("form", [0, 1])
def test_precision_workload_full_size(form, cuda_lib):
    scene = scenes.precision(num_worlds=16384, bodies=32, seed=3)
    tuning = dict(resolver_lanes=16, resolver_contacts=96) if form == 1 else None
    gpu, ref, _ = _settled_pair(scene, form, settle=200, tuning=tuning)
    threads = hardware_threads()
    for _ in range(2):
        gpu.step(1, DT)
        ref.step(1, DT, 4, threads)
    assert_bodies_equal(gpu.download(), ref.bodies())
    gs, rs = gpu.stats(), ref.stats()
    assert rs["contacts"].sum() > 500_000
    np.testing.assert_array_equal(gpu.contact_counts(), rs["contacts"])
    np.testing.assert_array_equal(gs["vel_iterations"], rs["vel_iterations"])


def test_piles_full_size_one_frame(cuda_lib):
    scene = scenes.piles(num_worlds=256)
    gpu, ref, _ = _settled_pair(scene, 1, settle=60)
    gpu.step(1, DT)
    ref.step(1, DT, 4, hardware_threads())
    assert_bodies_equal(gpu.download(), ref.bodies())
    gs, rs = gpu.stats(), ref.stats()
    assert rs["contacts"].min() > 1000
    np.testing.assert_array_equal(gs["vel_iterations"], rs["vel_iterations"])


def test_batched_workload_full_size(cuda_lib):
    """The batched configuration: 4096 worlds of U{8..64} spheres and cubes in
    the plain float64 form, three frames from a settled state, bit for bit
    (the step order of examples/cubedrop.go:29-75 in every world)."""
    scene = scenes.mixed(num_worlds=4096, seed=2)
    gpu, ref, _ = _settled_pair(scene, 0, settle=150)
    threads = hardware_threads()
    for _ in range(3):
        gpu.step(1, DT)
        ref.step(1, DT, 4, threads)
    assert_bodies_equal(gpu.download(), ref.bodies())
    gs, rs = gpu.stats(), ref.stats()
    assert rs["contacts"].sum() > 100_000
    np.testing.assert_array_equal(gpu.contact_counts(), rs["contacts"])
    np.testing.assert_array_equal(gs["pos_iterations"], rs["pos_iterations"])
    np.testing.assert_array_equal(gs["vel_iterations"], rs["vel_iterations"])
