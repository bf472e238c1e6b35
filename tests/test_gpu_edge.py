"""Edge cases of the batch: empty worlds, single-body worlds, worlds with no
contacts and a world above the shared-memory slot, ragged in one batch; the
warm start on the same batch."""
import numpy as np
import pytest

from cubez_gb300 import scenes
from oracle.oracle import FP32 as ORC_FP32
from oracle.oracle import FP64 as ORC_FP64
from oracle.oracle import OracleBatch

from tests.test_gpu_parity import assert_bodies_equal, assert_contacts_equal

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0
COUNTS = [0, 1, 0, 5, 70, 0, 2, 33, 0]


def _ragged():
    parts = [scenes.mixed(num_worlds=1, seed=82 + i, min_bodies=n, max_bodies=n)
             for i, n in enumerate(c for c in COUNTS if c > 0)]
    return scenes.Scene.concat(parts, counts=COUNTS)


@pytest.mark.parametrize("form", [0, 1])
def test_ragged_batch_with_empty_worlds(form, cuda_lib):
    from cubez_gb300.batch import WorldBatch
    scene = _ragged()
    gpu = WorldBatch.from_scene(scene, form=form)
    ref = OracleBatch(scene, form=ORC_FP64 if form == 0 else ORC_FP32)
    gpu.step(200, DT)
    ref.step(200, DT)
    assert_bodies_equal(gpu.download(), ref.bodies())
    rs = ref.stats()
    np.testing.assert_array_equal(gpu.contact_counts(), rs["contacts"])
    np.testing.assert_array_equal(gpu.stats()["vel_iterations"], rs["vel_iterations"])
    assert_contacts_equal(gpu, ref, scene.num_worlds)
    empty = np.array(COUNTS) == 0
    assert (rs["contacts"][empty] == 0).all() and rs["contacts"][~empty].sum() > 100


def test_warm_start_on_ragged_batch(cuda_lib):
    """The warm start serves small worlds; empty worlds stay empty and the
    world above the slot is solved by the plain large-world resolver, so it
    ends exactly as without the warm start."""
    from cubez_gb300.batch import FORM_FP32, WorldBatch
    from cubez_gb300.learned import BLOB, OFF_B4, OFF_IS, OFF_OS, set_warm_start
    scene = _ragged()
    plain = WorldBatch.from_scene(scene, form=FORM_FP32)
    warm = WorldBatch.from_scene(scene, form=FORM_FP32)
    blob = np.zeros(BLOB, np.float32)
    blob[OFF_IS:OFF_IS + 18] = 1.0
    blob[OFF_OS:OFF_OS + 3] = 1.0
    blob[OFF_B4] = 0.2  # a small normal impulse everywhere
    set_warm_start(warm, blob)
    warm.counters(reset=True)
    plain.step(200, DT)
    warm.step(200, DT)
    assert warm.counters()["warm_bodies"] > 0
    p, w = plain.download(), warm.download()
    big = scene.world_slice(COUNTS.index(70))
    for k in ("position", "orientation", "velocity", "rotation"):
        np.testing.assert_array_equal(w[k][big], p[k][big])
        assert np.all(np.isfinite(w[k]))
