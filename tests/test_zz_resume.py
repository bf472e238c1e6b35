"""Checkpoint and resume (WorldBatch.save / WorldBatch.load over
cz_download_bodies / cz_upload_bodies): a batch loaded from a saved state
steps on bit for bit as the saved batch does, with sleeping on (the motion
average and awake flags are state) and with collider Offsets."""
import numpy as np
import pytest

from cubez_gb300 import scenes

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0


def _sleepy():
    sc = scenes.mixed(num_worlds=16, seed=81, min_bodies=8, max_bodies=40)
    sc.can_sleep[:] = 1
    return sc


@pytest.mark.parametrize("form", [0, 1])
@pytest.mark.parametrize("make", [_sleepy, lambda: scenes.offsets(num_worlds=8, bodies=20, seed=82)],
                         ids=["sleeping", "offsets"])
def test_resume_from_a_saved_state(form, make, cuda_lib, tmp_path):
    from cubez_gb300.batch import _WIDTH, WorldBatch
    a = WorldBatch.from_scene(make(), form=form)
    a.step(45, DT)
    path = str(tmp_path / "state.npz")
    a.save(path)
    b = WorldBatch.load(path)
    a.step(45, DT)
    b.step(45, DT)
    sa, sb = a.download(tuple(_WIDTH)), b.download(tuple(_WIDTH))
    for k in _WIDTH:
        np.testing.assert_array_equal(sa[k], sb[k], err_msg=k)
    a.close()
    b.close()
