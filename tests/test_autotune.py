"""The autotuner's search on a fake batch (CPU only): it keeps the fastest
setting of each knob, skips shapes the batch refuses, tries the large-world
lanes only when the batch has worlds of more than 64 bodies, and restores
the snapshot before every trial."""
import numpy as np

from cubez_gb300 import autotune


class FakeBatch:
    def __init__(self, counts):
        self.counts = np.asarray(counts, np.int32)
        self.cfg = {"narrowphase_threads": 128, "resolver_contacts": 128, "resolver_lanes": 8,
                    "large_world_lanes": 32, "warm_start_budget_shift": 2, "fused_frame": -1}
        self.restores = 0
        self.calls = []

    def set_tuning(self, **kw):
        kw = {k: v for k, v in kw.items() if v}
        if kw.get("resolver_contacts") == 192 and kw.get("resolver_lanes") == 32:
            raise RuntimeError("does not fit in shared memory")
        self.calls.append(kw)
        self.cfg.update(kw)

    def get_tuning(self):
        return dict(self.cfg)

    def restore(self):
        self.restores += 1

    def step_timed(self, frames, dt):
        c = self.cfg
        npm = {32: 1.0, 64: 2.0, 128: 3.0, 256: 4.0}[c["narrowphase_threads"]]
        rs = 10.0 + abs(c["resolver_lanes"] - 16) + abs(c["resolver_contacts"] - 96) / 32.0
        rs += 5.0 if c["large_world_lanes"] == 16 else 0.0
        if c["fused_frame"] == 1 and c["resolver_lanes"] == 32:
            return 8.0, np.array([0.0, 0.0, 8.0])
        ph = np.array([0.5, npm, rs])
        return float(ph.sum()), ph


def test_search_keeps_the_fastest_settings():
    b = FakeBatch([32] * 8)
    cfg, trials = autotune.tune(b, frames=2)
    assert cfg["narrowphase_threads"] == 32
    assert cfg["resolver_lanes"] == 16 and cfg["resolver_contacts"] == 96
    assert any("error" in t for t in trials)  # the refused shape is recorded, not fatal
    assert not any("large_world_lanes" in t for t in trials)  # no world above 64 bodies
    assert b.restores == len([t for t in trials if "error" not in t]) + 1


def test_large_world_lanes_tried_only_with_large_worlds():
    b = FakeBatch([32, 80, 1024])
    cfg, trials = autotune.tune(b, frames=2)
    tried = [t["large_world_lanes"] for t in trials if "large_world_lanes" in t]
    assert tried == list(autotune.DEFAULT_LARGE_LANES)
    assert cfg["large_world_lanes"] == 32


def test_fused_frame_tried_with_one_world_per_warp():
    b = FakeBatch([32] * 8)
    cfg, trials = autotune.tune(b, frames=2, lanes=(32,))
    tried = [t["fused_frame"] for t in trials if "fused_frame" in t]
    assert tried == [-1, 1]
    assert cfg["fused_frame"] == 1
    b = FakeBatch([32, 80])
    cfg, trials = autotune.tune(b, frames=2, lanes=(32,))
    assert not any("fused_frame" in t for t in trials)  # a world above the slot
    b = FakeBatch([32] * 8)
    b.warm_start = True
    cfg, trials = autotune.tune(b, frames=2, lanes=(32,))
    assert not any("fused_frame" in t for t in trials)  # the learned resolver
