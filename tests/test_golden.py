"""The oracle against the committed golden fixtures (tests/golden/*.json,
written by tests/golden/make_golden.py): the cubedrop and ballistic frame
loops and colliders with Offsets in float64, and a bench-scene world and the
cubedrop scene in the precision form, bit for bit at the listed frames.

The fixtures pin the oracle between changes; the GPU path is compared with
the oracle itself by the parity tests.  The path's only libm values are the
damping powers pow(damping, dt): on a host whose pow gives other bits the
fixture does not apply and the test says so."""
import json
import math
import os

import numpy as np
import pytest

from tests.golden import make_golden

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    with open(os.path.join(GOLDEN, name + ".json")) as f:
        return json.load(f)


@pytest.mark.parametrize("name", sorted(make_golden.FIXTURES))
def test_oracle_matches_golden(name, oracle_lib):
    doc = _load(name)
    spec = make_golden.FIXTURES[name]
    assert doc["scene"]["generator"] == spec["scene"][0] and doc["scene"]["args"] == spec["scene"][1]
    dt = float.fromhex(doc["dt"])
    for base, p in doc["pow_dt"].items():
        if math.pow(float.fromhex(base), dt) != float.fromhex(p):
            pytest.skip("this host's pow(%r, dt) differs from the fixture's" % float.fromhex(base))
    _, out = make_golden.run(spec)
    assert sorted(out) == sorted(int(f) for f in doc["frames"])
    for fr, (count, state) in out.items():
        want = doc["frames"][str(fr)]
        assert count == want["contacts"], "frame %d: %d contacts vs %d" % (fr, count, want["contacts"])
        for k in make_golden.STATE:
            w = np.array([[float.fromhex(x) for x in row] for row in want[k]])
            assert np.array_equal(state[k], w), "frame %d: %s differs" % (fr, k)


def test_golden_fixtures_are_complete():
    names = {f[:-5] for f in os.listdir(GOLDEN) if f.endswith(".json")}
    assert names == set(make_golden.FIXTURES)
    for name in names:
        doc = _load(name)
        n = None
        for fr, st in doc["frames"].items():
            for k in make_golden.STATE:
                rows = st[k]
                n = len(rows) if n is None else n
                assert len(rows) == n and all(len(r) == {"orientation": 4}.get(k, 3) for r in rows)
