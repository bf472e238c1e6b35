"""Writes the golden fixtures of tests/golden/ from the oracle (the
restatement of the reference's path: float64, and for the *_precision
fixtures its float32 instantiation with the float64 islands), for the tests
and, for the float64 ones, for a later run of the reference itself where a Go
toolchain exists.

    python tests/golden/make_golden.py

Each fixture is JSON: the scene's generator and arguments, the frame loop, the
damping powers the host's std::pow gave (the only libm values the path
depends on), and per listed frame the contact count and the body state
(position, orientation, velocity, rotation) as float.hex strings.
"""
import json
import math
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from cubez_gb300 import scenes  # noqa: E402
from oracle.oracle import FP32, FP64, OracleBatch  # noqa: E402

DT = 1.0 / 60.0
STATE = ("position", "orientation", "velocity", "rotation")

FIXTURES = {
    # examples/cubedrop.go's loop: 20 cubes dropped on the plane
    "cubedrop_seed1": {"scene": ("cubedrop", {"seed": 1}), "loop": "cubedrop", "frames": [1, 10, 60, 240]},
    # examples/ballistic.go's loop: cube, static backboard, six bullets
    "ballistic_seed74": {"scene": ("ballistic", {"num_worlds": 1, "bullets": 6, "seed": 74}), "loop": "ballistic",
                         "frames": [1, 40, 120]},
    # colliders with Offsets (some scaled) in the cubedrop loop
    "offsets_seed73": {"scene": ("offsets", {"num_worlds": 1, "bodies": 14, "seed": 73, "nonrigid": 0.3}),
                       "loop": "cubedrop", "frames": [1, 60, 150]},
    # the precision form: a world of the bench scene (16 spheres + 16 cubes)
    # and the cubedrop scene, in float32 with the float64 islands
    "precision_seed3_precision": {"scene": ("precision", {"num_worlds": 1, "seed": 3}), "loop": "cubedrop",
                                  "frames": [1, 30, 120, 300], "form": FP32},
    "cubedrop_seed1_precision": {"scene": ("cubedrop", {"seed": 1}), "loop": "cubedrop", "frames": [1, 60, 240],
                                 "form": FP32},
}


def build_scene(spec):
    name, kw = spec
    return getattr(scenes, name)(**kw)


def run(spec):
    """Frames of the fixture's loop on the oracle: {frame: (contacts, state)}."""
    sc = build_scene(spec["scene"])
    o = OracleBatch(sc, form=spec.get("form", FP64))
    units = scenes.ballistic_units(int(sc.counts[0])) if spec["loop"] == "ballistic" else None
    out = {}
    for fr in range(1, max(spec["frames"]) + 1):
        if units is None:
            o.step(1, DT)
        else:
            o.integrate(DT)
            o.collide(0, units)
            o.resolve(DT, iter_mult=8)
        if fr in spec["frames"]:
            b = o.bodies()
            out[fr] = (int(o.stats()["contacts"][0]), {k: np.asarray(b[k]) for k in STATE})
    return sc, out


def damping_powers(sc):
    vals = sorted(set(sc.linear_damping.tolist()) | set(sc.angular_damping.tolist()) | {0.5})
    return {float.hex(v): float.hex(math.pow(v, DT)) for v in vals}


def main():
    for name, spec in FIXTURES.items():
        sc, out = run(spec)
        doc = {"scene": {"generator": spec["scene"][0], "args": spec["scene"][1]}, "loop": spec["loop"],
               "dt": float.hex(DT),
               "form": "float64" if spec.get("form", FP64) == FP64 else "float32 with float64 islands",
               "pow_dt": damping_powers(sc),
               "frames": {str(fr): {"contacts": c, **{k: [[float.hex(float(x)) for x in row] for row in st[k]]
                                                      for k in STATE}}
                          for fr, (c, st) in out.items()}}
        with open(os.path.join(HERE, name + ".json"), "w") as f:
            json.dump(doc, f, indent=1)
            f.write("\n")
        print(name, {fr: c for fr, (c, _) in out.items()})


if __name__ == "__main__":
    main()
