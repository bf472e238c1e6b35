"""One-step outliers of the precision form, classified (TEST INFRASTRUCTURE:
an analysis tool, not on the product path).

Steps the bench scene (the precision workload: 32 bodies per world, 16
spheres + 16 cubes) one frame from its initial state in both of the oracle's
instantiations (float64, and float32 with the float64 islands: the GPU's two
forms bit for bit), computes each body's relative error per quantity as
bench.py's accuracy block does (|x - x64|_inf / max(|x64|_inf, 1)), and
classifies every world holding a body above 1e-4:

  contacts differ      the frame's contact lists differ (count or the pair
                       sequence): a narrowphase threshold decided differently;
  iterations differ    same contact pairs, but adjustPositions or
                       adjustVelocities used a different number of iterations:
                       the sequential resolver took another path;
  same path            same pairs and iteration counts: the difference is the
                       float32 arithmetic along the same path, or a different
                       choice among contacts that left the counts equal.

With --trace N, the first N worlds of the velocity outliers are replayed on
the second restatement (oracle/rigidbody_ref.py, bit-identical with the
oracle) in both arithmetics, recording which contact each iteration
resolved: "other choice" when the two sequences differ, "same choices" when
they are identical (the arithmetic of the same resolutions drifted apart).

    python -m oracle.accuracy_outliers [--worlds N] [--seed S] [--threads T] [--trace N]
"""
import argparse
import collections

import numpy as np

from cubez_gb300 import scenes
from oracle.oracle import FP32, FP64, OracleBatch, hardware_threads

QUANTITIES = ("position", "orientation", "velocity", "rotation")


def world_bodies(sc, w, real):
    """World w's bodies as the second restatement's dicts, derived data
    computed (in the type `real`)."""
    from oracle import rigidbody_ref
    offs = sc.collider_offset if sc.collider_offset is not None else np.tile(scenes.IDENTITY_OFFSET,
                                                                              (sc.num_bodies, 1))

    def v(a):
        return [real(x) for x in np.ravel(a)]

    bodies = []
    for i in range(sc.world_slice(w).start, sc.world_slice(w).stop):
        b = {"shape": int(sc.shape[i]), "half": v(sc.half_size[i]), "radius": real(sc.radius[i]),
             "position": v(sc.position[i]), "orientation": v(sc.orientation[i]),
             "velocity": v(sc.velocity[i]), "rotation": v(sc.rotation[i]),
             "acceleration": v(sc.acceleration[i]), "iit_body": v(sc.inverse_inertia[i]),
             "inverse_mass": real(sc.inverse_mass[i]), "linear_damping": float(sc.linear_damping[i]),
             "angular_damping": float(sc.angular_damping[i]), "can_sleep": bool(sc.can_sleep[i]),
             "awake": bool(sc.is_awake[i]), "lfa": [real(0.0)] * 3, "offset": v(offs[i]),
             "motion": real(sc.motion[i])}
        rigidbody_ref.calculate_derived_data(b)
        bodies.append(b)
    return bodies


def resolution_trace(sc, w, real, dt=1.0 / 60.0):
    """The contacts world w's first frame resolves, in order, in arithmetic `real`."""
    from oracle import rigidbody_ref
    trace = []
    rigidbody_ref.step(world_bodies(sc, w, real), [real(x) for x in sc.plane], dt, trace=trace)
    return trace


def classify(num_worlds=16384, seed=3, threads=0, dt=1.0 / 60.0, trace=0):
    sc = scenes.precision(num_worlds=num_worlds, seed=seed)
    threads = threads or hardware_threads()
    ref, low = OracleBatch(sc, form=FP64), OracleBatch(sc, form=FP32)
    ref.step(1, dt, 4, threads)
    low.step(1, dt, 4, threads)
    r, a = ref.bodies(), low.bodies()
    world_of = np.repeat(np.arange(sc.num_worlds), sc.counts)
    rs, ls = ref.stats(), low.stats()
    kinds = {}

    def kind(w):
        if w not in kinds:
            cr, cl = ref.contacts(int(w)), low.contacts(int(w))
            if len(cr["penetration"]) != len(cl["penetration"]) or not np.array_equal(cr["bodies"], cl["bodies"]):
                kinds[w] = "contacts differ"
            elif rs["pos_iterations"][w] != ls["pos_iterations"][w] or rs["vel_iterations"][w] != ls["vel_iterations"][w]:
                kinds[w] = "iterations differ"
            else:
                kinds[w] = "same path"
        return kinds[w]

    out = {}
    for q in QUANTITIES:
        den = np.maximum(np.abs(r[q]).max(axis=1), 1.0)
        e = np.abs(a[q] - r[q]).max(axis=1) / den
        bad = np.nonzero(e > 1e-4)[0]
        worlds = np.unique(world_of[bad])
        by_kind = collections.Counter(kind(w) for w in worlds)
        bodies_by_kind = collections.Counter(kind(world_of[i]) for i in bad)
        out[q] = {"bodies": int(len(bad)), "of": int(len(e)), "max": float(e.max()),
                  "worlds": int(len(worlds)), "worlds_by_kind": dict(by_kind),
                  "bodies_by_kind": dict(bodies_by_kind)}
        if q == "velocity" and trace:
            choices = collections.Counter()
            for w in worlds[:trace]:
                same = resolution_trace(sc, int(w), float, dt) == resolution_trace(sc, int(w), np.float32, dt)
                choices["same choices" if same else "other choice"] += 1
            out[q]["traced"] = dict(choices)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--worlds", type=int, default=16384)
    ap.add_argument("--seed", type=int, default=3)
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--trace", type=int, default=0)
    a = ap.parse_args()
    res = classify(a.worlds, a.seed, a.threads, trace=a.trace)
    print("| quantity | bodies above 1e-4 | max | worlds | contacts differ | iterations differ | same path |")
    print("|---|---:|---:|---:|---:|---:|---:|")
    for q, v in res.items():
        k = v["worlds_by_kind"]
        print("| %s | %d of %d | %.2g | %d | %d | %d | %d |" % (
            q, v["bodies"], v["of"], v["max"], v["worlds"], k.get("contacts differ", 0),
            k.get("iterations differ", 0), k.get("same path", 0)))
    if "traced" in res["velocity"]:
        print("velocity outlier worlds replayed with a resolution trace:", res["velocity"]["traced"])


if __name__ == "__main__":
    main()
