"""Operation counts of the narrowphase (TEST INFRASTRUCTURE: an analysis
tool, not on the product path).

Runs the second restatement of the colliders (oracle/colliders_ref.py) with
counting floats, so every floating-point add, subtract, multiply, divide and
square root of the reference's tests is counted as it would execute, plus
the float32 culls of the GPU narrowphase (restated from k_narrowphase's
pair_test).  The result is the algorithmic floating-point work of one frame's
narrowphase on a scene: the figure a floating-point roofline of the kernel
divides by its time.

    python -m oracle.opcount [frames ...]

prints, for the precision workload's distribution (32 bodies per world,
16 spheres + 16 cubes), the operations per frame and world at the given
frames of a rollout (default 30 150 300 600).
"""
import math
import sys

import numpy as np

from oracle import colliders_ref as cr
from oracle import contact_ref


class Counter:
    flops = 0
    compares = 0


class CF:
    """A float that counts the arithmetic done on it (IEEE float64 values)."""
    __slots__ = ("v",)

    def __init__(self, v):
        self.v = float(v.v if isinstance(v, CF) else v)

    @staticmethod
    def _val(o):
        return o.v if isinstance(o, CF) else float(o)

    def _op(self, r):
        Counter.flops += 1
        return CF(r)

    def __add__(self, o): return self._op(self.v + CF._val(o))
    def __radd__(self, o): return self._op(CF._val(o) + self.v)
    def __sub__(self, o): return self._op(self.v - CF._val(o))
    def __rsub__(self, o): return self._op(CF._val(o) - self.v)
    def __mul__(self, o): return self._op(self.v * CF._val(o))
    def __rmul__(self, o): return self._op(CF._val(o) * self.v)
    def __truediv__(self, o): return self._op(self.v / CF._val(o))
    def __rtruediv__(self, o): return self._op(CF._val(o) / self.v)
    def __neg__(self): return CF(-self.v)
    def __abs__(self): return CF(abs(self.v))
    def __float__(self): return self.v

    def _cmp(self, r):
        Counter.compares += 1
        return r

    def __lt__(self, o): return self._cmp(self.v < CF._val(o))
    def __le__(self, o): return self._cmp(self.v <= CF._val(o))
    def __gt__(self, o): return self._cmp(self.v > CF._val(o))
    def __ge__(self, o): return self._cmp(self.v >= CF._val(o))
    def __eq__(self, o): return self._cmp(self.v == CF._val(o))
    def __ne__(self, o): return self._cmp(self.v != CF._val(o))
    __hash__ = None


def _sqrt(x):
    if isinstance(x, CF):
        Counter.flops += 1
        return CF(math.sqrt(x.v))
    return math.sqrt(x)


def _cull_radii(body):
    """The bounding radii of np_build_tile, once per body: |h|_2 and |h|_1
    (each times 1.0001), or the sphere's radius."""
    if body["shape"] == cr.SPHERE:
        return body["radius"], body["radius"]
    h = body["half"]
    return _sqrt(h[0] * h[0] + h[1] * h[1] + h[2] * h[2]) * 1.0001, (h[0] + h[1] + h[2]) * 1.0001


def _cull(a, b):
    """pair_test's float32 culls (Cull in k_narrowphase), counted: True when
    the full test is skipped."""
    ca, cb = cr.get_axis(a["T"], 3), cr.get_axis(b["T"], 3)
    d = [cb[k] - ca[k] for k in range(3)]
    sc = 1.0 + abs(ca[0]) + abs(ca[1]) + abs(ca[2]) + abs(cb[0]) + abs(cb[1]) + abs(cb[2])
    d2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2]
    (rba, rla), (rbb, rlb) = a["cull"], b["cull"]
    if a["shape"] == cr.SPHERE and b["shape"] == cr.SPHERE:
        t = rba + rbb + 1e-3 + 1e-5 * sc
    elif a["shape"] == cr.CUBE and b["shape"] == cr.CUBE:
        t = (rba + rbb) * 1.1 + 1e-3 + 1e-5 * sc
    else:
        box_rl, sph_rb = (rla, rbb) if a["shape"] == cr.CUBE else (rlb, rba)
        t = box_rl + 3.0 * sph_rb + 1e-3 + 1e-5 * sc
    return d2 > t * t


def count_world(bodies, plane):
    """Counts for one world's ordered narrowphase: (flops, compares,
    pair tests, pair tests the cull let through)."""
    contact_ref_sqrt, cr_sqrt = contact_ref.sqrt_, cr.sqrt_
    contact_ref.sqrt_, cr.sqrt_ = _sqrt, _sqrt
    try:
        Counter.flops = Counter.compares = 0
        cb = []
        for b in bodies:
            c = dict(b)
            for k in ("half", "position", "orientation", "velocity", "offset"):
                c[k] = [CF(x) for x in b[k]]
            c["radius"] = CF(b["radius"])
            c["T"] = cr.collider_transform(c)  # the tile build, once per body
            c["cull"] = _cull_radii(c)
            cb.append(c)
        pl = [CF(x) for x in plane]
        full = 0
        out = []
        for i, a in enumerate(cb):
            if a["shape"] == cr.SPHERE:
                cr.sphere_half_space(a, i, pl, out)
            else:
                cr.cube_half_space(a, i, pl, out)
            for j, o in enumerate(cb):
                if j == i:
                    continue
                if _cull(a, o):
                    continue
                full += 1
                cr.check_for_collisions(a, i, o, j, out)
        n = len(bodies)
        return Counter.flops, Counter.compares, n * (n - 1), full
    finally:
        contact_ref.sqrt_, cr.sqrt_ = contact_ref_sqrt, cr_sqrt


def main(frames):
    from cubez_gb300 import scenes
    from oracle.oracle import FP64, OracleBatch
    sc = scenes.precision(num_worlds=8, bodies=32, seed=3)
    ident = scenes.IDENTITY_OFFSET.tolist()
    for fr in frames:
        o = OracleBatch(sc, form=FP64)
        o.step(fr - 1, 1.0 / 60.0)
        o.integrate(1.0 / 60.0)  # the state frame fr's narrowphase sees
        st = o.bodies()
        tot = np.zeros(4)
        for w in range(sc.num_worlds):
            sl = sc.world_slice(w)
            bodies = [{"shape": int(sc.shape[i]), "half": sc.half_size[i].tolist(), "radius": float(sc.radius[i]),
                       "position": st["position"][i].tolist(), "orientation": st["orientation"][i].tolist(),
                       "velocity": st["velocity"][i].tolist(), "offset": ident} for i in range(sl.start, sl.stop)]
            tot += count_world(bodies, sc.plane.tolist())
        f, c, pairs, full = tot / sc.num_worlds
        print("frame %4d: %8.0f flops, %7.0f compares per world; %4.0f of %4.0f pair tests past the cull"
              % (fr, f, c, full, pairs))


if __name__ == "__main__":
    main([int(x) for x in sys.argv[1:]] or [30, 150, 300, 600])
