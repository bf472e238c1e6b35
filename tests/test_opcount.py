"""The operation counter of oracle/opcount.py on a test whose count is known
by hand: CheckAgainstSphere for two touching spheres (colliders.go:216-254)
is 22 floating-point operations (the midline 3, its magnitude 6, the radius
sum 1, the point 6, the normal 4, the penetration 2).  CPU only."""
from oracle import colliders_ref as cr
from oracle import contact_ref, opcount


def test_sphere_sphere_count():
    def body(x, r):
        b = {"shape": cr.SPHERE, "half": [opcount.CF(0)] * 3, "radius": opcount.CF(r),
             "position": [opcount.CF(x), opcount.CF(0), opcount.CF(0)],
             "orientation": [opcount.CF(1), opcount.CF(0), opcount.CF(0), opcount.CF(0)],
             "velocity": [opcount.CF(0)] * 3, "offset": [opcount.CF(v) for v in (1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0)]}
        b["T"] = [opcount.CF(v) for v in (1, 0, 0, 0, 1, 0, 0, 0, 1, x, 0, 0)]
        return b
    a, b = body(0.0, 1.0), body(1.5, 1.0)
    saved = contact_ref.sqrt_, cr.sqrt_
    contact_ref.sqrt_ = cr.sqrt_ = opcount._sqrt
    try:
        opcount.Counter.flops = opcount.Counter.compares = 0
        out = []
        cr.sphere_sphere(a, 0, b, 1, out)
    finally:
        contact_ref.sqrt_, cr.sqrt_ = saved
    assert len(out) == 1 and float(out[0][4]) == 0.5
    assert opcount.Counter.flops == 22
    assert opcount.Counter.compares == 2


def test_counts_grow_with_contact():
    """A settled world costs more than the same bodies spread apart (fewer
    pairs pass the cull when the bodies are far from one another)."""
    from cubez_gb300 import scenes
    sc = scenes.precision(num_worlds=1, bodies=32, seed=3)
    ident = scenes.IDENTITY_OFFSET.tolist()
    bodies = [{"shape": int(sc.shape[i]), "half": sc.half_size[i].tolist(), "radius": float(sc.radius[i]),
               "position": sc.position[i].tolist(), "orientation": sc.orientation[i].tolist(),
               "velocity": sc.velocity[i].tolist(), "offset": ident} for i in range(32)]
    flops, compares, pairs, full = opcount.count_world(bodies, sc.plane.tolist())
    assert pairs == 32 * 31 and 0 <= full < pairs
    far = [dict(b, position=[p * 100.0 for p in b["position"]]) for b in bodies]
    flops_far, _, _, full_far = opcount.count_world(far, sc.plane.tolist())
    assert full_far <= full and flops_far <= flops
