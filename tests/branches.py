"""Which branch of the reference's narrowphase a scene's tests take, found by
running the second restatement (oracle/colliders_ref.py) in the form's
arithmetic with its branch points observed.  Test infrastructure."""
import contextlib

import numpy as np

from cubez_gb300 import scenes


@contextlib.contextmanager
def observed():
    """Record contactPoint's branch (colliders.go:519-573) and box-sphere's
    zero-normal fallback (colliders.go:414-421) while the block runs."""
    from oracle import colliders_ref as cr
    from oracle.contact_ref import EPSILON, dot, real_type
    seen = []
    contact_point, cube_sphere = cr._contact_point, cr.cube_sphere
    point_face, cube_cube = cr._point_face, cr.cube_cube
    current = []

    def cp(p_one, d_one, one_size, p_two, d_two, two_size, use_one):
        sm_one = d_one[0] * d_one[0] + d_one[1] * d_one[1] + d_one[2] * d_one[2]
        sm_two = d_two[0] * d_two[0] + d_two[1] * d_two[1] + d_two[2] * d_two[2]
        dp = dot(d_two, d_one)
        to_st = [p_one[k] - p_two[k] for k in range(3)]
        a, b = dot(d_one, to_st), dot(d_two, to_st)
        denom = sm_one * sm_two - dp * dp
        if abs(denom) < real_type(denom)(EPSILON):
            seen.append("edge_parallel")
        else:
            mua = (dp * b - sm_two * a) / denom
            mub = (sm_one * b - dp * a) / denom
            out = mua > one_size or mua < -one_size or mub > two_size or mub < -two_size
            seen.append("edge_out_of_range" if out else "edge_cross")
        return contact_point(p_one, d_one, one_size, p_two, d_two, two_size, use_one)

    def cs(c, i, s, j, out):
        n = len(out)
        cube_sphere(c, i, s, j, out)
        if len(out) > n and out[-1][4] == 0.0 and list(out[-1][3]) != [0.0, 0.0, 0.0]:
            seen.append("sphere_centre_in_box")

    def cc(one, i, two, j, out):
        current.append(i)
        try:
            cube_cube(one, i, two, j, out)
        finally:
            current.pop()

    def pf(one, i, two, j, to_center, best, pen, out):
        # fillPointFaceBoxBox(one, two) for best < 3, (two, one) for best < 6 (colliders.go:628-640)
        seen.append("vertex_face" if current and current[-1] == i else "vertex_face_swapped")
        point_face(one, i, two, j, to_center, best, pen, out)

    cr._contact_point, cr.cube_sphere, cr._point_face, cr.cube_cube = cp, cs, pf, cc
    try:
        yield seen
    finally:
        cr._contact_point, cr.cube_sphere, cr._point_face, cr.cube_cube = (contact_point, cube_sphere, point_face,
                                                                          cube_cube)


def narrowphase_branches(sc, form):
    """The branches world 0 of `sc` takes in its narrowphase, as set up
    (CalculateDerivedData done), in form 0 (float64) or 1 (float32)."""
    from oracle import colliders_ref, rigidbody_ref
    real = float if form == 0 else np.float32
    offs = sc.collider_offset if sc.collider_offset is not None else np.tile(scenes.IDENTITY_OFFSET,
                                                                              (sc.num_bodies, 1))

    def v(a):
        return [real(x) for x in np.ravel(a)]

    bodies = []
    for i in range(sc.world_slice(0).start, sc.world_slice(0).stop):
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
    with observed() as seen:
        contacts = colliders_ref.generate_contacts(bodies, [real(x) for x in sc.plane])
    return set(seen), contacts
