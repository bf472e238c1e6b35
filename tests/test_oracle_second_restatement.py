"""The C++ oracle's resolver against a second, independent restatement of
contact.go in plain Python (oracle/contact_ref.py), bit for bit: the same
frames' contact lists resolved by both, then every body's state, the
iteration counts and the resolved contacts compared.  CPU only."""
import numpy as np
import pytest

from cubez_gb300 import scenes
from oracle import contact_ref
from oracle.oracle import FP32, FP64, OracleBatch

DT = 1.0 / 60.0


def _python_world(o, sc, w, st):
    sl = sc.world_slice(w)
    bodies = []
    for i in range(sl.start, sl.stop):
        bodies.append({"position": st["position"][i].tolist(), "orientation": st["orientation"][i].tolist(),
                       "velocity": st["velocity"][i].tolist(), "rotation": st["rotation"][i].tolist(),
                       "iit": st["iit_world"][i].tolist(), "inverse_mass": float(sc.inverse_mass[i]),
                       # right after Integrate with no forces: lastFrameAccelleration = Acceleration
                       "lfa": sc.acceleration[i].tolist(), "awake": bool(st["is_awake"][i])})
    c = o.contacts(w)
    contacts = [contact_ref.Contact(int(b[0]) if b[0] >= 0 else None, int(b[1]) if b[1] >= 0 else None,
                                    p.tolist(), n.tolist(), float(pen))
                for b, p, n, pen in zip(c["bodies"], c["point"], c["normal"], c["penetration"])]
    return bodies, contacts


SCENES = {
    "mixed_early": lambda: (scenes.mixed(num_worlds=8, seed=61, min_bodies=6, max_bodies=12), 40),
    "mixed_landed": lambda: (scenes.mixed(num_worlds=8, seed=63, min_bodies=6, max_bodies=12), 150),
    "mixed_crowded": lambda: (scenes.mixed(num_worlds=4, seed=64, min_bodies=20, max_bodies=24), 240),
    # 3 x 3 x 2 cubes dropped into a pile: box-box contacts in both orders
    "pile": lambda: (scenes.piles(num_worlds=3, seed=65, nx=3, nz=3, ny=2, spacing=1.1), 60),
}


@pytest.mark.parametrize("name", sorted(SCENES))
def test_resolver_matches_second_restatement(name, oracle_lib):
    sc, settle = SCENES[name]()
    o = OracleBatch(sc, form=FP64)
    o.step(settle, DT)
    o.integrate(DT)
    o.narrowphase()
    st = o.bodies()
    worlds = [_python_world(o, sc, w, st) for w in range(sc.num_worlds)]
    o.resolve(DT, iter_mult=4)
    after = o.bodies()
    stats = o.stats()
    resolved_any = 0
    for w, (bodies, contacts) in enumerate(worlds):
        pos_used, vel_used = contact_ref.resolve_contacts(len(contacts) * 4, contacts, bodies, DT)
        assert (pos_used, vel_used) == (stats["pos_iterations"][w], stats["vel_iterations"][w]), w
        resolved_any += vel_used
        sl = sc.world_slice(w)
        for k in ("position", "orientation", "velocity", "rotation"):
            got = np.array([b[k] for b in bodies]).reshape(after[k][sl].shape)
            assert np.array_equal(got, after[k][sl]), "world %d: %s differs" % (w, k)
        rc = o.resolved_contacts(w)
        assert np.array_equal(np.array([c.penetration for c in contacts]), rc["penetration"])
        assert np.array_equal(np.array([c.normal for c in contacts]).reshape(-1, 3), rc["normal"])
        assert [[c.bodies[0], -1 if c.bodies[1] is None else c.bodies[1]] for c in contacts] == rc["bodies"].tolist()
    assert resolved_any > 0


NARROW_SCENES = {
    "mixed": lambda: (scenes.mixed(num_worlds=6, seed=66, min_bodies=10, max_bodies=16), 120),
    "pile": lambda: (scenes.piles(num_worlds=2, seed=67, nx=3, nz=3, ny=2, spacing=1.1), 60),
    "offsets": lambda: (scenes.offsets(num_worlds=4, bodies=14, seed=68, nonrigid=0.3), 120),
    "cubedrop": lambda: (scenes.cubedrop(seed=1), 150),
    # 16 spheres + 16 cubes per world: box-sphere contacts in both orders
    "precision": lambda: (scenes.precision(num_worlds=3, bodies=32, seed=69), 200),
}


@pytest.mark.parametrize("name", sorted(NARROW_SCENES))
def test_narrowphase_matches_second_restatement(name, oracle_lib):
    """The oracle's contact lists (every narrowphase branch the scenes reach,
    in the reference's order) against oracle/colliders_ref.py."""
    from oracle import colliders_ref
    sc, settle = NARROW_SCENES[name]()
    o = OracleBatch(sc, form=FP64)
    o.step(settle, DT)
    o.integrate(DT)
    o.narrowphase()
    st = o.bodies()
    offs = sc.collider_offset if sc.collider_offset is not None else np.tile(scenes.IDENTITY_OFFSET,
                                                                              (sc.num_bodies, 1))
    kinds = set()
    for w in range(sc.num_worlds):
        sl = sc.world_slice(w)
        bodies = [{"shape": int(sc.shape[i]), "half": sc.half_size[i].tolist(), "radius": float(sc.radius[i]),
                   "position": st["position"][i].tolist(), "orientation": st["orientation"][i].tolist(),
                   "velocity": st["velocity"][i].tolist(), "offset": offs[i].tolist()}
                  for i in range(sl.start, sl.stop)]
        got = colliders_ref.generate_contacts(bodies, sc.plane.tolist())
        want = o.contacts(w)
        assert len(got) == len(want["penetration"]), "world %d: %d vs %d contacts" % (w, len(got),
                                                                                    len(want["penetration"]))
        for k, (b0, b1, p, n, pen) in enumerate(got):
            assert [b0, -1 if b1 is None else b1] == want["bodies"][k].tolist(), (w, k)
            assert np.array_equal(p, want["point"][k]) and np.array_equal(n, want["normal"][k]), (w, k)
            assert pen == want["penetration"][k], (w, k)
            kinds.add((bodies[b0]["shape"], None if b1 is None else bodies[b1]["shape"]))
    assert len(kinds) >= 2 and sum(len(o.contacts(w)["penetration"]) for w in range(sc.num_worlds)) > 0
    if name == "precision":
        assert (scenes.CUBE, scenes.SPHERE) in kinds


def _frame_bodies(sc, w, real=float):
    """The scene's bodies of world w as set up (CalculateDerivedData done), in
    the form's real type (the dampings stay float64: their powers are taken in
    float64)."""
    from oracle import rigidbody_ref
    sl = sc.world_slice(w)
    offs = sc.collider_offset if sc.collider_offset is not None else np.tile(scenes.IDENTITY_OFFSET,
                                                                              (sc.num_bodies, 1))

    def v(a):
        return [real(x) for x in np.ravel(a)]

    bodies = []
    for i in range(sl.start, sl.stop):
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


def _sleepy(make):
    def f():
        sc = make()
        sc.can_sleep[:] = 1
        return sc
    return f


FRAME_SCENES = {
    "cubedrop": (lambda: scenes.cubedrop(seed=2), 90),
    "mixed": (lambda: scenes.mixed(num_worlds=3, seed=70, min_bodies=8, max_bodies=12), 90),
    "offsets": (lambda: scenes.offsets(num_worlds=2, bodies=10, seed=71, nonrigid=0.3), 90),
    # CanSleep on: the motion average and SetAwake (13 of 28 bodies asleep at
    # once), and in a pile matchAwakeState waking sleeping bodies (49 times)
    "sleeping": (_sleepy(lambda: scenes.mixed(num_worlds=2, seed=74, min_bodies=12, max_bodies=14)), 400),
    "sleeping_pile": (_sleepy(lambda: scenes.piles(num_worlds=1, seed=73, nx=3, nz=3, ny=2, spacing=1.1)), 300),
}


@pytest.mark.parametrize("form", [FP64, FP32])
@pytest.mark.parametrize("name", sorted(FRAME_SCENES))
def test_frames_match_second_restatement(name, form, oracle_lib, monkeypatch):
    """Whole frames (Integrate, the ordered narrowphase, ResolveContacts) of
    the Python restatement against the oracle's step, every frame."""
    from oracle import rigidbody_ref
    transitions = {"sleep": 0, "wake": 0}
    set_awake = rigidbody_ref.set_awake

    def counting_set_awake(b, awake):
        if awake != b["awake"]:
            transitions["wake" if awake else "sleep"] += 1
        set_awake(b, awake)

    monkeypatch.setattr(rigidbody_ref, "set_awake", counting_set_awake)
    make, frames = FRAME_SCENES[name]
    sc = make()
    real = float if form == FP64 else np.float32
    o = OracleBatch(sc, form=form)
    worlds = [_frame_bodies(sc, w, real) for w in range(sc.num_worlds)]
    plane = [real(x) for x in sc.plane]
    total = 0
    for fr in range(frames):
        o.step(1, DT)
        st, stats = o.bodies(), o.stats()
        for w, bodies in enumerate(worlds):
            n, pit, vit = rigidbody_ref.step(bodies, plane, DT)
            assert (n, pit, vit) == (stats["contacts"][w], stats["pos_iterations"][w],
                                     stats["vel_iterations"][w]), (fr, w)
            total += n
            sl = sc.world_slice(w)
            for k in ("position", "orientation", "velocity", "rotation"):
                got = np.array([b[k] for b in bodies], dtype=np.float64)
                assert np.array_equal(got, st[k][sl]), "frame %d world %d: %s differs" % (fr, w, k)
            assert np.array_equal(np.array([b["iit"] for b in bodies], dtype=np.float64), st["iit_world"][sl])
            assert np.array_equal(np.array([b["motion"] for b in bodies], dtype=np.float64), st["motion"][sl])
            assert [int(b["awake"]) for b in bodies] == st["is_awake"][sl].tolist()
    assert total > 50
    if name == "sleeping":
        assert transitions["sleep"] > 10
    if name == "sleeping_pile":
        assert transitions["wake"] > 10  # matchAwakeState woke sleeping bodies


def test_resolver_materials_match_second_restatement(oracle_lib):
    """Per-contact friction and restitution (the fields the resolver reads;
    the colliders write 0.9 and 0.1): frictionless two-body contacts take
    calculateFrictionlessImpulse with its inverted nil test (only the first
    body's response), the others the friction solve with varied friction and
    restitution."""
    sc = scenes.mixed(num_worlds=6, seed=75, min_bodies=16, max_bodies=20)
    o = OracleBatch(sc, form=FP64)
    o.step(200, DT)
    o.integrate(DT)
    o.narrowphase()
    st = o.bodies()
    rng = np.random.default_rng(5)
    worlds = []
    for w in range(sc.num_worlds):
        bodies, contacts = _python_world(o, sc, w, st)
        c = o.contacts(w)
        n = len(contacts)
        two = c["bodies"][:, 1] >= 0
        fric = np.where(two, 0.0, rng.uniform(0.2, 1.0, n))
        rest = rng.uniform(0.0, 0.6, n)
        for k, ct in enumerate(contacts):
            ct.friction, ct.restitution = float(fric[k]), float(rest[k])
        o.set_contacts(w, {"bodies": c["bodies"], "point": c["point"], "normal": c["normal"],
                           "penetration": c["penetration"], "friction": fric, "restitution": rest})
        worlds.append((bodies, contacts, int((fric == 0).sum())))
    max_it = 200
    o.resolve_fixed(max_it, DT)
    after, stats = o.bodies(), o.stats()
    frictionless = 0
    for w, (bodies, contacts, nf) in enumerate(worlds):
        pit, vit = contact_ref.resolve_contacts(max_it, contacts, bodies, DT)
        assert (pit, vit) == (stats["pos_iterations"][w], stats["vel_iterations"][w]), w
        sl = sc.world_slice(w)
        for k in ("position", "orientation", "velocity", "rotation"):
            got = np.array([b[k] for b in bodies]).reshape(after[k][sl].shape)
            assert np.array_equal(got, after[k][sl]), "world %d: %s differs" % (w, k)
        frictionless += nf
    assert frictionless > 5


def test_frictionless_single_body_contact_is_the_nil_case(oracle_lib):
    """A frictionless contact with one body reaches the reference's nil
    dereference (contact.go:512): the Python restatement raises, the oracle
    reports it as a status bit (the C ABI's CZ_ERR_FRICTIONLESS)."""
    sc = scenes.cubedrop(seed=1)
    o = OracleBatch(sc, form=FP64)
    o.step(30, DT)
    o.integrate(DT)
    o.narrowphase()
    st = o.bodies()
    bodies, contacts = _python_world(o, sc, 0, st)
    c = o.contacts(0)
    one = c["bodies"][:, 1] < 0
    assert one.any()
    fric = np.where(one, 0.0, 0.9)
    for k, ct in enumerate(contacts):
        ct.friction = float(fric[k])
    o.set_contacts(0, {"bodies": c["bodies"], "point": c["point"], "normal": c["normal"],
                       "penetration": c["penetration"], "friction": fric, "restitution": np.full(len(fric), 0.1)})
    status = o.resolve_fixed(4 * len(fric), DT)
    assert status & 2  # the frictionless-nil bit
    with pytest.raises(contact_ref.NilBody):
        contact_ref.resolve_contacts(4 * len(fric), contacts, bodies, DT)


@pytest.mark.parametrize("form", [FP64, FP32])
def test_ballistic_frames_match_second_restatement(form, oracle_lib):
    """examples/ballistic.go's loop (the example's test order, ResolveContacts
    with len(contacts) * 8, the static backboard integrated as a static body)
    frame by frame against the oracle."""
    from oracle import rigidbody_ref
    sc = scenes.ballistic(num_worlds=2, bullets=6, seed=77)
    real = float if form == FP64 else np.float32
    o = OracleBatch(sc, form=form)
    units = scenes.ballistic_units(int(sc.counts[0]))
    worlds = [_frame_bodies(sc, w, real) for w in range(sc.num_worlds)]
    plane = [real(x) for x in sc.plane]
    total = 0
    for fr in range(150):
        o.integrate(DT)
        for w in range(sc.num_worlds):
            o.collide(w, units)
        o.resolve(DT, iter_mult=8)
        st, stats = o.bodies(), o.stats()
        for w, bodies in enumerate(worlds):
            n, pit, vit = rigidbody_ref.step(bodies, plane, DT, iter_mult=8, units=units.tolist())
            assert (n, pit, vit) == (stats["contacts"][w], stats["pos_iterations"][w],
                                     stats["vel_iterations"][w]), (fr, w)
            total += n
            sl = sc.world_slice(w)
            for k in ("position", "orientation", "velocity", "rotation"):
                got = np.array([b[k] for b in bodies], dtype=np.float64)
                assert np.array_equal(got, st[k][sl]), "frame %d world %d: %s differs" % (fr, w, k)
    assert total > 50
