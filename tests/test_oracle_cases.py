"""The oracle's narrowphase on hand-built scenes, checked against values
worked out by hand from colliders.go (including its quirks: the plane contact
point is the vertex moved by the penetration once more, the sphere-sphere point
is half the midline from the first centre)."""
import math

import numpy as np
import pytest

from oracle.oracle import OracleBatch
from tests import cases


def contacts_of(scene):
    ob = OracleBatch(scene)
    ob.narrowphase()
    return ob.contacts(0)


def test_cube_resting_four_vertex_contacts():
    c = contacts_of(cases.cube_resting())
    assert len(c["penetration"]) == 4
    assert np.all(c["bodies"] == [0, -1])
    np.testing.assert_allclose(c["penetration"], 0.01, atol=1e-12)
    np.testing.assert_array_equal(c["normal"], np.tile([0.0, 1.0, 0.0], (4, 1)))
    # vertices with a negative y sign in the reference's order: mults 2, 3, 6, 7
    want_xz = np.array([[0.5, 0.5], [-0.5, 0.5], [0.5, -0.5], [-0.5, -0.5]])
    np.testing.assert_allclose(c["point"][:, [0, 2]], want_xz, atol=1e-12)
    np.testing.assert_allclose(c["point"][:, 1], -0.02, atol=1e-12)


def test_sphere_resting():
    c = contacts_of(cases.sphere_resting())
    assert len(c["penetration"]) == 1
    np.testing.assert_allclose(c["penetration"], [0.1], atol=1e-12)
    np.testing.assert_allclose(c["point"][0], [2.0, -0.2, -1.0], atol=1e-12)
    assert list(c["bodies"][0]) == [0, -1]


def test_sphere_pair_both_orders():
    c = contacts_of(cases.sphere_pair())
    assert len(c["penetration"]) == 2
    assert c["bodies"].tolist() == [[0, 1], [1, 0]]
    np.testing.assert_allclose(c["penetration"], [0.5, 0.5], atol=1e-12)
    np.testing.assert_allclose(c["normal"], [[-1, 0, 0], [1, 0, 0]], atol=1e-15)
    np.testing.assert_allclose(c["point"], [[-0.75, 5, 0], [2.25, 5, 0]], atol=1e-12)


def test_cube_sphere_same_contact_from_both_orders():
    c = contacts_of(cases.cube_sphere())
    assert len(c["penetration"]) == 2
    # (cube, sphere) and (sphere, cube) both give Bodies = [cube, sphere] (colliders.go:209-213)
    assert c["bodies"].tolist() == [[0, 1], [0, 1]]
    for k in ("point", "normal", "penetration"):
        np.testing.assert_array_equal(c[k][0], c[k][1])
    np.testing.assert_allclose(c["point"][0], [1.0, 5.0, 0.0], atol=1e-12)
    np.testing.assert_allclose(c["normal"][0], [-1.0, 0.0, 0.0], atol=1e-12)
    np.testing.assert_allclose(c["penetration"][0], 0.2, atol=1e-12)


def test_sphere_inside_cube_uses_velocity_normal():
    c = contacts_of(cases.sphere_inside_cube())
    assert len(c["penetration"]) == 2
    np.testing.assert_allclose(c["normal"][0], [0.0, -1.0, 0.0], atol=1e-15)  # colliders.go:417-421
    assert c["penetration"][0] == 0.0  # colliders.go:425-429
    np.testing.assert_allclose(c["point"][0], [0.2, 5.0, 0.0], atol=1e-12)


def test_cube_on_cube_vertex_face():
    c = contacts_of(cases.cube_on_cube())
    assert len(c["penetration"]) == 2
    # the lower box's top face is the reference face in both orders: Bodies[0] = 0
    assert c["bodies"].tolist() == [[0, 1], [0, 1]]
    np.testing.assert_allclose(c["normal"][0], [0.0, -1.0, 0.0], atol=1e-12)
    for k in ("point", "normal", "penetration"):
        np.testing.assert_allclose(c[k][0], c[k][1], atol=1e-12)
    # the lowest vertex of box 1 touches the top face y = 6 of box 0
    pen = c["penetration"][0]
    assert 0.0 < pen < 0.5
    np.testing.assert_allclose(c["point"][0][1], 6.0 - pen, atol=1e-9)


def test_cube_edge_edge():
    sc = cases.cube_edge_edge()
    c = contacts_of(sc)
    assert len(c["penetration"]) == 2
    n = c["normal"][0]
    assert abs(np.linalg.norm(n) - 1.0) < 1e-12
    # the edges are along x (box 0) and z (box 1): the normal is perpendicular to both
    assert abs(n[0]) < 1e-9 and abs(n[2]) < 1e-9
    np.testing.assert_allclose(c["penetration"][0], 0.04, atol=1e-9)
    # the point is the midpoint of the two edges' closest points
    d = 0.5 * math.sqrt(2.0)
    np.testing.assert_allclose(c["point"][0], [0.05, 5.0 + d - 0.02, 0.0], atol=1e-9)


def test_tilted_cube_single_vertex():
    c = contacts_of(cases.tilted_cube_on_plane())
    assert len(c["penetration"]) == 1
    half_diag = 0.5 * math.sqrt(3.0)
    np.testing.assert_allclose(c["penetration"][0], half_diag - 0.85, atol=1e-9)


def test_cube_edge_down_two_vertex_contacts():
    c = contacts_of(cases.cube_edge_down())
    assert len(c["penetration"]) == 2
    np.testing.assert_allclose(c["penetration"], 0.01, atol=1e-9)
    np.testing.assert_allclose(c["point"][:, 0], 0.0, atol=1e-9)
    assert sorted(np.round(c["point"][:, 2], 12).tolist()) == [-0.5, 0.5]


def test_cube_below_plane_eight_vertex_contacts():
    c = contacts_of(cases.cube_below_plane())
    assert len(c["penetration"]) == 8
    # penetration = offset - vertex distance (colliders.go:348-355): 0.5 or 1.5
    assert sorted(c["penetration"].tolist()) == [0.5] * 4 + [1.5] * 4
    assert np.all(c["bodies"] == [0, -1])


@pytest.mark.parametrize("form", [0, 1])
def test_singular_friction_solve_spends_the_budget(form):
    sc = cases.static_cube_singular_friction()
    ob = OracleBatch(sc, form=form)
    ob.narrowphase()
    assert len(ob.contacts(0)["penetration"]) == 4
    ob.resolve(1.0 / 60.0, iter_mult=4)
    st = ob.stats()
    assert st["pos_iterations"][0] == 0            # 0.005 is under positionEpsilon
    assert st["vel_iterations"][0] == 4 * 4        # the whole budget, len(contacts) * 4
    b = ob.bodies()
    assert np.array_equal(b["velocity"][0], [0.0, -1.0, 0.0])   # zero impulses
    start = sc.position[0] if form == 0 else sc.position[0].astype(np.float32).astype(np.float64)
    assert np.array_equal(b["position"][0], start)


@pytest.mark.parametrize("name", sorted(cases.ALL))
def test_cases_deterministic(name):
    a = contacts_of(cases.ALL[name]())
    b = contacts_of(cases.ALL[name]())
    for k in a:
        np.testing.assert_array_equal(a[k], b[k])


@pytest.mark.parametrize("form", [0, 1])
@pytest.mark.parametrize("name", sorted(cases.ALL))
def test_cases_match_second_restatement(name, form):
    """Each hand-built scene's contact list from the oracle equals the second
    restatement's in the same arithmetic, and the scenes built for a branch
    take it (the near-parallel edges: in the precision form's rounding)."""
    from tests import branches
    sc = cases.ALL[name]()
    seen, got = branches.narrowphase_branches(sc, form)
    ob = OracleBatch(sc, form=form)
    ob.narrowphase()
    want = ob.contacts(0)
    assert len(got) == len(want["penetration"])
    for k, (b0, b1, p, n, pen) in enumerate(got):
        assert [b0, -1 if b1 is None else b1] == want["bodies"][k].tolist()
        assert [float(x) for x in p] == want["point"][k].tolist()
        assert [float(x) for x in n] == want["normal"][k].tolist()
        assert float(pen) == want["penetration"][k]
    expect = {"sphere_inside_cube": {"sphere_centre_in_box"}, "sphere_inside_turned_cube_far": {"sphere_centre_in_box"},
              "cube_edge_edge": {"edge_cross"},
              "cube_on_cube": {"vertex_face", "vertex_face_swapped"},
              "edge_parallel_fallback": [{"edge_cross"}, {"edge_parallel"}][form],
              "edge_range_fallback": [{"edge_cross"}, {"edge_out_of_range"}][form]}.get(name, set())
    assert expect <= seen
