"""The reference's rare branches forced through the CUDA kernels: every
hand-built scene of tests/cases.py, in both forms, through cz_narrowphase,
cz_resolve and whole frames of cz_step, bit for bit against the oracle, with
the branch each scene names checked on the second restatement in the same
arithmetic (tests/branches.py).

  sphere centred in a box: the velocity normal (colliders.go:414-421)
  edge-edge crossing, and the near-parallel fallbacks of contactPoint
    (colliders.go:545-573): the precision form's rounding takes the parallel
    and the out-of-range fallback; the float64 form crosses the same edges
  vertex-face in both orders (colliders.go:628-640)
  edge-down cube and a cube below the plane (colliders.go:308-366)
  the singular friction solve: Invert gives the zero matrix
    (math/matrix.go:133-138) and adjustVelocities spends its budget
"""
import numpy as np
import pytest

from oracle.oracle import OracleBatch
from tests import branches, cases

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0

# branch each scene must take, per form (None: the same in both)
EXPECTED = {
    "sphere_inside_cube": {"sphere_centre_in_box"},
    "sphere_inside_turned_cube_far": {"sphere_centre_in_box"},
    "cube_edge_edge": {"edge_cross"},
    "cube_on_cube": {"vertex_face", "vertex_face_swapped"},
    "edge_parallel_fallback": ({"edge_cross"}, {"edge_parallel"}),
    "edge_range_fallback": ({"edge_cross"}, {"edge_out_of_range"}),
}
PLANE_CONTACTS = {"cube_resting": 4, "tilted_cube_on_plane": 1, "cube_edge_down": 2, "cube_below_plane": 8,
                  "sphere_resting": 1, "static_cube_singular_friction": 4}


def _same_contacts(got, want):
    n = len(want["penetration"])
    assert len(got["penetration"]) == n
    np.testing.assert_array_equal(got["bodies"], want["bodies"])
    np.testing.assert_array_equal(got["point"], want["point"])
    np.testing.assert_array_equal(got["normal"], want["normal"])
    np.testing.assert_array_equal(got["penetration"], want["penetration"])


def _same_bodies(g, r):
    for k in ("position", "orientation", "velocity", "rotation", "is_awake"):
        np.testing.assert_array_equal(g[k], r[k], err_msg=k)
    np.testing.assert_array_equal(g["inverse_inertia_world"], r["iit_world"])


@pytest.mark.parametrize("form", [0, 1])
@pytest.mark.parametrize("name", sorted(cases.ALL))
def test_case_branch_bit_exact(name, form, cuda_lib):
    from cubez_gb300.batch import WorldBatch
    sc = cases.ALL[name]()
    seen, _ = branches.narrowphase_branches(sc, form)
    want = EXPECTED.get(name)
    if want is not None:
        want = want[form] if isinstance(want, tuple) else want
        assert want <= seen, (name, form, seen)
    gpu = WorldBatch.from_scene(sc, form=form)
    ref = OracleBatch(sc, form=form)
    # the narrowphase on the scene as built
    gpu.narrowphase()
    assert ref.narrowphase() == 0
    c = ref.contacts(0)
    _same_contacts(gpu.contacts(0), c)
    if name in PLANE_CONTACTS:
        assert len(c["penetration"]) == PLANE_CONTACTS[name]
    if name == "sphere_inside_cube":
        np.testing.assert_array_equal(c["normal"][0], [0.0, -1.0, 0.0])
        assert c["penetration"][0] == 0.0
    # ResolveContacts(4 * len(contacts)) on those contacts
    gpu.resolve(DT)
    assert ref.resolve(DT, 4) == 0
    gs, rs = gpu.stats(), ref.stats()
    assert gs["pos_iterations"][0] == rs["pos_iterations"][0]
    assert gs["vel_iterations"][0] == rs["vel_iterations"][0]
    _same_bodies(gpu.download(), ref.bodies())
    if name == "static_cube_singular_friction":
        assert rs["pos_iterations"][0] == 0 and rs["vel_iterations"][0] == 16   # the whole budget
        np.testing.assert_array_equal(gpu.download()["velocity"][0], [0.0, -1.0, 0.0])
    # then whole frames of the cubedrop loop
    gpu.step(5, DT)
    assert ref.step(5, DT) == 0
    _same_bodies(gpu.download(), ref.bodies())
    assert gpu.contact_counts()[0] == ref.stats()["contacts"][0]
    gpu.close()
