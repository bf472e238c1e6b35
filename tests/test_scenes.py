"""The seeded scene generator: deterministic, distributions as configured,
body setup as the reference's helpers compute it."""
import numpy as np

from cubez_gb300 import scenes


def test_deterministic_and_order_independent():
    a = scenes.mixed(num_worlds=64, seed=9)
    b = scenes.mixed(num_worlds=64, seed=9)
    for k in a.FIELDS:
        np.testing.assert_array_equal(getattr(a, k), getattr(b, k))
    # world w does not depend on how many worlds are generated
    c = scenes.mixed(num_worlds=16, seed=9)
    np.testing.assert_array_equal(a.counts[:16], c.counts)
    n16 = int(c.counts.sum())
    np.testing.assert_array_equal(a.position[:n16], c.position)
    d = scenes.mixed(num_worlds=64, seed=10)
    assert not np.array_equal(a.position[:10], d.position[:10])


def test_mixed_distributions():
    s = scenes.mixed(num_worlds=4096)
    assert s.counts.min() >= 8 and s.counts.max() <= 64
    assert abs(s.counts.mean() - 36) < 1.0
    frac = (s.shape == scenes.SPHERE).mean()
    assert 0.48 < frac < 0.52
    sph = s.shape == scenes.SPHERE
    assert s.radius[sph].min() >= 0.25 and s.radius[sph].max() <= 1.0
    assert s.half_size[~sph].min() >= 0.25 and s.half_size[~sph].max() <= 1.0
    assert s.position[:, 1].min() >= 0.5 and s.position[:, 1].max() <= 25.0
    assert np.abs(s.velocity).max() <= 2.0 and np.abs(s.rotation).max() <= 1.0
    np.testing.assert_allclose(np.linalg.norm(s.orientation, axis=1), 1.0, atol=1e-12)


def test_precision_split_and_setup():
    s = scenes.precision(num_worlds=128)
    assert np.all(s.counts == 32)
    per_world = (s.shape == scenes.SPHERE).reshape(128, 32).sum(axis=1)
    assert np.all(per_world == 16)
    cube = s.shape == scenes.CUBE
    h = s.half_size[cube]
    mass = 8.0 * h[:, 0] * h[:, 1] * h[:, 2]
    np.testing.assert_allclose(1.0 / s.inverse_mass[cube], mass, rtol=1e-15)
    # inverse of SetBlockInertiaTensor: 1 / (0.3 m (hy^2 + hz^2)) on the diagonal
    np.testing.assert_allclose(s.inverse_inertia[cube][:, 0], 1.0 / (0.3 * mass * (h[:, 1] ** 2 + h[:, 2] ** 2)),
                               rtol=1e-14)
    sph = ~cube
    r = s.radius[sph]
    m = 4.0 / 3.0 * np.pi * r ** 3
    np.testing.assert_allclose(s.inverse_inertia[sph][:, 4], 1.0 / (0.4 * m * r * r), rtol=1e-14)
    assert np.all(s.can_sleep == 0) and np.all(s.is_awake == 1)
    np.testing.assert_array_equal(s.acceleration[:, 1], -9.8)
    np.testing.assert_array_equal(s.linear_damping, 0.95)
    np.testing.assert_array_equal(s.angular_damping, 0.8)


def test_cubedrop_and_piles():
    c = scenes.cubedrop()
    assert c.num_worlds == 1 and c.num_bodies == 20 and np.all(c.shape == scenes.CUBE)
    assert c.half_size.min() >= 0.5 and c.position[:, 1].min() >= 1.0
    np.testing.assert_array_equal(c.velocity, 0.0)
    p = scenes.piles(num_worlds=2)
    assert np.all(p.counts == 1024)
    assert p.half_size.min() >= 0.3 and p.half_size.max() <= 0.6
    q = p.orientation
    tilt = 2 * np.arccos(np.clip(np.abs(q[:, 0]), 0, 1))
    assert tilt.max() <= 0.2 + 1e-9
    bottom = p.position[:, 1] - 0.6
    assert bottom.min() >= 0.5 - 0.1 - 1e-12


def test_subset():
    s = scenes.mixed(num_worlds=10, seed=4)
    sub = s.subset([2, 5])
    assert sub.num_worlds == 2
    np.testing.assert_array_equal(sub.position, np.concatenate([s.position[s.world_slice(2)],
                                                                s.position[s.world_slice(5)]]))


def test_concat_with_empty_worlds():
    parts = [scenes.mixed(num_worlds=1, seed=90 + i, min_bodies=n, max_bodies=n) for i, n in enumerate((3, 4))]
    s = scenes.Scene.concat(parts, counts=[0, 3, 0, 4])
    assert list(s.counts) == [0, 3, 0, 4] and s.num_bodies == 7
    np.testing.assert_array_equal(s.position[s.world_slice(3)], parts[1].position)
    assert s.world_slice(0) == slice(0, 0)


def test_ballistic_setup_matches_the_example():
    """examples/ballistic.go:149-231: cube mass 8 with the block inertia of
    half size 1, bullets of mass 1.5 with 0.4 m r^2, a backboard of infinite
    mass and zero inverse inertia, NewRigidBody's dampings."""
    sc = scenes.ballistic(num_worlds=2, bullets=3, seed=5)
    assert sc.counts.tolist() == [5, 5]
    w0 = sc.world_slice(0)
    inv_m = sc.inverse_mass[w0]
    assert inv_m.tolist() == [1.0 / 8.0, 0.0, 1.0 / 1.5, 1.0 / 1.5, 1.0 / 1.5]
    ii = sc.inverse_inertia[w0].reshape(-1, 3, 3)
    assert np.array_equal(np.diag(ii[0]), np.full(3, 1.0 / (0.3 * 8.0 * 2.0)))
    assert not ii[1].any()
    assert np.array_equal(np.diag(ii[2]), np.full(3, 1.0 / (((0.4 * 1.5) * 0.2) * 0.2)))
    assert sc.shape[w0].tolist() == [scenes.CUBE, scenes.CUBE] + [scenes.SPHERE] * 3
    assert sc.can_sleep[w0].tolist() == [1, 0, 1, 1, 1]
    assert not sc.acceleration[w0][1].any() and not sc.velocity[w0][1].any()
    assert np.all(sc.velocity[w0][2:] == [0.0, 0.0, -40.0])
    assert np.all(sc.linear_damping == 0.95) and np.all(sc.angular_damping == 0.95)


def test_offsets_rigid_and_scaled():
    sc = scenes.offsets(num_worlds=16, bodies=24, seed=6, nonrigid=0.25)
    o = sc.collider_offset
    assert o.shape == (sc.num_bodies, 12)
    cols = o[:, :9].reshape(-1, 3, 3)
    norms = np.linalg.norm(cols, axis=2)
    rigid = np.all(np.abs(norms - 1.0) < 1e-12, axis=1)
    assert 0 < (~rigid).sum() < len(rigid)
    assert np.all((norms[~rigid] >= 0.7 - 1e-12) & (norms[~rigid] <= 1.3 + 1e-12))
    assert np.all(np.abs(o[:, 9:]) <= 0.3)
    again = scenes.offsets(num_worlds=16, bodies=24, seed=6, nonrigid=0.25)
    assert np.array_equal(again.collider_offset, o)
