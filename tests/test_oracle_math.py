"""The reference's own known-answer tests (math/*_test.go), re-asserted on the
oracle's math layer.  Comparisons use the reference's RealEqual
(relative 1e-7, math/math.go:64-78), as its tests do."""
import ctypes as C
import math

import numpy as np
import pytest

from oracle import oracle as O

MAX = np.finfo(np.float64).max


@pytest.fixture(scope="module")
def L():
    return O.lib()


def arr(*v):
    return np.array(v, dtype=np.float64)


def p(a):
    return a.ctypes.data_as(C.c_void_p)


def req(L, a, b):
    return bool(L.orc_real_equal(float(a), float(b)))


def all_req(L, got, want):
    return all(req(L, g, w) for g, w in zip(got, want))


def test_real_equal_rules(L):
    assert req(L, 1.0, 1.0)
    assert req(L, math.inf, math.inf)
    assert req(L, 0.0, 1e-15)            # near zero: absolute 1e-14
    assert not req(L, 0.0, 1e-13)
    assert req(L, 1.0, 1.0 + 1e-8)       # relative 1e-7
    assert not req(L, 1.0, 1.0 + 1e-6)
    assert not req(L, math.nan, math.nan)


def test_quat_mul_identity(L):  # quaternion_test.go:11-21
    a, b = arr(1, 0, 0, 0), arr(1, 0, 0, 0)
    L.orc_quat_mul(p(a), p(b))
    assert all_req(L, a, [1, 0, 0, 0])


def test_quat_len(L):  # quaternion_test.go:23-47
    assert req(L, L.orc_quat_len(p(arr(0, 1, 0, 0))), 1.0)
    assert req(L, L.orc_quat_len(p(arr(0, 1e-13, 0, 0))), 1e-13)
    assert req(L, L.orc_quat_len(p(arr(0, MAX, 1, 0))), math.inf)
    assert req(L, L.orc_quat_len(p(arr(4, 1, 2, 3))), math.sqrt(1 * 1 + 2 * 2 + 3 * 3 + 4 * 4))


def test_quat_normalize(L):  # quaternion_test.go:49-73
    for q, want in [((0, 0, 0, 0), (1, 0, 0, 0)), ((0, 1, 0, 0), (0, 1, 0, 0)),
                    ((0, 1e-13, 0, 0), (0, 1, 0, 0)), ((0, MAX, 1, 0), (0, 1, 0, 0))]:
        a = arr(*q)
        L.orc_quat_normalize(p(a))
        assert all_req(L, a, want), (q, a)


def test_quat_mul(L):  # quaternion_test.go:75-84
    a, b = arr(1.0, 0.5, -3.0, 4.0), arr(6.0, 2.0, 1.0, -9.0)
    L.orc_quat_mul(p(a), p(b))
    assert all_req(L, a, [44.0, 28.0, -4.5, 21.5])


ROTATIONS = [  # quaternion_test.go:86-181: (angle deg, axis, v, expected)
    (0, (0, 1, 0), (1, 0, 0), (1, 0, 0)), (90, (0, 1, 0), (1, 0, 0), (0, 0, -1)),
    (180, (0, 1, 0), (1, 0, 0), (-1, 0, 0)), (270, (0, 1, 0), (0, 0, 1), (-1, 0, 0)),
    (0, (0, 0, 1), (0, 1, 0), (0, 1, 0)), (90, (1, 0, 0), (0, 1, 0), (0, 0, 1)),
    (180, (1, 0, 0), (0, 1, 0), (0, -1, 0)), (270, (1, 0, 0), (0, 1, 0), (0, 0, -1)),
    (0, (0, 0, 1), (0, 1, 0), (0, 1, 0)), (90, (0, 0, 1), (0, 1, 0), (-1, 0, 0)),
    (180, (0, 0, 1), (0, 1, 0), (0, -1, 0)), (270, (0, 0, 1), (0, 1, 0), (1, 0, 0)),
]


@pytest.mark.parametrize("deg,axis,v,want", ROTATIONS)
def test_quat_rotate(L, deg, axis, v, want):
    q = np.zeros(4)
    L.orc_quat_from_axis(deg * math.pi / 180.0, *map(float, axis), p(q))
    out = np.zeros(3)
    L.orc_quat_rotate(p(q), p(arr(*v)), p(out))
    assert all_req(L, out, want), (deg, axis, out)


def test_quat_rotate_unnormalised_start(L):  # quaternion_test.go:87-94
    q = arr(1.0, 0.0, 1.0, 0.0)
    L.orc_quat_normalize(p(q))
    out = np.zeros(3)
    L.orc_quat_rotate(p(q), p(arr(1, 0, 0)), p(out))
    assert all_req(L, out, [0, 0, -1])


def test_mat3_identity(L):  # matrix_test.go:10-22
    i = arr(1, 0, 0, 0, 1, 0, 0, 0, 1)
    out = np.zeros(9)
    L.orc_m3_mul(p(i), p(i.copy()), p(out))
    assert all_req(L, out, i)


def test_mat3x4_identity(L):  # matrix_test.go:24-36
    i = arr(1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0)
    out = np.zeros(12)
    L.orc_m34_mul(p(i), p(i.copy()), p(out))
    assert all_req(L, out, i)


def test_mat3_inverse_roundtrip(L):  # matrix_test.go:38-53
    m = arr(0.6, 0.2, 0.3, 0.2, 0.7, 0.5, 0.3, 0.5, 0.7)
    inv = np.zeros(9)
    L.orc_m3_invert(p(m), p(inv))
    out = np.zeros(9)
    L.orc_m3_mul(p(m), p(inv), p(out))
    assert all_req(L, out, [1, 0, 0, 0, 1, 0, 0, 0, 1])


def test_mat3_singular_inverse_is_zero(L):  # matrix.go:135-137
    m = arr(1, 2, 3, 2, 4, 6, 0, 0, 1)
    inv = np.full(9, 7.0)
    L.orc_m3_invert(p(m), p(inv))
    assert np.all(inv == 0.0)


VECTOR_CASES = [  # vector_test.go
    (0, (1.0, 2.5, 3.75), (0.0, 1.0, 7.0), 0, (1.0, 3.5, 10.75)),     # Add :12-32
    (1, (1.0, 2.5, 3.75), (0.0, 1.0, 7.0), 3.0, (1.0, 5.5, 24.75)),   # AddScaled :34-48
    (2, (1.0, 2.5, 3.5), (0.0, 1.0, 7.0), 0, (0.0, 2.5, 24.5)),       # ComponentProduct :60-72
    (3, (1.0, 2.0, 3.0), (10.0, 11.0, 12.0), 0, (-9.0, 18.0, -9.0)),  # Cross :74-90
    (4, (-1.0, -5.0, -7.0), (10.0, 20.0, 30.0), 0, (-11.0, -25.0, -37.0)),  # Sub
    (5, (1.0, 2.5, 3.5), (0, 0, 0), 10.0, (10.0, 25.0, 35.0)),        # MulWith
]


@pytest.mark.parametrize("op,a,b,s,want", VECTOR_CASES)
def test_vector_ops(L, op, a, b, s, want):
    v = arr(*a)
    L.orc_v3_op(op, p(v), p(arr(*b)), s)
    assert all_req(L, v, want)


def test_vector_scalars(L):
    assert req(L, L.orc_v3_dot(p(arr(-1, -5, -7)), p(arr(10, 20, 30))), -320.0)  # vector_test.go:92-107
    assert req(L, L.orc_v3_magnitude(p(arr(2, -5, 4))), 6.708203932499369)    # :109-121
    assert req(L, L.orc_v3_square_magnitude(p(arr(2, -5, 4))), 4.0 + 25 + 16)  # :123-135
    v = arr(1.0, 2.5, 3.5)
    L.orc_v3_op(6, p(v), p(arr(0, 0, 0)), 0)  # Normalize :146-152
    assert req(L, L.orc_v3_magnitude(p(v)), 1.0)


def test_quat_add_scaled_vector_matches_formula(L):
    q = arr(0.8, 0.2, -0.4, 0.4)
    v = arr(0.3, -1.2, 2.0)
    s = 1.0 / 60.0
    L.orc_quat_add_scaled_vector(p(q), p(v), s)
    # q += 0.5 * (0, v*s) (x) q  (quaternion.go:18-33)
    w0, x0, y0, z0 = 0.8, 0.2, -0.4, 0.4
    a, b, c = 0.3 * s, -1.2 * s, 2.0 * s
    want = [w0 + 0.5 * (-a * x0 - b * y0 - c * z0), x0 + 0.5 * (a * w0 + b * z0 - c * y0),
            y0 + 0.5 * (b * w0 + c * x0 - a * z0), z0 + 0.5 * (c * w0 + a * y0 - b * x0)]
    assert np.allclose(q, want, rtol=1e-14, atol=1e-15)


def test_block_inertia_tensor(L):
    # SetBlockInertiaTensor uses 0.3*m*(h^2+h^2) (math/matrix.go:68-77)
    out = np.zeros(9)
    L.orc_block_inverse_inertia(p(arr(0.5, 0.5, 0.5)), 8.0, p(out))
    i = 0.3 * 8.0 * (0.25 + 0.25)
    assert np.allclose(out[[0, 4, 8]], 1.0 / i, rtol=1e-15)
    assert np.all(out[[1, 2, 3, 5, 6, 7]] == 0.0)
