"""The resolver's argmax (k_resolve, k_resolve_big) restated on the CPU and
checked against the reference's own scan (contact.go:238-245, 394-402:
`max := epsilon; index := len; if c > max {...}`): order-preserving integer
keys of the float bits, each lane's contacts in four interleaved chains
merged by key then the smaller index, and the first-maximum butterfly over
the lanes.  Random values with ties, NaN, infinities, signed zeros,
subnormals and values at the epsilon.  CPU only."""
import numpy as np
import pytest

EPS = 0.01


def key_of(values, dtype):
    """key_of (cz_resolve.cuh): the value's bits when it is above eps and not
    NaN (positive IEEE values sort like their bit patterns), else 0."""
    it = np.int32 if dtype == np.float32 else np.int64
    b = np.asarray(values, dtype).view(it).astype(np.int64)
    e = int(np.asarray(EPS, dtype).view(it))
    inf = int(np.asarray(np.inf, dtype).view(it))
    return np.where((b > e) & (b <= inf), b, 0)


def reference_scan(values):
    """The reference's scan: the first strict maximum above epsilon."""
    best, index = EPS, len(values)
    for i, c in enumerate(values):
        if c > best:
            best, index = c, i
    return index


def lane_first_max(keys, lane, G):
    """Four interleaved chains over k = lane, lane + G, ..., merged."""
    b, ix = [0] * 4, [0x7FFFFFFF] * 4
    C = len(keys)
    k = lane
    while k + 3 * G < C:
        for q in range(4):
            if keys[k + G * q] > b[q]:
                b[q], ix[q] = keys[k + G * q], k + G * q
        k += 4 * G
    for q in range(3):
        kq = k + G * q
        if kq < C and keys[kq] > b[q]:
            b[q], ix[q] = keys[kq], kq
    for q in range(1, 4):
        if b[q] > b[0] or (b[q] == b[0] and ix[q] < ix[0]):
            b[0], ix[0] = b[q], ix[q]
    return b[0], ix[0]


def group_first_max(pairs):
    """The butterfly over G lanes: every lane ends with the largest key and,
    among equal keys, the smallest index."""
    G = len(pairs)
    pairs = list(pairs)
    off = G // 2
    while off > 0:
        nxt = []
        for lane in range(G):
            k, i = pairs[lane]
            ok, oi = pairs[lane ^ off]
            nxt.append((ok, oi) if (ok > k or (ok == k and oi < i)) else (k, i))
        pairs = nxt
        off //= 2
    assert len(set(pairs)) == 1
    return pairs[0]


def _values(rng, n, dtype):
    pool = np.array([0.0, -0.0, EPS, np.nextafter(np.asarray(EPS, dtype), np.asarray(1, dtype)), 0.5, 0.5, 3.0,
                     np.inf, -np.inf, np.nan, -1.0, 1e-40, np.finfo(dtype).max], dtype)
    v = np.where(rng.random(n) < 0.5, rng.choice(pool, n), rng.uniform(-1, 1, n).astype(dtype) ** 3 * 2)
    return v.astype(dtype)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("G", [4, 8, 16, 32])
def test_argmax_matches_the_reference_scan(dtype, G):
    rng = np.random.default_rng(G + (0 if dtype == np.float32 else 100))
    for trial in range(400):
        n = int(rng.integers(0, 300))
        v = _values(rng, n, dtype)
        keys = key_of(v, dtype).tolist()
        best, idx = group_first_max([lane_first_max(keys, lane, G) for lane in range(G)])
        want = reference_scan([float(x) for x in v])
        if want == n:
            assert best == 0, (trial, v.tolist())
        else:
            assert best != 0 and idx == want, (trial, idx, want)
