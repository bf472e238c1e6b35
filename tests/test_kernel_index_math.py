"""Index arithmetic of the narrowphase and resolver kernels restated on the
CPU, lane by lane, as the kernels compute it (CPU only):

* np_world's cull rounds: upt consecutive units per thread, one scan of the
  threads' counts per round, the kept units appended in unit order, and the
  list never longer than its capacity (cz_kernels.cuh, all-pairs branch);
* np_flush's stable sort of a chunk by kind of test (ballot ranks and
  per-kind warp counts) and the emission offsets scanned in list order;
* update_touching's per-group gather (a ballot masked to the group, the rank
  below the lane) for G = 8, 16, 32: each group's list holds exactly its
  world's touching contacts, in contact order;
* apply_velocity_change_spread's lane map (c = gl % 3, i = gl / 3) and the
  cross product's component c = a_p b_q - a_q b_p against cross();
* k_reorder's counting sort: a permutation of the worlds by descending
  cost, the warm start's worlds first when it is on.

Every contact's position in the reference's order depends on these, and the
GPU parity tests check the results bit for bit; these checks pin the index
arithmetic on its own, for sizes the GPU tests do not reach."""
import numpy as np
import pytest

K_TOUCH_LIST = 64


def cull_rounds(keep, bd, scap):
    """np_world's all-pairs loop over `keep` (one flag per unit): returns the
    kept units in list order, and the largest list length reached."""
    U = len(keep)
    upt = max(1, min(8, (scap - bd) // bd))
    rnd = bd * upt
    out, surv, longest = [], [], 0
    base = 0
    while base < U:
        counts, picks = [], []
        for t in range(bd):
            u0 = base + t * upt
            mine = [u0 + q for q in range(upt) if u0 + q < U and keep[u0 + q]]
            counts.append(len(mine))
            picks.append(mine)
        excl = np.concatenate([[0], np.cumsum(counts)[:-1]])
        start = len(surv)
        surv.extend([None] * int(sum(counts)))
        for t in range(bd):
            for j, u in enumerate(picks[t]):
                surv[start + int(excl[t]) + j] = u
        longest = max(longest, len(surv))
        if len(surv) <= scap - rnd and base + rnd < U:
            base += rnd
            continue
        out.extend(surv)
        surv = []
        base += rnd
    return out, longest


@pytest.mark.parametrize("bd,scap", [(32, 1280), (64, 1280), (128, 1280), (256, 1280), (32, 128), (128, 1088)])
def test_cull_rounds_keep_unit_order_within_capacity(bd, scap):
    rng = np.random.default_rng(bd + scap)
    for n in (3, 32, 64, 100):
        U = n * n
        for density in (0.0, 0.05, 0.5, 1.0):
            keep = rng.random(U) < density
            out, longest = cull_rounds(keep, bd, scap)
            assert out == [u for u in range(U) if keep[u]]
            assert longest <= scap


def sort_chunk(keys, bd):
    """np_flush's order of a chunk: thread t (key keys[t], 5 = no unit) gets
    slot dst[t]; perm[dst[t]] = t."""
    nw = (bd + 31) // 32
    wcnt = np.zeros((6, 8), np.int64)
    rank = np.zeros(bd, np.int64)
    for w in range(nw):
        lanes = range(32 * w, min(32 * w + 32, bd))
        for q in range(6):
            mask = [t for t in lanes if keys[t] == q]
            wcnt[q, w] = len(mask)
            for r, t in enumerate(mask):
                rank[t] = r
    perm = np.full(bd, -1)
    for t in range(bd):
        w = t // 32
        dst = rank[t] + wcnt[:keys[t], :nw].sum() + wcnt[keys[t], :w].sum()
        assert perm[dst] == -1
        perm[dst] = t
    return perm


@pytest.mark.parametrize("bd", [32, 64, 128, 256])
def test_flush_sort_is_stable_by_kind_and_emission_keeps_list_order(bd):
    rng = np.random.default_rng(bd)
    for m in (0, 1, 7, bd // 2, bd):
        keys = np.full(bd, 5)
        keys[:m] = rng.integers(0, 5, m)
        perm = sort_chunk(keys, bd)
        assert sorted(perm.tolist()) == list(range(bd))
        # sorted by kind, and stable (list order within a kind)
        assert all((keys[perm[s]], perm[s]) < (keys[perm[s + 1]], perm[s + 1]) for s in range(bd - 1))
        # contacts per unit, scanned in list order: slot offsets as the unsorted scan gives
        cnt = np.where(np.arange(bd) < m, rng.integers(0, 9, bd), 0)
        excl = np.concatenate([[0], np.cumsum(cnt)[:-1]])
        slots = {}
        for s in range(bd):
            src = perm[s]  # the thread in sorted slot s tests unit src and writes at excl[src]
            for j in range(cnt[src]):
                slots[excl[src] + j] = (src, j)
        assert [slots[o] for o in range(int(cnt.sum()))] == [(u, j) for u in range(bd) for j in range(cnt[u])]


def touching(bodies, d0, d1):
    return [k for k, (kb0, kb1) in enumerate(bodies)
            if kb0 == d0 or (d1 >= 0 and kb0 == d1) or (kb1 >= 0 and (kb1 == d0 or kb1 == d1))]


@pytest.mark.parametrize("G", [8, 16, 32])
def test_group_gather_lists_each_worlds_touching_contacts_in_order(G):
    """update_touching<G>: 32 / G worlds per warp, each group's ballot bits
    masked to its lanes; flushes when any group's list could overflow."""
    rng = np.random.default_rng(G)
    NG = 32 // G
    for trial in range(50):
        worlds = []
        for g in range(NG):
            n = int(rng.integers(2, 40))
            C = int(rng.integers(0, 200))
            b0 = rng.integers(0, n, C)
            b1 = np.where(rng.random(C) < 0.4, -1, rng.integers(0, n, C))
            b1 = np.where(b1 == b0, -1, b1)
            d0 = int(rng.integers(0, n))
            d1 = int(rng.integers(-1, n))
            if d1 == d0:
                d1 = -1
            on = bool(rng.random() < 0.8)
            worlds.append((list(zip(b0.tolist(), b1.tolist())), d0, d1, on))
        Cg = [len(wd[0]) if wd[3] else 0 for wd in worlds]
        Cmax = max(Cg)
        visited = [[] for _ in range(NG)]
        m = [0] * NG
        ml = [[None] * K_TOUCH_LIST for _ in range(NG)]
        base = 0
        while base < Cmax:
            bal = 0
            hits = [False] * 32
            for lane in range(32):
                g, gl = divmod(lane, G)
                bodies, d0, d1, on = worlds[g]
                k = base + gl
                if k < Cg[g]:
                    kb0, kb1 = bodies[k]
                    hits[lane] = kb0 == d0 or (d1 >= 0 and kb0 == d1) or (kb1 >= 0 and (kb1 == d0 or kb1 == d1))
                if hits[lane]:
                    bal |= 1 << lane
            for lane in range(32):
                g, gl = divmod(lane, G)
                gmask = ((1 << G) - 1) << (lane - gl)
                gb = bal & gmask
                if hits[lane]:
                    idx = m[g] + bin(gb & ((1 << lane) - 1)).count("1")
                    assert idx < K_TOUCH_LIST
                    ml[g][idx] = base + gl
            for g in range(NG):
                gmask = ((1 << G) - 1) << (g * G)
                m[g] += bin(bal & gmask).count("1")
            if any(mm > K_TOUCH_LIST - G for mm in m) or base + G >= Cmax:
                for g in range(NG):
                    visited[g].extend(ml[g][:m[g]])
                    m[g] = 0
            base += G
        for g in range(NG):
            bodies, d0, d1, on = worlds[g]
            want = touching(bodies, d0, d1) if on else []
            assert visited[g] == want


def test_spread_velocity_change_lane_map():
    rng = np.random.default_rng(3)
    for _ in range(20):
        a, b = rng.normal(size=3), rng.normal(size=3)
        ref = [a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]]
        for gl in range(6):
            c, i = gl % 3, gl // 3
            p = 0 if c == 2 else c + 1
            q = 2 if c == 0 else c - 1
            assert a[p] * b[q] - a[q] * b[p] == ref[c]
            assert 3 * i + c == gl
        # the triple of body i reads its cross components from lanes 3i..3i+2
        for gl in range(32):
            i = gl // 3
            t0 = 3 * (i if gl < 6 else 0)
            assert t0 in (0, 3)


def reorder(pos_it, vel_it, plain_next=None, buckets=2048):
    """k_reorder's counting sort: worlds by last frame's iterations,
    descending; with the warm start on, the worlds it will serve
    (plain_next == 0) first.  Order within a bucket is free."""
    key = np.minimum(np.asarray(pos_it) + np.asarray(vel_it), buckets - 1)
    if plain_next is not None:
        key = np.where(np.asarray(plain_next) == 0, buckets - 1, key)
    hist = np.bincount(buckets - 1 - key, minlength=buckets)
    start = np.concatenate([[0], np.cumsum(hist)[:-1]])
    order = np.full(len(key), -1)
    for w in range(len(key)):
        b = buckets - 1 - key[w]
        order[start[b]] = w
        start[b] += 1
    return order, key


def test_reorder_is_a_permutation_by_descending_cost_warm_first():
    rng = np.random.default_rng(11)
    for warm in (False, True):
        W = 5000
        pos, vel = rng.integers(0, 300, W), rng.integers(0, 3000, W)
        plain_next = rng.integers(0, 2, W) if warm else None
        order, key = reorder(pos, vel, plain_next)
        assert sorted(order.tolist()) == list(range(W))
        k = key[order]
        assert np.all(k[:-1] >= k[1:])
        if warm:
            served = plain_next[order] == 0
            # every world the warm start serves precedes every other with a lower key
            first_plain = np.argmax(~served) if (~served).any() else W
            assert served[:first_plain].all()
