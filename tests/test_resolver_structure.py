"""The large-world resolver's per-body contact lists (k_resolve_big) restated
on the CPU: built as the kernel builds them (count, exclusive scan, fill) and
walked as for_pair_contacts walks them (body d0's list, then d1's list
without the contacts that also touch d0), they visit exactly the contacts the
reference's update loop changes (contact.go:254-280, 412-440: every contact
with a body equal to one of the resolved contact's bodies), each once.
CPU only."""
import numpy as np
import pytest


def build_lists(bodies, n):
    cnt = np.zeros(n, np.int64)
    for b0, b1 in bodies:
        cnt[b0] += 1
        if b1 >= 0:
            cnt[b1] += 1
    off = np.concatenate([[0], np.cumsum(cnt)[:-1]])
    cursor = off.copy()
    adj = np.zeros(int(cnt.sum()), np.int64)
    for k, (b0, b1) in enumerate(bodies):
        adj[cursor[b0]] = k
        cursor[b0] += 1
        if b1 >= 0:
            adj[cursor[b1]] = k
            cursor[b1] += 1
    return off, cursor, adj  # cursor ends at each list's end


def pair_contacts(bodies, off, end, adj, d0, d1, G):
    """for_pair_contacts with G lanes: the union of the visits of all lanes."""
    l0 = end[d0] - off[d0]
    l1 = end[d1] - off[d1] if d1 >= 0 else 0
    seen = []
    for lane in range(G):
        for e in range(lane, l0 + l1, G):
            if e < l0:
                k = adj[off[d0] + e]
            else:
                k = adj[off[d1] + e - l0]
                b0, b1 = bodies[k]
                if b0 == d0 or b1 == d0:
                    continue
            seen.append(int(k))
    return seen


@pytest.mark.parametrize("G", [16, 32])
def test_contact_lists_visit_what_the_reference_updates(G):
    rng = np.random.default_rng(G)
    for trial in range(300):
        n = int(rng.integers(2, 80))
        C = int(rng.integers(1, 400))
        b0 = rng.integers(0, n, C)
        b1 = rng.integers(-1, n, C)
        b1 = np.where(b1 == b0, -1, b1)  # a contact's two bodies differ
        bodies = list(zip(b0.tolist(), b1.tolist()))
        off, end, adj = build_lists(bodies, n)
        for _ in range(5):
            k = int(rng.integers(0, C))
            d0, d1 = bodies[k]
            seen = pair_contacts(bodies, off, end, adj, d0, d1, G)
            # the reference's loop: c.Bodies[b] != nil and == contact.Bodies[d]
            want = [c for c in range(C) if bodies[c][0] == d0 or (d1 >= 0 and bodies[c][0] == d1)
                    or (bodies[c][1] >= 0 and (bodies[c][1] == d0 or (d1 >= 0 and bodies[c][1] == d1)))]
            assert sorted(seen) == want, (trial, d0, d1)
            assert len(seen) == len(set(seen))
