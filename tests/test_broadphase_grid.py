"""The narrowphase's grid (np_grid_build in csrc/cz_kernels.cuh), restated in
float32 as the kernel evaluates it: on random worlds of spheres and boxes of
mixed sizes, spread out and packed, every ordered pair the float32 culls keep
lies in neighbouring cells, so the grid loses no pair the all-pairs path
tests.  CPU only; the GPU tests check the contact lists bit for bit."""
import numpy as np
import pytest

from oracle import colliders_ref as cr
from tests.test_cull_conservative import F, _body, _cull_radii, _quat, _rejects


def _grid_cells(bodies):
    """Cell coordinates of each body, or None where the kernel falls back to
    all pairs (non-finite values; the cell count above the scratch is not
    restated: it only chooses the path)."""
    c = np.array([[F(x) for x in cr.get_axis(b["T"], 3)] for b in bodies], dtype=np.float32)
    reach = []
    for b in bodies:
        rb, rl = _cull_radii(b)
        reach.append(F(3) * rb if b["shape"] == cr.SPHERE else max(F(1.1) * rb, rl))
    reach = np.array(reach, dtype=np.float32)
    if not (np.isfinite(c).all() and np.isfinite(reach).all()):
        return None
    hi, lo = c.max(axis=0), c.min(axis=0)
    m1 = F(0)
    for a in range(3):
        m1 = m1 + max(abs(hi[a]), abs(lo[a]))
    L = (F(2) * reach.max() + F(1e-3) + F(1e-5) * (F(1) + F(2) * m1)) * F(1.001) + F(1e-6)
    dims = [int((hi[a] - lo[a]) / L) + 1 for a in range(3)]
    cells = np.array([[min(int((c[i, a] - lo[a]) / L), dims[a] - 1) for a in range(3)] for i in range(len(bodies))])
    return cells


@pytest.mark.parametrize("spread", [2.0, 8.0, 60.0])
def test_kept_pairs_are_in_neighbouring_cells(spread):
    rng = np.random.default_rng(int(spread * 10))
    kept = 0
    for world in range(12):
        n = 40
        shapes = rng.choice([cr.CUBE, cr.SPHERE], n)
        centre = rng.uniform(-200, 200, 3) * (world % 2)
        bodies = [_body(rng, int(s), (centre + rng.uniform(-spread, spread, 3)).tolist(), _quat(rng)) for s in shapes]
        cells = _grid_cells(bodies)
        assert cells is not None
        for i in range(n):
            for j in range(n):
                if i == j or _rejects(bodies[i], bodies[j])[0]:
                    continue
                kept += 1
                assert np.abs(cells[i] - cells[j]).max() <= 1, (world, i, j)
    assert kept > (100 if spread < 50 else 3)
