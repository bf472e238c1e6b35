"""Autotuner for the batched step's launch shapes.

Searches, on the caller's own batch and scene state, over
  * resolver lanes per world G (worlds per warp = 32 / G),
  * the resolver's shared-memory contact tile (contacts per world kept on chip),
  * the narrowphase CTA size,
  * with worlds of more than 64 bodies in the batch, the large-world
    resolver's lanes per world (32, or 16 = two worlds per warp),
  * with one world per warp, the fused frame (one launch per frame) or the
    three launches (it compares whole frames: the fused frame has no phases),
  * with the learned warm start enabled, optionally the warm-start budget
    threshold (which worlds are warm-started; it changes which of two valid
    solutions a world gets, within the resolver's epsilon, and the speed),
timing a short captured rollout for each candidate with CUDA events, and
leaves the batch set to the fastest.  The launch-shape candidates all compute the same
bits (the parity tests run all lanes settings), so they change only speed.

The state is restored from the batch snapshot before every trial, so the
search is reproducible; the snapshot should hold a representative
(settled) state.
"""
import itertools

import numpy as np

DEFAULT_LANES = (4, 8, 16, 32)
DEFAULT_TILES = (64, 96, 128, 192)
DEFAULT_NP_THREADS = (32, 64, 128, 256)
DEFAULT_LARGE_LANES = (32, 16)
BIG_WORLD = 64  # worlds of more bodies than this go to the large-world resolver


def tune(batch, frames=30, dt=1.0 / 60.0, lanes=DEFAULT_LANES, tiles=DEFAULT_TILES, np_threads=DEFAULT_NP_THREADS,
         warm_shifts=(), large_lanes=DEFAULT_LARGE_LANES, fused=True, repeats=1, log=None):
    """Returns (best_config, trials); the batch is left at best_config."""
    trials = []

    def measure():
        best = None
        for _ in range(repeats):
            batch.restore()
            total, phases = batch.step_timed(frames, dt)
            best = phases if best is None or phases.sum() < best.sum() else best
        return best

    # narrowphase CTA size first (independent of the resolver settings)
    np_best, np_time = None, None
    for t in np_threads:
        batch.set_tuning(narrowphase_threads=t)
        ph = measure()
        trials.append({"narrowphase_threads": t, "narrowphase_ms": float(ph[1])})
        if np_time is None or ph[1] < np_time:
            np_best, np_time = t, ph[1]
    batch.set_tuning(narrowphase_threads=np_best)
    best, best_ms = None, None
    for g, cs in itertools.product(lanes, tiles):
        try:
            batch.set_tuning(resolver_lanes=g, resolver_contacts=cs)
        except Exception as e:  # a tile that does not fit in shared memory
            trials.append({"resolver_lanes": g, "resolver_contacts": cs, "error": str(e)})
            continue
        ph = measure()
        cfg = batch.get_tuning()
        trials.append({"resolver_lanes": g, "resolver_contacts": cfg["resolver_contacts"],
                       "resolver_ms": float(ph[2])})
        if log:
            log("lanes=%d tile=%d resolve %.3f ms" % (g, cfg["resolver_contacts"], ph[2]))
        if best_ms is None or ph[2] < best_ms:
            best, best_ms = (g, cfg["resolver_contacts"]), ph[2]
    batch.set_tuning(resolver_lanes=best[0], resolver_contacts=best[1])
    # one launch per frame, where the batch allows it (one world per warp, no
    # world above the slot, the plain resolver): the batch ignores it otherwise
    if (fused and best[0] == 32 and not getattr(batch, "warm_start", False)
            and not (np.asarray(batch.counts) > BIG_WORLD).any()):
        best_f, f_ms = None, None
        for f in (-1, 1):
            batch.set_tuning(fused_frame=f)
            ph = measure()
            trials.append({"fused_frame": f, "step_ms": float(ph.sum())})
            if f_ms is None or ph.sum() < f_ms:
                best_f, f_ms = f, ph.sum()
        batch.set_tuning(fused_frame=best_f)
    if large_lanes and (np.asarray(batch.counts) > BIG_WORLD).any():
        best_ll, ll_ms = None, None
        for g in large_lanes:
            batch.set_tuning(large_world_lanes=g)
            ph = measure()
            trials.append({"large_world_lanes": g, "resolver_ms": float(ph[2])})
            if ll_ms is None or ph[2] < ll_ms:
                best_ll, ll_ms = g, ph[2]
        batch.set_tuning(large_world_lanes=best_ll)
    if warm_shifts:
        best_shift, shift_ms = None, None
        for sh in warm_shifts:
            batch.set_tuning(warm_start_budget_shift=sh)
            ph = measure()
            trials.append({"warm_start_budget_shift": sh, "resolver_ms": float(ph[2])})
            if shift_ms is None or ph[2] < shift_ms:
                best_shift, shift_ms = sh, ph[2]
        batch.set_tuning(warm_start_budget_shift=best_shift)
    batch.restore()
    cfg = batch.get_tuning()
    return cfg, trials
