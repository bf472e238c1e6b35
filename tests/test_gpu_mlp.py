"""The learned warm start on the GPU: the hand-written tensor-core training
kernels against the CPU reference (gradient check), inference, training,
harvesting, and the warm start's guarantees inside the resolver."""
import numpy as np
import pytest

from cubez_gb300 import scenes
from oracle import mlp_ref

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0


def _data(n, seed=0):
    rng = np.random.default_rng(seed)
    x = rng.normal(0, 1, (n, 18)).astype(np.float32) * np.linspace(0.2, 3.0, 18, dtype=np.float32)
    x[:, 16:] = np.abs(np.round(x[:, 16:] * 3))
    w = rng.normal(0, 1, (18, 3))
    y = (np.tanh(x @ w) + 0.3 * x[:, :3]).astype(np.float32)
    return x, y


def test_gradient_matches_cpu_reference(cuda_lib):
    from cubez_gb300.learned import Trainer
    x, y = _data(300)
    t = Trainer(seed=5)
    t.set_data(x, y, normalize=True)
    loss, g = t.loss_and_grad(300)
    ref_loss, ref_g = mlp_ref.loss_and_grad(t.params(), x, y)
    assert abs(loss - ref_loss) <= 1e-4 * abs(ref_loss)
    # float32 accumulation order and occasional BF16 rounding of backward
    # operands differ from the float64 reference: compare as vectors
    err = np.linalg.norm(g - ref_g) / np.linalg.norm(ref_g)
    cos = float(g @ ref_g / (np.linalg.norm(g) * np.linalg.norm(ref_g)))
    assert err < 1e-2 and cos > 0.9999, (err, cos)
    for name, (a, b) in {"W1": (mlp_ref.OFF_W1, mlp_ref.OFF_B1), "b4": (mlp_ref.OFF_B4, mlp_ref.NPARAM),
                         "W4": (mlp_ref.OFF_W4, mlp_ref.OFF_B4), "b1": (mlp_ref.OFF_B1, mlp_ref.OFF_W2)}.items():
        e = np.linalg.norm(g[a:b] - ref_g[a:b]) / max(np.linalg.norm(ref_g[a:b]), 1e-12)
        assert e < 2e-2, (name, e)


def test_inference_matches_cpu_reference(cuda_lib):
    from cubez_gb300.learned import Trainer
    x, y = _data(500, seed=1)
    t = Trainer(seed=6)
    t.set_data(x, y, normalize=True)
    out = t.predict(x)
    ref = mlp_ref.predict(t.params(), x)
    np.testing.assert_allclose(out, ref, rtol=2e-2, atol=2e-2 * np.abs(ref).max())


def test_training_reduces_loss(cuda_lib):
    from cubez_gb300.learned import Trainer
    x, y = _data(20000, seed=2)
    t = Trainer(seed=7)
    t.set_data(x, y, normalize=True)
    losses = t.train(epochs=20, batch=2048, lr=2e-3)
    assert losses[-1] < 0.2 * losses[0], losses


def test_harvest_features_and_labels(cuda_lib):
    from cubez_gb300.batch import FORM_FP32, WorldBatch
    from cubez_gb300.learned import harvest
    scene = scenes.precision(num_worlds=64, seed=40)
    b = WorldBatch.from_scene(scene, form=FORM_FP32)
    b.step(150, DT)
    x, y = harvest(b, 40, DT, every=10, capacity=200000)
    assert len(x) > 1000
    assert np.all(np.isfinite(x)) and np.all(np.isfinite(y))
    assert set(np.unique(x[:, 1])) <= {0.0, 1.0}             # half-space flag
    half = x[:, 1] == 1.0
    assert half.any() and (~half).any()
    assert np.all(x[:, 0] == np.round(x[:, 0])) and np.all(x[:, 0] >= 0)
    assert np.all(x[~half, 0] >= 1.0)                        # body 0 touches body 1
    assert (x[half, 0] == 0).any()                           # some bodies touch only the ground
    assert np.all(x[:, 7:10] > 0.0)                          # response matrix diagonal
    # a symmetric positive definite response: each 2x2 minor positive
    assert np.all(x[:, 7] * x[:, 8] - x[:, 10] ** 2 > -1e-4 * x[:, 7] * x[:, 8])
    np.testing.assert_allclose(x[:, 13], x[:, 6] / x[:, 7], rtol=1e-5, atol=1e-6)
    assert np.all(x[:, 14] >= 1.0)                           # each contact touches its first body
    assert np.all(x[half, 15] == 0.0) and np.all(x[~half, 15] >= 1.0)
    assert np.all(x[:, 16] >= np.maximum(x[:, 6], 0) - 1e-5)  # a body's load includes this contact
    assert np.median(y[:, 0]) >= 0.0                         # normal impulses push apart


def _pair_batches(scene, **kw):
    from cubez_gb300.batch import FORM_FP32, WorldBatch
    a = WorldBatch.from_scene(scene, form=FORM_FP32, **kw)
    b = WorldBatch.from_scene(scene, form=FORM_FP32, **kw)
    return a, b


def _settled(seed, frames=150):
    from cubez_gb300.batch import FORM_FP32, WorldBatch
    scene = scenes.precision(num_worlds=64, seed=seed)
    b = WorldBatch.from_scene(scene, form=FORM_FP32)
    b.step(frames, DT)
    state = b.download(("position", "orientation", "velocity", "rotation"))
    settled = scene.copy()
    for k, v in state.items():
        setattr(settled, k, v)
    return settled


def _bias_blob(b4):
    from cubez_gb300.learned import BLOB, OFF_B4, OFF_IS, OFF_OS
    blob = np.zeros(BLOB, np.float32)
    blob[OFF_IS:OFF_IS + 18] = 1.0
    blob[OFF_OS:OFF_OS + 3] = 1.0
    blob[OFF_B4:OFF_B4 + 3] = b4
    return blob


def test_zero_network_equals_plain_resolver(cuda_lib):
    from cubez_gb300.learned import BLOB, OFF_IS, OFF_OS, set_warm_start
    scene = scenes.precision(num_worlds=64, seed=41)
    plain, warm = _pair_batches(scene)
    blob = np.zeros(BLOB, np.float32)
    blob[OFF_IS:OFF_IS + 18] = 1.0
    blob[OFF_OS:OFF_OS + 3] = 1.0
    set_warm_start(warm, blob)
    plain.step(120, DT)
    warm.step(120, DT)
    p, w = plain.download(), warm.download()
    for k in ("position", "orientation", "velocity", "rotation"):
        np.testing.assert_array_equal(w[k], p[k])  # a zero warm start changes no value
    # no body was warm-started, so no world is re-solved either
    np.testing.assert_array_equal(warm.stats()["vel_iterations"], plain.stats()["vel_iterations"])


def test_wild_network_is_scaled_back(cuda_lib):
    """Absurd predicted impulses everywhere: the line search scales them
    back so that no contact is pushed past its resolved velocity, and the
    step's kinetic energy stays that of the plain resolver."""
    from cubez_gb300.learned import set_warm_start
    settled = _settled(42)
    for b4 in ([50.0, 40.0, -40.0], [-50.0, 0.0, 0.0]):
        plain, warm = _pair_batches(settled)
        set_warm_start(warm, _bias_blob(b4))
        warm.counters(reset=True)
        plain.step(1, DT)
        warm.step(1, DT)
        c = warm.counters()
        assert c["warm_worlds"] > 0
        if b4[0] > 0:
            assert c["warm_bodies"] > 0
            assert c["warm_scale_sum"] / c["warm_bodies"] < 0.2     # scaled far back
        else:
            assert c["warm_bodies"] == 0                             # negative normal impulses project to 0
        p, w = plain.download(), warm.download()
        ke_p = np.square(p["velocity"]).sum()
        ke_w = np.square(w["velocity"]).sum()
        assert ke_w <= 1.05 * ke_p + 1e-3, (ke_w, ke_p)
        if b4[0] <= 0:
            for k in ("position", "orientation", "velocity", "rotation"):
                np.testing.assert_array_equal(w[k], p[k])


def test_exhausted_worlds_fall_back_to_plain(cuda_lib):
    """With a two-iteration budget most worlds exhaust it in the warm solve
    too; they are re-solved from the saved state by the plain path and end
    exactly where the plain resolver ends."""
    from cubez_gb300.learned import set_warm_start
    settled = _settled(43)
    plain, warm = _pair_batches(settled, max_iterations=2)
    set_warm_start(warm, _bias_blob([0.3, 0.0, 0.0]))
    warm.counters(reset=True)
    plain.step(1, DT)
    warm.step(1, DT)
    c = warm.counters()
    assert c["warm_fallbacks"] > 0
    fell_back = warm.stats()["vel_iterations"] > 2
    assert fell_back.sum() == c["warm_fallbacks"]
    p, w = plain.download(), warm.download()
    for wi in np.nonzero(fell_back)[0]:
        sl = settled.world_slice(int(wi))
        for k in ("position", "orientation", "velocity", "rotation"):
            np.testing.assert_array_equal(w[k][sl], p[k][sl])  # the plain path decided these worlds


def test_trained_network_ablation(cuda_lib):
    """The ablation: a network trained on harvested contacts of some scenes,
    applied to a held-out scene, against the same FP32 form without it
    (adjustVelocities iterations, and the physics)."""
    from cubez_gb300.batch import FORM_FP32, WorldBatch
    from cubez_gb300.learned import Trainer, harvest, set_warm_start
    xs, ys = [], []
    for seed in (60, 61):
        b = WorldBatch.from_scene(scenes.precision(num_worlds=1024, seed=seed), form=FORM_FP32)
        b.step(60, DT)
        x, y = harvest(b, 240, DT, every=4, capacity=3_000_000)
        xs.append(x)
        ys.append(y)
    x, y = np.concatenate(xs), np.concatenate(ys)
    grounded = (x[:, 0] == 0) & (x[:, 1] == 1)   # the contacts the warm start serves
    t = Trainer(seed=3)
    t.set_data(x[grounded], y[grounded], normalize=True)
    losses = np.concatenate([t.train(epochs=12, batch=4096, lr=2e-3), t.train(epochs=8, batch=4096, lr=5e-4)])
    assert losses[-1] < 0.5 * losses[0], losses
    blob = t.params()

    held_out = _settled(62, frames=60)
    runs = {}
    for name in ("plain", "zero", "trained"):
        b = WorldBatch.from_scene(held_out, form=FORM_FP32)
        # warm-start every world whose last solve used at most half its budget
        # (the default quarter keeps the warm start to the easiest worlds)
        b.set_tuning(warm_start_budget_shift=1)
        if name == "zero":
            set_warm_start(b, _bias_blob([0.0, 0.0, 0.0]))
        elif name == "trained":
            set_warm_start(b, blob)
        b.counters(reset=True)
        ys, kes = [], []
        for _ in range(24):  # time averages over the rollout, sampled every 10 frames
            b.step(10, DT)
            d = b.download(("position", "velocity"))
            ys.append(d["position"][:, 1].mean())
            kes.append(np.square(d["velocity"]).sum(1).mean())
        c = b.counters()
        runs[name] = dict(it=c["vel_iterations"], fb=c["warm_fallbacks"], y=float(np.mean(ys)),
                          ke=float(np.mean(kes)), bodies=c["warm_bodies"])
    p, z, w = runs["plain"], runs["zero"], runs["trained"]
    print("ablation", runs)
    assert z["bodies"] == 0 and w["bodies"] > 0
    # Iterations count both solves of a re-solved world.  Training is not
    # bit-reproducible (float atomics accumulate the gradients; the harvest's
    # rows land in the order the worlds finish), and across five trainings the
    # trained network's iterations ranged from 0.96x to 1.03x of no warm start
    # (mean 0.99x), with 130-142 re-solves over the 240 frames: the gain is
    # within the spread of training, so the bound is that the warm start
    # costs at most a few per cent of iterations while it serves the bodies
    # above.
    assert w["it"] <= 1.06 * z["it"]
    assert abs(w["y"] - p["y"]) <= 0.01 * abs(p["y"])
    assert abs(w["ke"] - p["ke"]) <= 0.03 * p["ke"]
