"""The learned warm start of adjustVelocities (host side).

  harvest(batch, ...)   features and total applied contact-frame impulses of
                        the plain resolver (the training set)
  Trainer               the GPU trainer (hand-written BF16 tensor-core
                        forward/backward kernels, Adam on FP32 masters)
  batch.set_warm_start  enable the network inside the resolver

The network: 18 features -> 64 -> 64 -> 64 -> 3, ReLU.  Parameter blobs are
float32 arrays of BLOB floats in the layout of include/cubez_gpu.h.
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import check

IN, H, OUT = 18, 64, 3
OFF_W1 = 0
OFF_B1 = OFF_W1 + H * IN
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H * H
OFF_W4 = OFF_B3 + H
OFF_B4 = OFF_W4 + OUT * H
NPARAM = OFF_B4 + OUT
OFF_MU = NPARAM
OFF_IS = OFF_MU + IN
OFF_OS = OFF_IS + IN
BLOB = OFF_OS + OUT

# The columns of the harvested features (contact_features in cz_resolve.cuh),
# all in the contact basis: body 0's contacts with other bodies, a half-space
# flag, the contact velocity, penetration, desired delta velocity, the
# velocity-per-impulse matrix (nn, tt, ss, nt, ns, ts), the impulse that would
# resolve the contact alone, and per body its contact count and the sum of its
# contacts' positive desired delta velocities.
FEATURES = ("body0_pair_contacts", "half_space", "cv_n", "cv_t", "cv_s", "penetration", "desired_dv",
            "k_nn", "k_tt", "k_ss", "k_nt", "k_ns", "k_ts", "alone_impulse",
            "contacts_body_0", "contacts_body_1", "load_body_0", "load_body_1")
assert len(FEATURES) == IN


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def lib():
    return _lib.load()


def harvest(batch, nsteps, dt=1.0 / 60.0, every=10, capacity=1 << 20):
    """Step `batch` nsteps frames with the plain resolver; every `every`
    frames record each contact's features and the impulse adjustVelocities
    applied to it in total.  Returns (features [n,18], labels [n,3])."""
    L = lib()
    f = np.zeros((capacity, IN), np.float32)
    y = np.zeros((capacity, OUT), np.float32)
    n = C.c_int64(0)
    check(L.cz_harvest(batch.h, int(nsteps), float(dt), int(every), _ptr(f), _ptr(y), int(capacity), C.byref(n)))
    return f[:n.value].copy(), y[:n.value].copy()


def set_warm_start(batch, blob):
    """Enable the warm start with a parameter blob, or disable it (None)."""
    L = lib()
    if blob is None:
        check(L.cz_set_warm_start(batch.h, None))
    else:
        b = np.ascontiguousarray(blob, np.float32)
        assert b.shape == (BLOB,)
        check(L.cz_set_warm_start(batch.h, _ptr(b)))
    batch.warm_start = blob is not None


class Trainer:
    """GPU trainer of the warm-start network (cz_mlp_*)."""

    def __init__(self, seed=0, device=0):
        self.L = lib()
        h = C.c_void_p()
        check(self.L.cz_mlp_create(device, seed, C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.cz_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def params(self):
        b = np.zeros(BLOB, np.float32)
        check(self.L.cz_mlp_get_params(self.h, _ptr(b)))
        return b

    def set_params(self, blob):
        b = np.ascontiguousarray(blob, np.float32)
        check(self.L.cz_mlp_set_params(self.h, _ptr(b)))

    def set_data(self, x, y, normalize=True):
        self._x = np.ascontiguousarray(x, np.float32)
        self._y = np.ascontiguousarray(y, np.float32)
        check(self.L.cz_mlp_set_data(self.h, _ptr(self._x), _ptr(self._y), len(self._x), 1 if normalize else 0))

    def train(self, epochs, batch=4096, lr=1e-3, seed=1):
        losses = np.zeros(epochs, np.float32)
        check(self.L.cz_mlp_train(self.h, int(epochs), int(batch), float(lr), int(seed), _ptr(losses)))
        return losses

    def loss_and_grad(self, n):
        loss = C.c_float(0.0)
        g = np.zeros(NPARAM, np.float32)
        check(self.L.cz_mlp_loss_and_grad(self.h, int(n), C.byref(loss), _ptr(g)))
        return loss.value, g

    def predict(self, x):
        x = np.ascontiguousarray(x, np.float32)
        out = np.zeros((len(x), OUT), np.float32)
        check(self.L.cz_mlp_predict(self.h, _ptr(x), len(x), _ptr(out)))
        return out


def train_warm_start(seeds=(100, 101), num_worlds=4096, settle=60, frames=540, every=20, epochs=(16, 16),
                     lr=(2e-3, 5e-4), batch=8192, max_rows=3_000_000, seed=1, device=0):
    """The training procedure of the warm-start network: harvest the plain
    precision-form resolver on seeded precision scenes (settle frames first,
    then every `every` frames over `frames`), keep the contacts of grounded
    bodies (all their contacts with the half-space: the ones the warm start
    serves), train on the GPU in two phases of (epochs, learning rate).
    Returns (blob, info)."""
    from . import scenes
    from .batch import FORM_FP32, WorldBatch
    xs, ys = [], []
    for s in seeds:
        b = WorldBatch.from_scene(scenes.precision(num_worlds=num_worlds, seed=s), form=FORM_FP32, device=device)
        b.step(settle, 1.0 / 60.0)
        x, y = harvest(b, frames, 1.0 / 60.0, every=every, capacity=max(1, 2 * max_rows // len(seeds)))
        b.close()
        xs.append(x)
        ys.append(y)
    x, y = np.concatenate(xs), np.concatenate(ys)
    grounded = (x[:, 0] == 0) & (x[:, 1] == 1)
    x, y = x[grounded][:max_rows], y[grounded][:max_rows]
    t = Trainer(seed=seed, device=device)
    t.set_data(x, y, normalize=True)
    losses = [t.train(epochs=e, batch=batch, lr=r) for e, r in zip(epochs, lr)]
    blob = t.params()
    t.close()
    return blob, {"rows": int(len(x)), "grounded_fraction": float(grounded.mean()),
                  "loss_first": float(losses[0][0]), "loss_last": float(losses[-1][-1]), "seeds": list(seeds)}
