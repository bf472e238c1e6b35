"""CPU reference of the warm-start network (TEST INFRASTRUCTURE).

The checker for the GPU kernels of cubez_gb300/csrc/cz_mlp.cu: the same
forward pass, loss and backward pass in numpy, rounding weights, activations
and backward operands to BF16 (round to nearest even) where the tensor-core
kernels do, accumulating in float64 here (the kernels accumulate in float32,
so results agree to float32 rounding of sums, not bit for bit).
"""
import numpy as np

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


def bf16(a):
    """Round float32 values to the nearest BF16 (ties to even), as float32."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    rounded = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return (rounded.astype(np.uint32) << 16).view(np.float32).reshape(a.shape)


def unpack(blob, dtype=np.float32):
    b = np.asarray(blob, dtype)
    return {
        "W1": b[OFF_W1:OFF_B1].reshape(H, IN), "b1": b[OFF_B1:OFF_W2],
        "W2": b[OFF_W2:OFF_B2].reshape(H, H), "b2": b[OFF_B2:OFF_W3],
        "W3": b[OFF_W3:OFF_B3].reshape(H, H), "b3": b[OFF_B3:OFF_W4],
        "W4": b[OFF_W4:OFF_B4].reshape(OUT, H), "b4": b[OFF_B4:NPARAM],
        "mu": b[OFF_MU:OFF_IS], "inv_sigma": b[OFF_IS:OFF_OS], "out_scale": b[OFF_OS:OFF_OS + OUT],
    }


def forward(blob, x, rounding=True):
    """rounding=False evaluates the same network in float64 without the BF16
    roundings (for finite-difference checks of the gradient formulas)."""
    p = unpack(blob, np.float32 if rounding else np.float64)
    f64 = np.float64
    r = bf16 if rounding else (lambda a: np.asarray(a, f64))
    xn = r(((x - p["mu"]) * p["inv_sigma"]).astype(np.float32 if rounding else f64))
    W = {k: r(p[k]).astype(f64) for k in ("W1", "W2", "W3", "W4")}
    z1 = xn.astype(f64) @ W["W1"].T + p["b1"]
    h1 = r(np.maximum(z1, 0).astype(np.float32 if rounding else f64))
    z2 = h1.astype(f64) @ W["W2"].T + p["b2"]
    h2 = r(np.maximum(z2, 0).astype(np.float32 if rounding else f64))
    z3 = h2.astype(f64) @ W["W3"].T + p["b3"]
    h3 = r(np.maximum(z3, 0).astype(np.float32 if rounding else f64))
    o = h3.astype(f64) @ W["W4"].T + p["b4"]
    return {"xn": xn, "h1": h1, "h2": h2, "h3": h3, "o": o, "W": W, "p": p, "r": r}


def predict(blob, x):
    f = forward(blob, x)
    return (f["o"] * f["p"]["out_scale"]).astype(np.float32)


def loss_and_grad(blob, x, y, rounding=True):
    """Mean squared error of the normalised outputs and its gradient with
    respect to the trainable parameters (flat, NPARAM floats)."""
    f = forward(blob, x, rounding)
    p, W = f["p"], f["W"]
    bf16 = f["r"]
    n = len(x)
    t = y / p["out_scale"]
    d = f["o"] - t
    loss = float((d * d).sum() / (OUT * n))
    do = (2.0 * d / (OUT * n)).astype(np.float32 if rounding else np.float64)
    dob = bf16(do).astype(np.float64)
    g = np.zeros(NPARAM, np.float64)
    g[OFF_B4:NPARAM] = do.astype(np.float64).sum(axis=0)
    g[OFF_W4:OFF_B4] = (dob.T @ f["h3"].astype(np.float64)).ravel()
    dh3 = dob @ W["W4"]
    dz3 = np.where(f["h3"] > 0, dh3, 0.0)
    dz3b = bf16(dz3.astype(np.float32) if rounding else dz3).astype(np.float64)
    g[OFF_B3:OFF_W4] = dz3.astype(np.float64).sum(axis=0)
    g[OFF_W3:OFF_B3] = (dz3b.T @ f["h2"].astype(np.float64)).ravel()
    dh2 = dz3b @ W["W3"]
    dz2 = np.where(f["h2"] > 0, dh2, 0.0)
    dz2b = bf16(dz2.astype(np.float32) if rounding else dz2).astype(np.float64)
    g[OFF_B2:OFF_W3] = dz2.astype(np.float64).sum(axis=0)
    g[OFF_W2:OFF_B2] = (dz2b.T @ f["h1"].astype(np.float64)).ravel()
    dh1 = dz2b @ W["W2"]
    dz1 = np.where(f["h1"] > 0, dh1, 0.0)
    dz1b = bf16(dz1.astype(np.float32) if rounding else dz1).astype(np.float64)
    g[OFF_B1:OFF_W2] = dz1.astype(np.float64).sum(axis=0)
    g[OFF_W1:OFF_B1] = (dz1b.T @ f["xn"].astype(np.float64)).ravel()
    return loss, (g.astype(np.float32) if rounding else g)
