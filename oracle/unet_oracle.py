"""CPU oracle of the learned preconditioner network (test infrastructure only).

A float64 numpy restatement of the 4-level U-Net of csrc/unet.cu (the library's own design; the
reference has no network): forward pass and the gradients of a scalar loss with respect to
every weight and bias, used to check the GPU forward and backward kernels.  Tensors are
[batch][channel][height][width]; convolutions are 3x3 with zero padding.
"""
import numpy as np

# (cin, cout, level, relu) of the twelve convolutions
LAYERS = [(2, 16, 0, True), (16, 16, 0, True), (16, 32, 1, True), (32, 32, 1, True), (32, 64, 2, True),
          (64, 64, 2, True), (64, 64, 3, True), (64, 64, 3, True), (128, 64, 2, True), (96, 32, 1, True),
          (48, 16, 0, True), (16, 1, 0, False)]


def conv3(x, w, b):
    """out[b, co] = bias[co] + sum_ci sum_k w[co, ci, ky, kx] x[b, ci, y + ky - 1, x + kx - 1]"""
    B, C, H, W = x.shape
    xp = np.zeros((B, C, H + 2, W + 2))
    xp[:, :, 1:-1, 1:-1] = x
    out = np.zeros((B, w.shape[0], H, W)) + (b[None, :, None, None] if b is not None else 0.0)
    for ky in range(3):
        for kx in range(3):
            out += np.einsum('oc,bchw->bohw', w[:, :, ky, kx], xp[:, :, ky:ky + H, kx:kx + W])
    return out


def conv3_back(x, w, g):
    """Gradients of conv3 for the output gradient g: (dx, dw, db)."""
    B, C, H, W = x.shape
    xp = np.zeros((B, C, H + 2, W + 2))
    xp[:, :, 1:-1, 1:-1] = x
    dxp = np.zeros_like(xp)
    dw = np.zeros_like(w)
    for ky in range(3):
        for kx in range(3):
            dw[:, :, ky, kx] = np.einsum('bohw,bchw->oc', g, xp[:, :, ky:ky + H, kx:kx + W])
            dxp[:, :, ky:ky + H, kx:kx + W] += np.einsum('oc,bohw->bchw', w[:, :, ky, kx], g)
    return dxp[:, :, 1:-1, 1:-1], dw, g.sum(axis=(0, 2, 3))


def pool(x):
    return 0.25 * (x[:, :, 0::2, 0::2] + x[:, :, 0::2, 1::2] + x[:, :, 1::2, 0::2] + x[:, :, 1::2, 1::2])


def pool_back(g):
    return 0.25 * np.repeat(np.repeat(g, 2, axis=2), 2, axis=3)


def up(x):
    return np.repeat(np.repeat(x, 2, axis=2), 2, axis=3)


def up_back(g):
    return g[:, :, 0::2, 0::2] + g[:, :, 0::2, 1::2] + g[:, :, 1::2, 0::2] + g[:, :, 1::2, 1::2]


def forward(x, ws, bs):
    """Network output and the saved activations."""
    a = [None] * 12
    inp = [None] * 12
    h = x
    for k in range(8):
        if k in (2, 4, 6):
            h = pool(a[k - 1])
        inp[k] = h
        z = conv3(h, ws[k], bs[k])
        a[k] = np.maximum(z, 0.0)
        h = a[k]
    for d, (k, prev, skip) in enumerate(((8, 7, 5), (9, 8, 3), (10, 9, 1))):
        inp[k] = np.concatenate((up(a[prev]), a[skip]), axis=1)
        a[k] = np.maximum(conv3(inp[k], ws[k], bs[k]), 0.0)
    inp[11] = a[10]
    a[11] = conv3(a[10], ws[11], bs[11])
    return a[11], (a, inp)


def backward(saved, ws, dy):
    """Weight and bias gradients for dL/dy = dy."""
    a, inp = saved
    ga = [np.zeros_like(t) for t in a]
    dws, dbs = [None] * 12, [None] * 12
    ga[11] = dy

    def back(k):
        g = ga[k] if not LAYERS[k][3] else ga[k] * (a[k] > 0)
        dx, dws[k], dbs[k] = conv3_back(inp[k], ws[k], g)
        return dx

    ga[10] += back(11)
    for k, prev, skip in ((10, 9, 1), (9, 8, 3), (8, 7, 5)):
        dcat = back(k)
        cu = a[prev].shape[1]
        ga[prev] += up_back(dcat[:, :cu])
        ga[skip] += dcat[:, cu:]
    for k in range(7, -1, -1):
        dx = back(k)
        if k in (2, 4, 6):
            ga[k - 1] += pool_back(dx)
        elif k > 0:
            ga[k - 1] += dx
    return dws, dbs
