"""Learned preconditioner for the GMRES pressure path (no reference counterpart).

The network is the 4-level convolutional U-Net of csrc/unet.cu (BF16 weights, FP32
activations and accumulation, hand-written forward and backward kernels).  It learns the part
of the pressure solve that the separable rectangle inverse T^-1 misses: for a right-hand side
b with s = max |b| it maps [b / s, mask] to (A^-1 b - T^-1 b) / s.  Attached to a
``MAC_CylinderFlow(pressure_solver='iterative')`` case, flexible GMRES preconditions its first
direction (the right-hand side itself, the distribution the network was trained on) with
z = T^-1 b + s net([b / s, mask]) and every later direction with T^-1; GMRES still iterates to
the reference's true-residual tolerance, so the network only changes the iteration count.

Training pairs are the solver's own pressure solves (``record_pressure_pairs``).  Training
runs on the GPU through ``UNetFunction`` (a ``torch.autograd.Function`` over the library's
forward and backward kernels) with Adam on FP32 master weights; the kernels read BF16 copies.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import lib


def layer_shapes():
    """[(cin, cout)] of the twelve 3x3 convolutions."""
    n = C.c_int32()
    lib.gm_unet_layers(C.byref(n), None, None)
    cin = (C.c_int32 * n.value)()
    cout = (C.c_int32 * n.value)()
    lib.gm_unet_layers(None, cin, cout)
    return [(cin[k], cout[k]) for k in range(n.value)]


def _torch():
    import torch
    return torch


class UNetWeights:
    """FP32 master weights (torch parameters on the GPU) and their BF16 copies."""

    def __init__(self, seed=0, device='cuda'):
        torch = _torch()
        g = torch.Generator().manual_seed(seed)
        self.w, self.b = [], []
        for k, (cin, cout) in enumerate(layer_shapes()):
            std = (2.0 / (9 * cin)) ** 0.5 if k < 11 else 1e-2 / (9 * cin) ** 0.5
            self.w.append(torch.nn.Parameter((torch.randn(cout, cin, 3, 3, generator=g) * std).to(device)))
            self.b.append(torch.nn.Parameter(torch.zeros(cout, device=device)))
        self.refresh()

    def parameters(self):
        return self.w + self.b

    def refresh(self):
        """BF16 copies of the master weights (called after every optimizer step)."""
        torch = _torch()
        self.w16 = [w.detach().to(torch.bfloat16).contiguous() for w in self.w]
        self.wp = (C.c_void_p * len(self.w16))(*[t.data_ptr() for t in self.w16])
        self.bp = (C.c_void_p * len(self.b))(*[t.data_ptr() for t in self.b])

    def count(self):
        return sum(int(p.numel()) for p in self.parameters())

    def state_dict(self):
        return {f'w{k}': w.detach().cpu().numpy() for k, w in enumerate(self.w)} | \
               {f'b{k}': b.detach().cpu().numpy() for k, b in enumerate(self.b)}

    def load(self, state):
        torch = _torch()
        with torch.no_grad():
            for k, w in enumerate(self.w):
                w.copy_(torch.from_numpy(np.asarray(state[f'w{k}'], np.float32)))
            for k, b in enumerate(self.b):
                b.copy_(torch.from_numpy(np.asarray(state[f'b{k}'], np.float32)))
        self.refresh()


class UNet:
    """Activation workspace of the network for a (batch, height, width) shape."""

    def __init__(self, batch, height, width):
        h = C.c_void_p()
        rc = lib.gm_unet_create(int(batch), int(height), int(width), C.byref(h))
        if rc != _lib.GM_OK:
            raise _lib.error_for(rc, lib.gm_unet_last_error(None).decode(errors='replace'))
        self._u, self.shape = h, (int(batch), int(height), int(width))

    def _check(self, rc):
        if rc != _lib.GM_OK:
            raise _lib.error_for(rc, lib.gm_unet_last_error(self._u).decode(errors='replace'))

    def forward(self, weights, x, stream=0):
        torch = _torch()
        B, H, W = self.shape
        y = torch.empty(B, 1, H, W, device=x.device, dtype=torch.float32)
        self._check(lib.gm_unet_forward(self._u, weights.wp, weights.bp, C.c_void_p(x.data_ptr()),
                                        C.c_void_p(y.data_ptr()), C.c_void_p(stream)))
        return y

    def backward(self, weights, dy, stream=0):
        torch = _torch()
        dw = [torch.zeros_like(w) for w in weights.w]
        db = [torch.zeros_like(b) for b in weights.b]
        dwp = (C.c_void_p * len(dw))(*[t.data_ptr() for t in dw])
        dbp = (C.c_void_p * len(db))(*[t.data_ptr() for t in db])
        self._check(lib.gm_unet_backward(self._u, weights.wp, C.c_void_p(dy.contiguous().data_ptr()), dwp, dbp,
                                         C.c_void_p(stream)))
        return dw, db

    def close(self):
        if getattr(self, '_u', None):
            lib.gm_unet_destroy(self._u)
            self._u = None

    def __del__(self):
        self.close()


def _make_function():
    torch = _torch()

    class UNetFunction(torch.autograd.Function):
        """y = net(x) with the library's kernels; backward returns the weight gradients."""

        @staticmethod
        def forward(ctx, x, net, weights, *params):
            torch.cuda.synchronize()
            y = net.forward(weights, x.contiguous(), torch.cuda.current_stream().cuda_stream)
            ctx.net, ctx.weights = net, weights
            return y

        @staticmethod
        def backward(ctx, dy):
            dw, db = ctx.net.backward(ctx.weights, dy, torch.cuda.current_stream().cuda_stream)
            return (None, None, None, *dw, *db)

    return UNetFunction


UNetFunction = None


def apply(net, weights, x):
    """Differentiable network output (the activations of this call are kept by `net`)."""
    global UNetFunction
    if UNetFunction is None:
        UNetFunction = _make_function()
    return UNetFunction.apply(x, net, weights, *weights.w, *weights.b)


def record_pressure_pairs(solver, n_steps, dt, capacity=None):
    """Runs n_steps of a MAC_CylinderFlow case and returns the right-hand sides and solutions
    of its pressure solves as torch tensors [k, ny, nx] (the solver's own training pairs)."""
    torch = _torch()
    cap = capacity or 2 * n_steps + 1
    ny, nx = solver.ny, solver.nx
    rhs = torch.zeros(cap, ny, nx, dtype=torch.float64, device='cuda')
    sol = torch.zeros_like(rhs)
    _lib.check(lib.gm_set_pressure_recorder(solver._h, C.c_void_p(rhs.data_ptr()), C.c_void_p(sol.data_ptr()),
                                            cap), solver._h)
    try:
        solver.solve(n_steps=n_steps, dt=dt, perturb_transient=False, save_artifacts=False, verbose=False)
    finally:
        count = int(lib.gm_pressure_recorded(solver._h))
        lib.gm_set_pressure_recorder(solver._h, None, None, 0)
    return rhs[:count], sol[:count]


def training_set(solver, rhs, sol):
    """Network inputs [k, 2, ny, nx] and targets [k, 1, ny, nx] (float32) from recorded pairs:
    x = [b / s, mask], y = (A^-1 b - T^-1 b) / s on the active cells, s = max |b|."""
    torch = _torch()
    mask = torch.from_numpy(np.ascontiguousarray(~solver.mask, dtype=np.float64)).cuda()
    active = np.zeros(solver.ny * solver.nx, bool)
    active[solver.gg.pi] = True
    act = torch.from_numpy(active.reshape(solver.ny, solver.nx).astype(np.float64)).cuda()
    xs, ys = [], []
    for b, x in zip(rhs, sol):
        s = float(torch.max(torch.abs(b * act)))
        if not s > 0:
            continue
        rect = torch.from_numpy(solver.gg.rectangle_solve('pressure', (b * act).cpu().numpy())).cuda()
        xs.append(torch.stack(((b * act / s), act)).float())
        ys.append(((x - rect * act) * act / s)[None].float())
    del mask
    return torch.stack(xs), torch.stack(ys), act.float()


def train(weights, x, y, mask, epochs=200, lr=2e-3, batch=4, seed=0, log=None):
    """Adam on the masked mean-squared error with a cosine learning-rate decay to lr / 20;
    returns the loss history."""
    torch = _torch()
    import math
    k, _, H, W = x.shape
    net = UNet(min(batch, k), H, W)
    opt = torch.optim.Adam(weights.parameters(), lr=lr)
    gen = torch.Generator(device='cpu').manual_seed(seed)
    hist = []
    B = net.shape[0]
    for ep in range(epochs):
        for gparam in opt.param_groups:
            gparam['lr'] = lr * (0.05 + 0.95 * 0.5 * (1 + math.cos(math.pi * ep / max(epochs, 1))))
        idx = torch.randperm(k, generator=gen)[:B]
        xb, yb = x[idx].contiguous(), y[idx].contiguous()
        opt.zero_grad()
        pred = apply(net, weights, xb)
        loss = (((pred - yb) * mask) ** 2).sum() / (mask.sum() * B)
        loss.backward()
        opt.step()
        weights.refresh()
        hist.append(float(loss.detach()))
        if log and ep % 50 == 0:
            log(ep, hist[-1])
    net.close()
    return hist


def relative_error(weights, x, y, mask):
    """Masked relative L2 error of the network on inputs x against targets y (per sample)."""
    torch = _torch()
    k, _, H, W = x.shape
    net = UNet(1, H, W)
    out = []
    with torch.no_grad():
        for i in range(k):
            pred = net.forward(weights, x[i:i + 1].contiguous(), torch.cuda.current_stream().cuda_stream)
            torch.cuda.synchronize()
            num = float(torch.linalg.vector_norm((pred - y[i:i + 1]) * mask))
            den = float(torch.linalg.vector_norm(y[i:i + 1] * mask))
            out.append(num / max(den, 1e-300))
    net.close()
    return out


class LearnedPreconditioner:
    """Trained network attached to a GMRES case: keeps the workspace and weights alive."""

    def __init__(self, solver, weights):
        if solver.pressure_solver != 'iterative':
            raise ValueError("the learned preconditioner serves pressure_solver='iterative'")
        self.solver, self.weights = solver, weights
        self.net = UNet(1, solver.ny, solver.nx)
        _lib.check(lib.gm_set_learned_preconditioner(solver._h, self.net._u, weights.wp, weights.bp), solver._h)

    def detach(self):
        lib.gm_set_learned_preconditioner(self.solver._h, None, None, None)
