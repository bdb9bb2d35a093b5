"""Learned initial guess for the ECP contact parameter: training-set
generation from plain-Newton trajectories and training with the library's
tensor-core kernels (no counterpart in the reference).

Samples are (features of a listed pair, converged lambda) taken from the
device list after an ECP force call with the plain Newton solver, at several
temperatures. Features and labels stay on the device (BF16 / FP32 buffers
held as torch tensors, which serve only as device memory here).
"""
import ctypes as C

import numpy as np

from . import capi

_F = C.POINTER(C.c_float)


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def generate(g, pair_newton, step_langevin, temps=(0.8, 1.2, 1.6), samples=1_000_000, every=25, equil=200,
             device="cuda"):
    """Run Langevin MD at each temperature with the plain Newton solver and
    collect the (features, lambda) of every listed pair every `every` steps
    until `samples` are gathered. `step_langevin(T)` configures the context's
    captured step for temperature T. Returns (X bf16 [S,16], y fp32 [S])."""
    import torch
    X = torch.empty((samples, 16), dtype=torch.bfloat16, device=device)
    y = torch.empty((samples,), dtype=torch.float32, device=device)
    torch.cuda.synchronize()
    per_t = samples // len(temps)
    got = 0
    for ti, T in enumerate(temps):
        step_langevin(T)
        g.step(equil)
        target = samples if ti == len(temps) - 1 else (ti + 1) * per_t
        while got < target:
            g.step(every)
            g.zero_forces()
            g.pair_forces(pair_newton)
            cnt = C.c_int64(0)
            room = target - got
            capi.check(g.ctx, g.L.sg_mlp_features(g.ctx, _ptr(X[got:]), _ptr(y[got:]), room, C.byref(cnt)))
            got += cnt.value
        g.step_check()
    return X, y


def train(g, X, y, epochs=4, batch=65536, lr=2e-3, seed=1, init=True, log=None):
    """Adam on minibatches of a fixed random permutation; returns the loss history."""
    import torch
    if init:
        capi.check(g.ctx, g.L.sg_mlp_init(g.ctx, seed))
    n = X.shape[0]
    gen = torch.Generator(device=X.device)
    gen.manual_seed(seed)
    hist = []
    loss = C.c_float(0.0)
    for ep in range(epochs):
        perm = torch.randperm(n, device=X.device, generator=gen)
        Xs = X[perm].contiguous()
        ys = y[perm].contiguous()
        torch.cuda.synchronize()   # the library works on its own (non-blocking) stream
        acc = 0.0
        nb = 0
        for b0 in range(0, n - batch + 1, batch):
            capi.check(g.ctx, g.L.sg_mlp_train_step(g.ctx, _ptr(Xs[b0:]), _ptr(ys[b0:]), batch, lr, C.byref(loss)))
            acc += loss.value
            nb += 1
        hist.append(acc / max(nb, 1))
        if log:
            log(f"epoch {ep} mse {hist[-1]:.3e}")
    return hist


def grad(g, X, y):
    import torch
    torch.cuda.synchronize()
    loss = C.c_float(0.0)
    out = np.zeros(g.L.sg_mlp_weight_count(), dtype=np.float32)
    capi.check(g.ctx, g.L.sg_mlp_grad(g.ctx, _ptr(X), _ptr(y), X.shape[0], out.ctypes.data_as(_F), C.byref(loss)))
    return out, loss.value


def predict(g, X):
    import torch
    out = torch.empty(X.shape[0], dtype=torch.float32, device=X.device)
    torch.cuda.synchronize()
    capi.check(g.ctx, g.L.sg_mlp_predict(g.ctx, _ptr(X), X.shape[0], _ptr(out)))
    g.synchronize()
    return out


def guess_tc(g):
    """The tensor-core guess pass (tcgen05) for the current list, same order as guess()."""
    import torch
    k = g.npairs()
    out = torch.empty(max(k, 1), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    capi.check(g.ctx, g.L.sg_mlp_guess_tc(g.ctx, _ptr(out), out.numel()))
    return out[:k]


def guess(g):
    """The ECP kernel's in-kernel guesses for the current list (sg_nlist_pairs order)."""
    import torch
    k = g.npairs()
    out = torch.empty(max(k, 1), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    capi.check(g.ctx, g.L.sg_mlp_guess(g.ctx, _ptr(out), out.numel()))
    return out[:k]
