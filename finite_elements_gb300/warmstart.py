"""Learned warm start for the PCG solve: the graph network of libfe_gb300.so
(fe_gnn_*), its weights, and its training loop.

The network predicts the shape of the displacement field of an assembled
elasticity problem; the library scales it optimally in the A-norm and adds the
prescribed values, giving x0 for ``GpuSystem.solve(x0=...)``.  PCG from x0 to the same
tolerance decides the accuracy: a poor prediction only costs iterations.

Training uses solutions the solver itself produces: each training problem is solved
once by the library's PCG and the network is fitted to that solution, normalised by
its RMS (fe_gnn_fit_grad, mean-squared error on the free DOFs).  The energy loss of
fe_gnn_loss_grad -- the share of the solution's energy the warm start leaves to PCG
-- is what the scaled warm start minimises at inference and is reported beside it.
Forward, backward and Adam run on the GPU in the library's own kernels.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _lib
from .engine import GpuSystem

WEIGHTS_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights")
DEFAULT_WEIGHTS = os.path.join(WEIGHTS_DIR, "warmstart_gnn.npz")

HIDDEN, FEATURES, LAYERS = 64, 16, 6


def num_params():
    n = ctypes.c_int64()
    _lib.check(_lib.load().fe_gnn_num_params(ctypes.byref(n)), "fe_gnn_num_params")
    return n.value


def init_params(seed=0, gain=1.0):
    """He-uniform initial weights in the library's parameter layout: encoder
    W0 [16x64], b0; per layer W [128x64], b [64], U [64x64]; decoder Wd [64x2], bd."""
    rng = np.random.default_rng(seed)

    def uni(fan_in, shape, scale=1.0):
        lim = scale * np.sqrt(6.0 / fan_in)
        return rng.uniform(-lim, lim, shape)

    parts = [uni(FEATURES, FEATURES * HIDDEN) * gain, np.zeros(HIDDEN)]
    for _ in range(LAYERS):
        parts += [uni(2 * HIDDEN, 2 * HIDDEN * HIDDEN, 0.5) * gain, np.zeros(HIDDEN),
                  uni(HIDDEN, HIDDEN * HIDDEN, 0.1) * gain]
    parts += [uni(HIDDEN, HIDDEN * 2, 0.5) * gain, np.zeros(2)]
    p = np.concatenate(parts).astype(np.float32)
    assert p.size == num_params(), (p.size, num_params())
    return p


class WarmStartNet:
    """One network on the device (fe_gnn handle)."""

    def __init__(self, params=None, weights=None, seed=0):
        lib = _lib.load()
        self._lib = lib
        g = ctypes.c_void_p()
        _lib.check(lib.fe_gnn_create(ctypes.byref(g)), "fe_gnn_create")
        self.g = g
        if weights is not None:
            params = load_weights(weights)
        if params is None:
            params = init_params(seed)
        self.set_params(params)

    def close(self):
        if getattr(self, "g", None):
            self._lib.fe_gnn_destroy(self.g)
            self.g = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        _lib.check(self._lib.fe_gnn_set_params(self.g, _lib.ptr(p), p.size), "fe_gnn_set_params")

    def get_params(self):
        p = np.empty(num_params(), np.float32)
        _lib.check(self._lib.fe_gnn_get_params(self.g, _lib.ptr(p), p.size), "fe_gnn_get_params")
        return p

    def features(self, system: GpuSystem):
        out = np.empty((system.prob.n_nodes, FEATURES), np.float32)
        _lib.check(self._lib.fe_gnn_features(self.g, system.handle.h, _lib.ptr(out)), "fe_gnn_features")
        return out

    def predict(self, system: GpuSystem, host=False):
        """x0 for the system: (device address of n_dof doubles, valid until the next
        call, or a host copy with host=True) and the scale s."""
        x0 = ctypes.c_void_p()
        s = ctypes.c_double()
        out = np.empty(system.prob.n_dof) if host else None
        _lib.check(self._lib.fe_gnn_predict(self.g, system.handle.h, _lib.ptr(out) if host else None,
                                            ctypes.byref(x0), ctypes.byref(s)), "fe_gnn_predict")
        return (out if host else x0.value), s.value

    def predict_async(self, system: GpuSystem):
        """x0 for the system, enqueued on the network's own stream: returns at once with
        the device address of n_dof doubles; the system's next solve waits for the
        prediction before it reads x0 (its multigrid setup runs meanwhile)."""
        x0 = ctypes.c_void_p()
        _lib.check(self._lib.fe_gnn_predict_async(self.g, system.handle.h, ctypes.byref(x0)),
                   "fe_gnn_predict_async")
        return x0.value

    def target_energy(self, system: GpuSystem):
        e = ctypes.c_double()
        _lib.check(self._lib.fe_gnn_target_energy(self.g, system.handle.h, ctypes.byref(e)),
                   "fe_gnn_target_energy")
        return e.value

    def loss_grad(self, system: GpuSystem, energy, want_grad=False):
        loss = ctypes.c_double()
        grad = np.empty(num_params(), np.float32) if want_grad else None
        _lib.check(self._lib.fe_gnn_loss_grad(self.g, system.handle.h, float(energy), ctypes.byref(loss),
                                              _lib.ptr(grad) if want_grad else None), "fe_gnn_loss_grad")
        return loss.value, grad

    def fit_grad(self, system: GpuSystem, want_grad=False):
        """Mean-squared error against the system's last solution (normalised), and
        its gradient."""
        loss = ctypes.c_double()
        grad = np.empty(num_params(), np.float32) if want_grad else None
        _lib.check(self._lib.fe_gnn_fit_grad(self.g, system.handle.h, ctypes.byref(loss),
                                             _lib.ptr(grad) if want_grad else None), "fe_gnn_fit_grad")
        return loss.value, grad

    def adam_step(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        _lib.check(self._lib.fe_gnn_adam_step(self.g, lr, beta1, beta2, eps), "fe_gnn_adam_step")


def save_weights(path, params, meta=None):
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    np.savez_compressed(path, params=np.asarray(params, np.float32),
                        **{k: np.asarray(v) for k, v in (meta or {}).items()})


def load_weights(path=DEFAULT_WEIGHTS):
    return np.load(path)["params"].astype(np.float32)


def solve_with_warm_start(system: GpuSystem, net: WarmStartNet, **solve_kw):
    """Predict x0 with the network and run PCG from it."""
    ptr, _ = net.predict(system)
    return system.solve(x0_device_ptr=ptr, **solve_kw)


def train(problems, net: WarmStartNet, steps=2000, lr=1e-3, seed=0, solve_kw=None, log_every=200, log=print):
    """Train on a list of Problems: solve each once with the library's PCG (the
    targets), then Adam steps over randomly drawn problems.  Returns the loss history."""
    solve_kw = dict(precision="mixed", tol=1e-8, cheb_degree=3, **(solve_kw or {}))
    rng = np.random.default_rng(seed)
    systems = []
    for p in problems:
        s = GpuSystem(p)
        _, st = s.solve(want_host=False, **solve_kw)
        if st.status != 0:
            s.close()
            continue
        systems.append(s)
    hist = []
    run = 0.0
    for k in range(steps):
        i = int(rng.integers(len(systems)))
        loss, _ = net.fit_grad(systems[i])
        net.adam_step(lr=lr * (0.1 if k > 0.8 * steps else 1.0))
        run = loss if k == 0 else 0.98 * run + 0.02 * loss
        hist.append(loss)
        if log and (k % log_every == 0 or k == steps - 1):
            log(f"step {k}: loss {loss:.4f} (running {run:.4f})")
    for s in systems:
        s.close()
    return np.array(hist)
