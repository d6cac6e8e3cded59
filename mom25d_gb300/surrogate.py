"""Learned layered-Green's remainder.

The Green's tables of a frequency are the closed-form leading terms plus a
remainder, the Sommerfeld integral of the spectral remainder against J0
(mom25d: Engine/mom25d/greens.py:157-173, layered.py:360-372), evaluated at
every tabulation radius; the integral is the cost of a table. GreensSurrogate
trains a small network (3 x 64 tanh, fp32) on the engine's own Sommerfeld
integrals over a frequency band of one stack, the inputs a logarithmic radius
coordinate and the frequency, the outputs the real and imaginary parts of the
remainder of every kernel and level pair. With it attached the engine

  - integrates at the radii below `near` x a (a: the thinnest layer, the
    scale of the remainder's structure near the source), then at every
    `stride`-th radius (the knots) and at the middle radius of each gap
    between knots (validation radii),
  - corrects the network with a not-a-knot spline of its residual through the
    knots and judges the corrected network at the validation radii: accepted
    when the largest error there is <= tol x max |remainder|,
  - and when accepted fills the other radii with the network plus the spline
    of its residual through all integrated radii; else integrates there too
    (the plain tabulation, no integral wasted).

The network (mom25d_gb300/csrc/mlp.cu) is trained on the GPU by the engine's
forward, backward and Adam kernels; tests/test_gpu_surrogate.py checks their
gradients against oracle/mlp.py.

Measured on the two-layer via transition on one GB300 (1-20 GHz, 1024 x
1024 = 1.05e6 samples, 20000 Adam steps in 2.9 s; stride 4, near 8 a,
tol 5e-6; tests/test_gpu_surrogate.py): accepted at 9 of 10 frequencies;
judged error 1.9-3.9e-6 of the largest remainder, where a spline of the
integral alone through the same knots is off by 6.3-8.0e-6; 115-223 of the
149-365 radii integrated; table time 0.68-1.14 ms against 0.72-1.61 ms
without the network; S of a sweep within 1.9e-6 of the plain tabulation's.
"""

import ctypes as C
import time

import numpy as np

from . import engine as E

_f32p = C.POINTER(C.c_float)


def _f32(a):
    return np.ascontiguousarray(a, np.float32)


class MLP:
    """tanh network n_in -> 64 x layers -> n_out on the device (fp32)."""

    def __init__(self, ctx, n_in, n_out, layers=3, seed=0):
        self.ctx, self.n_in, self.n_out, self.layers = ctx, n_in, n_out, layers
        h = C.c_void_p()
        E.check(ctx.lib.m25_mlp_create(ctx.h, n_in, 64, layers, n_out, seed, C.byref(h)))
        self._h = E.Handle(ctx, h, ctx.lib.m25_mlp_destroy)
        self.h = h
        cnt = C.c_int64()
        E.check(ctx.lib.m25_mlp_params(h, C.byref(cnt), None, None))
        self.count = cnt.value

    def params(self):
        p = np.zeros(self.count, np.float32)
        E.check(self.ctx.lib.m25_mlp_params(self.h, None, p.ctypes.data_as(_f32p), None))
        return p

    def set_params(self, p):
        p = _f32(p)
        assert p.size == self.count
        E.check(self.ctx.lib.m25_mlp_params(self.h, None, None, p.ctypes.data_as(_f32p)))

    def loss_grad(self, X, Y):
        X, Y = _f32(X), _f32(Y)
        loss = C.c_double()
        g = np.zeros(self.count, np.float32)
        E.check(self.ctx.lib.m25_mlp_loss_grad(self.h, X.shape[0], X.ctypes.data_as(_f32p), Y.ctypes.data_as(_f32p),
                                               C.byref(loss), g.ctypes.data_as(_f32p)))
        return loss.value, g

    def train(self, X, Y, steps, batch=4096, lr=2e-3, lr_min=1e-5, seed=0):
        X, Y = _f32(X), _f32(Y)
        loss = C.c_double()
        E.check(self.ctx.lib.m25_mlp_train(self.h, X.shape[0], X.ctypes.data_as(_f32p), Y.ctypes.data_as(_f32p),
                                           int(steps), int(batch), float(lr), float(lr_min), int(seed),
                                           C.byref(loss)))
        return loss.value

    def __call__(self, X):
        X = _f32(X)
        Y = np.zeros((X.shape[0], self.n_out), np.float32)
        E.check(self.ctx.lib.m25_mlp_forward(self.h, X.shape[0], X.ctypes.data_as(_f32p), Y.ctypes.data_as(_f32p)))
        return Y

    def close(self):
        self._h.close()


class GreensSurrogate:
    """Network for the Green's remainder of `solver`'s stack over [fmin, fmax].

    Training samples: the engine's Sommerfeld remainder at `nfreq` frequencies
    x `nrad` radii (quadratically spaced from 0 past the tabulation range).
    Attach with solver.surrogate = GreensSurrogate(solver, ...); every Greens
    of a frequency in the band then goes through the learned path and its
    judge (Greens.remainder() reports which table was used).
    """

    def __init__(self, solver, fmin, fmax, nfreq=64, nrad=256, layers=3, steps=12000, batch=4096, lr=2e-3,
                 lr_min=1e-5, seed=0, near=8.0, stride=4, tol=5e-6):
        from .solver import Greens

        self.fmin, self.fmax = float(fmin), float(fmax)
        # samples over the band widened by 5 % at either end: the network is
        # least accurate at the edges of its inputs
        pad = 0.05 * (self.fmax - self.fmin)
        self.flo, self.fhi = max(self.fmin - pad, 0.5 * self.fmin), self.fmax + pad
        self.near, self.stride, self.tol = float(near), int(stride), float(tol)
        st = solver.stack
        t = np.array([d.t for d in st.layers], float)
        self.a = float(t[0] if solver.single else t.min())  # the radius scale of the remainder's structure
        self.rho_ref = 1.1 * solver.rho_max
        t0 = time.perf_counter()
        rho = self.rho_ref * np.linspace(0.0, 1.0, nrad) ** 2
        F = np.linspace(self.flo, self.fhi, nfreq)
        Xs, Ys = [], []
        for f in F:
            g = Greens(solver, f, rho=rho, surrogate=False)
            res, _ = g.remainder()
            g.close()
            Xs.append(self.features(rho, f))
            Ys.append(np.concatenate([res.real, res.imag], 1)[:, self._order(res.shape[1])])
        X, Y = np.concatenate(Xs), np.concatenate(Ys)
        self.nc = Y.shape[1] // 2
        self.scale = np.abs(Y).max(0)
        self.scale[self.scale == 0] = 1.0
        self.sample_seconds = time.perf_counter() - t0
        self.nsamples = X.shape[0]
        t1 = time.perf_counter()
        self.net = MLP(solver.ctx, 2, 2 * self.nc, layers=layers, seed=seed)
        self.train_loss = self.net.train(X, Y / self.scale, steps, batch=batch, lr=lr, lr_min=lr_min, seed=seed)
        self.train_seconds = time.perf_counter() - t1
        self.X, self.Y = X, Y

    @staticmethod
    def _order(nc):
        # interleave: output 2c = Re(res[:, c]), 2c + 1 = Im(res[:, c])
        return np.stack([np.arange(nc), nc + np.arange(nc)], 1).ravel()

    def features(self, rho, f):
        s = 2.0 * np.log1p(np.asarray(rho, float) / self.a) / np.log1p(self.rho_ref / self.a) - 1.0
        u = np.full_like(s, 2.0 * (float(f) - self.flo) / (self.fhi - self.flo) - 1.0)
        return np.stack([s, u], 1)

    def predict(self, rho, f):
        """The network's remainder (uncorrected) at radii rho: (n, NC) complex."""
        Y = self.net(self.features(rho, f)).astype(float) * self.scale
        return Y[:, 0::2] + 1j * Y[:, 1::2]

    def covers(self, f):
        return self.fmin <= f <= self.fmax

    def fill_desc(self, d, scale_ptr):
        d.surrogate = self.net.h.value
        d.sur_a, d.sur_rho_ref, d.sur_fmin, d.sur_fmax = self.a, self.rho_ref, self.flo, self.fhi
        d.sur_scale = scale_ptr
        d.sur_near = self.near * self.a
        d.sur_stride = self.stride
        d.sur_tol = self.tol

    def close(self):
        self.net.close()
