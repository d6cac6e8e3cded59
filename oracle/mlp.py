"""ORACLE (test infrastructure only; never imported by the product path).

float64 restatement of the engine's learned-remainder network
(mom25d_gb300/csrc/mlp.cu): tanh hidden layers of width 64, a linear output
layer, parameters in one flat array layer by layer (W_l (out, in) row-major,
then b_l), loss = mean over samples and outputs of (f(x) - y)^2. mom25d has
no learned part; this checks the CUDA forward and backward kernels.
"""

import numpy as np

HIDDEN = 64


def layout(n_in, n_layers, n_out):
    """[(offset, out, in)] of every layer and the parameter count."""
    out, off = [], 0
    for l in range(n_layers + 1):
        fi = n_in if l == 0 else HIDDEN
        fo = n_out if l == n_layers else HIDDEN
        out.append((off, fo, fi))
        off += fo * fi + fo
    return out, off


def unpack(p, n_in, n_layers, n_out):
    lay, _ = layout(n_in, n_layers, n_out)
    Ws, bs = [], []
    for off, fo, fi in lay:
        Ws.append(p[off:off + fo * fi].reshape(fo, fi))
        bs.append(p[off + fo * fi:off + fo * fi + fo])
    return Ws, bs


def forward(p, X, n_layers, n_out):
    Ws, bs = unpack(np.asarray(p, float), X.shape[1], n_layers, n_out)
    a = np.asarray(X, float)
    acts = [a]
    for l, (W, b) in enumerate(zip(Ws, bs)):
        z = a @ W.T + b
        a = np.tanh(z) if l < n_layers else z
        acts.append(a)
    return a, acts


def loss_grad(p, X, Y, n_layers):
    """(loss, dloss/dp) of the mean squared error."""
    n_out = Y.shape[1]
    Ws, _ = unpack(np.asarray(p, float), X.shape[1], n_layers, n_out)
    f, acts = forward(p, X, n_layers, n_out)
    e = f - Y
    loss = np.mean(e ** 2)
    delta = 2.0 * e / e.size
    grads = [None] * (n_layers + 1)
    for l in range(n_layers, -1, -1):
        grads[l] = (delta.T @ acts[l], delta.sum(0))
        if l > 0:
            delta = (delta @ Ws[l]) * (1.0 - acts[l] ** 2)
    flat = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return loss, flat
