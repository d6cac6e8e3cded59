"""ORACLE (test infrastructure only; never imported by the product path).

numpy restatement of mom25d's FreqInterp transform
(Engine/mom25d/freqinterp.py:93-165): an anchor matrix is
W = j w Z exp(+j k_e R) (_anchor, 107-122), R the distance of the basis
centres with 0 between two via unknowns (_R_block, 93-105), and the
interpolated Z = (sum_a L_a W_a) exp(-j k_e R) / (j w) (impedance,
145-165). Used to check the device kernels (m25_interp_store / _eval) and,
with the oracle's own fill at the anchors, against the reference's
interpolated Z (tests/golden/*_interp.npz).
"""

import numpy as np


def distances(pos, nb):
    """R (n, n) float64 between the basis centres, 0 in the via-via block."""
    d = pos[:, None, :] - pos[None, :, :]
    R = np.sqrt((d * d).sum(-1))
    R[nb:, nb:] = 0.0
    return R


def store(Z, pos, nb, freq, ke, dtype=np.complex128):
    w = 2 * np.pi * freq
    return (1j * w * Z * np.exp(1j * ke * distances(pos, nb))).astype(dtype)


def evaluate(Ws, L, pos, nb, freq, ke):
    w = 2 * np.pi * freq
    acc = sum(Li * Wi.astype(complex) for Li, Wi in zip(L, Ws))
    return acc * np.exp(-1j * ke * distances(pos, nb)) / (1j * w)


def window(anchors, order, f):
    """freqinterp.py:124-132."""
    n, k = len(anchors), order + 1
    j = int(np.clip(np.searchsorted(anchors, f, side="right") - 1, 0, n - 2))
    i0 = min(max(j - (k - 1) // 2, 0), n - k)
    return list(range(i0, i0 + k))


def weights(anchors, f, idx):
    """freqinterp.py:134-141."""
    fa = anchors[idx]
    L = np.ones(len(idx))
    for a in range(len(idx)):
        for b in range(len(idx)):
            if a != b:
                L[a] *= (f - fa[b]) / (fa[a] - fa[b])
    return L
