"""Decoding of the X16 tensor-core operand layout (test infrastructure):
X16[kc][c][e][128 B], row = [re(32 spectra) | im(32 spectra)] as f16/bf16,
16-byte chunk j stored at j ^ (e & 7)."""
import numpy as np


def phys_index(L, e):
    """Half-word position of logical value L (0..63) of row e."""
    return (((L >> 3) ^ (e & 7)) << 3) | (L & 7)


def unswizzle_x16(buf, nch, nsp, ne, nep, bf16=False):
    """X16 bytes -> float32 [c][s][e][2] (re, im)."""
    nkc = (nsp + 31) // 32
    if bf16:
        h = buf.view(np.uint16).astype(np.uint32) << 16
        rows = h.view(np.float32).reshape(nkc, nch, nep, 64)
    else:
        rows = buf.view(np.float16).reshape(nkc, nch, nep, 64)
    rows = rows.transpose(1, 0, 2, 3)  # [c][kc][e][64]
    X = np.zeros((nch, nkc * 32, ne, 2), np.float32)
    L = np.arange(64)
    for e in range(ne):
        p = phys_index(L, e)
        logical = rows[:, :, e, :][:, :, p]
        X[:, :, e, 0] = logical[:, :, :32].reshape(nch, -1)
        X[:, :, e, 1] = logical[:, :, 32:].reshape(nch, -1)
    return X[:, :nsp]


def swizzle_x16(X, nep):
    """Logical values X[c][s][e][2] (re, im; representable in f16) -> X16 bytes."""
    nch, nsp, ne, _ = X.shape
    nkc = (nsp + 31) // 32
    rows = np.zeros((nkc, nch, nep, 64), np.float16)
    L = np.arange(64)
    for e in range(ne):
        p = phys_index(L, e)
        for kc in range(nkc):
            s = np.arange(kc * 32, min(nsp, kc * 32 + 32))
            vals = np.zeros((nch, 64), np.float16)
            vals[:, :len(s)] = X[:, s, e, 0]
            vals[:, 32:32 + len(s)] = X[:, s, e, 1]
            rk = rows[kc]          # view [c][e][64]
            rk[:, e, p] = vals
    return rows.view(np.uint8).reshape(-1)
