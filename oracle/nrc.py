"""TEST INFRASTRUCTURE ONLY (the oracle): FP64 restatement of the neural radiance cache of
vkrt_gb300/csrc/nrc.cuh / nrc.cu, for checking the tensor-core kernels' outputs and gradients.

Given the cache's FP16 parameters (as uint16 bit patterns) and grid placement, it evaluates in double precision:
hash-grid encoding (16 levels x 2 features, trilinear, dense or hashed indexing), degree-3 real spherical harmonics
of the direction, the remaining inputs, the 64-64-64-64-64-64-16 ReLU MLP without biases, the relative L2 loss
mean((y - t)^2 / (y^2 + 0.01)) over records and RGB, and its gradients with respect to the weights and the table.
"""
from __future__ import annotations

import numpy as np

LEVELS, FEATURES, TABLE = 16, 2, 1 << 19
PRIMES = (1, 2654435761, 805459861)


def halves(u16: np.ndarray) -> np.ndarray:
    return np.asarray(u16, np.uint16).view(np.float16).astype(np.float64)


def weights_from_halves(w16: np.ndarray) -> list[np.ndarray]:
    w = halves(w16)
    mats = [w[l * 4096:(l + 1) * 4096].reshape(64, 64) for l in range(5)]
    mats.append(w[20480:].reshape(16, 64))
    return mats


def sh16(d: np.ndarray) -> np.ndarray:
    x, y, z = d[:, 0], d[:, 1], d[:, 2]
    xx, yy, zz = x * x, y * y, z * z
    return np.stack([
        np.full_like(x, 0.28209479177387814), -0.48860251190291987 * y, 0.48860251190291987 * z,
        -0.48860251190291987 * x, 1.0925484305920792 * x * y, -1.0925484305920792 * y * z,
        0.94617469575755997 * zz - 0.31539156525251999, -1.0925484305920792 * x * z,
        0.54627421529603959 * (xx - yy), 0.59004358992664352 * y * (-3 * xx + yy), 2.8906114426405538 * x * y * z,
        0.45704579946446572 * y * (1 - 5 * zz), 0.3731763325901154 * z * (5 * zz - 3),
        0.45704579946446572 * x * (1 - 5 * zz), 1.4453057213202769 * z * (xx - yy),
        0.59004358992664352 * x * (-xx + 3 * yy)], axis=1)


def _index(res: int, dense: bool, c: np.ndarray) -> np.ndarray:
    c = c.astype(np.uint64)
    if dense:
        r1 = np.uint64(res + 1)
        return (c[:, 0] + r1 * (c[:, 1] + r1 * c[:, 2])).astype(np.int64)
    h = c[:, 0] * np.uint64(PRIMES[0])
    h ^= (c[:, 1] * np.uint64(PRIMES[1])) & np.uint64(0xFFFFFFFF)
    h ^= (c[:, 2] * np.uint64(PRIMES[2])) & np.uint64(0xFFFFFFFF)
    return (h & np.uint64(TABLE - 1)).astype(np.int64)


class Cache:
    """FP64 evaluation of one cache state: inputs (n, 16) float32 records as the C ABI takes them."""

    def __init__(self, weights16, table16, lo, hi, res, dense):
        self.W = weights_from_halves(weights16)
        self.table = halves(table16).reshape(LEVELS, TABLE, FEATURES)
        self.lo = np.asarray(lo, np.float64)
        self.inv = 1.0 / (np.asarray(hi, np.float64) - self.lo)
        self.res = [int(r) for r in res]
        self.dense = [bool(d) for d in dense]

    def _corners(self, pos):
        u = np.clip((pos - self.lo) * self.inv, 0.0, 1.0)
        out = []
        for l in range(LEVELS):
            r = float(self.res[l])
            p = u * r
            fl = np.clip(np.floor(p), 0.0, r - 1.0)
            f = np.clip(p - fl, 0.0, 1.0)
            c0 = fl.astype(np.int64)
            idx, wts = [], []
            for k in range(8):
                d = np.array([k & 1, (k >> 1) & 1, (k >> 2) & 1])
                w = np.prod(np.where(d[None, :] == 1, f, 1.0 - f), axis=1)
                idx.append(_index(self.res[l], self.dense[l], c0 + d[None, :]))
                wts.append(w)
            out.append((np.stack(idx, 1), np.stack(wts, 1)))
        return out

    def encode(self, inputs):
        x = np.asarray(inputs, np.float64).reshape(-1, 16)
        n = len(x)
        corners = self._corners(x[:, 0:3])
        enc = np.zeros((n, 64))
        for l, (idx, w) in enumerate(corners):
            feats = self.table[l][idx]  # (n, 8, 2)
            enc[:, 2 * l:2 * l + 2] = np.einsum("nk,nkf->nf", w, feats)
        enc[:, 32:48] = sh16(x[:, 4:7])
        enc[:, 48:51] = x[:, 8:11]
        enc[:, 51] = x[:, 3]
        enc[:, 52:55] = x[:, 12:15]
        enc[:, 55] = x[:, 7]
        enc[:, 56] = 1.0
        return enc, corners

    def forward(self, inputs):
        x0, corners = self.encode(inputs)
        acts = [x0]
        h = x0
        for l in range(5):
            h = np.maximum(h @ self.W[l].T, 0.0)
            acts.append(h)
        y = h @ self.W[5].T
        return y, acts, corners

    def loss_and_grads(self, inputs, targets):
        y, acts, corners = self.forward(inputs)
        n = len(y)
        t = np.asarray(targets, np.float64)[:, :3]
        den = y[:, :3] ** 2 + 0.01
        diff = y[:, :3] - t
        loss = float(np.mean(diff * diff / den))
        dy = np.zeros_like(y)
        dy[:, :3] = 2.0 * diff / den / (3.0 * n)
        gW = [None] * 6
        gW[5] = dy.T @ acts[5]
        dx = dy @ self.W[5]
        for l in range(4, -1, -1):
            dz = dx * (acts[l + 1] > 0.0)
            gW[l] = dz.T @ acts[l]
            dx = dz @ self.W[l]
        gtable = np.zeros_like(self.table)
        for l, (idx, w) in enumerate(corners):
            for f in range(2):
                np.add.at(gtable[l, :, f], idx.reshape(-1), (w * dx[:, 2 * l + f][:, None]).reshape(-1))
        gw_flat = np.concatenate([g.reshape(-1) for g in gW])
        return loss, y, gw_flat, gtable.reshape(-1)
