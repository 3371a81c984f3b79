"""CPU statement of the learned surrogate (test infrastructure only: the
oracle libsdem_surrogate.so is compared with, never called by the product path).

The surrogate has no counterpart in the reference; this module restates the
library's contract (include/sdem_surrogate.h) in numpy:

- graph(): the neighbour graph of the uniform cell grid (edges j != i with
  |x_j - x_i|^2 < cutoff^2, CSR by receiver, senders ordered by neighbour
  cell dz, dy, dx = -1..1 then by index) and its bf16 edge features, found by
  brute force over all pairs, so the cell search is checked against a
  method that does not use it;
- node_features(): the bf16 node features;
- forward() / backward(): the network in float64 with the bf16 roundings at
  the points where the library stores bf16 (bf16=True), or exact float64
  (bf16=False, for finite-difference checks of backward itself).

Parity is unpinned: there is no reference implementation to pin it to; the
tests check this statement against finite differences and brute force.
"""
from __future__ import annotations

import numpy as np

from sdem_gb300.surrogate import (DCLIP, EDGE_IN, NODE_IN, OUT, OUT_USED, OVERLAP_GAIN, bf16_round,
                                  param_layout)


def _bf(x: np.ndarray, on: bool = True) -> np.ndarray:
    """float64 -> float32 -> bf16, returned as float64 (identity when off)."""
    if not on:
        return np.asarray(x, np.float64)
    return bf16_round(np.asarray(x, np.float64).astype(np.float32)).astype(np.float64)


def cells(posR: np.ndarray, lo, cell: float, dim) -> np.ndarray:
    """(n, 3) clamped cell coordinates: floor((x - lo)/cell) in [0, dim)."""
    out = np.zeros((posR.shape[0], 3), np.int64)
    for a in range(3):
        q = (posR[:, a] - lo[a]) / cell
        k = np.where(q >= 0.0, np.where(q < dim[a], np.floor(q), dim[a] - 1), 0)
        out[:, a] = k.astype(np.int64)
    return out


def graph(posR: np.ndarray, lo, cell: float, cutoff: float, scale: float, dim):
    """(row_off, dst, src, efeat (E, 16) float32 bf16 values)."""
    n = posR.shape[0]
    c = cells(posR, lo, cell, dim)
    rc2 = cutoff * cutoff
    ii, jj = [], []
    for i0 in range(0, n, 512):
        i1 = min(n, i0 + 512)
        ex = posR[None, :, 0] - posR[i0:i1, None, 0]
        ey = posR[None, :, 1] - posR[i0:i1, None, 1]
        ez = posR[None, :, 2] - posR[i0:i1, None, 2]
        d2 = ex * ex + ey * ey + ez * ez
        a, b = np.nonzero(d2 < rc2)
        keep = (a + i0) != b
        ii.append(a[keep] + i0)
        jj.append(b[keep])
    i = np.concatenate(ii) if ii else np.zeros(0, np.int64)
    j = np.concatenate(jj) if jj else np.zeros(0, np.int64)
    dc = c[j] - c[i]
    if dc.size and np.abs(dc).max() > 1:
        raise AssertionError("an edge spans more than one cell")
    rank = ((dc[:, 2] + 1) * 3 + (dc[:, 1] + 1)) * 3 + (dc[:, 0] + 1)
    order = np.lexsort((j, rank, i))
    i, j = i[order], j[order]
    row_off = np.zeros(n + 1, np.int64)
    row_off[1:] = np.cumsum(np.bincount(i, minlength=n))
    ex = posR[j, 0] - posR[i, 0]
    ey = posR[j, 1] - posR[i, 1]
    ez = posR[j, 2] - posR[i, 2]
    d = np.sqrt(ex * ex + ey * ey + ez * ez)
    ov = np.maximum(posR[i, 3] + posR[j, 3] - d, 0.0)
    f = np.zeros((len(i), EDGE_IN), np.float64)
    f[:, 0], f[:, 1], f[:, 2] = ex / scale, ey / scale, ez / scale
    f[:, 3] = d / scale
    f[:, 4] = OVERLAP_GAIN * ov / scale
    return row_off, i, j, _bf(f).astype(np.float32)


def node_features(posR, vel, omega, planes, scale: float, vscale: float) -> np.ndarray:
    """(n, 32) float32 bf16 values; vel (3, n, 3), planes (nw, 4)."""
    n = posR.shape[0]
    f = np.zeros((n, NODE_IN), np.float64)
    for fr in range(3):
        f[:, 3 * fr:3 * fr + 3] = vel[fr] / vscale
    r = posR[:, 3]
    f[:, 9:12] = omega * r[:, None] / vscale
    f[:, 12] = 2.0 * r / scale
    for w in range(min(5, planes.shape[0])):
        nx, ny, nz, d = planes[w]
        dist = nx * posR[:, 0] + ny * posR[:, 1] + nz * posR[:, 2] + d
        q = np.minimum(np.maximum(dist / scale, -DCLIP), DCLIP)
        f[:, 13 + w] = q / DCLIP
    return _bf(f).astype(np.float32)


class Net:
    """The network on a flat float32 parameter vector (layout of
    sdem_gb300.surrogate.param_layout)."""

    def __init__(self, params: np.ndarray, latent: int = 128, layers: int = 6, bf16: bool = True):
        self.p = np.asarray(params, np.float64)
        self.L, self.layers, self.bf16 = latent, layers, bf16
        self.lay = {name: (shape, off) for name, shape, off in param_layout(latent, layers)}

    def W(self, name):
        shape, off = self.lay[name]
        w = self.p[off:off + int(np.prod(shape))].reshape(shape)
        return _bf(w, self.bf16)

    def b(self, name):
        shape, off = self.lay[name]
        return self.p[off:off + shape[0]]

    def _lin(self, x, name):
        return x @ self.W(name).T + self.b(name[:-2] + "b" + name[-1])

    def forward(self, xn, efeat, dst, src, row_off):
        r = self.bf16
        n = xn.shape[0]
        s = {"xn": np.asarray(xn, np.float64), "xe": np.asarray(efeat, np.float64)}
        z = _bf(np.maximum(self._lin(s["xn"], "enc_n.w1"), 0.0), r)
        h = self._lin(z, "enc_n.w2")
        hb = _bf(h, r)
        ze = _bf(np.maximum(self._lin(s["xe"], "enc_e.w1"), 0.0), r)
        e = self._lin(ze, "enc_e.w2")
        eb = _bf(e, r)
        s.update(z_enc=z, ze_enc=ze, hb=[hb], eb=[eb], ze=[], zn=[], agg=[])
        for l in range(self.layers):
            x_in = np.concatenate([hb[dst], hb[src], eb], axis=1)
            zl = _bf(np.maximum(self._lin(x_in, f"edge{l}.w1"), 0.0), r)
            m = self._lin(zl, f"edge{l}.w2")
            e = e + m
            eb = _bf(e, r)
            agg = np.zeros((n, self.L))
            np.add.at(agg, dst, m)
            aggb = _bf(agg, r)
            zn = _bf(np.maximum(self._lin(np.concatenate([hb, aggb], axis=1), f"node{l}.w1"), 0.0), r)
            h = h + self._lin(zn, f"node{l}.w2")
            hb = _bf(h, r)
            s["ze"].append(zl)
            s["zn"].append(zn)
            s["agg"].append(aggb)
            s["hb"].append(hb)
            s["eb"].append(eb)
        zd = _bf(np.maximum(self._lin(hb, "dec.w1"), 0.0), r)
        y = self._lin(zd, "dec.w2")
        s["zd"] = zd
        self.s = s
        self.graph = (dst, src)
        return y

    def loss(self, y, target):
        n = y.shape[0]
        d = y[:, :OUT_USED] - target
        dy = np.zeros((n, OUT))
        dy[:, :OUT_USED] = 2.0 * d / (n * OUT_USED)
        return float((d * d).sum() / (n * OUT_USED)), dy

    def backward(self, dy) -> np.ndarray:
        r = self.bf16
        s = self.s
        dst, src = self.graph
        L = self.L
        n = dy.shape[0]
        E = len(dst)
        g = np.zeros_like(self.p)

        def add(name, val):
            shape, off = self.lay[name]
            g[off:off + val.size] += val.reshape(-1)

        dyb = _bf(dy, r)
        add("dec.w2", dyb.T @ s["zd"])
        add("dec.b2", dy.sum(0))
        dz = (dyb @ self.W("dec.w2")) * (s["zd"] > 0)
        dzb = _bf(dz, r)
        add("dec.w1", dzb.T @ s["hb"][-1])
        add("dec.b1", dz.sum(0))
        dh = dzb @ self.W("dec.w1")
        dhb = _bf(dh, r)
        de = np.zeros((E, L))
        for l in reversed(range(self.layers)):
            hb, eb = s["hb"][l], s["eb"][l]
            zn, ze, aggb = s["zn"][l], s["ze"][l], s["agg"][l]
            add(f"node{l}.w2", dhb.T @ zn)
            add(f"node{l}.b2", dh.sum(0))
            dz = (dhb @ self.W(f"node{l}.w2")) * (zn > 0)
            dzb = _bf(dz, r)
            add(f"node{l}.w1", dzb.T @ np.concatenate([hb, aggb], axis=1))
            add(f"node{l}.b1", dz.sum(0))
            din = dzb @ self.W(f"node{l}.w1")
            dh_prev = dh + din[:, :L]
            dm = de + din[dst, L:]
            dmb = _bf(dm, r)
            add(f"edge{l}.w2", dmb.T @ ze)
            add(f"edge{l}.b2", dm.sum(0))
            dze = (dmb @ self.W(f"edge{l}.w2")) * (ze > 0)
            dzeb = _bf(dze, r)
            add(f"edge{l}.w1", dzeb.T @ np.concatenate([hb[dst], hb[src], eb], axis=1))
            add(f"edge{l}.b1", dze.sum(0))
            din_e = dzeb @ self.W(f"edge{l}.w1")
            de = de + din_e[:, 2 * L:]
            np.add.at(dh_prev, dst, din_e[:, :L])
            np.add.at(dh_prev, src, din_e[:, L:2 * L])
            dh = dh_prev
            dhb = _bf(dh, r)
        add("enc_n.w2", dhb.T @ s["z_enc"])
        add("enc_n.b2", dh.sum(0))
        dz = (dhb @ self.W("enc_n.w2")) * (s["z_enc"] > 0)
        dzb = _bf(dz, r)
        add("enc_n.w1", dzb.T @ s["xn"])
        add("enc_n.b1", dz.sum(0))
        deb = _bf(de, r)
        add("enc_e.w2", deb.T @ s["ze_enc"])
        add("enc_e.b2", de.sum(0))
        dze = (deb @ self.W("enc_e.w2")) * (s["ze_enc"] > 0)
        dzeb = _bf(dze, r)
        add("enc_e.w1", dzeb.T @ s["xe"])
        add("enc_e.b1", dze.sum(0))
        return g
