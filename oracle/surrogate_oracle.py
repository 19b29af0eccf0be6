"""CPU oracle of the surrogate network (test infrastructure only).

A NumPy restatement of floodgb.surrogate.model.MPNN: the same architecture,
the same points where values are rounded to bfloat16 (weights, GEMM inputs,
saved activations, back-propagated GEMM inputs) and fp32 everywhere else, so
the GPU's forward outputs and parameter gradients can be checked against it.
There is no reference counterpart (the reference ships no learned model);
the oracle is pinned by finite differences of its own loss.
"""

from __future__ import annotations

import numpy as np

H = 128
FIN = 64
FOUT = 64


ROUND = True  # False: plain fp32 (finite-difference check of the oracle itself)


def bf16(x) -> np.ndarray:
    """Round to the nearest bfloat16 (ties to even), returned as float32."""

    x = np.ascontiguousarray(x, dtype=np.float32)
    if not ROUND:
        return x
    u = x.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def relu(x):
    return np.maximum(x, 0.0).astype(np.float32)


class OracleMPNN:
    """Parameters as a list of (w [out, in], b [out]) in MPNN.layers() order:
    enc_n (2), enc_e (2), dec (2), then per layer edge (2) and node (2)."""

    def __init__(self, params, n_layers):
        self.p = [(np.asarray(w, np.float32), np.asarray(b, np.float32)) for w, b in params]
        self.L = n_layers

    def _dense(self, k):
        w, b = self.p[k]
        return bf16(w), b

    def idx(self, name, l=0, j=0):
        base = {"enc_n": 0, "enc_e": 2, "dec": 4}
        if name in base:
            return base[name] + j
        return 6 + 4 * l + (0 if name == "edge" else 2) + j

    def forward(self, x, ef, src, dst):
        C, E = x.shape[0], ef.shape[0]
        s = {}
        w, b = self._dense(self.idx("enc_n", j=0))
        s["x"] = bf16(x)
        s["zn"] = bf16(relu(s["x"] @ w.T + b))
        w, b = self._dense(self.idx("enc_n", j=1))
        h = (s["zn"] @ w.T + b).astype(np.float32)
        w, b = self._dense(self.idx("enc_e", j=0))
        s["ef"] = bf16(ef)
        s["ze"] = bf16(relu(s["ef"] @ w.T + b))
        w, b = self._dense(self.idx("enc_e", j=1))
        s["e"] = bf16(s["ze"] @ w.T + b)
        s["h"], s["z1e"], s["agg"], s["z1n"] = [], [], [], []
        for l in range(self.L):
            hb = bf16(h)
            s["h"].append(hb)
            cat = np.concatenate([hb[dst], hb[src], s["e"]], axis=1)
            w, b = self._dense(self.idx("edge", l, 0))
            z1e = bf16(relu(cat @ w.T + b))
            s["z1e"].append(z1e)
            w, b = self._dense(self.idx("edge", l, 1))
            m = (z1e @ w.T + b).astype(np.float32)
            agg = np.zeros((C, H), np.float32)
            np.add.at(agg, dst, m)
            aggb = bf16(agg)
            s["agg"].append(aggb)
            w, b = self._dense(self.idx("node", l, 0))
            z1n = bf16(relu(np.concatenate([hb, aggb], axis=1) @ w.T + b))
            s["z1n"].append(z1n)
            w, b = self._dense(self.idx("node", l, 1))
            h = (h + (z1n @ w.T + b)).astype(np.float32)
        s["hL"] = bf16(h)
        w, b = self._dense(self.idx("dec", j=0))
        s["zd"] = bf16(relu(s["hL"] @ w.T + b))
        w, b = self._dense(self.idx("dec", j=1))
        y = (s["zd"] @ w.T + b).astype(np.float32)
        self.saved = s
        return y

    def backward(self, dy, src, dst):
        s = self.saved
        C = dy.shape[0]
        grads = [None] * len(self.p)

        def put(k, dzb, x, dzf):
            grads[k] = ((dzb.T @ x).astype(np.float32), dzf.sum(0).astype(np.float32))

        k1, k2 = self.idx("dec", j=0), self.idx("dec", j=1)
        dyb = bf16(dy)
        put(k2, dyb, s["zd"], dy)
        d = (dyb @ bf16(self.p[k2][0])).astype(np.float32)
        d = np.where(s["zd"] > 0, d, 0.0).astype(np.float32)
        db = bf16(d)
        put(k1, db, s["hL"], d)
        dh = (db @ bf16(self.p[k1][0])).astype(np.float32)
        de = np.zeros_like(s["e"])
        for l in reversed(range(self.L)):
            e1, e2 = self.idx("edge", l, 0), self.idx("edge", l, 1)
            n1, n2 = self.idx("node", l, 0), self.idx("node", l, 1)
            dhb = bf16(dh)
            put(n2, dhb, s["z1n"][l], dh)
            d = (dhb @ bf16(self.p[n2][0])).astype(np.float32)
            d = np.where(s["z1n"][l] > 0, d, 0.0).astype(np.float32)
            db = bf16(d)
            put(n1, db, np.concatenate([s["h"][l], s["agg"][l]], axis=1), d)
            dx = (db @ bf16(self.p[n1][0])).astype(np.float32)
            dh_in = (dh + dx[:, :H]).astype(np.float32)
            dagg = dx[:, H:]
            daggb = bf16(dagg)
            dm = daggb[dst]
            grads[e2] = ((dm.T @ s["z1e"][l]).astype(np.float32), dagg[dst].sum(0).astype(np.float32))
            d = (dm @ bf16(self.p[e2][0])).astype(np.float32)
            d = np.where(s["z1e"][l] > 0, d, 0.0).astype(np.float32)
            db = bf16(d)
            cat = np.concatenate([s["h"][l][dst], s["h"][l][src], s["e"]], axis=1)
            put(e1, db, cat, d)
            dcat = (db @ bf16(self.p[e1][0])).astype(np.float32)
            np.add.at(dh_in, dst, dcat[:, :H])
            np.add.at(dh_in, src, dcat[:, H:2 * H])
            de += dcat[:, 2 * H:]
            dh = dh_in
        k1, k2 = self.idx("enc_n", j=0), self.idx("enc_n", j=1)
        dhb = bf16(dh)
        put(k2, dhb, s["zn"], dh)
        d = (dhb @ bf16(self.p[k2][0])).astype(np.float32)
        d = np.where(s["zn"] > 0, d, 0.0).astype(np.float32)
        put(k1, bf16(d), s["x"], d)
        k1, k2 = self.idx("enc_e", j=0), self.idx("enc_e", j=1)
        deb = bf16(de)
        put(k2, deb, s["ze"], de)
        d = (deb @ bf16(self.p[k2][0])).astype(np.float32)
        d = np.where(s["ze"] > 0, d, 0.0).astype(np.float32)
        put(k1, bf16(d), s["ef"], d)
        return grads
