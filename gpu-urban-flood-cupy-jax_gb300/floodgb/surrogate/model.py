"""Mesh message-passing network on the triangle dual graph.

Architecture (hidden width H = 128, every MLP Linear-ReLU-Linear):
  node encoder  x (12 features, padded to 64) -> h0
  edge encoder  e (4 features, padded to 64)  -> e
  8 processor layers, each
      m_ij = MLP_e([h_i, h_j, e_ij])         messages on directed dual edges j -> i
      a_i  = sum_j m_ij                       fixed-order CSR sum at the receiving cell
      h_i <- h_i + MLP_n([h_i, a_i])          residual node update
  decoder       h -> 64 outputs (two used: next-hour depth change, hour max above it)

Every dense product runs on the tcgen05 GEMM (bf16 operands, fp32
accumulation in TMEM); the concatenated edge-MLP input is gathered inside the
GEMM.  The backward pass is written out by hand: dX = dZ W on the GEMM with
the transposed weight copy, dW = dZ^T X as a split-K GEMM over rows of
transposed bf16 copies, bias gradients as column sums, input gradients
scattered back to cells with fixed-order CSR sums.  Weights are fp32 masters
updated by Adam, with bf16 copies (and transposes) refreshed by the same
kernel.  PyTorch only allocates the device tensors.
"""

from __future__ import annotations

import math

import numpy as np

from . import ops

H = 128
FIN = 64
FOUT = 64
N_NODE_FEATURES = 12
N_EDGE_FEATURES = 4


def round64(x: int) -> int:
    return (int(x) + 63) // 64 * 64


class DualGraph:
    """Directed dual graph of a triangle mesh: one edge per direction of every
    interior mesh edge, sorted by receiving cell (then sending cell)."""

    def __init__(self, topo, device: str = "cuda"):
        import torch

        left = np.asarray(topo.edge_left_cell, np.int64)
        right = np.asarray(topo.edge_right_cell, np.int64)
        inner = right >= 0
        l, r = left[inner], right[inner]
        nx = np.asarray(topo.edge_normal_x, np.float32)[inner]
        ny = np.asarray(topo.edge_normal_y, np.float32)[inner]
        ln = np.asarray(topo.edge_length_m, np.float32)[inner]
        src = np.concatenate([l, r])
        dst = np.concatenate([r, l])
        # unit vector from the sending to the receiving cell (the edge normal points left -> right)
        ux = np.concatenate([nx, -nx])
        uy = np.concatenate([ny, -ny])
        lens = np.concatenate([ln, ln])
        order = np.lexsort((src, dst))
        self.C = int(topo.cell_count)
        self.E = int(src.size)
        self.src_h = src[order].astype(np.int32)
        self.dst_h = dst[order].astype(np.int32)
        recv_start = np.zeros(self.C + 1, np.int64)
        np.add.at(recv_start, self.dst_h.astype(np.int64) + 1, 1)
        recv_start = np.cumsum(recv_start)
        send_order = np.argsort(self.src_h, kind="stable").astype(np.int32)
        send_start = np.zeros(self.C + 1, np.int64)
        np.add.at(send_start, self.src_h.astype(np.int64) + 1, 1)
        send_start = np.cumsum(send_start)
        bed = np.asarray(topo.bed_elevation_m, np.float32)
        mean_len = float(lens.mean()) if lens.size else 1.0
        ef = np.zeros((self.E, FIN), np.float32)
        ef[:, 0] = ux[order]
        ef[:, 1] = uy[order]
        ef[:, 2] = lens[order] / mean_len
        ef[:, 3] = bed[self.dst_h] - bed[self.src_h]
        self.edge_features_h = ef
        self.indeg_h = np.diff(recv_start).astype(np.float32)
        t = lambda a, dt: torch.as_tensor(a, dtype=dt, device=device).contiguous()  # noqa: E731
        self.src = t(self.src_h, torch.int32)
        self.dst = t(self.dst_h, torch.int32)
        self.recv_start = t(recv_start.astype(np.int32), torch.int32)
        self.send_order = t(send_order, torch.int32)
        self.send_start = t(send_start.astype(np.int32), torch.int32)
        self.row_start = t(np.arange(self.E + 1, dtype=np.int32), torch.int32)  # identity segments (row copies)
        self.indeg = t(self.indeg_h, torch.float32)
        self.ef_bf = t(ef, torch.float32).to(torch.bfloat16).contiguous()

    def replicate(self, copies: int) -> "DualGraph":
        """The disjoint union of `copies` copies of this graph (cell c of copy k
        is cell k * C + c): many members of an ensemble in one forward pass."""

        import torch

        g = DualGraph.__new__(DualGraph)
        C, E, k = self.C, self.E, int(copies)
        off_c = (np.arange(k, dtype=np.int64) * C)[:, None]
        off_e = (np.arange(k, dtype=np.int64) * E)[:, None]
        g.C, g.E = C * k, E * k
        g.src_h = (self.src_h[None, :] + off_c).reshape(-1).astype(np.int32)
        g.dst_h = (self.dst_h[None, :] + off_c).reshape(-1).astype(np.int32)
        rs = self.recv_start.cpu().numpy().astype(np.int64)
        ss = self.send_start.cpu().numpy().astype(np.int64)
        so = self.send_order.cpu().numpy().astype(np.int64)
        recv = np.concatenate([(rs[:-1][None, :] + off_e).reshape(-1), [E * k]])
        send = np.concatenate([(ss[:-1][None, :] + off_e).reshape(-1), [E * k]])
        order = (so[None, :] + off_e).reshape(-1)
        g.edge_features_h = np.tile(self.edge_features_h, (k, 1))
        g.indeg_h = np.tile(self.indeg_h, k)
        dev = self.src.device
        t = lambda a, dt: torch.as_tensor(a, dtype=dt, device=dev).contiguous()  # noqa: E731
        g.src, g.dst = t(g.src_h, torch.int32), t(g.dst_h, torch.int32)
        g.recv_start = t(recv.astype(np.int32), torch.int32)
        g.send_order = t(order.astype(np.int32), torch.int32)
        g.send_start = t(send.astype(np.int32), torch.int32)
        g.row_start = t(np.arange(g.E + 1, dtype=np.int32), torch.int32)
        g.indeg = t(g.indeg_h, torch.float32)
        g.ef_bf = self.ef_bf.repeat(k, 1).contiguous()
        return g


class Dense:
    """One linear layer: fp32 master weights, bf16 copy and transpose, Adam state."""

    def __init__(self, n_out: int, n_in: int, rng: np.random.Generator, device: str = "cuda", n_in_real=None):
        import torch

        fan_in = n_in_real if n_in_real is not None else n_in
        w = np.zeros((n_out, n_in), np.float32)
        w[:, :fan_in] = rng.normal(0.0, math.sqrt(2.0 / fan_in), size=(n_out, fan_in)).astype(np.float32)
        z = lambda *s: torch.zeros(*s, device=device, dtype=torch.float32)  # noqa: E731
        self.w = torch.as_tensor(w, device=device)
        self.b = z(n_out)
        self.gw, self.gb = z(n_out, n_in), z(n_out)
        self.m1w, self.m2w, self.m1b, self.m2b = z(n_out, n_in), z(n_out, n_in), z(1, n_out), z(1, n_out)
        self.w_bf = self.w.to(torch.bfloat16).contiguous()
        self.wt_bf = self.w.t().contiguous().to(torch.bfloat16).contiguous()
        self.n_out, self.n_in = n_out, n_in

    def zero_grad(self):
        self.gw.zero_()
        self.gb.zero_()

    def step(self, lr: float, t: int, weight_decay: float = 0.0):
        ops.adam(self.w, self.m1w, self.m2w, self.gw, lr, t, weight_decay=weight_decay, w_bf16=self.w_bf,
                 wt_bf16=self.wt_bf)
        ops.adam(self.b.view(1, -1), self.m1b, self.m2b, self.gb.view(1, -1), lr, t)

    def state(self) -> dict:
        return {"w": self.w.cpu().numpy(), "b": self.b.cpu().numpy()}

    def load(self, st: dict):
        import torch

        self.w.copy_(torch.as_tensor(st["w"]))
        self.b.copy_(torch.as_tensor(st["b"]))
        self.w_bf.copy_(self.w.to(torch.bfloat16))
        self.wt_bf.copy_(self.w.t().to(torch.bfloat16))


class Workspace:
    """Activations of the forward pass for one graph size; for training also
    every layer's saved activations and the backward scratch."""

    def __init__(self, C: int, E: int, n_layers: int, train: bool = True, device: str = "cuda"):
        import torch

        bf = lambda *s: torch.empty(*s, device=device, dtype=torch.bfloat16)  # noqa: E731
        f32 = lambda *s: torch.empty(*s, device=device, dtype=torch.float32)  # noqa: E731
        self.C, self.E, self.train = C, E, train
        keep = n_layers if train else 1  # inference reuses one set of layer buffers
        self.zn, self.ze, self.e_bf = bf(C, H), bf(E, H), bf(E, H)
        self.h_bf = [bf(C, H) for _ in range(n_layers + 1 if train else 2)]
        self.h_f32 = [f32(C, H), f32(C, H)]
        self.z1e = [bf(E, H) for _ in range(keep)]
        self.agg_bf = [bf(C, H) for _ in range(keep)]
        self.z1n = [bf(C, H) for _ in range(keep)]
        self.zd = bf(C, H)
        self.y = f32(C, FOUT)
        self.m_f32 = f32(E, H)
        if not train:
            return
        # backward scratch
        self.dz_bf_e = bf(E, H)
        self.dzf_e = f32(E, H)
        self.dcat = f32(E, 3 * H)
        self.de = f32(E, H)
        self.dh = [f32(C, H), f32(C, H)]
        self.dx_c = f32(C, 2 * H)
        self.dz_bf_c, self.dzf_c = bf(C, H), f32(C, H)
        self.dagg_bf = bf(C, H)
        self.dy_bf = bf(C, FOUT)
        Mp = round64(max(C, E))
        self.tA = bf(H, Mp)          # dZ^T
        self.tB = bf(3 * H, Mp)      # X^T
        self.cs_scratch = f32(256 * 3 * H * H)
        self.part = f32(512 * H * 3 * H)


class MPNN:
    def __init__(self, n_layers: int = 8, seed: int = 0, device: str = "cuda"):
        rng = np.random.default_rng(seed)
        self.n_layers = n_layers
        self.device = device
        mk = lambda o, i, real=None: Dense(o, i, rng, device, real)  # noqa: E731
        self.enc_n = [mk(H, FIN, N_NODE_FEATURES), mk(H, H)]
        self.enc_e = [mk(H, FIN, N_EDGE_FEATURES), mk(H, H)]
        self.edge = [[mk(H, 3 * H), mk(H, H)] for _ in range(n_layers)]
        self.node = [[mk(H, 2 * H), mk(H, H)] for _ in range(n_layers)]
        self.dec = [mk(H, H), mk(FOUT, H)]
        for d in (self.edge + self.node):
            d[1].w.mul_(0.1)  # small residual updates at start
            d[1].load(d[1].state())
        self.dec[1].w.mul_(0.1)
        self.dec[1].load(self.dec[1].state())
        self.ws = None
        self._ws = {}
        self.t = 0

    def layers(self):
        out = list(self.enc_n) + list(self.enc_e) + list(self.dec)
        for a, b in zip(self.edge, self.node):
            out += list(a) + list(b)
        return out

    def workspace(self, g: DualGraph, train: bool) -> Workspace:
        key = (g.C, g.E, train)
        if key not in self._ws:
            self._ws[key] = Workspace(g.C, g.E, self.n_layers, train, self.device)
        self.ws = self._ws[key]
        return self.ws

    # -------------------------------------------------------------- forward
    def forward(self, g: DualGraph, x_bf, train: bool = True):
        """x_bf: bf16 [C, 64] node inputs; returns fp32 [C, 64] outputs (view
        into the workspace).  train=False keeps no activations for backward."""

        ws = self.workspace(g, train)
        C, E = g.C, g.E
        a, b = self.enc_n
        ops.gemm([(x_bf, None, FIN)], a.w_bf, bias=a.b, out_bf16=ws.zn, relu=True)
        ops.gemm([(ws.zn, None, H)], b.w_bf, bias=b.b, out_f32=ws.h_f32[0], out_bf16=ws.h_bf[0])
        a, b = self.enc_e
        ops.gemm([(g.ef_bf, None, FIN)], a.w_bf, bias=a.b, out_bf16=ws.ze, relu=True)
        ops.gemm([(ws.ze, None, H)], b.w_bf, bias=b.b, out_bf16=ws.e_bf)
        cur = 0
        nh = len(ws.h_bf)
        for l in range(self.n_layers):
            e1, e2 = self.edge[l]
            n1, n2 = self.node[l]
            k = l if train else 0
            hb = ws.h_bf[l % nh]
            ops.gemm([(hb, g.dst, H), (hb, g.src, H), (ws.e_bf, None, H)], e1.w_bf, bias=e1.b, out_bf16=ws.z1e[k],
                     relu=True)
            ops.gemm([(ws.z1e[k], None, H)], e2.w_bf, bias=e2.b, out_f32=ws.m_f32)
            # aggregation, written as bf16 only: both the next GEMM and backward read that copy
            ops.segment_sum(ws.m_f32, 0, g.recv_start, None, C, H, None, dst_bf16=ws.agg_bf[k])
            ops.gemm([(hb, None, H), (ws.agg_bf[k], None, H)], n1.w_bf, bias=n1.b, out_bf16=ws.z1n[k], relu=True)
            ops.gemm([(ws.z1n[k], None, H)], n2.w_bf, bias=n2.b, residual=ws.h_f32[cur], out_f32=ws.h_f32[cur ^ 1],
                     out_bf16=ws.h_bf[(l + 1) % nh])
            cur ^= 1
        a, b = self.dec
        ops.gemm([(ws.h_bf[self.n_layers % nh], None, H)], a.w_bf, bias=a.b, out_bf16=ws.zd, relu=True)
        ops.gemm([(ws.zd, None, H)], b.w_bf, bias=b.b, out_f32=ws.y)
        return ws.y

    # -------------------------------------------------------------- backward
    def _wgrad(self, dense: Dense, dz_segments, x_segments, m: int):
        """dense.gw += dZ^T X over m rows (split-K GEMM over transposed copies)."""

        ws = self.ws
        mp = round64(m)
        n_out, n_in = dense.n_out, dense.n_in
        tA = ws.tA[:n_out, :mp]
        tB = ws.tB[:n_in, :mp]
        ops.transpose(dz_segments, m, tA)
        ops.transpose(x_segments, m, tB)
        chunks = mp // 64
        tiles = (n_in + 127) // 128
        splits = max(1, min(chunks, 512, (4 * 152) // tiles))
        per = -(-chunks // splits)
        splits = -(-chunks // per)
        part = ws.part[: splits * n_out * n_in].view(splits, n_out, n_in)
        ops.gemm([(tA, None, mp)], tB, out_f32=part, k_splits=splits)
        ops.colsum(part.view(splits, n_out * n_in), splits, n_out * n_in, ws.cs_scratch, dense.gw.view(-1),
                   accumulate=True)

    def _bgrad(self, dense: Dense, dz_f32, m: int):
        ops.colsum(dz_f32, m, dense.n_out, self.ws.cs_scratch, dense.gb, accumulate=True)

    def backward(self, g: DualGraph, x_bf, dy):
        """Accumulate parameter gradients for dLoss/dy (fp32 [C, 64])."""

        ws = self.ws
        C, E, L = g.C, g.E, self.n_layers
        # decoder
        a, b = self.dec
        ops.cast_bf16(dy, ws.dy_bf)
        self._wgrad(b, [(ws.dy_bf, None, FOUT)], [(ws.zd, None, H)], C)
        self._bgrad(b, dy, C)
        ops.gemm([(ws.dy_bf, None, FOUT)], b.wt_bf, out_f32=ws.dzf_c)
        ops.relu_bwd(ws.dzf_c, ws.zd, ws.dz_bf_c, ws.dzf_c)
        self._wgrad(a, [(ws.dz_bf_c, None, H)], [(ws.h_bf[L], None, H)], C)
        self._bgrad(a, ws.dzf_c, C)
        dh = ws.dh[0]
        ops.gemm([(ws.dz_bf_c, None, H)], a.wt_bf, out_f32=dh)
        ws.de.zero_()
        cur = 0
        for l in reversed(range(L)):
            e1, e2 = self.edge[l]
            n1, n2 = self.node[l]
            dh = ws.dh[cur]
            # node update h' = h + n2(relu(n1([h, agg])))
            ops.cast_bf16(dh, ws.dz_bf_c)
            self._wgrad(n2, [(ws.dz_bf_c, None, H)], [(ws.z1n[l], None, H)], C)
            self._bgrad(n2, dh, C)
            ops.gemm([(ws.dz_bf_c, None, H)], n2.wt_bf, out_f32=ws.dzf_c)
            ops.relu_bwd(ws.dzf_c, ws.z1n[l], ws.dz_bf_c, ws.dzf_c)
            self._wgrad(n1, [(ws.dz_bf_c, None, H)], [(ws.h_bf[l], None, H), (ws.agg_bf[l], None, H)], C)
            self._bgrad(n1, ws.dzf_c, C)
            ops.gemm([(ws.dz_bf_c, None, H)], n1.wt_bf, out_f32=ws.dx_c)
            dh_in = ws.dh[cur ^ 1]
            dh_in.copy_(dh)
            dh_in.add_(ws.dx_c[:, :H])
            # messages: agg_i = sum_j m_ij, so dm_e = dagg[dst(e)] (gathered inside the GEMMs)
            dagg = ws.dx_c[:, H:]
            ops.cast_bf16(dagg, ws.dagg_bf)
            self._wgrad(e2, [(ws.dagg_bf, g.dst, H)], [(ws.z1e[l], None, H)], E)
            e2.gb.add_((dagg * g.indeg[:, None]).sum(0))
            ops.gemm([(ws.dagg_bf, g.dst, H)], e2.wt_bf, out_f32=ws.dzf_e)
            ops.relu_bwd(ws.dzf_e, ws.z1e[l], ws.dz_bf_e, ws.dzf_e)
            hb = ws.h_bf[l]
            self._wgrad(e1, [(ws.dz_bf_e, None, H)], [(hb, g.dst, H), (hb, g.src, H), (ws.e_bf, None, H)], E)
            self._bgrad(e1, ws.dzf_e, E)
            ops.gemm([(ws.dz_bf_e, None, H)], e1.wt_bf, out_f32=ws.dcat)
            ops.segment_sum(ws.dcat, 0, g.recv_start, None, C, H, dh_in, accumulate=True)
            ops.segment_sum(ws.dcat, H, g.send_start, g.send_order, C, H, dh_in, accumulate=True)
            ops.segment_sum(ws.dcat, 2 * H, g.row_start, None, E, H, ws.de, accumulate=True)
            cur ^= 1
        dh = ws.dh[cur]
        # encoders
        a, b = self.enc_n
        ops.cast_bf16(dh, ws.dz_bf_c)
        self._wgrad(b, [(ws.dz_bf_c, None, H)], [(ws.zn, None, H)], C)
        self._bgrad(b, dh, C)
        ops.gemm([(ws.dz_bf_c, None, H)], b.wt_bf, out_f32=ws.dzf_c)
        ops.relu_bwd(ws.dzf_c, ws.zn, ws.dz_bf_c, ws.dzf_c)
        self._wgrad(a, [(ws.dz_bf_c, None, H)], [(x_bf, None, FIN)], C)
        self._bgrad(a, ws.dzf_c, C)
        a, b = self.enc_e
        ops.cast_bf16(ws.de, ws.dz_bf_e)
        self._wgrad(b, [(ws.dz_bf_e, None, H)], [(ws.ze, None, H)], E)
        self._bgrad(b, ws.de, E)
        ops.gemm([(ws.dz_bf_e, None, H)], b.wt_bf, out_f32=ws.dzf_e)
        ops.relu_bwd(ws.dzf_e, ws.ze, ws.dz_bf_e, ws.dzf_e)
        self._wgrad(a, [(ws.dz_bf_e, None, H)], [(g.ef_bf, None, FIN)], E)
        self._bgrad(a, ws.dzf_e, E)

    def zero_grad(self):
        for d in self.layers():
            d.zero_grad()

    def step(self, lr: float, weight_decay: float = 0.0):
        self.t += 1
        for d in self.layers():
            d.step(lr, self.t, weight_decay)

    def state(self) -> list:
        return [d.state() for d in self.layers()]

    def load(self, st: list):
        for d, s in zip(self.layers(), st):
            d.load(s)
