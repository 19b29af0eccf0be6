"""Training data, training, hourly rollout and ensemble screening.

The surrogate maps the state at one hourly snapshot and the coming hour's
rainfall to the next snapshot's depth and the maximum depth reached in
between.  Training pairs come from the solver's own trajectories (batched
runs of seeded storms on one mesh); screening rolls the network out hour by
hour from a dry start, flags members it should not be trusted on, and the
plain solver re-runs the flagged members plus a random audit and scores the
surrogate on them.

Node inputs (12 features, padded to 64): depth, previous-snapshot depth and
window maximum (x10, m -> dm), bed relative to the mesh mean, Manning n
(x10), log cell area relative to its mean, characteristic length relative to
its mean, exterior-boundary flag, rain depth of the coming window and of the
last window (mm / 100), peak intensity of the coming window (mm/h / 100), and
the window length in hours.  Targets: 10 x (depth change) and 10 x (window
maximum above the new depth).
"""

from __future__ import annotations

import math
import time
from dataclasses import dataclass

import numpy as np

from . import ops
from .model import FIN, FOUT, MPNN, DualGraph

SCALE = 10.0


@dataclass
class Trajectory:
    times_s: np.ndarray     # snapshot times
    h: np.ndarray           # [n_snap, C]
    hmax: np.ndarray        # [n_snap, C] window maxima
    storm: object           # RainfallEvent
    duration_s: float


class MeshFeatures:
    """Static per-cell inputs and the dual graph of one mesh (device-resident)."""

    def __init__(self, topo, device: str = "cuda"):
        import torch

        self.topo = topo
        self.C = int(topo.cell_count)
        bed = np.asarray(topo.bed_elevation_m, np.float64)
        area = np.asarray(topo.cell_area_m2, np.float64)
        cl = np.asarray(topo.characteristic_length_m, np.float64)
        boundary = np.zeros(self.C, np.float32)
        right = np.asarray(topo.edge_right_cell)
        boundary[np.asarray(topo.edge_left_cell)[right < 0]] = 1.0
        st = np.zeros((self.C, FIN), np.float32)
        st[:, 3] = bed - bed.mean()
        st[:, 4] = 10.0 * np.asarray(topo.manning_n, np.float64)
        st[:, 5] = np.log(area) - np.log(area).mean()
        st[:, 6] = cl / cl.mean()
        st[:, 7] = boundary
        self.area = area.astype(np.float32)
        self.active = np.asarray(topo.active_mask) > 0 if topo.active_mask is not None else np.ones(self.C, bool)
        self.graph = DualGraph(topo, device)
        self.device = device
        self.static = torch.as_tensor(st, device=device)
        self.active_dev = torch.as_tensor(self.active, device=device)

    def inputs(self, h, h_prev, hmax, rain_next_mm, peak_next_mmhr, rain_prev_mm, window_h):
        """bf16 [C, 64] network inputs from device depth vectors and window scalars."""

        import torch

        x = self.static.clone()
        x[:, 0] = SCALE * h
        x[:, 1] = SCALE * h_prev
        x[:, 2] = SCALE * hmax
        x[:, 8] = rain_next_mm / 100.0
        x[:, 9] = rain_prev_mm / 100.0
        x[:, 10] = peak_next_mmhr / 100.0
        x[:, 11] = window_h
        return x.to(torch.bfloat16).contiguous()


def rain_window(event, t0_s: float, t1_s: float) -> tuple[float, float]:
    """(depth mm, peak intensity mm/h) of a hyetograph over [t0, t1)."""

    s = np.asarray(event.start_min, float) * 60.0
    e = np.asarray(event.end_min, float) * 60.0
    i = np.asarray(event.intensity_mmhr, float)
    ov = np.clip(np.minimum(e, t1_s) - np.maximum(s, t0_s), 0.0, None)
    depth = float(np.sum(i * ov / 3600.0))
    peak = float(i[ov > 0].max()) if np.any(ov > 0) else 0.0
    return depth, peak


def windows(duration_s: float) -> list[tuple[float, float]]:
    """Nominal hourly snapshot windows of a run: [0, 1 h), [1 h, 2 h), ..., [.., end)."""

    edges = [0.0] + [3600.0 * k for k in range(1, int(math.ceil(duration_s / 3600.0 - 1e-9)))] + [duration_s]
    return [(edges[k], edges[k + 1]) for k in range(len(edges) - 1)]


# ------------------------------------------------------------------ data
def solve_members(city, cfg, storms, durations_s, batch_size: int = 64, shape=None, device: str = "cuda"):
    """Solver trajectories (hourly snapshots + window maxima, kept on the
    device) of storms on one mesh, batched; returns (trajectories, solver
    seconds, scenario hours)."""

    import torch

    from ..batch import BatchSolver, Member

    out = []
    seconds = 0.0
    for k0 in range(0, len(storms), batch_size):
        members = [Member(city, storms[k], cfg, durations_s[k]) for k in range(k0, min(len(storms), k0 + batch_size))]
        with BatchSolver(members, shape=shape) as b:
            torch.cuda.synchronize()
            t = time.perf_counter()
            b.run()
            torch.cuda.synchronize()
            seconds += time.perf_counter() - t
            for j, m in enumerate(members):
                ts, h, hm = b.snapshots(j)
                out.append(Trajectory(ts, torch.as_tensor(h, device=device), torch.as_tensor(hm, device=device),
                                      m.rainfall, m.duration_s))
    return out, seconds, float(sum(durations_s)) / 3600.0


def transitions(tr: Trajectory):
    """Training windows of one trajectory: (snapshot j, rain next mm, peak
    mm/h, rain previous mm, window hours) for j -> j + 1.  Snapshot 0 is the
    state after the first step, snapshot k the first state at or after k
    hours, the last the end state."""

    out = []
    for j in range(len(tr.times_s) - 1):
        t0, t1 = float(tr.times_s[j]), float(tr.times_s[j + 1])
        rn, pk = rain_window(tr.storm, t0, t1)
        rp = rain_window(tr.storm, float(tr.times_s[j - 1]), t0)[0] if j > 0 else 0.0
        out.append((j, rn, pk, rp, (t1 - t0) / 3600.0))
    return out


def sample_tensors(mf: MeshFeatures, tr: Trajectory, w):
    """(inputs bf16 [C, 64], targets fp32 [C, 2]) of one training window."""

    import torch

    j, rn, pk, rp, wh = w
    h = tr.h[j]
    hp = tr.h[j - 1] if j > 0 else h
    hm = tr.hmax[j] if j > 0 else h
    x = mf.inputs(h, hp, hm, rn, pk, rp, wh)
    y = torch.stack([SCALE * (tr.h[j + 1] - h), SCALE * (tr.hmax[j + 1] - tr.h[j + 1])], dim=1).contiguous()
    return x, y


# ------------------------------------------------------------------ training
def train(model: MPNN, mf: MeshFeatures, trajectories, epochs: int = 10, lr: float = 1e-3, seed: int = 0,
          log=None, max_seconds: float | None = None):
    """Full-graph steps over every window of every trajectory; MSE on active cells."""

    import torch

    rng = np.random.default_rng(seed)
    g = mf.graph
    mask = mf.active_dev[:, None].float()
    n_act = float(mask.sum().item()) * 2.0
    samples = [(tr, w) for tr in trajectories for w in transitions(tr)]
    dy = torch.zeros(g.C, FOUT, device=mf.device)
    history = []
    steps = epochs * len(samples)
    k = 0
    t_start = time.perf_counter()
    for ep in range(epochs):
        total = torch.zeros((), device=mf.device)
        for i in rng.permutation(len(samples)):
            rate = lr * 0.5 * (1.0 + math.cos(math.pi * k / max(steps, 1)))  # cosine decay
            x, yt = sample_tensors(mf, *samples[i])
            y = model.forward(g, x)
            diff = (y[:, :2] - yt) * mask
            total += (diff * diff).sum() / n_act
            dy[:, :2] = diff * (2.0 / n_act)
            model.zero_grad()
            model.backward(g, x, dy)
            model.step(rate)
            k += 1
        history.append(float(total.item()) / len(samples))
        if log:
            log(f"epoch {ep}: loss {history[-1]:.5f}")
        if max_seconds is not None and time.perf_counter() - t_start > max_seconds:
            break
    ops.status()
    return history


# ------------------------------------------------------------------ inference
def rollout(model: MPNN, mf: MeshFeatures, storm, duration_s: float):
    """Hourly surrogate trajectory from a dry start, on the device:
    (window ends, h [n, C], hmax [n, C]) as host arrays."""

    import torch

    g = mf.graph
    act = mf.active_dev
    h = torch.zeros(mf.C, device=mf.device)
    hp, hm = h.clone(), h.clone()
    rp = 0.0
    ends, hs, hms = [], [], []
    for t0, t1 in windows(duration_s):
        rn, pk = rain_window(storm, t0, t1)
        y = model.forward(g, mf.inputs(h, hp, hm, rn, pk, rp, (t1 - t0) / 3600.0), train=False)
        hn = torch.clamp(h + y[:, 0] / SCALE, min=0.0) * act
        hmn = torch.maximum(hn + torch.clamp(y[:, 1], min=0.0) / SCALE, torch.maximum(h, hn)) * act
        ends.append(t1)
        hs.append(hn)
        hms.append(hmn)
        hp, h, hm, rp = h, hn, hmn, rn
    return np.asarray(ends), torch.stack(hs).cpu().numpy(), torch.stack(hms).cpu().numpy()


def rollout_batch(model: MPNN, mf: MeshFeatures, storms, durations_s, copies: int = 32):
    """Rollouts of many members, `copies` at a time in one forward pass over
    the replicated graph; same results as rollout() member by member."""

    import torch

    out = [None] * len(storms)
    graphs = {}
    # members of one forward pass run for the longest one's windows: group
    # members of equal window count so few passes are padding
    order = sorted(range(len(storms)), key=lambda i: (len(windows(durations_s[i])), i))
    for k0 in range(0, len(storms), copies):
        idx = order[k0:k0 + copies]
        B = len(idx)
        if B not in graphs:
            graphs[B] = mf.graph.replicate(B)
        g = graphs[B]
        static = mf.static.repeat(B, 1)
        act = mf.active_dev.repeat(B)
        wins = [windows(durations_s[i]) for i in idx]
        n_w = max(len(w) for w in wins)
        h = torch.zeros(B * mf.C, device=mf.device)
        hp, hm = h.clone(), h.clone()
        rp = np.zeros(B)
        hs, hms = [], []
        for w in range(n_w):
            sc = np.zeros((B, 5), np.float32)
            for b, i in enumerate(idx):
                t0, t1 = wins[b][min(w, len(wins[b]) - 1)]
                rn, pk = rain_window(storms[i], t0, t1) if w < len(wins[b]) else (0.0, 0.0)
                sc[b] = (rn / 100.0, rp[b] / 100.0, pk / 100.0, (t1 - t0) / 3600.0, rn)
            col = torch.as_tensor(sc, device=mf.device).repeat_interleave(mf.C, dim=0)
            x = static.clone()
            x[:, 0] = SCALE * h
            x[:, 1] = SCALE * hp
            x[:, 2] = SCALE * hm
            x[:, 8:12] = col[:, :4]
            y = model.forward(g, x.to(torch.bfloat16).contiguous(), train=False)
            hn = torch.clamp(h + y[:, 0] / SCALE, min=0.0) * act
            hmn = torch.maximum(hn + torch.clamp(y[:, 1], min=0.0) / SCALE, torch.maximum(h, hn)) * act
            hs.append(hn.view(B, mf.C))
            hms.append(hmn.view(B, mf.C))
            hp, h, hm, rp = h, hn, hmn, sc[:, 4]
        H = torch.stack(hs, 1).cpu().numpy()
        HM = torch.stack(hms, 1).cpu().numpy()
        for b, i in enumerate(idx):
            n = len(wins[b])
            out[i] = (np.asarray([w[1] for w in wins[b]]), H[b, :n], HM[b, :n])
    return out


# ------------------------------------------------------------------ scoring
def score(mf: MeshFeatures, pred, tr: Trajectory, threshold: float = 0.05) -> dict:
    """Surrogate vs solver over the member's hourly windows: depth and window
    maximum RMSE (m), flood-extent CSI of the max-depth envelope, and the
    final surface-volume error."""

    ends, hp, hmp = pred
    # solver snapshot k (k >= 1) closes window k - 1
    hs = tr.h[1:1 + len(ends)].cpu().numpy()
    hms = tr.hmax[1:1 + len(ends)].cpu().numpy()
    act = mf.active
    rm_h = float(np.sqrt(np.mean((hp[:, act] - hs[:, act]) ** 2)))
    rm_max = float(np.sqrt(np.mean((hmp[:, act] - hms[:, act]) ** 2)))
    env_p = hmp.max(0)[act] >= threshold
    env_s = hms.max(0)[act] >= threshold
    union = int((env_p | env_s).sum())
    csi = float((env_p & env_s).sum() / union) if union else 1.0
    vp = float(np.sum(hp[-1] * mf.area))
    vs = float(np.sum(hs[-1] * mf.area))
    return {"rmse_h_m": rm_h, "rmse_hmax_m": rm_max, "csi": csi, "volume_error": (vp - vs) / max(abs(vs), 1.0)}


def flags(mf: MeshFeatures, storm, pred, limits: dict) -> bool:
    """Members the surrogate should not be trusted on: storms outside the
    training range (peak or total depth), or a predicted envelope deeper than
    anything seen in training."""

    depth = float(np.sum(np.asarray(storm.intensity_mmhr) * (np.asarray(storm.end_min) - np.asarray(storm.start_min))) / 60.0)
    peak = float(np.max(storm.intensity_mmhr))
    deepest = float(pred[2].max())
    return peak > limits["peak_mmhr"] or depth > limits["depth_mm"] or deepest > limits["max_depth_m"]
