"""Training data, training, hourly rollout and ensemble screening.

The surrogate maps the state at one hourly snapshot and the coming hour's
rainfall to the next snapshot's state and the maximum depth reached in
between.  Training pairs come from the solver's own trajectories (batched
runs of seeded storms on one mesh); screening rolls an ensemble of networks
out hour by hour from a dry start, flags the members on which the networks
disagree beyond a threshold calibrated on held-out training storms, and the
plain solver re-runs the flagged members plus a random audit and scores the
surrogate on them.

Node inputs (12 features, padded to 64): depth h, momenta hu and hv, the
window maximum depth (all x10: m -> dm, m^2/s -> 0.1 m^2/s), bed relative to
the mesh mean, Manning n (x10), infiltration state (the fraction of the
Horton capacity above its floor, 1 - wet-time decay; 0 without
infiltration), exterior-boundary flag, rain depth of the coming and of the
last window (mm / 100), peak intensity of the coming window (mm/h / 100),
and the window length in hours.  Outputs: 10 x (depth change), 10 x (window
maximum above the new depth), 10 x the new hu and hv.
"""

from __future__ import annotations

import math
import time
from dataclasses import dataclass

import numpy as np

from . import ops
from .model import FIN, FOUT, MPNN, DualGraph

SCALE = 10.0
N_OUT = 4
THRESHOLD_M = 0.05


@dataclass
class Trajectory:
    times_s: np.ndarray     # snapshot times
    h: object               # [n_snap, C] device tensors
    hmax: object            # [n_snap, C] window maxima
    hu: object              # [n_snap, C]
    hv: object              # [n_snap, C]
    storm: object           # RainfallEvent
    duration_s: float


class MeshFeatures:
    """Static per-cell inputs and the dual graph of one mesh (device-resident)."""

    def __init__(self, topo, device: str = "cuda", infiltration_state=None):
        import torch

        self.topo = topo
        self.C = int(topo.cell_count)
        bed = np.asarray(topo.bed_elevation_m, np.float64)
        area = np.asarray(topo.cell_area_m2, np.float64)
        boundary = np.zeros(self.C, np.float32)
        right = np.asarray(topo.edge_right_cell)
        boundary[np.asarray(topo.edge_left_cell)[right < 0]] = 1.0
        st = np.zeros((self.C, FIN), np.float32)
        st[:, 4] = bed - bed.mean()
        st[:, 5] = 10.0 * np.asarray(topo.manning_n, np.float64)
        if infiltration_state is not None:
            st[:, 6] = np.asarray(infiltration_state, np.float32)
        st[:, 7] = boundary
        self.area = area.astype(np.float32)
        self.active = np.asarray(topo.active_mask) > 0 if topo.active_mask is not None else np.ones(self.C, bool)
        self.graph = DualGraph(topo, device)
        self.device = device
        self.static = torch.as_tensor(st, device=device)
        self.active_dev = torch.as_tensor(self.active, device=device)

    def inputs(self, h, hu, hv, hmax, rain_next_mm, peak_next_mmhr, rain_prev_mm, window_h):
        """bf16 [C, 64] network inputs from device state vectors and window scalars."""

        import torch

        x = self.static.clone()
        x[:, 0] = SCALE * h
        x[:, 1] = SCALE * hu
        x[:, 2] = SCALE * hv
        x[:, 3] = SCALE * hmax
        x[:, 8] = rain_next_mm / 100.0
        x[:, 9] = rain_prev_mm / 100.0
        x[:, 10] = peak_next_mmhr / 100.0
        x[:, 11] = window_h
        return x.to(torch.bfloat16).contiguous()


def advance(y, h, act):
    """The state after a window from the network outputs y [C, >=4] and the
    depth h at its start: (h, hmax, hu, hv), dry and inactive cells zeroed."""

    import torch

    hn = torch.clamp(h + y[:, 0] / SCALE, min=0.0) * act
    hmn = torch.maximum(hn + torch.clamp(y[:, 1], min=0.0) / SCALE, torch.maximum(h, hn)) * act
    wet = (hn > 1.0e-4) & act
    hun = torch.where(wet, y[:, 2] / SCALE, torch.zeros_like(hn))
    hvn = torch.where(wet, y[:, 3] / SCALE, torch.zeros_like(hn))
    return hn, hmn, hun, hvn


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
def solve_members(city, cfg, storms, durations_s, batch_size: int = 64, shape=None, device: str = "cuda",
                  stream=None):
    """Solver trajectories (hourly snapshots, window maxima and momenta, as
    tensors on `device`) of storms on one mesh, batched; returns (trajectories in
    the order of `storms`, solver seconds, scenario hours).  A batch runs
    until its longest member ends, so members go into batches longest storm
    first.  With `stream` the solver runs on that stream (and only it is
    synchronised), so other work can overlap it."""

    import torch

    from ..batch import BatchSolver, Member

    out = [None] * len(storms)
    seconds = 0.0
    sync = stream.synchronize if stream is not None else torch.cuda.synchronize
    order = sorted(range(len(storms)), key=lambda k: (-float(durations_s[k]), k))
    dev = lambda a: torch.as_tensor(a, device=device)  # noqa: E731
    for k0 in range(0, len(storms), batch_size):
        idx = order[k0:k0 + batch_size]
        members = [Member(city, storms[k], cfg, durations_s[k]) for k in idx]
        with BatchSolver(members, shape=shape) as b:
            sync()
            t = time.perf_counter()
            b.run(stream=stream)
            sync()
            seconds += time.perf_counter() - t
            for j, (k, m) in enumerate(zip(idx, members)):
                ts, h, hm, hu, hv = b.snapshots(j, momentum=True)
                out[k] = Trajectory(ts, dev(h), dev(hm), dev(hu), dev(hv), m.rainfall, m.duration_s)
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


def sample_tensors(mf: MeshFeatures, tr: Trajectory, w, state=None):
    """(inputs bf16 [C, 64], targets fp32 [C, 4], target depths for the loss
    weights [C, 2]) of one training window; `state` = (h, hu, hv, hmax) at its
    start replaces the solver's (the network's own prediction)."""

    import torch

    j, rn, pk, rp, wh = w
    if state is None:
        h, hu, hv = tr.h[j], tr.hu[j], tr.hv[j]
        hm = tr.hmax[j] if j > 0 else h
    else:
        h, hu, hv, hm = state
    x = mf.inputs(h, hu, hv, hm, rn, pk, rp, wh)
    y = torch.stack([SCALE * (tr.h[j + 1] - h), SCALE * (tr.hmax[j + 1] - tr.h[j + 1]), SCALE * tr.hu[j + 1],
                     SCALE * tr.hv[j + 1]], dim=1).contiguous()
    return x, y, torch.stack([tr.h[j + 1], tr.hmax[j + 1]], dim=1)


# ------------------------------------------------------------------ training
CHANNEL_WEIGHTS = (1.0, 1.0, 0.5, 0.5)


def loss_weights(mf: MeshFeatures, depths, extent_weight: float):
    """Per-cell, per-output loss weights: active cells; the depth and window
    maximum channels weigh cells near the 0.05 m extent threshold
    1 + extent_weight x exp(-((d - 0.05) / 0.025)^2) of their target depth d."""

    import torch

    act = mf.active_dev[:, None].float()
    w = torch.tensor(CHANNEL_WEIGHTS, device=mf.device)[None, :].repeat(mf.C, 1)
    if extent_weight > 0.0:
        near = 1.0 + extent_weight * torch.exp(-((depths - THRESHOLD_M) / 0.025) ** 2)
        w[:, :2] = w[:, :2] * near
    return w * act


def cosine(progress: float, t_start: float, max_seconds: float | None) -> float:
    """Cosine learning-rate factor at the larger of the step progress and,
    with a time budget, the fraction of it spent: training stopped by the
    budget ends with the rate decayed as if its last epoch were planned."""

    if max_seconds:
        progress = max(progress, (time.perf_counter() - t_start) / max_seconds)
    return 0.5 * (1.0 + math.cos(math.pi * min(progress, 1.0)))


def train(model: MPNN, mf: MeshFeatures, trajectories, epochs: int = 10, lr: float = 1e-3, seed: int = 0,
          log=None, max_seconds: float | None = None, extent_weight: float = 3.0, pushforward: float = 0.5,
          teacher: list | None = None, batch: int = 1):
    """Full-graph steps over every window of every trajectory; weighted MSE on
    active cells.  From the second epoch, a window after the first starts
    with probability `pushforward` from the network's own one-window
    prediction (from the solver's state a window earlier) instead of the
    solver's state, so the network learns to correct its own errors in a
    rollout.

    Returns the mean loss of each epoch over all its windows.  The first
    epoch has no pushforward windows, so that figure rises when they start;
    `teacher`, when given, receives each epoch's mean loss over the windows
    that started from the solver's state, which is comparable across
    epochs.  With `max_seconds` training stops when that much time is
    spent (within an epoch too), the cosine rate decaying over the budget.

    With batch > 1 every optimizer step takes `batch` windows in one pass
    over the replicated graph (the mean of their losses, each normalised by
    its own weights); the single-window step is launch-bound on a mesh of
    this size, so a batch costs little more than one window."""

    if batch > 1:
        return _train_batched(model, mf, trajectories, epochs, lr, seed, log, max_seconds, extent_weight,
                              pushforward, teacher, batch)

    import torch

    rng = np.random.default_rng(seed)
    g = mf.graph
    samples = [(tr, w) for tr in trajectories for w in transitions(tr)]
    dy = torch.zeros(g.C, FOUT, device=mf.device)
    act = mf.active_dev
    history = []
    steps = epochs * len(samples)
    k = 0
    t_start = time.perf_counter()
    for ep in range(epochs):
        total = torch.zeros((), device=mf.device)
        forced = torch.zeros((), device=mf.device)
        n_forced = n_done = 0
        for i in rng.permutation(len(samples)):
            if max_seconds is not None and time.perf_counter() - t_start > max_seconds:
                break
            rate = lr * cosine(k / max(steps, 1), t_start, max_seconds)
            tr, w = samples[i]
            state = None
            if ep > 0 and w[0] > 0 and rng.random() < pushforward:
                j = w[0] - 1
                xp, _, _ = sample_tensors(mf, tr, transitions(tr)[j])
                with torch.no_grad():
                    yp = model.forward(g, xp, train=False)
                    hn, hmn, hun, hvn = advance(yp, tr.h[j], act)
                state = (hn.clone(), hun.clone(), hvn.clone(), hmn.clone())
            x, yt, depths = sample_tensors(mf, tr, w, state)
            wts = loss_weights(mf, depths, extent_weight)
            norm = wts.sum()
            y = model.forward(g, x)
            diff = y[:, :N_OUT] - yt
            loss = (wts * diff * diff).sum() / norm
            total += loss
            if state is None:
                forced += loss
                n_forced += 1
            dy[:, :N_OUT] = wts * diff * (2.0 / norm)
            model.zero_grad()
            model.backward(g, x, dy)
            model.step(rate)
            k += 1
            n_done += 1
        if n_done == 0:
            break
        history.append(float(total.item()) / n_done)
        if teacher is not None:
            teacher.append(float(forced.item()) / max(n_forced, 1))
        if log:
            log(f"epoch {ep}: loss {history[-1]:.5f}")
        if max_seconds is not None and time.perf_counter() - t_start > max_seconds:
            break
    ops.status()
    return history


def _train_batched(model: MPNN, mf: MeshFeatures, trajectories, epochs, lr, seed, log, max_seconds, extent_weight,
                   pushforward, teacher, batch):
    import torch

    rng = np.random.default_rng(seed)
    C = mf.C
    samples = [(tr, w) for tr in trajectories for w in transitions(tr)]
    trans = {id(tr): transitions(tr) for tr in trajectories}
    act = mf.active_dev
    graphs, dys = {}, {}  # per batch size: the replicated graph and the output-gradient buffer

    def graph(b):
        if b not in graphs:
            graphs[b] = mf.graph.replicate(b)
            dys[b] = torch.zeros(b * C, FOUT, device=mf.device)
        return graphs[b], dys[b]

    history = []
    per_epoch = (len(samples) + batch - 1) // batch
    steps = epochs * per_epoch
    k = 0
    t_start = time.perf_counter()
    for ep in range(epochs):
        total = torch.zeros((), device=mf.device)
        forced = torch.zeros((), device=mf.device)
        n_forced = n_done = 0
        order = rng.permutation(len(samples))
        for b0 in range(0, len(samples), batch):
            if max_seconds is not None and time.perf_counter() - t_start > max_seconds:
                break
            idx = order[b0:b0 + batch]
            B = len(idx)
            rate = lr * cosine(k / max(steps, 1), t_start, max_seconds)
            push = [bool(ep > 0 and samples[i][1][0] > 0 and rng.random() < pushforward) for i in idx]
            states = [None] * B
            if any(push):
                # the network's own one-window predictions from the solver's
                # state a window earlier, in one pass at the batch's size (the
                # windows that start from the solver's state repeat a pushed one)
                src = [j if push[j] else push.index(True) for j in range(B)]
                xs = []
                for j in src:
                    tr, w = samples[idx[j]]
                    xs.append(sample_tensors(mf, tr, trans[id(tr)][w[0] - 1])[0])
                gp, _ = graph(B)
                with torch.no_grad():
                    yp = model.forward(gp, torch.cat(xs), train=False)
                    for j in range(B):
                        if push[j]:
                            tr, w = samples[idx[j]]
                            hn, hmn, hun, hvn = advance(yp[j * C:(j + 1) * C], tr.h[w[0] - 1], act)
                            states[j] = (hn.clone(), hun.clone(), hvn.clone(), hmn.clone())
            xs, ys, ws, norms = [], [], [], []
            for j in range(B):
                tr, w = samples[idx[j]]
                x, yt, depths = sample_tensors(mf, tr, w, states[j])
                wt = loss_weights(mf, depths, extent_weight)
                xs.append(x)
                ys.append(yt)
                ws.append(wt)
                norms.append(wt.sum())
            g, dy = graph(B)
            x = torch.cat(xs)
            wts = torch.cat(ws)
            norm = torch.stack(norms)
            y = model.forward(g, x)
            diff = y[:, :N_OUT] - torch.cat(ys)
            per = (wts * diff * diff).view(B, C, N_OUT).sum((1, 2)) / norm
            total += per.sum()
            keep = [j for j in range(B) if not push[j]]
            if keep:
                forced += per[keep].sum()
                n_forced += len(keep)
            scale = (2.0 / (norm * B)).repeat_interleave(C)[:, None]
            dy[:, :N_OUT] = wts * diff * scale
            model.zero_grad()
            model.backward(g, x, dy)
            model.step(rate)
            k += 1
            n_done += B
        if n_done == 0:
            break
        history.append(float(total.item()) / n_done)
        if teacher is not None:
            teacher.append(float(forced.item()) / max(n_forced, 1))
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
    hu, hv, hm = h.clone(), h.clone(), h.clone()
    rp = 0.0
    ends, hs, hms = [], [], []
    for t0, t1 in windows(duration_s):
        rn, pk = rain_window(storm, t0, t1)
        y = model.forward(g, mf.inputs(h, hu, hv, hm, rn, pk, rp, (t1 - t0) / 3600.0), train=False)
        hn, hmn, hun, hvn = advance(y, h, act)
        ends.append(t1)
        hs.append(hn)
        hms.append(hmn)
        h, hu, hv, hm, rp = hn, hun, hvn, hmn, rn
    return np.asarray(ends), torch.stack(hs).cpu().numpy(), torch.stack(hms).cpu().numpy()


def rollout_batch(model: MPNN, mf: MeshFeatures, storms, durations_s, copies: int = 32):
    """Rollouts of many members, `copies` at a time in one forward pass over
    the replicated graph; same results as rollout() member by member."""

    return ensemble_rollouts([model], mf, storms, durations_s, copies=copies)[0]


def ensemble_rollouts(models, mf: MeshFeatures, storms, durations_s, copies: int = 32):
    """Rollouts of every member by each network of an ensemble, `copies`
    members per forward pass over the replicated graph: (mean prediction
    (window ends, h [n, C], hmax [n, C]) per member as host arrays, and the
    disagreement per member = RMS over the member's windows, the networks and
    the active cells of the networks' window maxima about their mean).

    All networks advance the same members window by window, so the mean and
    the disagreement are formed on the device and only the mean comes back;
    members of one pass run for the longest one's windows, so members are
    grouped by window count and the padding windows are left out of the
    disagreement."""

    import torch

    out = [None] * len(storms)
    spread = np.zeros(len(storms))
    graphs = {}
    M = len(models)
    C = mf.C
    n_act = max(int(mf.active.sum()), 1)
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
        zero = torch.zeros(B * C, device=mf.device)
        states = [(zero, zero, zero, zero) for _ in range(M)]  # (h, hu, hv, hmax) per network
        rp = np.zeros(B)
        hs, hms = [], []
        d2 = torch.zeros(B, dtype=torch.float64, device=mf.device)
        for w in range(n_w):
            sc = np.zeros((B, 5), np.float32)
            live = np.zeros(B, np.float64)
            for b, i in enumerate(idx):
                t0, t1 = wins[b][min(w, len(wins[b]) - 1)]
                rn, pk = rain_window(storms[i], t0, t1) if w < len(wins[b]) else (0.0, 0.0)
                sc[b] = (rn / 100.0, rp[b] / 100.0, pk / 100.0, (t1 - t0) / 3600.0, rn)
                live[b] = 1.0 if w < len(wins[b]) else 0.0
            col = torch.as_tensor(sc, device=mf.device).repeat_interleave(C, dim=0)
            nxt = []
            for model, (h, hu, hv, hm) in zip(models, states):
                x = static.clone()
                x[:, 0] = SCALE * h
                x[:, 1] = SCALE * hu
                x[:, 2] = SCALE * hv
                x[:, 3] = SCALE * hm
                x[:, 8:12] = col[:, :4]
                y = model.forward(g, x.to(torch.bfloat16).contiguous(), train=False)
                hn, hmn, hun, hvn = advance(y, h, act)
                nxt.append((hn, hun, hvn, hmn))
            states = nxt
            h_mean = states[0][0] if M == 1 else sum(st[0] for st in states) / M
            hm_mean = states[0][3] if M == 1 else sum(st[3] for st in states) / M
            hs.append(h_mean.view(B, C))
            hms.append(hm_mean.view(B, C))
            if M > 1:
                dev2 = sum((st[3] - hm_mean) ** 2 for st in states).view(B, C)
                d2 += dev2.sum(1, dtype=torch.float64) * torch.as_tensor(live, device=mf.device)
            rp = sc[:, 4]
        H = torch.stack(hs, 1).cpu().numpy()
        HM = torch.stack(hms, 1).cpu().numpy()
        D2 = d2.cpu().numpy()
        for b, i in enumerate(idx):
            n = len(wins[b])
            out[i] = (np.asarray([w[1] for w in wins[b]]), H[b, :n], HM[b, :n])
            spread[i] = float(np.sqrt(D2[b] / (M * n * n_act))) if M > 1 else 0.0
    return out, spread


# ------------------------------------------------------------------ scoring
def score(mf: MeshFeatures, pred, tr: Trajectory, threshold: float = 0.05,
          extent_threshold: float | None = None) -> dict:
    """Surrogate vs solver over the member's hourly windows: depth and window
    maximum RMSE (m), flood-extent CSI of the max-depth envelopes (both at
    `threshold`), and the final surface-volume error; with
    `extent_threshold`, also "csi_calibrated": the surrogate's envelope at
    that depth against the solver's at `threshold`."""

    ends, hp, hmp = pred
    # solver snapshot k (k >= 1) closes window k - 1
    hs = tr.h[1:1 + len(ends)].cpu().numpy()
    hms = tr.hmax[1:1 + len(ends)].cpu().numpy()
    act = mf.active
    rm_h = float(np.sqrt(np.mean((hp[:, act] - hs[:, act]) ** 2)))
    rm_max = float(np.sqrt(np.mean((hmp[:, act] - hms[:, act]) ** 2)))
    env_p = hmp.max(0)[act]
    env_s = hms.max(0)[act] >= threshold
    vp = float(np.sum(hp[-1] * mf.area))
    vs = float(np.sum(hs[-1] * mf.area))
    out = {"rmse_h_m": rm_h, "rmse_hmax_m": rm_max, "csi": csi(env_p >= threshold, env_s),
           "volume_error": (vp - vs) / max(abs(vs), 1.0)}
    if extent_threshold is not None:
        out["csi_calibrated"] = csi(env_p >= extent_threshold, env_s)
    return out


def csi(pred: np.ndarray, truth: np.ndarray) -> float:
    """Critical success index hits / (hits + misses + false alarms) of two
    boolean extents; 1 when both are empty."""

    union = int((pred | truth).sum())
    return float((pred & truth).sum() / union) if union else 1.0


EXTENT_CANDIDATES_M = tuple(round(0.02 + 0.0025 * k, 4) for k in range(25))  # 0.02 .. 0.08 m


def calibrate_extent(mf: MeshFeatures, preds, trajectories, threshold: float = 0.05) -> dict:
    """Depth at which the surrogate's max-depth envelope best matches the
    solver's extent at `threshold`: the candidate (0.02-0.08 m) with the
    highest mean CSI over held-out training storms."""

    act = mf.active
    env_p, env_s = [], []
    for (ends, _, hmp), tr in zip(preds, trajectories):
        env_p.append(hmp.max(0)[act])
        env_s.append(tr.hmax[1:1 + len(ends)].cpu().numpy().max(0)[act] >= threshold)
    mean_csi = [float(np.mean([csi(p >= t, s) for p, s in zip(env_p, env_s)])) for t in EXTENT_CANDIDATES_M]
    best = int(np.argmax(mean_csi))
    at = EXTENT_CANDIDATES_M.index(threshold) if threshold in EXTENT_CANDIDATES_M else None
    return {"extent_threshold_m": EXTENT_CANDIDATES_M[best], "validation_csi_calibrated": mean_csi[best],
            "validation_csi_at_threshold": mean_csi[at] if at is not None else None}


def flags(spread: np.ndarray, threshold: float) -> np.ndarray:
    """Members the surrogate should not be trusted on: the networks of the
    ensemble disagree on the window maxima by more than `threshold` (RMS, m),
    a level calibrated on held-out training storms (calibrate_flags)."""

    return np.asarray(spread) > threshold


def calibrate_flags(spread: np.ndarray, errors: np.ndarray, flag_fraction: float = 0.04) -> dict:
    """Flag threshold from held-out training storms: the disagreement level
    above which the `flag_fraction` most uncertain members lie; also reports
    how well disagreement ranks the true window-maximum errors there."""

    spread = np.asarray(spread, np.float64)
    errors = np.asarray(errors, np.float64)
    thr = float(np.quantile(spread, 1.0 - flag_fraction)) if spread.size else float("inf")
    rank = lambda a: np.argsort(np.argsort(a))  # noqa: E731
    rho = float(np.corrcoef(rank(spread), rank(errors))[0, 1]) if spread.size > 2 else float("nan")
    sel = spread > thr
    return {"threshold_m": thr, "flag_fraction": flag_fraction, "spearman_spread_vs_error": rho,
            "validation_members": int(spread.size),
            "mean_error_flagged_m": float(errors[sel].mean()) if sel.any() else None,
            "mean_error_accepted_m": float(errors[~sel].mean()) if (~sel).any() else None}
