"""Learned surrogate: the CPU oracle pinned by finite differences, and the GPU
network (tcgen05 GEMMs + message-passing kernels) checked against the oracle
in its forward outputs and every parameter gradient."""

import numpy as np
import pytest

import surrogate_oracle as SO


def random_graph(rng, C=24, E=70):
    src = rng.integers(0, C, E).astype(np.int64)
    dst = rng.integers(0, C, E).astype(np.int64)
    return src, dst


def random_params(rng, n_layers, scale=0.3):
    shapes = [(SO.H, SO.FIN), (SO.H, SO.H), (SO.H, SO.FIN), (SO.H, SO.H), (SO.H, SO.H), (SO.FOUT, SO.H)]
    for _ in range(n_layers):
        shapes += [(SO.H, 3 * SO.H), (SO.H, SO.H), (SO.H, 2 * SO.H), (SO.H, SO.H)]
    return [(rng.normal(0, scale / np.sqrt(i), (o, i)).astype(np.float32), rng.normal(0, 0.1, o).astype(np.float32))
            for o, i in shapes]


def test_oracle_gradients_match_finite_differences(monkeypatch):
    monkeypatch.setattr(SO, "ROUND", False)
    rng = np.random.default_rng(0)
    C, E, L = 10, 26, 1
    src, dst = random_graph(rng, C, E)
    x = rng.normal(size=(C, SO.FIN)).astype(np.float32)
    ef = rng.normal(size=(E, SO.FIN)).astype(np.float32)
    params = random_params(rng, L)
    net = SO.OracleMPNN(params, L)
    y = net.forward(x, ef, src, dst)
    grads = net.backward(y.copy(), src, dst)  # loss = 0.5 * sum(y^2)

    def loss(p):
        n = SO.OracleMPNN(p, L)
        return 0.5 * float(np.sum(n.forward(x, ef, src, dst).astype(np.float64) ** 2))

    for k in [0, 3, 5, 6, 7, 8, 9]:
        w, b = params[k]
        for _ in range(3):
            i, j = rng.integers(w.shape[0]), rng.integers(w.shape[1])
            eps = 1e-2
            wp = w.copy(); wp[i, j] += eps
            wm = w.copy(); wm[i, j] -= eps
            pp = list(params); pp[k] = (wp, b)
            pm = list(params); pm[k] = (wm, b)
            fd = (loss(pp) - loss(pm)) / (2 * eps)
            an = float(grads[k][0][i, j])
            assert abs(fd - an) <= 2e-2 * max(1.0, abs(fd)), (k, i, j, fd, an)
        i = rng.integers(b.shape[0])
        bp = b.copy(); bp[i] += 1e-2
        bm = b.copy(); bm[i] -= 1e-2
        pp = list(params); pp[k] = (w, bp)
        pm = list(params); pm[k] = (w, bm)
        fd = (loss(pp) - loss(pm)) / 2e-2
        assert abs(fd - float(grads[k][1][i])) <= 2e-2 * max(1.0, abs(fd))


@pytest.mark.gpu
def test_gpu_network_matches_oracle_forward_and_gradients():
    torch = pytest.importorskip("torch")
    from floodgb import native
    from floodgb.build import build_library
    from floodgb.surrogate.model import MPNN, DualGraph
    from floodgb.synthetic import make_grid_city

    build_library()
    native.load()
    if native.device_count() < 1:
        pytest.skip("no CUDA device")
    sc = make_grid_city(n=9, size_m=90.0, seed=4)
    topo = sc.city.topologies.surface_topology
    g = DualGraph(topo)
    L = 2
    net = MPNN(n_layers=L, seed=3)
    rng = np.random.default_rng(1)
    # perturb biases so every path is exercised
    for d in net.layers():
        d.b.copy_(torch.as_tensor(rng.normal(0, 0.05, d.b.shape[0]).astype(np.float32)))
    x = np.zeros((g.C, SO.FIN), np.float32)
    x[:, :12] = rng.normal(size=(g.C, 12))
    x_bf = torch.as_tensor(x, device="cuda").to(torch.bfloat16).contiguous()
    y = net.forward(g, x_bf).clone()
    dy = torch.zeros_like(y)
    dy[:, :2] = y[:, :2] / g.C
    net.zero_grad()
    net.backward(g, x_bf, dy)
    torch.cuda.synchronize()
    from floodgb.surrogate import ops

    ops.status()
    params = [(d.w.cpu().numpy(), d.b.cpu().numpy()) for d in net.layers()]
    oracle = SO.OracleMPNN(params, L)
    yo = oracle.forward(x, g.edge_features_h, g.src_h.astype(np.int64), g.dst_h.astype(np.int64))
    yg = y.cpu().numpy()
    rel = np.linalg.norm(yg - yo) / np.linalg.norm(yo)
    assert rel < 1e-2, rel
    dyo = np.zeros_like(yo)
    dyo[:, :2] = yg[:, :2] / g.C  # the same upstream gradient
    go = oracle.backward(dyo, g.src_h.astype(np.int64), g.dst_h.astype(np.int64))
    for k, d in enumerate(net.layers()):
        for got, ref in ((d.gw.cpu().numpy(), go[k][0]), (d.gb.cpu().numpy(), go[k][1])):
            err = np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-12)
            assert err < 3e-2, (k, err)


def test_rain_window_and_windows():
    import sys

    from floodgb.rainfall import rainfall_event
    from floodgb.surrogate.pipeline import rain_window, windows

    ev = rainfall_event([0.0, 30.0, 90.0], [30.0, 90.0, 100.0], [60.0, 120.0, 10.0])
    d, p = rain_window(ev, 0.0, 3600.0)
    assert abs(d - (30.0 + 60.0)) < 1e-9 and p == 120.0
    d, p = rain_window(ev, 3600.0, 6000.0)
    assert abs(d - (120.0 * 0.5 + 10.0 * 10.0 / 60.0)) < 1e-9 and p == 120.0
    assert windows(3.5 * 3600.0) == [(0.0, 3600.0), (3600.0, 7200.0), (7200.0, 10800.0), (10800.0, 12600.0)]
    assert windows(2 * 3600.0) == [(0.0, 3600.0), (3600.0, 7200.0)]


@pytest.mark.gpu
def test_surrogate_trains_and_screens_small_ensemble():
    """End to end on a small mesh: the loss falls, the trained network beats
    'no change' and the untrained network on held-out members (throughput is
    measured at realistic sizes by the experiment, not on this tiny mesh)."""

    pytest.importorskip("torch")
    from floodgb import native
    from floodgb.build import build_library
    from floodgb.surrogate import experiment

    build_library()
    native.load()
    if native.device_count() < 1:
        pytest.skip("no CUDA device")
    # plain training (no pushforward windows): on a 512-cell mesh with two-hour
    # storms, windows started from the network's own early predictions raise
    # the loss of the others; the full-size experiment trains with them
    res = experiment.run(grid_n=16, n_train=56, n_eval=24, seed=5, epochs=30, lr=2e-3, n_layers=4,
                         plain_sample=4, duration_cap_h=2.0, log=lambda *_: None, baselines=True, n_val=8,
                         flag_fraction=0.25, pushforward=0.0)
    for loss, forced in zip(res["train"]["loss"], res["train"]["teacher_forced_loss"]):  # one per network
        assert len(forced) == len(loss) == 30
        assert forced == loss  # every window starts from the solver's state
        assert loss[-1] < 0.5 * loss[0], loss
    acc = res["surrogate_accepted"]
    assert acc is not None and acc["rmse_hmax_m"] < 0.10
    trained = float(np.mean([acc["rmse_hmax_m"]]))
    assert trained < 0.7 * res["no_change"] and trained < 0.7 * res["untrained"]
    # the two networks' disagreement flags members, and every flagged member is re-solved and scored
    assert res["ensemble_networks"] == 2 and res["calibration"]["validation_members"] == 8
    assert res["flagged"] >= 1 and res["surrogate_flagged"]["members"] == res["flagged"]
    assert res["re_solved"] >= res["flagged"]


def test_flag_calibration_on_held_out_storms():
    from floodgb.surrogate.pipeline import calibrate_flags, flags

    rng = np.random.default_rng(3)
    spread = rng.uniform(0.0, 0.02, 100)
    errors = 0.01 + 2.0 * spread + rng.normal(0.0, 1e-3, 100)  # disagreement tracks the true error
    cal = calibrate_flags(spread, errors, flag_fraction=0.1)
    f = flags(spread, cal["threshold_m"])
    assert 8 <= f.sum() <= 11
    assert cal["spearman_spread_vs_error"] > 0.9
    assert cal["mean_error_flagged_m"] > cal["mean_error_accepted_m"]
    assert not flags(np.zeros(5), cal["threshold_m"]).any()


def test_shipped_weights_load_into_the_current_network():
    """The trained ensemble the screening benchmark loads: one set of weights
    per network, each layer's shape that of the current MPNN, and a flag
    threshold calibrated on held-out training storms."""

    pytest.importorskip("torch")
    import json
    from pathlib import Path

    from floodgb.surrogate.model import MPNN

    path = Path(__file__).resolve().parents[1] / "gpu-urban-flood-cupy-jax_gb300" / "floodgb" / "surrogate" / \
        "weights" / "mpnn_grid224.npz"
    z = np.load(path)
    meta = json.loads(str(z["meta"]))
    assert meta["networks"] >= 2 and meta["grid_n"] == 224
    for j in range(meta["networks"]):
        model = MPNN(n_layers=meta["n_layers"], seed=0, device="cpu")
        layers = model.layers()
        assert sum(k.startswith(f"m{j}_w") for k in z.files) == len(layers)
        for k, d in enumerate(layers):
            assert z[f"m{j}_w{k}"].shape == tuple(d.w.shape) and z[f"m{j}_b{k}"].shape == tuple(d.b.shape), (j, k)
            assert np.isfinite(z[f"m{j}_w{k}"]).all()
    cal = json.loads(str(z["calibration"]))
    assert cal["threshold_m"] > 0 and cal["validation_members"] >= 8


def test_extent_calibration_finds_a_low_bias():
    """A surrogate whose window maxima read 1 cm low misses the cells just
    above 5 cm; calibrated on held-out storms its envelope is taken at 4 cm,
    where it matches the solver's 5 cm extent."""

    torch = pytest.importorskip("torch")
    from types import SimpleNamespace

    from floodgb.surrogate.pipeline import calibrate_extent, csi, score

    rng = np.random.default_rng(6)
    C = 4000
    mf = SimpleNamespace(active=rng.random(C) > 0.1, area=np.ones(C, np.float32))
    preds, trajs = [], []
    for _ in range(6):
        hms = rng.uniform(0.0, 0.12, (3, C)).astype(np.float32)
        hs = 0.8 * hms
        truth = SimpleNamespace(h=torch.as_tensor(np.vstack([np.zeros((1, C), np.float32), hs])),
                                hmax=torch.as_tensor(np.vstack([np.zeros((1, C), np.float32), hms])))
        preds.append((np.array([3600.0, 7200.0, 10800.0]), hs - 0.01, hms - 0.01))
        trajs.append(truth)
    cal = calibrate_extent(mf, preds, trajs)
    assert cal["extent_threshold_m"] == 0.04
    assert cal["validation_csi_calibrated"] == 1.0 > cal["validation_csi_at_threshold"]
    s = score(mf, preds[0], trajs[0], extent_threshold=cal["extent_threshold_m"])
    assert s["csi_calibrated"] == 1.0 and s["csi"] < 1.0
    assert abs(s["rmse_hmax_m"] - 0.01) < 1e-6
    assert csi(np.zeros(3, bool), np.zeros(3, bool)) == 1.0


@pytest.mark.gpu
def test_ensemble_rollouts_equal_member_rollouts():
    """The device ensemble (both networks advanced window by window over
    groups of members, padding windows left out of the disagreement) against
    each network's rollout of each member alone."""

    torch = pytest.importorskip("torch")
    from floodgb import native
    from floodgb.build import build_library
    from floodgb.rainfall import rainfall_event
    from floodgb.surrogate.model import MPNN
    from floodgb.surrogate.pipeline import MeshFeatures, ensemble_rollouts, rollout
    from floodgb.synthetic import make_grid_city

    build_library()
    native.load()
    if native.device_count() < 1:
        pytest.skip("no CUDA device")
    sc = make_grid_city(n=12, size_m=120.0, seed=2)
    mf = MeshFeatures(sc.city.topologies.surface_topology)
    models = [MPNN(n_layers=2, seed=s) for s in (1, 2)]
    storms = [rainfall_event([0.0, 20.0], [20.0, 90.0], [80.0, 30.0]),
              rainfall_event([0.0], [150.0], [45.0]),
              rainfall_event([10.0, 60.0], [60.0, 100.0], [110.0, 5.0])]
    durations = [5400.0, 10800.0, 7200.0]  # 2, 3 and 2 windows; groups of two carry a padding window
    preds, spread = ensemble_rollouts(models, mf, storms, durations, copies=2)
    act = mf.active
    for i, (storm, dur) in enumerate(zip(storms, durations)):
        alone = [rollout(m, mf, storm, dur) for m in models]
        ends, h, hm = preds[i]
        np.testing.assert_array_equal(ends, alone[0][0])
        np.testing.assert_allclose(h, np.mean([a[1] for a in alone], 0), atol=1e-6)
        np.testing.assert_allclose(hm, np.mean([a[2] for a in alone], 0), atol=1e-6)
        mean = np.mean([a[2] for a in alone], 0)
        want = np.sqrt(np.mean([(a[2][:, act] - mean[:, act]) ** 2 for a in alone]))
        assert abs(spread[i] - want) <= 1e-6 + 1e-4 * want, (i, spread[i], want)
        assert spread[i] > 0


@pytest.mark.gpu
def test_replicated_graph_gradient_is_the_sum_of_window_gradients():
    """The batched training step: one forward and backward pass over two
    copies of the graph gives each parameter the sum of the two windows'
    gradients taken one by one."""

    torch = pytest.importorskip("torch")
    from floodgb import native
    from floodgb.build import build_library
    from floodgb.surrogate.model import MPNN, DualGraph
    from floodgb.synthetic import make_grid_city

    build_library()
    native.load()
    if native.device_count() < 1:
        pytest.skip("no CUDA device")
    topo = make_grid_city(n=9, size_m=90.0, seed=4).city.topologies.surface_topology
    g = DualGraph(topo)
    g2 = g.replicate(2)
    net = MPNN(n_layers=2, seed=7)
    rng = np.random.default_rng(2)
    xs, dys = [], []
    for _ in range(2):
        x = np.zeros((g.C, SO.FIN), np.float32)
        x[:, :12] = rng.normal(size=(g.C, 12))
        xs.append(torch.as_tensor(x, device="cuda").to(torch.bfloat16).contiguous())
        dy = torch.zeros(g.C, SO.FOUT, device="cuda")
        dy[:, :4] = torch.as_tensor(rng.normal(0, 1e-2, (g.C, 4)).astype(np.float32), device="cuda")
        dys.append(dy)
    single = []
    for x, dy in zip(xs, dys):
        net.zero_grad()
        net.forward(g, x)
        net.backward(g, x, dy)
        single.append([(d.gw.clone(), d.gb.clone()) for d in net.layers()])
    net.zero_grad()
    xb = torch.cat(xs).contiguous()
    yb = net.forward(g2, xb).clone()
    net.backward(g2, xb, torch.cat(dys))
    torch.cuda.synchronize()
    for k, d in enumerate(net.layers()):
        for got, a, b in ((d.gw, single[0][k][0], single[1][k][0]), (d.gb, single[0][k][1], single[1][k][1])):
            want = (a + b).cpu().numpy()
            err = np.linalg.norm(got.cpu().numpy() - want) / max(np.linalg.norm(want), 1e-12)
            assert err < 1e-3, (k, err)
    # and the forward pass of each copy is the window's own
    for j, x in enumerate(xs):
        y = net.forward(g, x, train=False)
        np.testing.assert_allclose(yb[j * g.C:(j + 1) * g.C].cpu().numpy(), y.cpu().numpy(), atol=1e-5, rtol=1e-5)


def test_cosine_schedule_with_and_without_a_time_budget():
    import time

    from floodgb.surrogate.pipeline import cosine

    t0 = time.perf_counter()
    assert cosine(0.0, t0, None) == 1.0
    assert abs(cosine(0.5, t0, None) - 0.5) < 1e-12
    assert abs(cosine(1.0, t0, None)) < 1e-12
    # a budget already spent: the rate has decayed whatever the step progress
    assert abs(cosine(0.1, t0 - 10.0, 5.0)) < 1e-12
    # half the budget spent, a tenth of the steps done: the later of the two sets the rate
    r = cosine(0.1, time.perf_counter() - 5.0, 10.0)
    assert 0.45 < r < 0.5


class _FakeNet:
    """A stand-in network on CPU tensors: depth change from the coming
    window's rain and the current depth, a fixed window maximum above it,
    momenta from the depth; enough to check the rollout bookkeeping."""

    def __init__(self, k):
        self.k = k

    def forward(self, g, x, train=False):
        import torch

        x = x.float()
        y = torch.zeros(g.C, 64)
        y[:, 0] = self.k * x[:, 8] - 0.1 * x[:, 0]
        y[:, 1] = 0.02 * self.k + 0.01 * x[:, 9]
        y[:, 2] = 0.5 * x[:, 0]
        y[:, 3] = -0.25 * x[:, 0]
        return y


def test_ensemble_bookkeeping_against_member_rollouts_on_cpu():
    """Grouping by window count, padding windows and the device-side mean and
    disagreement of ensemble_rollouts against each network's rollout() of
    each member alone (a fake network, CPU tensors)."""

    pytest.importorskip("torch")
    from floodgb.rainfall import rainfall_event
    from floodgb.surrogate.pipeline import MeshFeatures, ensemble_rollouts, rollout
    from floodgb.synthetic import make_grid_city

    mf = MeshFeatures(make_grid_city(n=8, size_m=80.0, seed=2).city.topologies.surface_topology, device="cpu")
    nets = [_FakeNet(0.8), _FakeNet(1.3)]
    storms = [rainfall_event([0.0, 20.0], [20.0, 90.0], [80.0, 30.0]),
              rainfall_event([0.0], [150.0], [45.0]),
              rainfall_event([10.0, 60.0], [60.0, 100.0], [110.0, 5.0]),
              rainfall_event([0.0], [40.0], [20.0])]
    durations = [5400.0, 10800.0, 7200.0, 3000.0]  # 2, 3, 2 and 1 windows
    preds, spread = ensemble_rollouts(nets, mf, storms, durations, copies=2)
    act = mf.active
    for i, (storm, dur) in enumerate(zip(storms, durations)):
        alone = [rollout(n, mf, storm, dur) for n in nets]
        ends, h, hm = preds[i]
        np.testing.assert_array_equal(ends, alone[0][0])
        np.testing.assert_allclose(h, np.mean([a[1] for a in alone], 0), rtol=1e-6, atol=1e-7)
        np.testing.assert_allclose(hm, np.mean([a[2] for a in alone], 0), rtol=1e-6, atol=1e-7)
        mean = np.mean([a[2] for a in alone], 0)
        want = np.sqrt(np.mean([(a[2][:, act] - mean[:, act]) ** 2 for a in alone]))
        assert abs(spread[i] - want) <= 1e-6 * max(want, 1e-6), (i, spread[i], want)
    # one network: the mean is its rollout and there is no disagreement
    one, sp1 = ensemble_rollouts(nets[:1], mf, storms, durations, copies=3)
    assert not sp1.any()
    np.testing.assert_allclose(one[1][2], rollout(nets[0], mf, storms[1], durations[1])[2], rtol=1e-6, atol=1e-7)
