"""The surrogate's host orchestration (sdem_gb300.surrogate: graph build,
features, forward, backward, Adam, one stride) run on CPU tensors through a
numpy statement of the C ABI (tests/sg_mock.py) and compared with the
oracle: operand segments, gather indices, strides, offsets and the order of
the backward pass are checked without a GPU."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import surrogate_ref as ref
from sdem_gb300 import surrogate as sg
from tests.sg_mock import SgMock

LATENT, LAYERS = 32, 2


@pytest.fixture
def mock(monkeypatch):
    m = SgMock()
    monkeypatch.setattr(sg, "_lib", m)
    monkeypatch.setattr(sg, "_stream", lambda: 0)
    return m


def bed(n, seed):
    rng = np.random.default_rng(seed)
    d = rng.uniform(0.8e-3, 1.2e-3, n)
    pos = rng.uniform(0.5e-3, 5e-3, size=(n, 3))
    return np.concatenate([pos, (d / 2)[:, None]], axis=1)


def inputs(n=90, seed=1):
    posR = bed(n, seed)
    grid = sg.make_grid((0, 0, 0), (5.5e-3, 5.5e-3, 5.5e-3), 1.2e-3)
    g = sg.build_graph(torch.from_numpy(posR), grid)
    rng = np.random.default_rng(seed + 1)
    vel = rng.normal(scale=0.05, size=(3, n, 3))
    om = rng.normal(scale=10.0, size=(n, 3))
    planes = np.array([[0, 1, 0, 0.0], [1, 0, 0, 0.0], [-1, 0, 0, 5.5e-3]])
    xn = sg.node_features(torch.from_numpy(posR), torch.from_numpy(vel), torch.from_numpy(om),
                          torch.from_numpy(planes), 1.2e-3, 0.05)
    tgt = rng.normal(size=(n, sg.OUT_USED)).astype(np.float32)
    return posR, grid, g, xn, tgt


def test_graph_build_through_the_abi(mock):
    posR, grid, g, xn, _ = inputs()
    row_off, dst, src, ef = ref.graph(posR, grid.lo, grid.cell, grid.cutoff, grid.scale, list(grid.dim))
    assert g.E == len(dst) > 0
    np.testing.assert_array_equal(g.row_off.numpy(), row_off)
    np.testing.assert_array_equal(g.src.numpy(), src)
    perm = g.src_perm.numpy()
    assert np.all(np.diff(src[perm]) >= 0)
    np.testing.assert_array_equal(np.diff(g.src_off.numpy()), np.bincount(src, minlength=len(posR)))


def test_forward_backward_orchestration_matches_oracle(mock):
    posR, grid, g, xn, tgt = inputs()
    rng = np.random.default_rng(4)
    p = sg.init_params(2, LATENT, LAYERS)
    for name, shape, off in sg.param_layout(LATENT, LAYERS):
        if ".b" in name and name != "dec.b2":
            p[off:off + shape[0]] = rng.normal(scale=0.05, size=shape[0])
    net = sg.Network(device="cpu", latent=LATENT, layers=LAYERS, params=p)
    y = net.forward(g, xn, keep=True)
    loss, dy, dyb = net.loss(y, torch.from_numpy(tgt))
    net.grad.zero_()
    net.backward(dy, dyb)
    o = ref.Net(p, LATENT, LAYERS, bf16=True)
    y_ref = o.forward(xn.float().numpy(), g.efeat.float().numpy(), g.dst.numpy(), g.src.numpy(), g.row_off.numpy())
    loss_ref, dy_ref = o.loss(y_ref, tgt)
    g_ref = o.backward(dy_ref)
    rel = np.linalg.norm(y.numpy() - y_ref) / np.linalg.norm(y_ref)
    # the same bf16 rounding points; fp32 (stand-in) against float64 (oracle)
    # storage flips an occasional bf16 rounding: differences of 1e-3, where a
    # wrong operand, stride or order gives differences of order one
    assert rel < 1e-2, rel
    assert abs(float(loss) - loss_ref) <= 1e-2 * loss_ref
    grad = net.grad.numpy().astype(np.float64)
    worst = 0.0
    for name, shape, off in sg.param_layout(LATENT, LAYERS):
        k = int(np.prod(shape))
        a, b = grad[off:off + k], g_ref[off:off + k]
        nb = np.linalg.norm(b)
        if nb == 0:
            assert np.linalg.norm(a) == 0, name
        else:
            assert np.linalg.norm(a - b) <= 3e-2 * nb, (name, np.linalg.norm(a - b) / nb)
            worst = max(worst, np.linalg.norm(a - b) / nb)
    print(f"forward {rel:.2e}, worst gradient {worst:.2e}")


def test_training_steps_lower_the_loss(mock):
    _, _, g, xn, tgt = inputs(60, 3)
    net = sg.Network(seed=0, device="cpu", latent=LATENT, layers=LAYERS)
    t = torch.from_numpy(tgt)
    losses = [float(net.train_step(g, xn, t, lr=3e-3)) for _ in range(25)]
    assert losses[-1] < losses[0]


def test_stride_update(mock):
    posR, _, _, _, _ = inputs(20, 5)
    n = len(posR)
    rng = np.random.default_rng(6)
    pred = torch.from_numpy(rng.normal(size=(n, sg.OUT)).astype(np.float32))
    pos = torch.from_numpy(posR.copy())
    vel = torch.from_numpy(rng.normal(size=(3, n, 3)))
    om = torch.from_numpy(rng.normal(size=(n, 3)))
    v0, v1, p0, w0 = vel[0].clone(), vel[1].clone(), pos.clone(), om.clone()
    h = 2e-4
    box = sg.SgBox()
    for a in range(3):
        box.lo[a], box.hi[a] = -1e300, 1e300
    box.lo[1] = float(np.sort(posR[:, 1] - posR[:, 3])[n // 2])   # half of the spheres start against a floor
    assert sg.load().sdem_sg_advance(n, sg._ptr(pred), sg.OUT, 9.81, 0.0, -9.81, 0.0, h, ctypes.byref(box),
                                     sg._ptr(pos), sg._ptr(vel), sg._ptr(om), 0) == 0
    a = 9.81 * pred[:, :3].double() + torch.tensor([0.0, -9.81, 0.0], dtype=torch.float64)
    vfree = v0 + a * h
    xfree = p0[:, :3] + vfree * h
    floor = box.lo[1] + p0[:, 3]
    held = xfree[:, 1] < floor
    assert held.any() and (~held).any()
    torch.testing.assert_close(vel[1], v0)
    torch.testing.assert_close(vel[2], v1)
    torch.testing.assert_close(vel[0][:, [0, 2]], vfree[:, [0, 2]])
    torch.testing.assert_close(pos[:, [0, 2]], xfree[:, [0, 2]])
    torch.testing.assert_close(pos[~held, 1], xfree[~held, 1])
    torch.testing.assert_close(vel[0][~held, 1], vfree[~held, 1])
    torch.testing.assert_close(pos[held, 1], floor[held])
    torch.testing.assert_close(vel[0][held, 1], vfree[held, 1].clamp(min=0.0))
    torch.testing.assert_close(om, w0 + 9.81 * pred[:, 3:6].double() / p0[:, 3:4] * h)


def test_box_of_walls():
    from sdem_gb300 import beds
    case = beds.sandbox_case(np.random.default_rng(4), 0, n_lo=300, n_hi=300)
    b = sg.box_of(case.walls)
    lo, hi = case.opts.minpoint, case.opts.maxpoint
    for a in range(3):
        assert b.lo[a] == pytest.approx(lo[a], abs=1e-15)
    assert b.hi[0] == pytest.approx(hi[0]) and b.hi[2] == pytest.approx(hi[2])
    assert b.hi[1] == 1e300          # open top


def test_frames_aligned_by_id():
    now = np.array([5, 2, 9], np.int32)
    old = np.array([9, 5, 7], np.int32)
    v_old = np.array([[9.0] * 3, [5.0] * 3, [7.0] * 3])
    v_now = np.zeros((3, 3))
    np.testing.assert_array_equal(sg.align_frames(now, old, v_old, v_now)[:, 0], [5.0, 0.0, 9.0])


@pytest.mark.parametrize("bound,growth", [(1.0, 100.0), (0.0, 100.0), (1.0, 0.5)])
def test_runner_over_the_oracle(mock, bound, growth):
    # the runner's bookkeeping with the oracle as the plain DEM: judged
    # strides, fallbacks above the bound, divergence of the graph (a limit
    # below one edge-count ratio makes every second stride diverge), rewinds
    from oracle.oracle import OracleSystem
    from sdem_gb300 import beds
    case = beds.sandbox_case(np.random.default_rng(30), 0, n_lo=300, n_hi=300)
    dem = OracleSystem(case)
    dem.step(500)
    net = sg.Network(seed=1, device="cpu", latent=LATENT, layers=LAYERS)
    r = sg.SurrogateRunner(net, dem, case, stride=20, d_max=2.0 * float(case.tables.radius.max()), vscale=0.05,
                           judge_every=3, bound=bound, fallback_strides=2, edge_growth=growth)
    t0 = r.t
    st = r.run(9)
    assert r.t >= t0 + 9
    assert len(st["pressure_errors"]) == len(st["errors"]) == st["judged"]
    assert st["fallbacks"] == sum(1 for e, pe in zip(st["errors"], st["pressure_errors"])
                                  if e > bound or pe > r.pressure_bound) + st["diverged"]
    if bound == 0.0:
        assert st["fallbacks"] >= 1 and st["diverged"] == 0
    if growth < 1.0:
        assert st["diverged"] >= 1 and st["rewound_strides"] >= 1
    assert r.posR.shape[0] == dem.counters()["nlocal"] and torch.isfinite(r.posR).all()


def test_wall_pressure_known_answers():
    # one Hertz sphere pressed into the floor of a 0.1 x 0.6 x 0.1 m box, one
    # touching a side wall, one free: the pressure on each wall is
    # |Kn| delta^1.5 over the wall's area; LSD scales the overlap linearly
    from sdem_gb300 import beds, props
    case = beds.sandbox_case(np.random.default_rng(3), 0, n_lo=200, n_hi=200)
    nT = case.tables.n_types
    bpw = case.tables.bpw.reshape(-1, nT, props.BP_SIZE)
    lo, hi = np.asarray(case.opts.minpoint), np.asarray(case.opts.maxpoint)
    r = 1e-3
    mid = (lo + hi) / 2
    posR = np.array([[mid[0], lo[1] + r - 2e-5, mid[2], r],        # floor, delta 2e-5
                     [lo[0] + r - 1e-5, mid[1], mid[2], r],        # wall x = min, delta 1e-5
                     [mid[0], mid[1], mid[2], r]])                 # free
    ptype = np.array([1, 2, 1], dtype=np.int32)
    walls, flags = case.walls.arrays()
    W, F = walls.reshape(case.walls.n, -1), flags.reshape(case.walls.n, -1)
    p = sg.wall_pressure(posR, ptype, case)
    assert p.shape == (case.walls.n,)
    for k in range(case.walls.n):
        n = W[k, 12:15]
        area = float(np.linalg.norm(np.cross(W[k, 3:6] - W[k, 0:3], W[k, 9:12] - W[k, 0:3])))
        want = 0.0
        for (x, t) in ((posR[0], 1), (posR[1], 2)):
            delta = r - (x[:3] @ n + W[k, 15])
            if delta >= 0:
                kn = abs(bpw[F[k, 3] - 1, t - 1, 2])
                want += kn * delta ** 1.5 if case.opts.cf_type == props.CFT_NLIN else kn * 0.01 ** 0.4 * delta
        np.testing.assert_allclose(p[k], want / area, rtol=1e-12)
    assert np.count_nonzero(p) == 2
    # the relative error over the loaded walls only
    assert sg.pressure_error(p * 1.1, p) == pytest.approx(0.1)
    assert sg.pressure_error(p, np.zeros_like(p)) == 0.0


def test_graph_without_edges(mock):
    # spheres farther apart than the cutoff: an empty graph; forward, loss,
    # backward and Adam still run (encoder and node layers only)
    n = 8
    pos = np.stack([np.arange(n) * 5e-3 + 1e-3, np.full(n, 1e-3), np.full(n, 1e-3)], axis=1)
    posR = np.concatenate([pos, np.full((n, 1), 0.5e-3)], axis=1)
    grid = sg.make_grid((0, 0, 0), (0.05, 0.01, 0.01), 1.2e-3)
    g = sg.build_graph(torch.from_numpy(posR), grid)
    assert g.E == 0 and g.dst.numel() == 0 and g.src_perm.numel() == 0
    xn = sg.node_features(torch.from_numpy(posR), torch.zeros((3, n, 3), dtype=torch.float64),
                          torch.zeros((n, 3), dtype=torch.float64), torch.zeros((0, 4), dtype=torch.float64),
                          1.2e-3, 0.05)
    net = sg.Network(seed=0, device="cpu", latent=LATENT, layers=LAYERS)
    tgt = torch.ones((n, sg.OUT_USED))
    l0 = float(net.train_step(g, xn, tgt, lr=1e-2))
    for _ in range(10):
        l1 = float(net.train_step(g, xn, tgt, lr=1e-2))
    assert np.isfinite(l1) and l1 < l0
    # every edge-layer gradient of the last step is zero: no edge contributed
    for name, shape, off in sg.param_layout(LATENT, LAYERS):
        if name.startswith("edge") or name.startswith("enc_e"):
            assert float(net.grad[off:off + int(np.prod(shape))].abs().max()) == 0.0, name
