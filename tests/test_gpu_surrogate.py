"""The learned surrogate on the GPU, through libsdem_surrogate.so:

- the neighbour graph (CSR order) and the bf16 edge and node features equal
  the oracle's bit for bit;
- the tensor-core GEMM in all its operand forms (gathered segments,
  transposed operands, split reductions, fused epilogues) against float64
  products of the same bf16 values, within the fp32 accumulation bound;
- the network's forward pass and every parameter gradient of its backward
  pass against the oracle, which rounds to bf16 at the same points;
- training on trajectories of the plain DEM lowers the loss and beats the
  prediction without the network (free flight: a = g, alpha = 0) on frames
  it did not train on;
- the runner re-advances judged strides with the plain DEM and falls back
  to it when the bound is exceeded."""
import ctypes
import math

import numpy as np
import pytest
import torch

from oracle import surrogate_ref as ref
from sdem_gb300 import beds, build, surrogate as sg
from sdem_gb300.capi import DEMSystem

pytestmark = pytest.mark.gpu

DEV = "cuda"


@pytest.fixture(scope="module")
def sg_lib():
    build.build()
    return sg.load()


def bits(t: torch.Tensor) -> np.ndarray:
    return t.contiguous().view(torch.int16).cpu().numpy()


def settled_sandbox(n, index, steps):
    case = beds.sandbox_case(np.random.default_rng(100 + index), index, n_lo=n, n_hi=n)
    s = DEMSystem(case)
    if steps:
        s.step(steps)
    return case, s


def test_graph_and_features_match_oracle(sg_lib):
    case, s = settled_sandbox(1500, 0, 20000)
    st = s.state()
    s.close()
    dmax = 2.0 * float(case.tables.radius.max())
    grid = sg.make_grid(case.opts.minpoint, case.opts.maxpoint, dmax)
    g = sg.build_graph(torch.from_numpy(st.posR).to(DEV), grid)
    row_off, dst, src, ef = ref.graph(st.posR, grid.lo, grid.cell, grid.cutoff, grid.scale, list(grid.dim))
    assert g.E == len(dst) and g.E > 3 * st.posR.shape[0]
    np.testing.assert_array_equal(g.row_off.cpu().numpy(), row_off)
    np.testing.assert_array_equal(g.dst.cpu().numpy(), dst)
    np.testing.assert_array_equal(g.src.cpu().numpy(), src)
    np.testing.assert_array_equal(g.efeat.float().cpu().numpy(), ef)
    assert (ef[:, 4] > 0).sum() > 0, "no overlapping pair in the bed"
    # the sender-ordered permutation lists every edge once, by sender
    perm = g.src_perm.cpu().numpy()
    assert np.array_equal(np.sort(perm), np.arange(g.E)) and np.all(np.diff(src[perm]) >= 0)
    v = st.linVel[:, 0, :]
    vel = np.stack([v, 0.5 * v, -v])
    planes = sg.planes_of(case.walls)
    xn = sg.node_features(torch.from_numpy(st.posR).to(DEV), torch.from_numpy(vel).to(DEV),
                          torch.from_numpy(np.ascontiguousarray(st.rotVel[:, 0, :])).to(DEV),
                          torch.from_numpy(planes).to(DEV), dmax, 0.05)
    want = ref.node_features(st.posR, vel, st.rotVel[:, 0, :], planes, dmax, 0.05)
    np.testing.assert_array_equal(xn.float().cpu().numpy(), want)


def _bf16(rng, shape, scale=1.0):
    return torch.from_numpy((rng.normal(size=shape) * scale).astype(np.float32)).to(torch.bfloat16).to(DEV)


def _np(t):
    return t.float().cpu().numpy().astype(np.float64)


def _close(got, want, absbound):
    err = np.abs(got - want)
    assert np.all(err <= 1e-4 * absbound + 1e-30), float((err / (absbound + 1e-30)).max())


def test_gemm_operand_forms(sg_lib):
    rng = np.random.default_rng(1)
    lib = sg.load()

    def run(I, J, R, a, b, ep, splits=1):
        partial = torch.empty(splits * I * J, dtype=torch.float32, device=DEV) if splits > 1 else None
        rc = lib.sdem_sg_gemm(I, J, R, ctypes.byref(a.o), ctypes.byref(b.o), ctypes.byref(ep), splits,
                              sg._ptr(partial), sg._stream())
        assert rc == 0

    # forward form: three gathered segments (128 + 128 + 128) times W^T, bias,
    # ReLU, bf16 copy; then a residual epilogue
    M, rows = 1001, 300
    h = _bf16(rng, (rows, 128))
    e = _bf16(rng, (M, 128))
    i1 = torch.from_numpy(rng.integers(0, rows, M).astype(np.int32)).to(DEV)
    i2 = torch.from_numpy(rng.integers(0, rows, M).astype(np.int32)).to(DEV)
    W = _bf16(rng, (136, 384), 0.05)
    bias = torch.from_numpy(rng.normal(size=136).astype(np.float32)).to(DEV)
    out = torch.empty((M, 136), dtype=torch.float32, device=DEV)
    outb = torch.empty((M, 136), dtype=torch.bfloat16, device=DEV)
    A = sg._Op(0, (h, 0, 128, 128, i1), (h, 0, 128, 128, i2), (e, 0, 128, 128, None))
    B = sg._Op(0, (W, 0, 384, 384, None))
    run(M, 136, 384, A, B, sg._ep(bias=bias, relu=1, out=out, ld_out=136, out_bf=outb, ld_out_bf=136))
    x = np.concatenate([_np(h)[i1.cpu().numpy()], _np(h)[i2.cpu().numpy()], _np(e)], axis=1)
    w = _np(W)
    want = np.maximum(x @ w.T + _np(bias)[None, :], 0.0)
    _close(_np(out), want, np.abs(x) @ np.abs(w).T + np.abs(_np(bias))[None, :])
    np.testing.assert_array_equal(bits(outb), bits(out.to(torch.bfloat16)))
    resid = torch.from_numpy(rng.normal(size=(M, 136)).astype(np.float32)).to(DEV)
    res_out = torch.empty_like(resid)
    res_b = torch.empty((M, 136), dtype=torch.bfloat16, device=DEV)
    run(M, 136, 384, A, B, sg._ep(out=out, ld_out=136, resid=resid, ld_resid=136, res_out=res_out, ld_res_out=136,
                                  res_out_bf=res_b, ld_res_out_bf=136))
    np.testing.assert_array_equal(res_out.cpu().numpy(), resid.cpu().numpy() + out.cpu().numpy())
    np.testing.assert_array_equal(bits(res_b), bits(res_out.to(torch.bfloat16)))

    # input-gradient form: dY (trans 0) times W (trans 1), ReLU mask
    dy = _bf16(rng, (777, 16))
    W2 = _bf16(rng, (16, 128))
    mask = _bf16(rng, (777, 128))
    dx = torch.empty((777, 128), dtype=torch.float32, device=DEV)
    run(777, 128, 16, sg._Op(0, (dy, 0, 16, 16, None)), sg._Op(1, (W2, 0, 128, 128, None)),
        sg._ep(mask=mask, ld_mask=128, out=dx, ld_out=128))
    want = (_np(dy) @ _np(W2)) * (_np(mask) > 0)
    _close(_np(dx), want, np.abs(_np(dy)) @ np.abs(_np(W2)))

    # weight-gradient form: dY^T X over 5000 rows, both transposed, X in three
    # gathered segments, split over 23 blocks, accumulated onto a start value
    R = 5000
    dyr = _bf16(rng, (R, 128))
    xr = _bf16(rng, (400, 128))
    er = _bf16(rng, (R, 128))
    j1 = torch.from_numpy(rng.integers(0, 400, R).astype(np.int32)).to(DEV)
    j2 = torch.from_numpy(rng.integers(0, 400, R).astype(np.int32)).to(DEV)
    gw = torch.from_numpy(rng.normal(size=(128, 384)).astype(np.float32)).to(DEV)
    start = gw.cpu().numpy().astype(np.float64)
    run(128, 384, R, sg._Op(1, (dyr, 0, 128, 128, None)),
        sg._Op(1, (xr, 0, 128, 128, j1), (xr, 0, 128, 128, j2), (er, 0, 128, 128, None)),
        sg._ep(out=gw, ld_out=384, accumulate=1), splits=23)
    X = np.concatenate([_np(xr)[j1.cpu().numpy()], _np(xr)[j2.cpu().numpy()], _np(er)], axis=1)
    want = start + _np(dyr).T @ X
    _close(_np(gw), want, np.abs(start) + np.abs(_np(dyr)).T @ np.abs(X))

    # a 16-row output (decoder rows) over a ragged reduction, unsplit
    d16 = _bf16(rng, (333, 16))
    z = _bf16(rng, (333, 128))
    o16 = torch.empty((16, 128), dtype=torch.float32, device=DEV)
    run(16, 128, 333, sg._Op(1, (d16, 0, 16, 16, None)), sg._Op(1, (z, 0, 128, 128, None)),
        sg._ep(out=o16, ld_out=128))
    _close(_np(o16), _np(d16).T @ _np(z), np.abs(_np(d16)).T @ np.abs(_np(z)))


def test_gemm_tcgen05_and_mma_sync_paths(sg_lib):
    """The forward forms on both tensor paths: the tcgen05/TMEM kernel and
    the warp-level mma.sync kernel, each against float64 products of the same
    bf16 values within the fp32 accumulation bound, over ragged shapes (rows
    not a multiple of the 128-row tile, 16 and 136 output columns, reductions
    of 48 and 384 in up to three gathered segments); no bounded wait of the
    tcgen05 kernel expires."""
    rng = np.random.default_rng(7)
    lib = sg.load()
    shapes = [(1001, 136, 384, 3), (129, 16, 48, 1), (4096, 128, 256, 2), (77, 128, 128, 1)]
    try:
        for path in (1, 0):
            assert lib.sdem_sg_set_tensor_path(path) == 0
            for M, J, R, nseg in shapes:
                rows = 300
                w_seg = R // nseg
                segs, parts = [], []
                for k in range(nseg):
                    src = _bf16(rng, (rows, w_seg))
                    idx = torch.from_numpy(rng.integers(0, rows, M).astype(np.int32)).to(DEV)
                    segs.append((src, 0, w_seg, w_seg, idx))
                    parts.append(_np(src)[idx.cpu().numpy()])
                A = sg._Op(0, *segs)
                W = _bf16(rng, (J, R), 0.05)
                bias = torch.from_numpy(rng.normal(size=J).astype(np.float32)).to(DEV)
                out = torch.empty((M, J), dtype=torch.float32, device=DEV)
                rc = lib.sdem_sg_gemm(M, J, R, ctypes.byref(A.o), ctypes.byref(sg._Op(0, (W, 0, R, R, None)).o),
                                      ctypes.byref(sg._ep(bias=bias, out=out, ld_out=J)), 1, None, sg._stream())
                assert rc == 0
                x = np.concatenate(parts, axis=1)
                w = _np(W)
                want = x @ w.T + _np(bias)[None, :]
                _close(_np(out), want, np.abs(x) @ np.abs(w).T + np.abs(_np(bias))[None, :])
        cnt = ctypes.c_uint(99)
        assert lib.sdem_sg_tensor_timeouts(ctypes.byref(cnt)) == 0 and cnt.value == 0
    finally:
        lib.sdem_sg_set_tensor_path(1)


def _graph_sample(n, index, steps, seed):
    case, s = settled_sandbox(n, index, steps)
    st = s.state()
    s.close()
    dmax = 2.0 * float(case.tables.radius.max())
    grid = sg.make_grid(case.opts.minpoint, case.opts.maxpoint, dmax)
    posR = torch.from_numpy(st.posR).to(DEV)
    g = sg.build_graph(posR, grid)
    rng = np.random.default_rng(seed)
    v = st.linVel[:, 0, :]
    vel = np.stack([v, v, v])
    xn = sg.node_features(posR, torch.from_numpy(vel).to(DEV),
                          torch.from_numpy(np.ascontiguousarray(st.rotVel[:, 0, :])).to(DEV),
                          torch.from_numpy(sg.planes_of(case.walls)).to(DEV), dmax, 0.05)
    tgt = rng.normal(size=(n, sg.OUT_USED)).astype(np.float32)
    return g, xn, tgt


def test_network_forward_and_gradients_match_oracle(sg_lib):
    g, xn, tgt = _graph_sample(700, 1, 3000, 2)
    rng = np.random.default_rng(3)
    p = sg.init_params(11)
    for name, shape, off in sg.param_layout():
        if ".b" in name:
            p[off:off + shape[0]] = rng.normal(scale=0.05, size=shape[0]).astype(np.float32)
            if name == "dec.b2":
                p[off + sg.OUT_USED:off + shape[0]] = 0.0
    net = sg.Network(params=p)
    y = net.forward(g, xn, keep=True)
    loss, dy, dyb = net.loss(y, torch.from_numpy(tgt).to(DEV))
    net.grad.zero_()
    net.backward(dy, dyb)
    torch.cuda.synchronize()
    o = ref.Net(p, bf16=True)
    y_ref = o.forward(_np(xn), _np(g.efeat), g.dst.cpu().numpy(), g.src.cpu().numpy(), g.row_off.cpu().numpy())
    loss_ref, dy_ref = o.loss(y_ref, tgt)
    g_ref = o.backward(dy_ref)
    y_gpu = y.cpu().numpy().astype(np.float64)
    rel = np.linalg.norm(y_gpu - y_ref) / np.linalg.norm(y_ref)
    assert rel < 1e-2, rel
    assert abs(float(loss) - loss_ref) <= 1e-2 * loss_ref
    grad = net.grad.cpu().numpy().astype(np.float64)
    worst = 0.0
    for name, shape, off in sg.param_layout():
        k = int(np.prod(shape))
        a, b = grad[off:off + k], g_ref[off:off + k]
        nb = np.linalg.norm(b)
        if nb == 0.0:
            assert np.linalg.norm(a) == 0.0, name
            continue
        r = np.linalg.norm(a - b) / nb
        worst = max(worst, r)
        assert r < 3e-2, (name, r)
    print(f"forward rel err {rel:.2e}, worst gradient rel err {worst:.2e}")


def test_training_beats_free_flight(sg_lib):
    samples = []
    cases = []
    for k in range(3):
        case, s = settled_sandbox(1200 + 300 * k, 10 + k, 20000)
        cases.append(case)
        samples.append(sg.record_samples(s, case, stride=100, frames=12))
        s.close()
    dmax = max(2.0 * float(c.tables.radius.max()) for c in cases)
    dev_samples = [[sg.to_device(x, c, dmax, 0.05) for x in ss] for ss, c in zip(samples, cases)]
    train = [x for ss in dev_samples for x in ss[:-3]]
    held = [x for ss in dev_samples for x in ss[-3:]]
    net = sg.Network(seed=0)
    losses = []
    for it in range(300):
        d = train[it % len(train)]
        losses.append(float(net.train_step(d.graph, d.xn, d.target, lr=2e-3)))
    assert all(math.isfinite(x) for x in losses)
    assert np.mean(losses[-20:]) < np.mean(losses[:20])
    mse, mse_free = sg.evaluate(net, held)
    print(f"held-out mse {mse:.4g} vs free flight {mse_free:.4g}")
    assert mse < mse_free


def test_runner_judges_and_falls_back(sg_lib):
    # an untrained network: its strides let spheres close in on each other, so
    # a judged stride may also meet a state the plain DEM rejects (explosive
    # repulsion); the runner must restore the last plain state then
    for bound in (1.0, 0.0):
        case, s = settled_sandbox(1500, 20, 2000)
        dmax = 2.0 * float(case.tables.radius.max())
        net = sg.Network(seed=1)
        r = sg.SurrogateRunner(net, s, case, stride=100, d_max=dmax, vscale=0.05, judge_every=4, bound=bound,
                               fallback_strides=3)
        st = r.run(12)
        assert r.t >= 14 and st["judged"] >= 1
        errs, perrs = st["errors"], st["pressure_errors"]
        assert len(errs) == len(perrs) == st["judged"] and all(e >= 0.0 for e in errs + perrs)
        # a fallback exactly when a judged error exceeds its bound or the
        # graph outgrows its limit
        assert st["fallbacks"] == sum(1 for e, pe in zip(errs, perrs)
                                      if e > bound or pe > r.pressure_bound) + st["diverged"]
        if bound == 0.0:
            assert st["fallbacks"] >= 1
        assert torch.isfinite(r.posR).all() and r.posR.shape[0] == s.counters()["nlocal"]
        # the centres stay inside the box's walls (open top)
        box = sg.box_of(case.walls)
        p = r.posR.cpu().numpy()
        for a in range(3):
            assert np.all(p[:, a] >= box.lo[a]) and np.all(p[:, a] <= box.hi[a])
        s.close()


def test_batched_recording_equals_single_beds(sg_lib):
    # training frames recorded through the batched form (one graph per group
    # of beds) are the frames of each bed stepped alone, bit for bit
    from sdem_gb300 import props
    rng = np.random.default_rng(7)
    cases = [beds.sandbox_case(rng, k, n_lo=800, n_hi=1600, cf_type=props.CFT_NLIN) for k in range(3)]
    systems = [DEMSystem(c) for c in cases]
    batched = sg.record_samples_batch(systems, cases, stride=20, frames=5, settle=200, group_size=2)
    for s in systems:
        s.close()
    for c, got in zip(cases, batched):
        s = DEMSystem(c)
        want = sg.record_samples(s, c, 20, 5, settle=200)
        s.close()
        assert len(got) == len(want) == 2
        for a, b in zip(got, want):
            for f in ("posR", "vel", "omega", "target"):
                np.testing.assert_array_equal(getattr(a, f), getattr(b, f))
