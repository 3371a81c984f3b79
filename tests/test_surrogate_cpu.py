"""The learned surrogate without a GPU: the C ABI (header, exports, struct
layouts of the ctypes mirrors), the parameter layout and initialisation, the
bf16 rounding, the oracle's neighbour graph against an independent pair
search, and the oracle's backward pass against finite differences of its
forward pass."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest
import torch

from oracle import surrogate_ref as ref
from sdem_gb300 import build, surrogate as sg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    hdr = open(os.path.join(ROOT, "include", "sdem_surrogate.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    return sorted(set(re.findall(r"\b(sdem_sg_[a-z_0-9]+)\s*\(", hdr)))


def test_header_and_library_exports():
    assert set(sg.EXPORTED) == set(declared())
    build.build()
    lib = ctypes.CDLL(sg.LIB_PATH)
    assert [s for s in declared() if not hasattr(lib, s)] == []
    # host-only entry point: no GPU touched
    assert sg.load().sdem_sg_colsum_blocks() > 0


def test_struct_layouts_match_the_compiler(tmp_path):
    exe = tmp_path / "sg_layout"
    subprocess.run(["gcc", "-O0", "-o", str(exe), os.path.join(ROOT, "tests", "csrc", "sg_layout.c")], check=True)
    want = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n"):
        if line:
            k, v = line.split()
            want[k] = int(v)
    mirrors = {"sdem_sg_grid": sg.SgGrid, "sdem_sg_operand": sg.SgOperand, "sdem_sg_epilogue": sg.SgEpilogue,
               "sdem_sg_box": sg.SgBox}
    for key, val in want.items():
        if "." in key:
            s, f = key.split(".")
            assert getattr(mirrors[s], f).offset == val, key
        else:
            assert ctypes.sizeof(mirrors[key]) == val, key


def test_param_layout_and_init():
    lay = sg.param_layout()
    end = 0
    for name, shape, off in lay:
        assert off % 8 == 0 and off >= end, name
        end = off + int(np.prod(shape))
    assert sg.param_count() >= end
    p1, p2 = sg.init_params(3), sg.init_params(3)
    np.testing.assert_array_equal(p1, p2)
    shape, off = {n: (s, o) for n, s, o in lay}["dec.w2"]
    w = p1[off:off + shape[0] * shape[1]].reshape(shape)
    assert np.all(w[sg.OUT_USED:] == 0) and np.any(w[:sg.OUT_USED] != 0)


def test_bf16_rounding_matches_torch():
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.normal(size=10000), rng.normal(size=1000) * 1e-30, [0.0, -0.0, 1.0, 3.0039062]])
    x = x.astype(np.float32)
    want = torch.from_numpy(x).to(torch.bfloat16).float().numpy()
    np.testing.assert_array_equal(sg.bf16_round(x), want)


def small_bed(n, seed):
    rng = np.random.default_rng(seed)
    d = rng.uniform(0.8e-3, 1.2e-3, n)
    pos = rng.uniform(0.0, 6e-3, size=(n, 3))
    return np.concatenate([pos, (d / 2)[:, None]], axis=1)


def test_oracle_graph_against_pair_search():
    spatial = pytest.importorskip("scipy.spatial")
    posR = small_bed(600, 1)
    dmax = 1.2e-3
    grid = sg.make_grid((0, 0, 0), (6e-3, 6e-3, 6e-3), dmax)
    row_off, dst, src, ef = ref.graph(posR, grid.lo, grid.cell, grid.cutoff, grid.scale, list(grid.dim))
    pairs = spatial.cKDTree(posR[:, :3]).query_pairs(grid.cutoff * (1 - 1e-12))
    want = set(pairs) | {(j, i) for i, j in pairs}
    got = set(zip(dst.tolist(), src.tolist()))
    assert got == want
    assert np.all(np.diff(dst) >= 0) and row_off[-1] == len(dst)
    d = np.linalg.norm(posR[src, :3] - posR[dst, :3], axis=1)
    np.testing.assert_allclose(ef[:, 3], d / dmax, rtol=1e-2)
    assert np.all(ef[:, 5:] == 0)


def test_oracle_backward_against_finite_differences():
    latent, layers = 16, 2
    posR = small_bed(40, 2)
    grid = sg.make_grid((0, 0, 0), (6e-3, 6e-3, 6e-3), 1.2e-3)
    row_off, dst, src, ef = ref.graph(posR, grid.lo, grid.cell, grid.cutoff, grid.scale, list(grid.dim))
    assert len(dst) > 0
    rng = np.random.default_rng(5)
    xn = rng.normal(size=(40, sg.NODE_IN))
    tgt = rng.normal(size=(40, sg.OUT_USED))
    p = sg.init_params(7, latent, layers).astype(np.float64)
    # biases non-zero so every term is exercised
    for name, shape, off in sg.param_layout(latent, layers):
        if ".b" in name:
            p[off:off + shape[0]] = rng.normal(scale=0.1, size=shape[0])
            if name == "dec.b2":
                p[off + sg.OUT_USED:off + shape[0]] = 0.0
    net = ref.Net(p, latent, layers, bf16=False)

    def loss(pp):
        nn = ref.Net(pp, latent, layers, bf16=False)
        return nn.loss(nn.forward(xn, ef, dst, src, row_off), tgt)[0]

    y = net.forward(xn, ef, dst, src, row_off)
    _, dy = net.loss(y, tgt)
    g = net.backward(dy)
    used = np.concatenate([np.arange(off, off + int(np.prod(shape))) for name, shape, off in
                           sg.param_layout(latent, layers)])
    dshape, doff = {n: (s, o) for n, s, o in sg.param_layout(latent, layers)}["dec.w2"]
    unused = set(range(doff + sg.OUT_USED * dshape[1], doff + dshape[0] * dshape[1]))
    used = np.array([k for k in used if k not in unused])      # zero decoder rows: no loss gradient
    pick = rng.choice(used, size=60, replace=False)
    for k in pick:
        h = 1e-6 * max(1.0, abs(p[k]))
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (loss(pp) - loss(pm)) / (2 * h)
        assert abs(fd - g[k]) <= 1e-7 + 1e-4 * abs(fd), (k, fd, g[k])


def test_forward_flop_count_of_the_bench():
    # the tensor roofline's flop figure equals 2 M kin kout summed over the
    # weights of the layout (M = edges for edge layers, spheres otherwise)
    import bench
    n, E = 1000, 24000
    want = 0
    for name, shape, off in sg.param_layout():
        if len(shape) != 2:
            continue
        rows = E if (name.startswith("edge") or name.startswith("enc_e")) else n
        want += 2 * rows * shape[0] * shape[1]
    assert bench.surrogate_forward_flop(n, E) == float(want)
