"""Learned surrogate of the particle step, driven through libsdem_surrogate.so
(include/sdem_surrogate.h).

A message-passing network over the neighbour graph of the cell search
(radius 1.5 d_max) predicts each sphere's mean linear and angular
acceleration over a stride of S DEM steps:

- node features (32): velocity frames v(t), v(t-S), v(t-2S), spin omega r,
  diameter and the distances to the five planes of the box;
- edge features (16): relative displacement, distance, overlap;
- encoders: 2-layer MLPs to a latent width of 128 (nodes and edges);
- 6 processor layers: edge MLP over [h_dst, h_src, e] -> message m, e += m;
  node MLP over [h, sum of incoming m] -> h += u;
- decoder: 2-layer MLP to 6 outputs, (a - g)/|g| and alpha r/|g|.

Every layer runs on the tensor cores of the library's GEMM (bf16 operands,
fp32 accumulation, fused bias/ReLU/residual epilogues), forward and
backward; the aggregation and its adjoints, the loss, Adam and the stride
update are the library's kernels too.  PyTorch holds the device memory and
provides the sorts and prefix sums of the graph build.  The product path has
no CPU fallback: loading fails loudly when the library is missing.

SurrogateRunner advances a bed by surrogate strides and, every `judge_every`
strides, re-advances one stride with the plain FP64 DEM (include/sdem_gpu.h)
from the surrogate's state as the error judge; when the relative bed-height
difference or the mean relative wall-pressure difference exceeds its bound,
when the plain DEM rejects the state, or when the neighbour graph outgrows its
limit, the plain DEM takes over for the next strides (from its last own state
where the surrogate's was rejected).
"""
from __future__ import annotations

import ctypes as C
import math
import os
from dataclasses import dataclass
from typing import List, Optional, Tuple

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsdem_surrogate.so")

LATENT = 128
LAYERS = 6
NODE_IN = 32
EDGE_IN = 16
OUT = 16          # decoder rows (6 used, the rest stay zero)
OUT_USED = 6
CUTOFF_FACTOR = 1.5
DCLIP = 10.0
OVERLAP_GAIN = 100.0

EXPORTED = ("sdem_sg_cells", "sdem_sg_edge_count", "sdem_sg_edge_fill", "sdem_sg_node_features", "sdem_sg_gemm",
            "sdem_sg_segsum", "sdem_sg_gather_add", "sdem_sg_colsum_blocks", "sdem_sg_colsum", "sdem_sg_mse",
            "sdem_sg_adam", "sdem_sg_to_bf16", "sdem_sg_advance", "sdem_sg_set_tensor_path",
            "sdem_sg_tensor_timeouts")


class SgGrid(C.Structure):
    _fields_ = [("lo", C.c_double * 3), ("cell", C.c_double), ("cutoff", C.c_double), ("scale", C.c_double),
                ("dim", C.c_int * 3), ("pad_", C.c_int)]


class SgOperand(C.Structure):
    _fields_ = [("ptr", C.c_void_p * 3), ("idx", C.c_void_p * 3), ("ld", C.c_int * 3), ("width", C.c_int * 3),
                ("nseg", C.c_int), ("trans", C.c_int)]


class SgBox(C.Structure):
    _fields_ = [("lo", C.c_double * 3), ("hi", C.c_double * 3)]


class SgEpilogue(C.Structure):
    _fields_ = [("bias", C.c_void_p), ("relu", C.c_int), ("accumulate", C.c_int),
                ("mask", C.c_void_p), ("ld_mask", C.c_int),
                ("out", C.c_void_p), ("ld_out", C.c_int),
                ("out_bf", C.c_void_p), ("ld_out_bf", C.c_int),
                ("resid", C.c_void_p), ("ld_resid", C.c_int),
                ("res_out", C.c_void_p), ("ld_res_out", C.c_int),
                ("res_out_bf", C.c_void_p), ("ld_res_out_bf", C.c_int)]


_lib = None


def load(path: str = LIB_PATH):
    """Loads libsdem_surrogate.so (no fallback: a missing library raises)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with `python -m sdem_gb300.build` (sm_103a only)")
    lib = C.CDLL(path)
    P, I, D, LL, F = C.c_void_p, C.c_int, C.c_double, C.c_longlong, C.c_float
    sig = {
        "sdem_sg_cells": [I, P, C.POINTER(SgGrid), P, P],
        "sdem_sg_edge_count": [I, P, C.POINTER(SgGrid), P, P, P, P, P],
        "sdem_sg_edge_fill": [I, P, C.POINTER(SgGrid), P, P, P, P, P, P, P, P],
        "sdem_sg_node_features": [I, P, P, P, I, P, D, D, D, P, P],
        "sdem_sg_gemm": [I, I, I, C.POINTER(SgOperand), C.POINTER(SgOperand), C.POINTER(SgEpilogue), I, P, P],
        "sdem_sg_segsum": [I, I, P, P, P, I, P, I, I, P, I, P],
        "sdem_sg_gather_add": [I, I, P, P, I, P, I, P, I, P, I, P],
        "sdem_sg_colsum_blocks": [],
        "sdem_sg_colsum": [I, I, P, I, P, I, P, P],
        "sdem_sg_mse": [I, I, P, I, P, P, P, P, P],
        "sdem_sg_adam": [LL, P, P, P, P, P, F, F, F, F, F, I, P],
        "sdem_sg_to_bf16": [LL, P, P, P],
        "sdem_sg_advance": [I, P, I, D, D, D, D, D, C.POINTER(SgBox), P, P, P, P],
        "sdem_sg_set_tensor_path": [I],
        "sdem_sg_tensor_timeouts": [C.POINTER(C.c_uint)],
    }
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int
    _lib = lib
    return lib


def _check(rc: int, what: str) -> None:
    if rc:
        raise RuntimeError(f"{what} failed (code {rc})")


def _ptr(t: Optional[torch.Tensor], offset: int = 0) -> Optional[int]:
    """Address of element `offset` of t.  A zero-element view reports a null
    data pointer; its address inside its storage is used instead, so an
    empty slice of an allocated buffer still passes the library's checks."""
    if t is None:
        return None
    if t.numel():
        base = t.data_ptr()
    else:
        base = t.untyped_storage().data_ptr() + t.storage_offset() * t.element_size()
    return base + offset * t.element_size()


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


# ----------------------------------------------------------- parameters

def param_layout(latent: int = LATENT, layers: int = LAYERS) -> List[Tuple[str, Tuple[int, ...], int]]:
    """(name, shape, offset) of every tensor in the flat parameter vector;
    weights are (out, in) row-major, offsets multiples of 8 elements."""
    entries: List[Tuple[str, Tuple[int, ...]]] = []

    def mlp(prefix: str, kin: int, kout: int) -> None:
        entries.extend([(f"{prefix}.w1", (latent, kin)), (f"{prefix}.b1", (latent,)),
                        (f"{prefix}.w2", (kout, latent)), (f"{prefix}.b2", (kout,))])

    mlp("enc_n", NODE_IN, latent)
    mlp("enc_e", EDGE_IN, latent)
    for l in range(layers):
        mlp(f"edge{l}", 3 * latent, latent)
        mlp(f"node{l}", 2 * latent, latent)
    mlp("dec", latent, OUT)
    out, off = [], 0
    for name, shape in entries:
        out.append((name, shape, off))
        off += (int(np.prod(shape)) + 7) // 8 * 8
    return out


def param_count(latent: int = LATENT, layers: int = LAYERS) -> int:
    name, shape, off = param_layout(latent, layers)[-1]
    return off + (int(np.prod(shape)) + 7) // 8 * 8


def init_params(seed: int, latent: int = LATENT, layers: int = LAYERS) -> np.ndarray:
    """He-uniform first layers, 0.1-scaled second layers of the residual
    MLPs, zero biases, zero unused decoder rows (float32)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(param_count(latent, layers), np.float32)
    for name, shape, off in param_layout(latent, layers):
        if name.endswith(".b1") or name.endswith(".b2"):
            continue
        kin = shape[1]
        bound = math.sqrt(6.0 / kin)
        if name.endswith(".w2") and (name.startswith("edge") or name.startswith("node") or name.startswith("dec")):
            bound *= 0.1
        w = rng.uniform(-bound, bound, size=shape).astype(np.float32)
        if name == "dec.w2":
            w[OUT_USED:] = 0.0
        p[off:off + w.size] = w.reshape(-1)
    return p


def bf16_round(x: np.ndarray) -> np.ndarray:
    """float32 -> nearest bfloat16 (ties to even), returned as float32."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


# ---------------------------------------------------------------- graph

@dataclass
class Graph:
    n: int
    E: int
    row_off: torch.Tensor      # int32 (n+1): CSR by receiver
    dst: torch.Tensor          # int32 (E)
    src: torch.Tensor          # int32 (E)
    efeat: torch.Tensor        # bf16 (E, 16)
    src_perm: Optional[torch.Tensor]   # int32 (E): edges ordered by sender (backward only)
    src_off: Optional[torch.Tensor]    # int32 (n+1)


def make_grid(lo, hi, d_max: float) -> SgGrid:
    """Cells of edge 1.5 d_max covering [lo, hi] with one cell of margin."""
    cut = CUTOFF_FACTOR * d_max
    g = SgGrid()
    dims = []
    for a in range(3):
        g.lo[a] = float(lo[a]) - cut
        dims.append(max(1, int(math.floor((float(hi[a]) - float(lo[a]) + 2 * cut) / cut)) + 1))
    g.cell = cut
    g.cutoff = cut
    g.scale = float(d_max)
    for a in range(3):
        g.dim[a] = dims[a]
    return g


def build_graph(posR: torch.Tensor, grid: SgGrid, sender_order: bool = True) -> Graph:
    """Neighbour graph of the spheres in posR (cuda float64, n x 4); the
    sender-ordered permutation (needed by the backward pass only) is built
    when sender_order is set."""
    lib = load()
    n = posR.shape[0]
    dev = posR.device
    s = _stream()
    ncell = grid.dim[0] * grid.dim[1] * grid.dim[2]
    cell = torch.empty(n, dtype=torch.int32, device=dev)
    _check(lib.sdem_sg_cells(n, _ptr(posR), C.byref(grid), _ptr(cell), s), "sdem_sg_cells")
    key = cell.to(torch.int64) * max(n, 1) + torch.arange(n, device=dev, dtype=torch.int64)
    sorted_idx = torch.argsort(key).to(torch.int32)
    counts = torch.bincount(cell.to(torch.int64), minlength=ncell)
    cell_start = torch.zeros(ncell + 1, dtype=torch.int32, device=dev)
    cell_start[1:] = torch.cumsum(counts, 0).to(torch.int32)
    degree = torch.empty(n, dtype=torch.int32, device=dev)
    _check(lib.sdem_sg_edge_count(n, _ptr(posR), C.byref(grid), _ptr(cell), _ptr(cell_start), _ptr(sorted_idx),
                                  _ptr(degree), s), "sdem_sg_edge_count")
    csum = torch.cumsum(degree.to(torch.int64), 0)
    E = int(csum[-1].item()) if n else 0
    if E > 2**31 - 1:
        # the CSR offsets and edge indices are int32 on the device
        raise RuntimeError(f"{E} edges: more than the int32 offsets of the graph can address")
    row_off = torch.zeros(n + 1, dtype=torch.int32, device=dev)
    row_off[1:] = csum.to(torch.int32)
    # at least one row: an empty tensor has a null data pointer, which the
    # library refuses even when there is nothing to write
    dst = torch.empty(max(E, 1), dtype=torch.int32, device=dev)[:E]
    src = torch.empty(max(E, 1), dtype=torch.int32, device=dev)[:E]
    efeat = torch.empty((max(E, 1), EDGE_IN), dtype=torch.bfloat16, device=dev)
    _check(lib.sdem_sg_edge_fill(n, _ptr(posR), C.byref(grid), _ptr(cell), _ptr(cell_start), _ptr(sorted_idx),
                                 _ptr(row_off), _ptr(dst), _ptr(src), _ptr(efeat), s), "sdem_sg_edge_fill")
    src_perm = src_off = None
    if sender_order:
        skey = src.to(torch.int64) * max(E, 1) + torch.arange(E, device=dev, dtype=torch.int64)
        src_perm = torch.argsort(skey).to(torch.int32)
        src_off = torch.zeros(n + 1, dtype=torch.int32, device=dev)
        src_off[1:] = torch.cumsum(torch.bincount(src.to(torch.int64), minlength=n), 0).to(torch.int32)
    return Graph(n, E, row_off, dst, src, efeat[:E], src_perm, src_off)


def node_features(posR: torch.Tensor, vel: torch.Tensor, omega: torch.Tensor, planes: torch.Tensor, d_max: float,
                  vscale: float) -> torch.Tensor:
    """bf16 (n, 32) node features; vel (3, n, 3) frames, planes (nw, 4)."""
    lib = load()
    n = posR.shape[0]
    out = torch.empty((max(n, 1), NODE_IN), dtype=torch.bfloat16, device=posR.device)
    _check(lib.sdem_sg_node_features(n, _ptr(posR), _ptr(vel), _ptr(omega), int(planes.shape[0]), _ptr(planes),
                                     float(d_max), float(vscale), DCLIP, _ptr(out), _stream()),
           "sdem_sg_node_features")
    return out[:n]


def planes_of(walls) -> np.ndarray:
    """(nw, 4) plane normals and offsets (n.x + d) of a WallSet."""
    return np.array([[w[12], w[13], w[14], w[15]] for w in walls.walls], dtype=np.float64).reshape(-1, 4)


def box_of(walls) -> SgBox:
    """The axis-aligned walls of a WallSet as the box that holds the spheres
    in a surrogate stride: a plane n.x + d = 0 with n = +e_a (spheres on its
    positive side) bounds x_a from below at -d, with n = -e_a from above at d;
    open sides get -/+1e300."""
    b = SgBox()
    for a in range(3):
        b.lo[a], b.hi[a] = -1e300, 1e300
    for nx, ny, nz, d in planes_of(walls):
        nrm = (nx, ny, nz)
        for a in range(3):
            if nrm[a] > 0.999999:
                b.lo[a] = max(b.lo[a], -d / nrm[a])
            elif nrm[a] < -0.999999:
                b.hi[a] = min(b.hi[a], d / -nrm[a])
    return b


def align_frames(ids_now: np.ndarray, ids_old: np.ndarray, v_old: np.ndarray, v_now: np.ndarray) -> np.ndarray:
    """The velocities of the spheres `ids_now` in an older frame (ids_old,
    v_old); a sphere absent there keeps its current velocity (v_now)."""
    out = np.array(v_now, dtype=np.float64, copy=True)
    if len(ids_old) == 0 or len(ids_now) == 0:
        return out
    order = np.argsort(ids_old, kind="stable")
    pos = np.clip(np.searchsorted(ids_old[order], ids_now), 0, len(ids_old) - 1)
    hit = ids_old[order][pos] == ids_now
    out[hit] = np.asarray(v_old)[order][pos[hit]]
    return out


# --------------------------------------------------------------- network

class _Op:
    """Builder of an sdem_sg_operand: segments (tensor, element offset, ld,
    width, gather index)."""

    def __init__(self, trans: int, *segs):
        self.o = SgOperand()
        self.o.trans = trans
        self.o.nseg = len(segs)
        self.keep = segs
        for k, (t, off, ld, width, idx) in enumerate(segs):
            self.o.ptr[k] = _ptr(t, off)
            self.o.idx[k] = _ptr(idx) if idx is not None else None
            self.o.ld[k] = ld
            self.o.width[k] = width


def _ep(**kw) -> SgEpilogue:
    e = SgEpilogue()
    for k, v in kw.items():
        if isinstance(v, torch.Tensor):
            v = _ptr(v)
        setattr(e, k, v)
    return e


class Network:
    """Parameters (fp32 master + bf16 copy), forward, backward and Adam of
    the surrogate network on one CUDA device."""

    def __init__(self, seed: int = 0, device: str = "cuda", latent: int = LATENT, layers: int = LAYERS,
                 params: Optional[np.ndarray] = None):
        self.lib = load()
        self.latent, self.layers = latent, layers
        self.layout = {name: (shape, off) for name, shape, off in param_layout(latent, layers)}
        host = init_params(seed, latent, layers) if params is None else np.asarray(params, np.float32)
        self.p = torch.from_numpy(host.copy()).to(device)
        self.pb = torch.empty(self.p.numel(), dtype=torch.bfloat16, device=device)
        self.grad = torch.zeros_like(self.p)
        self.m = torch.zeros_like(self.p)
        self.v = torch.zeros_like(self.p)
        self.step_count = 0
        self.device = device
        self.colsum_partial = torch.empty(self.lib.sdem_sg_colsum_blocks() * 4 * latent, dtype=torch.float32,
                                          device=device)
        self.refresh_bf16()
        self.saved = None

    def refresh_bf16(self) -> None:
        _check(self.lib.sdem_sg_to_bf16(self.p.numel(), _ptr(self.p), _ptr(self.pb), _stream()), "sdem_sg_to_bf16")

    def host_params(self) -> np.ndarray:
        return self.p.cpu().numpy()

    def off(self, name: str) -> int:
        return self.layout[name][1]

    def shape(self, name: str):
        return self.layout[name][0]

    # -- GEMM helpers
    def _gemm(self, I, J, R, a: _Op, b: _Op, ep: SgEpilogue, splits: int = 1, partial=None) -> None:
        _check(self.lib.sdem_sg_gemm(I, J, R, C.byref(a.o), C.byref(b.o), C.byref(ep), splits, _ptr(partial),
                                     _stream()), "sdem_sg_gemm")

    def _w(self, name: str, trans: int) -> _Op:
        kout, kin = self.shape(name)
        return _Op(trans, (self.pb, self.off(name), kin, kin, None))

    def _linear(self, M, a: _Op, name: str, **ep) -> None:
        """act(A W^T + b): A is M x kin (trans 0 segments)."""
        kout, kin = self.shape(name)
        bias = name[:-2] + "b" + name[-1]
        self._gemm(M, kout, kin, a, self._w(name, 0), _ep(bias=_ptr(self.p, self.off(bias)), **ep))

    def _wgrad(self, name: str, R: int, dy: _Op, x: _Op) -> None:
        """grad[name] += dY^T X over R rows (dy, x: trans 1 operands)."""
        kout, kin = self.shape(name)
        gx, gy = (kout + 63) // 64, (kin + 63) // 64
        splits = max(1, min(R // 256, 608 // (gx * gy)))
        partial = torch.empty(splits * kout * kin, dtype=torch.float32, device=self.device) if splits > 1 else None
        self._gemm(kout, kin, R, dy, x, _ep(out=_ptr(self.grad, self.off(name)), ld_out=kin, accumulate=1),
                   splits, partial)

    def _dgrad(self, M, dy: _Op, name: str, **ep) -> None:
        """dX = dY W (M x kin)."""
        kout, kin = self.shape(name)
        self._gemm(M, kin, kout, dy, self._w(name, 1), _ep(**ep))

    def _bgrad(self, name: str, M: int, x: torch.Tensor, ldx: int) -> None:
        kout = self.shape(name)[0]
        _check(self.lib.sdem_sg_colsum(M, kout, _ptr(x), ldx, _ptr(self.grad, self.off(name)), 1,
                                       _ptr(self.colsum_partial), _stream()), "sdem_sg_colsum")

    # -- forward
    def forward(self, g: Graph, xn: torch.Tensor, keep: bool = True) -> torch.Tensor:
        """(n, 16) fp32 predictions; keep=True saves what backward needs."""
        L, n, E, dev = self.latent, g.n, g.E, self.device
        bf, f32 = torch.bfloat16, torch.float32
        zb = torch.empty((n, L), dtype=bf, device=dev)
        self._linear(n, _Op(0, (xn, 0, NODE_IN, NODE_IN, None)), "enc_n.w1", relu=1, out_bf=zb, ld_out_bf=L)
        h = torch.empty((n, L), dtype=f32, device=dev)
        hb = torch.empty((n, L), dtype=bf, device=dev)
        self._linear(n, _Op(0, (zb, 0, L, L, None)), "enc_n.w2", out=h, ld_out=L, out_bf=hb, ld_out_bf=L)
        zeb = torch.empty((max(E, 1), L), dtype=bf, device=dev)
        self._linear(E, _Op(0, (g.efeat, 0, EDGE_IN, EDGE_IN, None)), "enc_e.w1", relu=1, out_bf=zeb, ld_out_bf=L)
        e = torch.empty((max(E, 1), L), dtype=f32, device=dev)
        eb = torch.empty((max(E, 1), L), dtype=bf, device=dev)
        self._linear(E, _Op(0, (zeb, 0, L, L, None)), "enc_e.w2", out=e, ld_out=L, out_bf=eb, ld_out_bf=L)
        saved = {"xn": xn, "zb_enc": zb, "zeb_enc": zeb, "hb": [hb], "eb": [eb], "ze": [], "zn": [], "agg": []}
        m = torch.empty((max(E, 1), L), dtype=f32, device=dev)
        for l in range(self.layers):
            ze = torch.empty((max(E, 1), L), dtype=bf, device=dev)
            a_in = _Op(0, (hb, 0, L, L, g.dst), (hb, 0, L, L, g.src), (eb, 0, L, L, None))
            self._linear(E, a_in, f"edge{l}.w1", relu=1, out_bf=ze, ld_out_bf=L)
            e2 = torch.empty_like(e)
            eb2 = torch.empty_like(eb)
            self._linear(E, _Op(0, (ze, 0, L, L, None)), f"edge{l}.w2", out=m, ld_out=L, resid=e, ld_resid=L,
                         res_out=e2, ld_res_out=L, res_out_bf=eb2, ld_res_out_bf=L)
            aggb = torch.empty((n, L), dtype=bf, device=dev)
            _check(self.lib.sdem_sg_segsum(n, L, _ptr(g.row_off), None, _ptr(m), L, None, L, 0, _ptr(aggb), L,
                                           _stream()), "sdem_sg_segsum")
            zn = torch.empty((n, L), dtype=bf, device=dev)
            self._linear(n, _Op(0, (hb, 0, L, L, None), (aggb, 0, L, L, None)), f"node{l}.w1", relu=1, out_bf=zn,
                         ld_out_bf=L)
            h2 = torch.empty_like(h)
            hb2 = torch.empty_like(hb)
            self._linear(n, _Op(0, (zn, 0, L, L, None)), f"node{l}.w2", resid=h, ld_resid=L, res_out=h2,
                         ld_res_out=L, res_out_bf=hb2, ld_res_out_bf=L)
            if keep:
                saved["ze"].append(ze)
                saved["zn"].append(zn)
                saved["agg"].append(aggb)
                saved["hb"].append(hb2)
                saved["eb"].append(eb2)
            h, hb, e, eb = h2, hb2, e2, eb2
        zd = torch.empty((n, L), dtype=bf, device=dev)
        self._linear(n, _Op(0, (hb, 0, L, L, None)), "dec.w1", relu=1, out_bf=zd, ld_out_bf=L)
        y = torch.empty((n, OUT), dtype=f32, device=dev)
        self._linear(n, _Op(0, (zd, 0, L, L, None)), "dec.w2", out=y, ld_out=OUT)
        saved["zd"] = zd
        self.saved = saved if keep else None
        self.graph = g if keep else None
        return y

    def loss(self, y: torch.Tensor, target: torch.Tensor):
        """(mse, dy fp32, dy bf16) of predictions against (n, 6) targets."""
        n = y.shape[0]
        rowerr = torch.empty(n, dtype=torch.float32, device=self.device)
        dy = torch.empty((n, OUT), dtype=torch.float32, device=self.device)
        dyb = torch.empty((n, OUT), dtype=torch.bfloat16, device=self.device)
        _check(self.lib.sdem_sg_mse(n, OUT_USED, _ptr(y), OUT, _ptr(target), _ptr(rowerr), _ptr(dy), _ptr(dyb),
                                    _stream()), "sdem_sg_mse")
        return rowerr.sum() / (n * OUT_USED), dy, dyb

    # -- backward
    def backward(self, dy: torch.Tensor, dyb: torch.Tensor) -> None:
        """Accumulates d loss / d params into self.grad (zero it first)."""
        s, g = self.saved, self.graph
        if s is None:
            raise RuntimeError("backward needs a forward with keep=True")
        if g.src_perm is None:
            raise RuntimeError("backward needs a graph built with sender_order=True")
        L, n, E, dev = self.latent, g.n, g.E, self.device
        bf, f32 = torch.bfloat16, torch.float32
        lib = self.lib
        # decoder
        self._wgrad("dec.w2", n, _Op(1, (dyb, 0, OUT, OUT, None)), _Op(1, (s["zd"], 0, L, L, None)))
        self._bgrad("dec.b2", n, dy, OUT)
        dz = torch.empty((n, L), dtype=f32, device=dev)
        dzb = torch.empty((n, L), dtype=bf, device=dev)
        self._dgrad(n, _Op(0, (dyb, 0, OUT, OUT, None)), "dec.w2", mask=s["zd"], ld_mask=L, out=dz, ld_out=L,
                    out_bf=dzb, ld_out_bf=L)
        hb6 = s["hb"][-1]
        self._wgrad("dec.w1", n, _Op(1, (dzb, 0, L, L, None)), _Op(1, (hb6, 0, L, L, None)))
        self._bgrad("dec.b1", n, dz, L)
        dh = torch.empty((n, L), dtype=f32, device=dev)
        dhb = torch.empty((n, L), dtype=bf, device=dev)
        self._dgrad(n, _Op(0, (dzb, 0, L, L, None)), "dec.w1", out=dh, ld_out=L, out_bf=dhb, ld_out_bf=L)
        de = torch.zeros((max(E, 1), L), dtype=f32, device=dev)
        din_n = torch.empty((n, 2 * L), dtype=f32, device=dev)
        din_e = torch.empty((max(E, 1), 3 * L), dtype=f32, device=dev)
        dm = torch.empty((max(E, 1), L), dtype=f32, device=dev)
        dmb = torch.empty((max(E, 1), L), dtype=bf, device=dev)
        dze = torch.empty((max(E, 1), L), dtype=f32, device=dev)
        dzeb = torch.empty((max(E, 1), L), dtype=bf, device=dev)
        for l in reversed(range(self.layers)):
            hb_prev, eb_prev = s["hb"][l], s["eb"][l]
            zn, ze, aggb = s["zn"][l], s["ze"][l], s["agg"][l]
            # node MLP: h_l = h_{l-1} + W2 relu(W1 [h, agg] + b1) + b2
            self._wgrad(f"node{l}.w2", n, _Op(1, (dhb, 0, L, L, None)), _Op(1, (zn, 0, L, L, None)))
            self._bgrad(f"node{l}.b2", n, dh, L)
            self._dgrad(n, _Op(0, (dhb, 0, L, L, None)), f"node{l}.w2", mask=zn, ld_mask=L, out=dz, ld_out=L,
                        out_bf=dzb, ld_out_bf=L)
            self._wgrad(f"node{l}.w1", n, _Op(1, (dzb, 0, L, L, None)),
                        _Op(1, (hb_prev, 0, L, L, None), (aggb, 0, L, L, None)))
            self._bgrad(f"node{l}.b1", n, dz, L)
            self._dgrad(n, _Op(0, (dzb, 0, L, L, None)), f"node{l}.w1", out=din_n, ld_out=2 * L)
            dh_prev = torch.empty_like(dh)
            _check(lib.sdem_sg_gather_add(n, L, None, _ptr(din_n), 2 * L, _ptr(dh), L, _ptr(dh_prev), L, None, L,
                                          _stream()), "sdem_sg_gather_add")
            # messages: dm = de_l + dagg[dst]
            _check(lib.sdem_sg_gather_add(E, L, _ptr(g.dst), _ptr(din_n, L), 2 * L, _ptr(de), L, _ptr(dm), L,
                                          _ptr(dmb), L, _stream()), "sdem_sg_gather_add")
            # edge MLP: m = W2 relu(W1 [h_dst, h_src, e] + b1) + b2
            self._wgrad(f"edge{l}.w2", E, _Op(1, (dmb, 0, L, L, None)), _Op(1, (ze, 0, L, L, None)))
            self._bgrad(f"edge{l}.b2", E, dm, L)
            self._dgrad(E, _Op(0, (dmb, 0, L, L, None)), f"edge{l}.w2", mask=ze, ld_mask=L, out=dze, ld_out=L,
                        out_bf=dzeb, ld_out_bf=L)
            self._wgrad(f"edge{l}.w1", E, _Op(1, (dzeb, 0, L, L, None)),
                        _Op(1, (hb_prev, 0, L, L, g.dst), (hb_prev, 0, L, L, g.src), (eb_prev, 0, L, L, None)))
            self._bgrad(f"edge{l}.b1", E, dze, L)
            self._dgrad(E, _Op(0, (dzeb, 0, L, L, None)), f"edge{l}.w1", out=din_e, ld_out=3 * L)
            de_prev = torch.empty_like(de)
            _check(lib.sdem_sg_gather_add(E, L, None, _ptr(din_e, 2 * L), 3 * L, _ptr(de), L, _ptr(de_prev), L, None,
                                          L, _stream()), "sdem_sg_gather_add")
            _check(lib.sdem_sg_segsum(n, L, _ptr(g.row_off), None, _ptr(din_e), 3 * L, _ptr(dh_prev), L, 1, None, L,
                                      _stream()), "sdem_sg_segsum")
            _check(lib.sdem_sg_segsum(n, L, _ptr(g.src_off), _ptr(g.src_perm), _ptr(din_e, L), 3 * L, _ptr(dh_prev),
                                      L, 1, _ptr(dhb), L, _stream()), "sdem_sg_segsum")
            dh, de = dh_prev, de_prev
        # encoders
        self._wgrad("enc_n.w2", n, _Op(1, (dhb, 0, L, L, None)), _Op(1, (s["zb_enc"], 0, L, L, None)))
        self._bgrad("enc_n.b2", n, dh, L)
        self._dgrad(n, _Op(0, (dhb, 0, L, L, None)), "enc_n.w2", mask=s["zb_enc"], ld_mask=L, out=dz, ld_out=L,
                    out_bf=dzb, ld_out_bf=L)
        self._wgrad("enc_n.w1", n, _Op(1, (dzb, 0, L, L, None)), _Op(1, (s["xn"], 0, NODE_IN, NODE_IN, None)))
        self._bgrad("enc_n.b1", n, dz, L)
        deb = torch.empty((max(E, 1), L), dtype=bf, device=dev)
        _check(lib.sdem_sg_to_bf16(E * L, _ptr(de), _ptr(deb), _stream()), "sdem_sg_to_bf16")
        self._wgrad("enc_e.w2", E, _Op(1, (deb, 0, L, L, None)), _Op(1, (s["zeb_enc"], 0, L, L, None)))
        self._bgrad("enc_e.b2", E, de, L)
        self._dgrad(E, _Op(0, (deb, 0, L, L, None)), "enc_e.w2", mask=s["zeb_enc"], ld_mask=L, out=dze, ld_out=L,
                    out_bf=dzeb, ld_out_bf=L)
        self._wgrad("enc_e.w1", E, _Op(1, (dzeb, 0, L, L, None)), _Op(1, (g.efeat, 0, EDGE_IN, EDGE_IN, None)))
        self._bgrad("enc_e.b1", E, dze, L)

    def adam(self, lr: float = 1e-3, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8,
             weight_decay: float = 0.0) -> None:
        self.step_count += 1
        _check(self.lib.sdem_sg_adam(self.p.numel(), _ptr(self.p), _ptr(self.grad), _ptr(self.m), _ptr(self.v),
                                     _ptr(self.pb), lr, beta1, beta2, eps, weight_decay, self.step_count, _stream()),
               "sdem_sg_adam")

    def train_step(self, g: Graph, xn: torch.Tensor, target: torch.Tensor, lr: float = 1e-3) -> torch.Tensor:
        self.grad.zero_()
        y = self.forward(g, xn, keep=True)
        loss, dy, dyb = self.loss(y, target)
        self.backward(dy, dyb)
        self.adam(lr)
        self.saved = None
        return loss


# --------------------------------------------------------------- samples

@dataclass
class Sample:
    """One training frame: state at t, the two earlier velocity frames and
    the stride-mean accelerations over (t, t + S) as targets."""
    posR: np.ndarray      # (n, 4)
    vel: np.ndarray       # (3, n, 3): v(t), v(t-S), v(t-2S)
    omega: np.ndarray     # (n, 3)
    target: np.ndarray    # (n, 6) float32


def targets(v0, v1, w0, w1, r, h: float, gravity) -> np.ndarray:
    """((v1 - v0)/h - g)/|g| and ((w1 - w0)/h) r/|g|, float32 (n, 6)."""
    gm = float(np.linalg.norm(gravity))
    a = ((v1 - v0) / h - np.asarray(gravity)[None, :]) / gm
    al = (w1 - w0) / h * r[:, None] / gm
    return np.concatenate([a, al], axis=1).astype(np.float32)


def _frame(system):
    st = system.state()
    return st.posR.copy(), st.linVel[:, 0, :].copy(), st.rotVel[:, 0, :].copy(), st.id.copy()


def record_samples(system, case, stride: int, frames: int, settle: int = 0) -> List[Sample]:
    """Runs the plain DEM (a DEMSystem of `case`) and turns consecutive
    stride frames into samples (frames - 3 of them)."""
    if settle:
        system.step(settle)
    snaps = []
    for k in range(frames):
        if k:
            system.step(stride)
        snaps.append(_frame(system))
    return samples_from_frames(snaps, case, stride)


def record_samples_batch(systems, cases, stride: int, frames: int, settle: int = 0,
                         group_size: int = 0) -> List[List[Sample]]:
    """record_samples for many beds at once: the plain path's batched form
    (capi.DEMBatch, one captured graph per group of beds) advances all of
    them through the settling and from frame to frame; each bed's frames
    are downloaded between batch steps.  Even step counts keep the batch's
    two-step graphs whole."""
    from .capi import DEMBatch
    if stride % 2 or settle % 2:
        raise ValueError("record_samples_batch: stride and settle must be even")
    b = DEMBatch(systems, group_size=group_size)
    snaps = [[] for _ in systems]
    try:
        if settle:
            b.step(settle)
        for k in range(frames):
            if k:
                b.step(stride)
            for i, s in enumerate(systems):
                snaps[i].append(_frame(s))
    finally:
        b.close()
    return [samples_from_frames(sn, c, stride) for sn, c in zip(snaps, cases)]


def samples_from_frames(snaps, case, stride: int) -> List[Sample]:
    """Samples from consecutive frames (posR, v, omega, id) a stride apart."""
    frames = len(snaps)
    h = stride * case.opts.dt
    out = []
    for k in range(2, frames - 1):
        ids = snaps[k][3]
        if not all(np.array_equal(ids, snaps[j][3]) for j in (k - 2, k - 1, k + 1)):
            continue  # a sphere left the domain in between: the frames do not line up
        posR, v, w = snaps[k][0], snaps[k][1], snaps[k][2]
        vel = np.stack([v, snaps[k - 1][1], snaps[k - 2][1]])
        tgt = targets(v, snaps[k + 1][1], w, snaps[k + 1][2], posR[:, 3], h, case.opts.gravity)
        out.append(Sample(posR, vel, w, tgt))
    return out


@dataclass
class DeviceSample:
    graph: Graph
    xn: torch.Tensor
    target: torch.Tensor


def to_device(sample: Sample, case, d_max: float, vscale: float, device: str = "cuda") -> DeviceSample:
    posR = torch.from_numpy(np.ascontiguousarray(sample.posR)).to(device)
    vel = torch.from_numpy(np.ascontiguousarray(sample.vel)).to(device)
    om = torch.from_numpy(np.ascontiguousarray(sample.omega)).to(device)
    planes = torch.from_numpy(planes_of(case.walls)).to(device)
    grid = make_grid(case.opts.minpoint, case.opts.maxpoint, d_max)
    g = build_graph(posR, grid)
    xn = node_features(posR, vel, om, planes, d_max, vscale)
    return DeviceSample(g, xn, torch.from_numpy(sample.target).to(device))


def evaluate(net: Network, samples: List[DeviceSample]) -> Tuple[float, float]:
    """(network MSE, MSE of the prediction without the network: a = g,
    alpha = 0, i.e. zero output) over the samples, node-weighted."""
    num = den = base = 0.0
    for s in samples:
        y = net.forward(s.graph, s.xn, keep=False)
        loss, _, _ = net.loss(y, s.target)
        n = s.graph.n
        num += float(loss) * n
        base += float((s.target.double() ** 2).mean()) * n
        den += n
    return num / den, base / den


# ----------------------------------------------------------- wall pressure

def wall_pressure(posR: np.ndarray, ptype: np.ndarray, case) -> np.ndarray:
    """Pressure on each plane wall of `case` from the elastic normal forces of
    the spheres that overlap it (the state's static load): for a sphere at
    signed distance s = n.x + d from the wall's plane (|s| for a two-sided
    wall), overlap delta = r - s >= 0 and, for a finite wall, the foot of the
    perpendicular inside the wall's bounding box; the force is
    Kn delta^1.5 (Hertz) or Kn 0.01^0.4 delta (the reference's LSD stiffness
    at its lowest contact speed), Kn of the (wall type, sphere type) pair
    (Prtcl_Property.f90:200-247), and the pressure their sum over the wall's
    area |(p2 - p1) x (p4 - p1)|.  (nw,) float64 in Pa."""
    from . import props
    walls, flags = case.walls.arrays()
    nw = case.walls.n
    out = np.zeros(nw)
    if nw == 0 or len(posR) == 0:
        return out
    W = walls.reshape(nw, -1)
    F = flags.reshape(nw, -1)
    nT = case.tables.n_types
    bpw = case.tables.bpw.reshape(-1, nT, props.BP_SIZE)
    x, r = posR[:, :3], posR[:, 3]
    for k in range(nw):
        n, d = W[k, 12:15], W[k, 15]
        s = x @ n + d
        if F[k, 0]:
            s = np.abs(s)
        delta = r - s
        on = (delta >= 0.0) & (s >= 0.0)
        if not F[k, 1]:   # finite wall: the foot of the perpendicular inside its box
            foot = x - s[:, None] * n[None, :]
            lo, hi = W[k, 19:22] - 1e-12, W[k, 22:25] + 1e-12
            on &= np.all((foot >= lo) & (foot <= hi), axis=1)
        if not on.any():
            continue
        kn = np.abs(bpw[F[k, 3] - 1, ptype[on] - 1, 2])
        dl = delta[on]
        f = kn * (dl * np.sqrt(dl) if case.opts.cf_type == props.CFT_NLIN else 0.01 ** 0.4 * dl)
        p1, p2, p4 = W[k, 0:3], W[k, 3:6], W[k, 9:12]
        area = float(np.linalg.norm(np.cross(p2 - p1, p4 - p1)))
        out[k] = float(f.sum()) / area
    return out


def pressure_error(p: np.ndarray, ref: np.ndarray) -> float:
    """Mean over the walls that carry load in `ref` of |p - ref| / ref (0 when
    no wall carries load)."""
    loaded = ref > 0.0
    if not loaded.any():
        return 0.0
    return float(np.mean(np.abs(p[loaded] - ref[loaded]) / ref[loaded]))


# --------------------------------------------------------------- rollout

class Diverged(RuntimeError):
    """The surrogate's state has collapsed: its neighbour graph outgrew the
    limit set from the last plain-DEM state."""


class SurrogateRunner:
    """Advances a bed by surrogate strides with a plain-DEM judge.

    Every `judge_every` surrogate strides the plain DEM re-advances one
    stride from the surrogate's state; between that stride and the
    surrogate's own stride from the same state, the relative bed-height
    difference (mean sphere height above the floor, over the spheres both
    keep) and the mean relative wall-pressure difference (wall_pressure of
    either end state, over the walls the plain state loads) are the errors.
    Within both bounds the run continues from the plain DEM's state; above
    either, or when the plain stride fails (a state the DEM rejects), the
    last state the plain DEM produced is restored (simulated time rewinds to
    it) and the plain DEM advances the next `fallback_strides` strides
    itself.  Spheres the plain DEM deletes (out of the domain) leave the
    surrogate's state with it; velocity frames are matched by sphere id.
    A surrogate stride whose graph has more than `edge_growth` times the
    edges of the first graph after the last plain state counts as a failed
    judgement too (spheres interpenetrating without the contact repulsion
    the network has not learned: the graph and its memory would grow
    without bound)."""

    def __init__(self, net: Network, system, case, stride: int, d_max: float, vscale: float,
                 judge_every: int = 20, bound: float = 0.02, fallback_strides: int = 20, edge_growth: float = 3.0,
                 pressure_bound: float = 0.05):
        self.net, self.sys, self.case = net, system, case
        self.edge_growth = edge_growth
        self.edge_ref = None
        self.stride, self.d_max, self.vscale = stride, d_max, vscale
        self.judge_every, self.bound, self.fallback = judge_every, bound, fallback_strides
        self.pressure_bound = pressure_bound
        self.h = stride * case.opts.dt
        self.grid = make_grid(case.opts.minpoint, case.opts.maxpoint, d_max)
        self.planes = torch.from_numpy(planes_of(case.walls)).to(net.device)
        self.box = box_of(case.walls)
        self.floor = float(case.opts.minpoint[1])
        self.t = 0                    # strides of simulated time since the start
        self.since_judge = 0
        self.stats = {"surrogate_strides": 0, "dem_strides": 0, "judged": 0, "fallbacks": 0, "rewound_strides": 0,
                      "diverged": 0, "errors": [], "pressure_errors": []}
        self._seed_from_dem()

    def _dem_stride(self) -> None:
        self.sys.step(self.stride)
        self.stats["dem_strides"] += 1
        self.t += 1

    def _adopt(self, st, vframes) -> None:
        dev = self.net.device
        self.parts, self.good, self.good_t = st, st, self.t
        self.edge_ref = None
        self.since_judge = 0
        self.posR = torch.from_numpy(np.ascontiguousarray(st.posR)).to(dev)
        self.vel = torch.from_numpy(np.ascontiguousarray(np.stack(vframes))).to(dev)
        self.omega = torch.from_numpy(np.ascontiguousarray(st.rotVel[:, 0, :])).to(dev)

    def _seed_from_dem(self) -> None:
        """Two plain strides; the three frames (matched by id) seed the state."""
        frames = [self.sys.state()]
        for _ in range(2):
            self._dem_stride()
            frames.append(self.sys.state())
        st = frames[-1]
        v = st.linVel[:, 0, :]
        self._adopt(st, [v] + [align_frames(st.id, f.id, f.linVel[:, 0, :], v) for f in (frames[1], frames[0])])

    def bed_height(self, posR: torch.Tensor) -> float:
        return float((posR[:, 1] - self.floor).mean())

    def _surrogate_stride(self, posR, vel, omega) -> None:
        g = build_graph(posR, self.grid, sender_order=False)
        if self.edge_ref is None:
            self.edge_ref = max(g.E, 1)
        elif g.E > self.edge_growth * self.edge_ref:
            raise Diverged(f"{g.E} edges against {self.edge_ref} after the last plain state")
        xn = node_features(posR, vel, omega, self.planes, self.d_max, self.vscale)
        y = self.net.forward(g, xn, keep=False)
        gx, gy, gz = self.case.opts.gravity
        _check(self.net.lib.sdem_sg_advance(posR.shape[0], _ptr(y), OUT, float(np.linalg.norm(self.case.opts.gravity)),
                                            gx, gy, gz, self.h, C.byref(self.box), _ptr(posR), _ptr(vel), _ptr(omega),
                                            _stream()), "sdem_sg_advance")

    def _upload(self) -> None:
        """The surrogate state into the plain DEM (contact history restarts)."""
        p = self.parts.copy()
        p.posR[:] = self.posR.cpu().numpy()
        v = self.vel[0].cpu().numpy()
        w = self.omega.cpu().numpy()
        for k in range(p.linVel.shape[1]):
            p.linVel[:, k, :] = v
            p.linAcc[:, k, :] = np.asarray(self.case.opts.gravity)[None, :]
        for k in range(p.rotVel.shape[1]):
            p.rotVel[:, k, :] = w
            p.rotAcc[:, k, :] = 0.0
        self.sys.upload(p)

    def _fall_back(self, rewind: bool) -> None:
        """Restores the last plain state (rewind) or keeps the plain DEM's
        current one, then lets the plain DEM advance `fallback_strides`."""
        self.stats["fallbacks"] += 1
        if rewind:
            self.sys.upload(self.good)
            self.stats["rewound_strides"] += self.t - self.good_t
            self.t = self.good_t
        for _ in range(self.fallback):
            self._dem_stride()
        self._seed_from_dem()

    def _judged_stride(self) -> None:
        ids = self.parts.id
        self._upload()
        p2 = self.posR.clone()
        self._surrogate_stride(p2, self.vel.clone(), self.omega.clone())
        try:
            self._dem_stride()
            st = self.sys.state()
        except Exception:       # the plain DEM rejected the surrogate's state
            st = None
        self.stats["judged"] += 1
        self.stats["surrogate_strides"] += 1
        if st is None:
            err = perr = math.inf
        else:
            p_sur = p2.cpu().numpy()
            keep = np.isin(ids, st.id)
            h_sur = float((p_sur[keep, 1] - self.floor).mean())
            h_dem = float((st.posR[:, 1] - self.floor).mean())
            err = abs(h_sur - h_dem) / max(abs(h_dem), 1e-300)
            perr = pressure_error(wall_pressure(p_sur, self.parts.ptype, self.case),
                                  wall_pressure(st.posR, st.ptype, self.case))
        self.stats["errors"].append(err)
        self.stats["pressure_errors"].append(perr)
        if err > self.bound or perr > self.pressure_bound:
            self._fall_back(rewind=st is None)
        else:
            v = st.linVel[:, 0, :]
            vprev = self.vel.cpu().numpy()
            self._adopt(st, [v, align_frames(st.id, ids, vprev[0], v), align_frames(st.id, ids, vprev[1], v)])

    def run(self, strides: int) -> dict:
        """Advances the bed by at least `strides` strides of simulated time."""
        target = self.t + strides
        while self.t < target:
            self.since_judge += 1
            try:
                if self.since_judge % self.judge_every == 0:
                    self._judged_stride()
                    continue
                self._surrogate_stride(self.posR, self.vel, self.omega)
            except Diverged:
                self.stats["diverged"] += 1
                self._fall_back(rewind=True)
                continue
            self.stats["surrogate_strides"] += 1
            self.t += 1
        return self.stats
