"""A numpy statement of the C ABI of include/sdem_surrogate.h that works on
raw host pointers (test infrastructure).

It lets the host orchestration of sdem_gb300.surrogate (operand segments,
gather indices, strides, offsets, epilogue choices, the order of the
backward pass) run on CPU tensors against the oracle without a GPU: each
entry point reads and writes the memory its pointers name, with the
semantics the header states.  Graph entry points delegate to the oracle's
brute-force graph."""
from __future__ import annotations

import ctypes as C

import numpy as np

from oracle import surrogate_ref as ref
from sdem_gb300.surrogate import bf16_round


def _flat(ptr, dtype, count):
    dtype = np.dtype(dtype)
    if count <= 0 or not ptr:
        return np.zeros(0, dtype)
    buf = (C.c_char * (count * dtype.itemsize)).from_address(ptr)
    return np.frombuffer(buf, dtype=dtype, count=count)


def _mat(ptr, dtype, rows, cols, ld):
    """Writable (rows, cols) view of row-major memory with row stride ld."""
    if rows == 0 or cols == 0:
        return np.zeros((rows, cols), dtype)
    flat = _flat(ptr, dtype, (rows - 1) * ld + cols)
    it = np.dtype(dtype).itemsize
    return np.lib.stride_tricks.as_strided(flat, shape=(rows, cols), strides=(ld * it, it))


def _bf_dec(u16):
    return (np.asarray(u16, np.uint16).astype(np.uint32) << 16).view(np.float32)


def _bf_enc(x):
    return (bf16_round(np.asarray(x, np.float32)).view(np.uint32) >> 16).astype(np.uint16)


def _obj(ref_arg):
    return ref_arg._obj if hasattr(ref_arg, "_obj") else ref_arg


class SgMock:
    def sdem_sg_colsum_blocks(self):
        return 160

    # -- graph
    def _graph(self, n, posR, g):
        pos = _mat(posR, np.float64, n, 4, 4).copy()
        return pos, ref.graph(pos, list(g.lo), g.cell, g.cutoff, g.scale, list(g.dim))

    def sdem_sg_cells(self, n, posR, g, cell, stream):
        g = _obj(g)
        pos = _mat(posR, np.float64, n, 4, 4)
        c = ref.cells(pos, list(g.lo), g.cell, list(g.dim))
        _flat(cell, np.int32, n)[:] = (c[:, 2] * g.dim[1] + c[:, 1]) * g.dim[0] + c[:, 0]
        return 0

    def sdem_sg_edge_count(self, n, posR, g, cell, cell_start, sorted_idx, degree, stream):
        _, (row_off, dst, src, ef) = self._graph(n, posR, _obj(g))
        _flat(degree, np.int32, n)[:] = np.diff(row_off)
        return 0

    def sdem_sg_edge_fill(self, n, posR, g, cell, cell_start, sorted_idx, row_off, dst, src, efeat, stream):
        if n and not (posR and cell and cell_start and sorted_idx and row_off and dst and src and efeat):
            return 1          # SDEM_SG_E_ARG, as the library
        _, (ro, d, s, ef) = self._graph(n, posR, _obj(g))
        assert np.array_equal(_flat(row_off, np.int32, n + 1), ro)
        E = len(d)
        _flat(dst, np.int32, E)[:] = d
        _flat(src, np.int32, E)[:] = s
        _mat(efeat, np.uint16, E, 16, 16)[:] = _bf_enc(ef)
        return 0

    def sdem_sg_node_features(self, n, posR, vel, omega, nw, planes, scale, vscale, dclip, nfeat, stream):
        pos = _mat(posR, np.float64, n, 4, 4)
        v = _flat(vel, np.float64, 9 * n).reshape(3, n, 3)
        w = _mat(omega, np.float64, n, 3, 3)
        pl = _mat(planes, np.float64, nw, 4, 4)
        _mat(nfeat, np.uint16, n, 32, 32)[:] = _bf_enc(ref.node_features(pos, v, w, pl, scale, vscale))
        return 0

    # -- GEMM
    def _operand(self, op, rows, cover):
        """(rows, cover) float64 logical matrix of an operand."""
        parts = []
        assert all(op.ptr[s] for s in range(op.nseg)), "null operand pointer"
        for s in range(op.nseg):
            idx = _flat(op.idx[s], np.int32, rows) if op.idx[s] else np.arange(rows)
            nsrc = int(idx.max()) + 1 if rows else 0
            m = _mat(op.ptr[s], np.uint16, nsrc, op.width[s], op.ld[s])
            parts.append(_bf_dec(m[idx]).astype(np.float64))
        out = np.concatenate(parts, axis=1)
        assert out.shape == (rows, cover)
        return out

    def sdem_sg_gemm(self, I, J, R, a, b, ep, splits, partial, stream):
        a, b, ep = _obj(a), _obj(b), _obj(ep)
        if I == 0 or J == 0:
            return 0
        A = self._operand(a, R, I).T if a.trans else self._operand(a, I, R)
        B = self._operand(b, R, J).T if b.trans else self._operand(b, J, R)
        v = (A @ B.T).astype(np.float32)
        if splits > 1:
            assert not (ep.bias or ep.relu or ep.mask or ep.out_bf or ep.resid)
        if ep.bias:
            v = v + _flat(ep.bias, np.float32, J)[None, :]
        if ep.relu:
            v = np.maximum(v, np.float32(0))
        if ep.mask:
            mk = _mat(ep.mask, np.uint16, I, J, ep.ld_mask)
            v = np.where(((mk & 0x8000) == 0) & ((mk & 0x7FFF) != 0), v, np.float32(0))
        if ep.out:
            o = _mat(ep.out, np.float32, I, J, ep.ld_out)
            o[:] = o + v if ep.accumulate else v
        if ep.out_bf:
            _mat(ep.out_bf, np.uint16, I, J, ep.ld_out_bf)[:] = _bf_enc(v)
        if ep.resid:
            w = _mat(ep.resid, np.float32, I, J, ep.ld_resid) + v
            if ep.res_out:
                _mat(ep.res_out, np.float32, I, J, ep.ld_res_out)[:] = w
            if ep.res_out_bf:
                _mat(ep.res_out_bf, np.uint16, I, J, ep.ld_res_out_bf)[:] = _bf_enc(w)
        return 0

    # -- reductions and elementwise
    def sdem_sg_segsum(self, nrows, J, row_off, perm, x, ldx, out, ld_out, accumulate, out_bf, ld_out_bf, stream):
        ro = _flat(row_off, np.int32, nrows + 1)
        E = int(ro[-1])
        order = _flat(perm, np.int32, E) if perm else np.arange(E)
        xs = _mat(x, np.float32, E, J, ldx)[order] if E else np.zeros((0, J), np.float32)
        s = np.zeros((nrows, J), np.float32)
        for i in range(nrows):
            s[i] = xs[ro[i]:ro[i + 1]].sum(axis=0)
        if accumulate:
            s = _mat(out, np.float32, nrows, J, ld_out) + s
        if out:
            _mat(out, np.float32, nrows, J, ld_out)[:] = s
        if out_bf:
            _mat(out_bf, np.uint16, nrows, J, ld_out_bf)[:] = _bf_enc(s)
        return 0

    def sdem_sg_gather_add(self, rows, J, idx, x, ldx, y, ldy, out, ld_out, out_bf, ld_out_bf, stream):
        if rows == 0:
            return 0
        ix = _flat(idx, np.int32, rows) if idx else np.arange(rows)
        nsrc = int(ix.max()) + 1 if rows else 0
        v = _mat(x, np.float32, nsrc, J, ldx)[ix]
        if y:
            v = _mat(y, np.float32, rows, J, ldy) + v
        if out:
            _mat(out, np.float32, rows, J, ld_out)[:] = v
        if out_bf:
            _mat(out_bf, np.uint16, rows, J, ld_out_bf)[:] = _bf_enc(v)
        return 0

    def sdem_sg_colsum(self, M, J, x, ldx, out, accumulate, partial, stream):
        s = _mat(x, np.float32, M, J, ldx).sum(axis=0, dtype=np.float32)
        o = _flat(out, np.float32, J)
        o[:] = o + s if accumulate else s
        return 0

    def sdem_sg_mse(self, n, K, pred, ldp, target, rowerr, dpred, dpred_bf, stream):
        p = _mat(pred, np.float32, n, ldp, ldp)
        t = _mat(target, np.float32, n, K, K)
        r = p[:, :K] - t
        d = np.zeros((n, ldp), np.float32)
        d[:, :K] = r * np.float32(2.0 / (n * K))
        if rowerr:
            _flat(rowerr, np.float32, n)[:] = (r * r).sum(axis=1)
        if dpred:
            _mat(dpred, np.float32, n, ldp, ldp)[:] = d
        if dpred_bf:
            _mat(dpred_bf, np.uint16, n, ldp, ldp)[:] = _bf_enc(d)
        return 0

    def sdem_sg_adam(self, n, p, g, m, v, p_bf, lr, b1, b2, eps, wd, step, stream):
        P, G, M, V = (_flat(q, np.float32, n) for q in (p, g, m, v))
        M[:] = b1 * M + (1 - b1) * G
        V[:] = b2 * V + (1 - b2) * G * G
        mh = M / np.float32(1 - b1 ** step)
        vh = V / np.float32(1 - b2 ** step)
        P[:] = P - lr * (mh / (np.sqrt(vh) + eps) + wd * P)
        if p_bf:
            _flat(p_bf, np.uint16, n)[:] = _bf_enc(P)
        return 0

    def sdem_sg_to_bf16(self, n, x, y, stream):
        _flat(y, np.uint16, n)[:] = _bf_enc(_flat(x, np.float32, n))
        return 0

    def sdem_sg_advance(self, n, pred, ldp, ascale, gx, gy, gz, h, box, posR, vel, omega, stream):
        b = _obj(box)
        p = _mat(pred, np.float32, n, ldp, ldp).astype(np.float64)
        pos = _mat(posR, np.float64, n, 4, 4)
        v = _flat(vel, np.float64, 9 * n).reshape(3, n, 3)
        w = _mat(omega, np.float64, n, 3, 3)
        r = pos[:, 3:4]
        a = ascale * p[:, :3] + np.array([gx, gy, gz])[None, :]
        vn = v[0] + a * h
        x = pos[:, :3] + vn * h
        lo = np.array(list(b.lo))[None, :] + r
        hi = np.array(list(b.hi))[None, :] - r
        below, above = x < lo, x > hi
        x = np.where(below, lo, np.where(above, hi, x))
        vn = np.where(below, np.maximum(vn, 0.0), np.where(above, np.minimum(vn, 0.0), vn))
        v[2] = v[1]
        v[1] = v[0]
        v[0] = vn
        pos[:, :3] = x
        w += ascale * p[:, 3:6] / r * h
        return 0
