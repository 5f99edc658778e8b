"""Block-cyclic redistribution between processes (PDGEMR2D across ranks,
REDIST/SRC/pdgemr.c) and a gather - solve - scatter PDGESV for callers whose
matrix is distributed over a P x Q grid of processes.

The per-(source, destination) packing is native code (sl1x1_redist_count /
_pack / _unpack in libsl1x1gpu.so); this module only moves the buffers, with
one torch.distributed all_to_all_single over host tensors (gloo, or any
backend that supports it on CPU tensors). The reference moves the same
element sets with BLACS point-to-point messages in a ring.

Layouts follow the reference's descriptors: a global m x n matrix in MB x NB
blocks dealt round-robin over a P x Q grid starting at process (RSRC, CSRC);
grid position (i, j) is the rank ranks[i*Q + j]. Local arrays are
Fortran-ordered float64 numpy arrays with leading dimension >= the local row
count (LOCr = NUMROC(M, MB, i, RSRC, P)), as ScaLAPACK stores them.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import lib as _lib
from . import numroc as _numroc


class Layout:
    """2D block-cyclic layout of an m x n matrix on a p x q grid of ranks."""

    def __init__(self, m, n, mb, nb, p=1, q=1, ranks=None, rsrc=0, csrc=0):
        self.m, self.n, self.mb, self.nb = int(m), int(n), int(mb), int(nb)
        self.p, self.q, self.rsrc, self.csrc = int(p), int(q), int(rsrc), int(csrc)
        self.ranks = list(range(self.p * self.q)) if ranks is None else [int(r) for r in ranks]
        if len(self.ranks) != self.p * self.q:
            raise ValueError("ranks must list p*q ranks in row-major grid order")

    def coords(self, rank):
        """(prow, pcol) of a rank, or (-1, -1) if it is not in this grid."""
        if rank not in self.ranks:
            return -1, -1
        k = self.ranks.index(rank)
        return k // self.q, k % self.q

    def local_shape(self, prow, pcol):
        if prow < 0:
            return 0, 0
        return (_numroc(self.m, self.mb, prow, self.rsrc, self.p),
                _numroc(self.n, self.nb, pcol, self.csrc, self.q))

    def desc(self, lld=1):
        """The 9-entry descriptor (CTXT unused by the pack routines)."""
        return np.array([1, -1, self.m, self.n, self.mb, self.nb, self.rsrc, self.csrc,
                         max(1, int(lld))], dtype=np.int32)

    def empty_local(self, rank):
        r, c = self.local_shape(*self.coords(rank))
        return np.zeros((max(1, r), c), dtype=np.float64, order="F")

    def rows_of(self, prow):
        """Global rows (0-based) held by process row prow, in local order."""
        g = np.arange(self.m)
        return g[(self.rsrc + g // self.mb) % self.p == prow]

    def cols_of(self, pcol):
        g = np.arange(self.n)
        return g[(self.csrc + g // self.nb) % self.q == pcol]

    def local_from_global(self, G, rank):
        """This rank's local array of a global matrix G (a reference mapping)."""
        pr, pc = self.coords(rank)
        out = self.empty_local(rank)
        if pr >= 0:
            rr, cc = self.rows_of(pr), self.cols_of(pc)
            out[: len(rr), : len(cc)] = np.asarray(G)[np.ix_(rr, cc)]
        return out


def _sig(L):
    vp = C.c_void_p
    args = [C.c_int, C.c_int, C.c_int, C.c_int, vp, C.c_int, C.c_int, C.c_int, C.c_int,
            C.c_int, C.c_int, vp, C.c_int, C.c_int, C.c_int, C.c_int]
    L.sl1x1_redist_count.argtypes = args
    L.sl1x1_redist_count.restype = C.c_longlong
    L.sl1x1_redist_pack.argtypes = args + [vp, vp]
    L.sl1x1_redist_pack.restype = C.c_longlong
    L.sl1x1_redist_unpack.argtypes = args + [vp, vp]
    L.sl1x1_redist_unpack.restype = C.c_longlong
    return L


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def pair_count(m, n, ia, ja, la, src, ib, jb, lb, dst):
    """Elements of sub(A) that process src (of la's grid) sends to dst (of lb's)."""
    L = _sig(_lib())
    da, db = la.desc(), lb.desc()
    c = L.sl1x1_redist_count(m, n, ia, ja, _ptr(da), la.p, la.q, src[0], src[1], ib, jb, _ptr(db),
                             lb.p, lb.q, dst[0], dst[1])
    if c < 0:
        raise ValueError("invalid layout")
    return int(c)


def pack(m, n, ia, ja, la, src, a_local, ib, jb, lb, dst):
    L = _sig(_lib())
    a = np.asfortranarray(a_local, dtype=np.float64)
    da, db = la.desc(a.shape[0]), lb.desc()
    buf = np.empty(max(1, pair_count(m, n, ia, ja, la, src, ib, jb, lb, dst)), dtype=np.float64)
    k = L.sl1x1_redist_pack(m, n, ia, ja, _ptr(da), la.p, la.q, src[0], src[1], ib, jb, _ptr(db),
                            lb.p, lb.q, dst[0], dst[1], _ptr(a), _ptr(buf))
    return buf[:k]


def unpack(m, n, ia, ja, la, src, ib, jb, lb, dst, buf, b_local):
    L = _sig(_lib())
    if not (b_local.dtype == np.float64 and b_local.flags.f_contiguous):
        raise TypeError("b_local must be a Fortran-ordered float64 array")
    buf = np.ascontiguousarray(buf, dtype=np.float64)
    da, db = la.desc(), lb.desc(b_local.shape[0])
    k = L.sl1x1_redist_unpack(m, n, ia, ja, _ptr(da), la.p, la.q, src[0], src[1], ib, jb, _ptr(db),
                              lb.p, lb.q, dst[0], dst[1], _ptr(buf), _ptr(b_local))
    if k != buf.size:
        raise RuntimeError("redistribution buffer size mismatch")


def pdgemr2d(m, n, a_local, ia, ja, la, b_local, ib, jb, lb, group=None):
    """PDGEMR2D across the ranks of `group`: copies sub(A) (layout la, this
    rank's local array a_local, or a 1x1 dummy if the rank is not in la's grid)
    into sub(B) (layout lb, b_local updated in place). Every rank of the group
    calls it."""
    import torch
    import torch.distributed as dist

    if m == 0 or n == 0:
        return
    rank = dist.get_rank(group)
    world = dist.get_world_size(group)
    me_a, me_b = la.coords(rank), lb.coords(rank)
    send_parts, send_splits, recv_splits = [], [], []
    for r in range(world):
        dst = lb.coords(r)
        if me_a[0] >= 0 and dst[0] >= 0:
            part = pack(m, n, ia, ja, la, me_a, a_local, ib, jb, lb, dst)
        else:
            part = np.empty(0, dtype=np.float64)
        send_parts.append(part)
        send_splits.append(part.size)
        src = la.coords(r)
        recv_splits.append(pair_count(m, n, ia, ja, la, src, ib, jb, lb, me_b)
                           if (src[0] >= 0 and me_b[0] >= 0) else 0)
    send = torch.from_numpy(np.concatenate(send_parts) if sum(send_splits) else np.empty(0))
    recv = torch.empty(sum(recv_splits), dtype=torch.float64)
    dist.all_to_all_single(recv, send, recv_splits, send_splits, group=group)
    out = recv.numpy()
    off = 0
    for r in range(world):
        k = recv_splits[r]
        if k:
            unpack(m, n, ia, ja, la, la.coords(r), ib, jb, lb, me_b, out[off:off + k], b_local)
        off += k


def pdgesv_gather(n, nrhs, a_local, la, ipiv_local, b_local, lb, root=0, group=None):
    """PDGESV for a matrix distributed over a P x Q grid of ranks: sub(A) and
    sub(B) are gathered into a 1x1 layout on `root` (PDGEMR2D), factored and
    solved there on the GPU (pdgesv_), and the factors, X and IPIV are
    scattered back into the callers' layouts. Returns INFO on every rank.
    Only `root` touches the GPU."""
    import torch
    import torch.distributed as dist

    from . import blacs_gridinit, pdgesv

    rank = dist.get_rank(group)
    nb = la.nb
    ra = Layout(n, n, nb, nb, 1, 1, ranks=[root])
    rb = Layout(n, nrhs, lb.mb, lb.nb, 1, 1, ranks=[root])
    A = np.zeros((max(1, n) if rank == root else 1, n if rank == root else 1), order="F")
    B = np.zeros((max(1, n) if rank == root else 1, nrhs if rank == root else 1), order="F")
    pdgemr2d(n, n, a_local, 1, 1, la, A, 1, 1, ra, group=group)
    pdgemr2d(n, nrhs, b_local, 1, 1, lb, B, 1, 1, rb, group=group)
    info = torch.zeros(1, dtype=torch.int64)
    ipiv = torch.zeros(max(1, n), dtype=torch.int32)
    if rank == root:
        ctx = blacs_gridinit(1, 1)
        desca = np.array([1, ctx, n, n, nb, nb, 0, 0, max(1, n)], np.int32)
        descb = np.array([1, ctx, n, nrhs, nb, nb, 0, 0, max(1, n)], np.int32)
        ip = np.zeros(n + nb, np.int32)
        info[0] = pdgesv(n, nrhs, A, 1, 1, desca, ip, B, 1, 1, descb)
        ipiv[:n] = torch.from_numpy(ip[:n].copy())
    dist.broadcast(info, src=root, group=group)
    dist.broadcast(ipiv, src=root, group=group)
    pdgemr2d(n, n, A, 1, 1, ra, a_local, 1, 1, la, group=group)
    if int(info[0]) == 0:
        pdgemr2d(n, nrhs, B, 1, 1, rb, b_local, 1, 1, lb, group=group)
    # IPIV is tied to A's rows: local row i holds the pivot of global row g(i)
    pr, _ = la.coords(rank)
    if pr >= 0:
        rows = la.rows_of(pr)
        ipiv_local[: len(rows)] = ipiv.numpy()[rows]
    return int(info[0])
