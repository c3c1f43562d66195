"""One matrix split across ranks by contiguous chunks of tiles: the reference's partial load, partial SpMV
and the synchronisation of its MPI CG (libs/dim/io/h5.cpp:86-173, include/dim/mpi/csr5.h:20-70,
libs/dim/mpi/csr5.cpp:8-46, libs/dim/mpi/csr5/output_range.cpp:5-12, edge_sync.cpp, result_sync.cpp,
benchmarks/conjugate_gradient/dim/main.cpp:100-180).

Part p of P holds the chunk of the matrix's elements that the reference's loader gives rank p: the stored
tiles (64 elements: sigma 16 x omega 4) are cut into runs of ceil(T / P) (``calculate_partition``,
h5.cpp:95-103) and the last part also takes the CSR tail.  A part multiplies into the rows its chunk
touches, ``output_range`` = [row of its first element, row of its last element] (for the last part: up to
the last row, csr5.h:853-855).  A row cut by a chunk boundary is output by both neighbours (or by several
parts when one row spans whole chunks), each with the partial sum over its own elements; edge sync adds
them.  The part owns its first row only if its chunk begins with that row (``owns_first_row``,
csr5.h:845-848), and result sync all-gathers the owned rows into the full vector.

On the device a part is an ordinary CSR5 matrix: the CSR of its chunk (rows = its output range, global
column indices, the boundary rows clipped to the chunk) goes through the device converter, so the partial
product is the ordinary SpMV kernel with x of full length and y of output-range length.  Edge and result
sync run over ``torch.distributed`` (NCCL with device tensors, or any backend through host copies); the
sums over ranks are taken in rank order, so every rank computes the same bits.  Empty rows that no chunk
touches (between two chunks, or before the first element) are outside every output range; ``assemble``
gives them 0, the value of their product.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _native as N
from .csr5 import csr5
from .mat import csr, dimensions_t

REF_TILE = 64  # elements per tile of the reference's stored format (sigma 16 x omega 4)


@dataclass(frozen=True)
class partial_identifier_t:
    """Which part of how many (h5.h: partial_identifier_t)."""
    idx: int
    total_count: int


def calculate_partition(element_count: int, part: partial_identifier_t) -> tuple[int, int]:
    """(start, count) of part `idx` when `element_count` items are cut into runs of ceil(count / parts)
    (h5.cpp:95-103); parts past the end get count 0."""
    if part.total_count < 1 or not 0 <= part.idx < part.total_count:
        raise ValueError(f"part {part.idx} of {part.total_count}")
    size = -(-element_count // part.total_count)
    first = size * part.idx
    return first, max(0, min(size, element_count - first))


@dataclass(frozen=True)
class output_range_t:
    """The rows a part writes, first and last inclusive (output_range.h:12-40)."""
    first_row: int
    last_row: int

    def is_continuation_of(self, other: "output_range_t") -> bool:
        return other.last_row == self.first_row

    def count(self) -> int:
        return self.last_row - self.first_row + 1

    @staticmethod
    def syncs_downto(all_output_ranges, current: int) -> int:
        """Index of the first part that outputs to all_output_ranges[current].first_row
        (output_range.cpp:5-12)."""
        base = all_output_ranges[current]
        while current != 0 and base.is_continuation_of(all_output_ranges[current - 1]):
            current -= 1
        return current


@dataclass(frozen=True)
class partial_layout:
    """Host description of one part: its tiles, elements, rows and the CSR of its chunk."""
    part: partial_identifier_t
    tile_start: int
    tile_count: int
    element_begin: int
    element_end: int
    first_row: int
    last_row: int
    owns_first_row: bool
    local: csr  # rows first_row..last_row, global columns

    def output_range(self) -> output_range_t:
        return output_range_t(self.first_row, self.last_row)

    def owning_range(self) -> output_range_t:
        """The rows this part owns (csr5.h owning_range: the first row only when the chunk starts it)."""
        return output_range_t(self.first_row + (0 if self.owns_first_row else 1), self.last_row)

    @staticmethod
    def chunk_of(nnz: int, part: partial_identifier_t) -> tuple[int, int, int, int]:
        """(first tile, tiles, first element, end element) of the part's chunk."""
        tiles = nnz // REF_TILE
        if part.total_count > max(tiles, 1):
            raise ValueError(f"{part.total_count} parts for {tiles} tiles: every part needs at least one tile")
        start, count = calculate_partition(tiles, part)
        last = part.idx == part.total_count - 1
        return start, count, start * REF_TILE, nnz if last else (start + count) * REF_TILE

    @staticmethod
    def from_chunk(part: partial_identifier_t, rows: int, cols: int, nnz: int, row_ptr, row_base: int, vals,
                   col_idx) -> "partial_layout":
        """The part's layout from its chunk's values and column indices (CSR order) and row_ptr[row_base:]
        (a slab of the row offsets from some row at or before the chunk's first row, to its last row + 1 or
        further)."""
        start, count, e0, e1 = partial_layout.chunk_of(nnz, part)
        rp = np.asarray(row_ptr, np.int64)
        # the row holding element e: the last row whose offset is <= e (empty rows before it are skipped)
        first_row = row_base + int(np.searchsorted(rp, e0, side="right") - 1) if nnz else 0
        if part.idx == part.total_count - 1:
            last_row = rows - 1
        else:
            last_row = row_base + int(np.searchsorted(rp, e1 - 1, side="right") - 1)
        if last_row + 2 - row_base > rp.size:
            raise ValueError("the row_ptr slab ends before the chunk's last row")
        local_rp = np.clip(rp[first_row - row_base:last_row + 2 - row_base] - e0, 0, e1 - e0).astype(np.uint32)
        local = csr(dimensions_t(last_row - first_row + 1, cols), vals, local_rp, col_idx)
        owns = bool(rp[first_row - row_base] == e0)
        return partial_layout(part, start, count, e0, e1, first_row, last_row, owns, local)

    @staticmethod
    def of(m: csr, part: partial_identifier_t) -> "partial_layout":
        _, _, e0, e1 = partial_layout.chunk_of(m.nnz, part)
        return partial_layout.from_chunk(part, m.dimensions.rows, m.dimensions.cols, m.nnz, m.row_start_offsets, 0,
                                         m.values[e0:e1], m.col_indices[e0:e1])


class csr5_partial:
    """One part of a matrix on the device (the reference's dim::mpi::csr5::csr5_partial, without MPI):
    ``spmv_partial(x, y)`` is y := (the part's rows of A restricted to its chunk) x, x of full length,
    y of ``output_range().count()``."""

    def __init__(self, layout: partial_layout, matrix: csr5):
        self.layout = layout
        self.matrix = matrix

    @staticmethod
    def from_csr(m: csr, part: partial_identifier_t, stream=None) -> "csr5_partial":
        """The part of a whole host matrix."""
        return csr5_partial.from_layout(partial_layout.of(m, part), stream)

    @staticmethod
    def from_layout(lay: partial_layout, stream=None) -> "csr5_partial":
        """The part described by `lay` (e.g. from ``io.h5.load_csr5_partial``, which reads only its slabs)."""
        return csr5_partial(lay, csr5.from_csr(lay.local, stream=stream))

    def output_range(self) -> output_range_t:
        return self.layout.output_range()

    def owning_range(self) -> output_range_t:
        return self.layout.owning_range()

    def owns_first_row(self) -> bool:
        return self.layout.owns_first_row

    def local_nnz(self) -> int:
        return self.layout.local.nnz

    def spmv_partial(self, x, y, calibrator=None, stream=None):
        return self.matrix.spmv(x, y, calibrator, stream=stream)


# ---- summation of the boundary rows and assembly (pure host logic, shared by every transport) ----------

def boundary_totals(ranges, firsts, lasts):
    """For every part p: the full values of its first and last rows, summed over all parts that output to
    them, in part order (edge_sync.cpp: an all-reduce among the parts sharing a row).  firsts[p] / lasts[p]
    are part p's partial values of its first / last row (the same value when the part has one row)."""
    P = len(ranges)
    contrib = {}
    for p in range(P):
        r = ranges[p]
        contrib.setdefault(r.first_row, []).append(firsts[p])
        if r.last_row != r.first_row:
            contrib.setdefault(r.last_row, []).append(lasts[p])
    tot_first, tot_last = [], []
    for p in range(P):
        def total(row):
            acc = 0.0
            for v in contrib[row]:
                acc += float(v)
            return acc
        tot_first.append(total(ranges[p].first_row))
        tot_last.append(total(ranges[p].last_row))
    return tot_first, tot_last


def shared_rows(ranges, p):
    """(first row shared with another part, last row shared with another part) for part p."""
    r = ranges[p]
    first = any(q != p and (ranges[q].first_row == r.first_row or ranges[q].last_row == r.first_row)
                for q in range(len(ranges)))
    last = any(q != p and (ranges[q].first_row == r.last_row or ranges[q].last_row == r.last_row)
               for q in range(len(ranges)))
    return first, last


def owned_slices(ranges):
    """(global first row, count) of the rows each part contributes to the full vector (result_sync.cpp:
    a part skips its first row when it continues the previous part's last row)."""
    out = []
    for p, r in enumerate(ranges):
        overlap = 1 if p > 0 and r.is_continuation_of(ranges[p - 1]) else 0
        out.append((r.first_row + overlap, r.count() - overlap))
    return out


def assemble(ranges, ys, rows: int) -> np.ndarray:
    """The full y from every part's partial y (host arrays), in one process: boundary rows summed in part
    order, rows outside every output range 0."""
    firsts = [float(y[0]) for y in ys]
    lasts = [float(y[-1]) for y in ys]
    tf, tl = boundary_totals(ranges, firsts, lasts)
    full = np.zeros(rows)
    for p, (start, cnt) in enumerate(owned_slices(ranges)):
        y = np.array(ys[p], dtype=np.float64, copy=True)
        sf, sl = shared_rows(ranges, p)
        if sf:
            y[0] = tf[p]
        if sl:
            y[-1] = tl[p]
        off = ranges[p].count() - cnt
        full[start:start + cnt] = y[off:]
    return full


# ---- the same over torch.distributed -------------------------------------------------------------------

def _dist():
    import torch.distributed as dist
    return dist


def _stage(t, backend_is_nccl: bool):
    return t if backend_is_nccl else t.cpu()


def all_output_ranges(rng: output_range_t, group=None):
    """Every rank's output range (csr5.cpp:22-30: an all-gather of two u32 per rank)."""
    import torch
    dist = _dist()
    nccl = dist.get_backend(group) == "nccl"
    dev = torch.device("cuda", torch.cuda.current_device()) if nccl else torch.device("cpu")
    mine = torch.tensor([rng.first_row, rng.last_row], dtype=torch.int64, device=dev)
    allr = [torch.empty_like(mine) for _ in range(dist.get_world_size(group))]
    dist.all_gather(allr, mine, group=group)
    return [output_range_t(int(t[0]), int(t[1])) for t in allr]


class edge_sync_t:
    """Adds the partial values of the boundary rows a rank shares with others (edge_sync.cpp), in rank
    order: one all-gather of (first, last) values per call."""

    def __init__(self, ranges, rank: int, group=None):
        self.ranges, self.rank, self.group = list(ranges), rank, group
        self.shared_first, self.shared_last = shared_rows(self.ranges, rank)

    def sync(self, y) -> None:
        """y: this rank's partial y (a torch tensor, output-range length), updated in place."""
        import torch
        dist = _dist()
        nccl = dist.get_backend(self.group) == "nccl"
        ends = torch.stack([y[0], y[-1]]).to(torch.float64)
        ends = _stage(ends, nccl)
        allv = [torch.empty_like(ends) for _ in range(dist.get_world_size(self.group))]
        dist.all_gather(allv, ends, group=self.group)
        tf, tl = boundary_totals(self.ranges, [float(v[0]) for v in allv], [float(v[1]) for v in allv])
        if self.shared_first:
            y[0] = tf[self.rank]
        if self.shared_last:
            y[-1] = tl[self.rank]


class result_sync_t:
    """All-gathers the rows each rank owns into the full vector (result_sync.cpp: MPI_Allgatherv with
    the overlapping first rows skipped)."""

    def __init__(self, ranges, rank: int, group=None):
        self.ranges, self.rank, self.group = list(ranges), rank, group
        self.slices = owned_slices(self.ranges)
        self.width = max(c for _, c in self.slices)

    def sync(self, full, y) -> None:
        """full: the full vector (torch, rows long), y: this rank's output-range vector."""
        import torch
        dist = _dist()
        nccl = dist.get_backend(self.group) == "nccl"
        start, cnt = self.slices[self.rank]
        off = self.ranges[self.rank].count() - cnt
        buf = torch.zeros(self.width, dtype=full.dtype, device=y.device)
        buf[:cnt] = y[off:off + cnt]
        buf = _stage(buf, nccl)
        allb = [torch.empty_like(buf) for _ in range(dist.get_world_size(self.group))]
        dist.all_gather(allb, buf, group=self.group)
        for q, (s0, c) in enumerate(self.slices):
            full[s0:s0 + c] = allb[q][:c].to(full.device)


@dataclass
class cg_partial_result:
    iterations: int
    rel_residual: float  # recurrence ||r|| / ||b|| at exit
    converged: bool


def _dot(a, b) -> float:
    out = ctypes.c_double()
    N.check(N.lib().dimgpu_vec_dot(a.numel(), N.device_ptr(a, "<f8", a.numel()), N.device_ptr(b, "<f8", b.numel()),
                                   ctypes.byref(out), None))
    return out.value


def _allreduce(v: float, group=None) -> float:
    import torch
    dist = _dist()
    nccl = dist.get_backend(group) == "nccl"
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if nccl else "cpu")
    dist.all_reduce(t, group=group)
    return float(t[0])


def cg_partial(part: csr5_partial, b_own, x_own, tol: float = 1e-10, max_it: int = 100000, group=None):
    """The reference's multi-rank CG (benchmarks/conjugate_gradient/dim/main.cpp:100-180) on this rank's
    part, with the single-process solver's stop rule ||r|| <= tol ||b||.  b_own / x_own: this rank's owned
    rows of b and of the initial guess (torch CUDA float64; x_own is overwritten with the solution).
    Products run on the device (partial SpMV, C-ABI vector kernels); dots are all-reduced on the host."""
    import torch
    dist = _dist()
    L = N.lib()
    rank = dist.get_rank(group)
    ranges = all_output_ranges(part.output_range(), group)
    edge, res = edge_sync_t(ranges, rank, group), result_sync_t(ranges, rank, group)
    out_r, own_r = part.output_range(), part.owning_range()
    cols = part.matrix.dimensions.cols
    skip = 0 if part.owns_first_row() else 1
    dev = b_own.device
    # r = b - A x0 on the owned rows: s_full holds x0 for the product
    s = torch.zeros(cols, dtype=torch.float64, device=dev)
    res.sync(s, torch.cat([torch.zeros(skip, dtype=torch.float64, device=dev), x_own]))
    As = torch.empty(out_r.count(), dtype=torch.float64, device=dev)
    part.spmv_partial(s, As)
    edge.sync(As)
    r = (b_own - As[skip:]).contiguous()
    bb = _allreduce(_dot(b_own, b_own), group)
    rr = _allreduce(_dot(r, r), group)
    thresh2 = tol * tol * (bb if bb > 0 else 1.0)
    res.sync(s, torch.cat([torch.zeros(skip, dtype=torch.float64, device=dev), r]))  # s0 = r0
    it = 0
    while rr > thresh2 and it < max_it:
        part.spmv_partial(s, As)  # As = A s (partial on the boundary rows)
        # alpha before the edge sync: the partial boundary values of all ranks add up to s.As
        s_out = s[out_r.first_row:out_r.first_row + out_r.count()].contiguous()
        sAs = _allreduce(_dot(s_out, As), group)
        if not (sAs > 0.0):
            break
        alpha = rr / sAs
        s_own = s[own_r.first_row:own_r.first_row + own_r.count()].contiguous()
        N.check(L.dimgpu_vec_axpy(x_own.numel(), alpha, N.device_ptr(s_own, "<f8"), N.device_ptr(x_own, "<f8"),
                                  None))
        edge.sync(As)
        As_own = As[skip:].contiguous()
        N.check(L.dimgpu_vec_axpy(r.numel(), -alpha, N.device_ptr(As_own, "<f8"), N.device_ptr(r, "<f8"), None))
        rr_new = _allreduce(_dot(r, r), group)
        beta = rr_new / rr
        rr = rr_new
        # s_own = r + beta s_own, then the full s from every rank's owned rows
        N.check(L.dimgpu_vec_aypx(s_own.numel(), beta, N.device_ptr(r, "<f8"), N.device_ptr(s_own, "<f8"), None))
        res.sync(s, torch.cat([torch.zeros(skip, dtype=torch.float64, device=dev), s_own]))
        it += 1
    return x_own, cg_partial_result(it, (rr / (bb if bb > 0 else 1.0)) ** 0.5, rr <= thresh2)
