"""Mesh-only precomputation for the deterministic patch assembly.

This replaces the reference's ``from_mesh`` pattern build
(assemble/element_assembler.py:838-875: scipy coo->csr->coo dedup of the
element (row, col) pairs plus the per-entry slot map ``elem_eids``) with a
device-side build (the CSR pattern by the project's own kernels, the patch
plan by torch ops) that produces:

* the node-level CSR pattern (indptr, indices) in canonical order -- the
  same unique, row-major, column-sorted pairs the reference's ``edges`` hold;
* a partition of the nodes into *patches* by recursive coordinate bisection
  (RCB); each patch owns a set of CSR rows and lists every element touching
  them, with a patch-local vertex table and, for each owned row, its
  incidences (element, local vertex) sorted by element together with the
  position of every column inside the row.

Everything is computed with torch ops, so it runs on the GPU when the mesh
lives there (and on the CPU in unit tests).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import torch

from . import _lib


# elements staged per chunk by the patch kernels (their block size)
PATCH_CHUNK = 256


@dataclass
class NodePattern:
    n_points: int
    indptr: torch.Tensor    # int64 [N+1]
    indices: torch.Tensor   # int32 [nnz]
    slots: torch.Tensor     # int64 [E, B, B] global slot of each element entry

    @property
    def nnz(self) -> int:
        return int(self.indices.shape[0])


def node_pattern(elements: torch.Tensor, n_points: int) -> NodePattern:
    """Unique element (row, col) pairs in canonical CSR order
    (element_assembler.py:838-866).  On a CUDA device the project's pattern
    kernels build it (tm_pattern_count / tm_pattern_fill); a mesh kept on the
    host (host-side planning and its unit tests) uses the same definition in
    torch ops."""
    if elements.is_cuda:
        return _node_pattern_gpu(elements, n_points)
    E, B = elements.shape
    el = elements.long()
    u = el.unsqueeze(2).expand(E, B, B).reshape(-1)
    v = el.unsqueeze(1).expand(E, B, B).reshape(-1)
    key = u * n_points + v
    uniq, inv = torch.unique(key, sorted=True, return_inverse=True)
    rows = torch.div(uniq, n_points, rounding_mode="floor")
    cols = uniq - rows * n_points
    counts = torch.bincount(rows, minlength=n_points)
    indptr = torch.zeros(n_points + 1, dtype=torch.int64, device=elements.device)
    indptr[1:] = torch.cumsum(counts, 0)
    return NodePattern(n_points, indptr, cols.to(torch.int32), inv.view(E, B, B))


def _node_pattern_gpu(elements: torch.Tensor, n_points: int) -> NodePattern:
    E, B = elements.shape
    dev = elements.device
    el = elements.to(torch.int32).contiguous()
    lib = _lib.load()
    work = torch.empty(int(lib.tm_pattern_workspace_bytes(E, B, n_points)), dtype=torch.uint8, device=dev)
    indptr = torch.empty(n_points + 1, dtype=torch.int64, device=dev)
    stream = _lib.stream_handle(dev)
    _lib.call("tm_pattern_count", el.data_ptr(), E, B, n_points, work.data_ptr(), indptr.data_ptr(), stream)
    nnz = int(indptr[-1])
    indices = torch.empty(nnz, dtype=torch.int32, device=dev)
    slots = torch.empty((E, B, B), dtype=torch.int64, device=dev)
    _lib.call("tm_pattern_fill", el.data_ptr(), E, B, n_points, work.data_ptr(), indptr.data_ptr(),
              indices.data_ptr(), slots.data_ptr(), stream)
    return NodePattern(n_points, indptr, indices, slots)


def block_pattern(indptr: torch.Tensor, indices: torch.Tensor, H: int):
    """Dof-level canonical CSR of the H x H block expansion
    row = H*i + a, col = H*j + b (sparse/matrix.py:355-375 followed by the
    canonical sort).  Row (H*i + a) lists cols H*j + b for j in row i,
    b in 0..H-1."""
    if H == 1:
        return indptr, indices
    n = indptr.shape[0] - 1
    deg = indptr[1:] - indptr[:-1]
    dof_deg = (deg * H).repeat_interleave(H)
    dptr = torch.zeros(n * H + 1, dtype=torch.int64, device=indptr.device)
    dptr[1:] = torch.cumsum(dof_deg, 0)
    # node row i -> H copies of [H*c + b for c in cols(i) for b]
    blk = (indices.long().unsqueeze(1) * H + torch.arange(H, device=indptr.device)).reshape(-1)  # [nnz*H]
    # for each node row, repeat its block row H times
    node_of_slot = torch.repeat_interleave(torch.arange(n, device=indptr.device), deg)
    start_blk = indptr[:-1] * H
    out = torch.empty(int(dptr[-1]), dtype=torch.int32, device=indptr.device)
    # dof row (i, a) occupies out[dptr[i*H+a] : +deg_i*H] = blk[start_blk[i] : start_blk[i] + deg_i*H]
    pos_in_row = torch.arange(blk.shape[0], device=indptr.device) - start_blk[node_of_slot.repeat_interleave(H)]
    node_blk = node_of_slot.repeat_interleave(H)
    for a in range(H):
        dst = dptr[node_blk * H + a] + pos_in_row
        out[dst] = blk.to(torch.int32)
    return dptr, out


def rcb_partition(coords: torch.Tensor, n_levels: int = None, n_parts: int = None) -> torch.Tensor:
    """Recursive coordinate bisection into ``n_parts`` parts (default
    ``2**n_levels``).  A segment that must become k parts is cut along its
    longest extent at the point count k_left / k of its points, where
    k_left = k // 2, and the two sides go on to become k_left and k - k_left
    parts; so parts hold floor or ceil of N / n_parts points whatever
    n_parts is.  Returns the part id of each point (parts numbered in RCB
    leaf order, spatially coherent)."""
    N = coords.shape[0]
    dev = coords.device
    if n_parts is None:
        n_parts = 1 << int(n_levels or 0)
    n_parts = max(1, int(n_parts))
    c = coords.to(torch.float64)
    D = c.shape[1]
    perm = torch.arange(N, device=dev)
    seg = torch.zeros(N, dtype=torch.int64, device=dev)        # first part id of the point's segment
    kpart = torch.zeros(n_parts, dtype=torch.int64, device=dev)  # parts still to make, at first-part ids
    kpart[0] = n_parts
    ar = torch.arange(N, device=dev)
    while N and int(kpart.max()) > 1:
        cp = c[perm]
        idx = seg.unsqueeze(1).expand(N, D)
        mx = torch.full((n_parts, D), -math.inf, dtype=torch.float64, device=dev).scatter_reduce(0, idx, cp, "amax")
        mn = torch.full((n_parts, D), math.inf, dtype=torch.float64, device=dev).scatter_reduce(0, idx, cp, "amin")
        axis = torch.argmax(mx - mn, dim=1)
        val = cp[ar, axis[seg]]
        o1 = torch.argsort(val, stable=True)
        o2 = torch.argsort(seg[o1], stable=True)
        order = o1[o2]
        perm = perm[order]
        seg = seg[order]
        counts = torch.bincount(seg, minlength=n_parts)
        start = torch.cumsum(counts, 0) - counts
        pos = ar - start[seg]
        k = kpart[seg]
        kl = k // 2
        cut = (counts[seg] * kl) // torch.clamp(k, min=1)
        seg = seg + ((k > 1) & (pos >= cut)).long() * kl
        firsts = torch.nonzero(kpart > 1, as_tuple=True)[0]
        kk = kpart[firsts]
        kpart[firsts + kk // 2] = kk - kk // 2
        kpart[firsts] = kk // 2
    part = torch.empty(N, dtype=torch.int64, device=dev)
    part[perm] = seg
    return part


def morton_keys(c: torch.Tensor, lo: torch.Tensor, hi: torch.Tensor, bits: int) -> torch.Tensor:
    """Z-order keys of the float64 points c [N, D]: coordinate d quantised to
    q = round((x - lo_d) / max(hi_d - lo_d, 1e-300) * (2^bits - 1)) (half to
    even), bit b of q at key bit b D + d.  One kernel on the device
    (tm_morton_keys); CPU tensors (host-side planning) take the same
    arithmetic in torch."""
    N, D = c.shape
    if c.is_cuda:
        key = torch.empty(N, dtype=torch.int64, device=c.device)
        _lib.call("tm_morton_keys", N, D, c.data_ptr(), lo.data_ptr(), hi.data_ptr(), bits, key.data_ptr(),
                  _lib.stream_handle(c.device))
        return key
    q = ((c - lo) / torch.clamp(hi - lo, min=1e-300) * ((1 << bits) - 1)).round().long()
    key = torch.zeros(N, dtype=torch.int64, device=c.device)
    for b in range(bits):
        for d in range(D):
            key |= ((q[:, d] >> b) & 1) << (b * D + d)
    return key


def morton_parts(coords: torch.Tensor, target: int) -> torch.Tensor:
    """Spatially compact parts of about ``target`` points: the cells of an
    octree (quadtree in 2D) over the bounding box, refined where a cell holds
    more than 2 * target points.  Points are sorted once along the Z-order
    (Morton) curve of their coordinates quantised to 2^(63 // D) steps per
    axis; every cell is then a run of that order, identified by a key prefix.
    Part ids follow the curve."""
    N, D = coords.shape
    dev = coords.device
    if N == 0:
        return torch.zeros(0, dtype=torch.int64, device=dev)
    c = coords.to(torch.float64).contiguous()
    lo, hi = c.min(0).values.contiguous(), c.max(0).values.contiguous()
    bits = 63 // D
    key = morton_keys(c, lo, hi, bits)
    order = torch.argsort(key, stable=True)
    k = key[order]
    level0 = max(0, min(bits, int(math.floor(math.log(max(1.0, N / target)) / math.log(2 ** D)))))
    level = torch.full((N,), level0, dtype=torch.int64, device=dev)
    for _ in range(bits + 1):
        prefix = k >> (D * (bits - level))
        new = torch.ones(N, dtype=torch.bool, device=dev)
        new[1:] = (prefix[1:] != prefix[:-1]) | (level[1:] != level[:-1])
        seg = torch.cumsum(new.long(), 0) - 1
        counts = torch.bincount(seg)
        over = (counts[seg] > 2 * target) & (level < bits)
        if not bool(over.any()):
            break
        level = level + over.long()
    part = torch.empty(N, dtype=torch.int64, device=dev)
    part[order] = seg
    return part


def rcb_partition_grouped(coords: torch.Tensor, groups: torch.Tensor, weight: torch.Tensor,
                          budget: float, max_rows: int):
    """RCB inside fixed groups (e.g. the instances of a batch): segments start
    as the groups and are bisected along their longest extent until each
    holds at most ``budget`` weight (CSR slots) and ``max_rows`` points.
    Parts never straddle groups; part ids are dense and ordered by group."""
    N = coords.shape[0]
    dev = coords.device
    c = coords.to(torch.float64)
    D = c.shape[1]
    seg = groups.long().clone()
    ar = torch.arange(N, device=dev)
    w = weight.to(torch.float64)
    for _ in range(64):
        nseg = int(seg.max()) + 1 if N else 0
        cnt = torch.bincount(seg, minlength=nseg)
        wsum = torch.zeros(nseg, dtype=torch.float64, device=dev).index_add_(0, seg, w)
        split = (wsum > budget) | (cnt > max_rows)
        split &= cnt > 1
        if not bool(split.any()):
            break
        idx = seg.unsqueeze(1).expand(N, D)
        mx = torch.full((nseg, D), -math.inf, dtype=torch.float64, device=dev).scatter_reduce(0, idx, c, "amax")
        mn = torch.full((nseg, D), math.inf, dtype=torch.float64, device=dev).scatter_reduce(0, idx, c, "amin")
        axis = torch.argmax(mx - mn, dim=1)
        val = c[ar, axis[seg]]
        o1 = torch.argsort(val, stable=True)
        order = o1[torch.argsort(seg[o1], stable=True)]
        start = torch.cumsum(cnt, 0) - cnt
        pos = torch.empty(N, dtype=torch.int64, device=dev)
        pos[order] = ar - start[seg[order]]
        side = ((pos >= (cnt[seg] + 1) // 2) & split[seg]).long()
        seg = 2 * seg + side
    _, part = torch.unique(seg, sorted=True, return_inverse=True)
    return part


class PatchPlan:
    """Device arrays of the patch structure plus the ctypes view of them."""

    def __init__(self, elements: torch.Tensor, coords: torch.Tensor, pattern: NodePattern,
                 slot_budget: int = 6144, max_rows_cap: int = 256, groups: torch.Tensor = None):
        dev = elements.device
        E, B = elements.shape
        N = pattern.n_points
        self.n_elements, self.n_basis, self.n_points = E, B, N
        el = elements.long()
        indptr = pattern.indptr
        deg = indptr[1:] - indptr[:-1]
        if E > 0 and int(deg.max()) > 255:
            raise NotImplementedError("a CSR row longer than 255 entries is not supported by the patch plan")

        # -- partition: enough RCB levels that every patch fits the slot budget
        if groups is not None:
            part = rcb_partition_grouped(coords, groups, deg, slot_budget, max_rows_cap)
            n_parts = int(part.max()) + 1 if N else 0
            slots_per_part = torch.zeros(n_parts, dtype=torch.int64, device=dev).index_add_(0, part, deg)
            rows_per_part = torch.bincount(part, minlength=n_parts)
            self.part = part
        else:
            avg_deg = float(deg.float().mean()) if N else 1.0
            target_rows = max(16, min(max_rows_cap, int(slot_budget / max(avg_deg, 1.0))))
            n_parts = max(1, math.ceil(N / target_rows))
            while True:
                part = rcb_partition(coords, n_parts=n_parts) if N else torch.zeros(0, dtype=torch.int64, device=dev)
                slots_per_part = torch.zeros(n_parts, dtype=torch.int64, device=dev).index_add_(0, part, deg)
                rows_per_part = torch.bincount(part, minlength=n_parts)
                if N == 0 or (int(slots_per_part.max()) <= 2 * slot_budget and
                              int(rows_per_part.max()) <= max_rows_cap):
                    break
                n_parts = n_parts + max(1, n_parts // 32)
            self.part = part
        self.n_patches = n_parts

        # -- owned rows, sorted by (patch, node id)
        row_order = torch.argsort(part * N + torch.arange(N, device=dev))
        rows = row_order
        rptr = torch.zeros(n_parts + 1, dtype=torch.int64, device=dev)
        rptr[1:] = torch.cumsum(rows_per_part, 0)
        row_deg = deg[rows]
        cum = torch.zeros(N + 1, dtype=torch.int64, device=dev)
        cum[1:] = torch.cumsum(row_deg, 0)                             # global exclusive prefix
        racc = cum[:-1] - cum[rptr[:-1]].repeat_interleave(rows_per_part)  # patch-relative
        row_rank = torch.empty(N, dtype=torch.int64, device=dev)
        row_rank[rows] = torch.arange(N, device=dev)

        # -- (patch, element) pairs: elements touching each patch
        pe_key = (part[el] * E + torch.arange(E, device=dev).unsqueeze(1)).reshape(-1)
        pairs = torch.unique(pe_key, sorted=True)
        pair_patch = torch.div(pairs, E, rounding_mode="floor")
        pair_elem = pairs - pair_patch * E
        elems_per_part = torch.bincount(pair_patch, minlength=n_parts)
        eptr = torch.zeros(n_parts + 1, dtype=torch.int64, device=dev)
        eptr[1:] = torch.cumsum(elems_per_part, 0)
        if E and int(elems_per_part.max()) > 65535:
            raise NotImplementedError("patch with more than 65535 elements")
        # processing order inside a patch: the kernels stage PATCH_CHUNK
        # elements at a time, and a row's incidences come in runs of
        # neighbouring element ids; dealing the sorted elements out over the
        # m = ceil(n / PATCH_CHUNK) chunks (element k goes to chunk k mod m)
        # gives every row a similar number of incidences in every chunk
        if E:
            rank = torch.arange(pairs.shape[0], device=dev) - eptr[pair_patch]
            m = torch.clamp((elems_per_part[pair_patch] + PATCH_CHUNK - 1) // PATCH_CHUNK, min=1)
            deal = torch.argsort(pair_patch * (1 << 32) + (rank % m) * (1 << 16) + rank // m)
            pair_patch, pair_elem = pair_patch[deal], pair_elem[deal]

        # -- patch-local vertex tables
        pconn = el[pair_elem]                                           # [n_pairs, B]
        pv_key = pair_patch.unsqueeze(1) * N + pconn
        vkeys = torch.unique(pv_key.reshape(-1), sorted=True)
        vtx_patch = torch.div(vkeys, N, rounding_mode="floor")
        vtx = vkeys - vtx_patch * N
        verts_per_part = torch.bincount(vtx_patch, minlength=n_parts)
        vptr = torch.zeros(n_parts + 1, dtype=torch.int64, device=dev)
        vptr[1:] = torch.cumsum(verts_per_part, 0)
        if E and int(verts_per_part.max()) > 65535:
            raise NotImplementedError("patch with more than 65535 vertices")
        local = torch.searchsorted(vkeys, pv_key) - vptr[pair_patch].unsqueeze(1)

        # -- incidences of owned rows
        owned = part[pconn] == pair_patch.unsqueeze(1)                 # [n_pairs, B]
        pi, a = torch.nonzero(owned, as_tuple=True)
        inc_row = pconn[pi, a]
        inc_local_elem = pi - eptr[pair_patch[pi]]
        order = torch.argsort(row_rank[inc_row] * (1 << 20) + inc_local_elem)
        pi, a, inc_row, inc_local_elem = pi[order], a[order], inc_row[order], inc_local_elem[order]
        ge = pair_elem[pi]
        inc_pos = pattern.slots[ge, a, :] - indptr[inc_row].unsqueeze(1)  # [n_inc, B]
        inc_per_row = torch.bincount(row_rank[inc_row], minlength=N)
        iptr = torch.zeros(N + 1, dtype=torch.int64, device=dev)
        iptr[1:] = torch.cumsum(inc_per_row, 0)

        i32 = torch.int32
        self.vptr = vptr.to(i32)
        self.vtx = vtx.to(i32)
        self.eptr = eptr.to(i32)
        self.elem = pair_elem.to(i32)
        self.econn = local.to(i32).to(torch.int16).contiguous()        # uint16 bit pattern
        self.rptr = rptr.to(i32)
        self.rows = rows.to(i32)
        self.racc = racc.to(i32)
        self.iptr = iptr.to(i32)
        self.inc_elem = inc_local_elem.to(i32).to(torch.int16).contiguous()
        self.inc_a = a.to(torch.uint8).contiguous()
        self.inc_pos = inc_pos.to(torch.uint8).contiguous()
        # P1 tetrahedra: one record per incidence, so the row owner issues one
        # load per incidence.  With o_j = (a + 1 + j) mod 4 the record holds the
        # positions of the three off-diagonal columns conn[e, o_j] in the row:
        #   64-bit: local element (bits 0-15) | a (16-17) | pos o_0, o_1, o_2
        #           (8 bits each from bit 18);
        #   32-bit (rows of at most 32 entries, at most 32767 elements per
        #           patch): local element (0-14) | a (15-16) | pos o_0, o_1,
        #           o_2 (5 bits each from bit 17).
        # rdiag holds the position of each owned row's own column (rows order).
        self.inc_pack = self.inc_pack32 = self.rdiag = None
        if B == 4:
            others = (a.unsqueeze(1) + 1 + torch.arange(3, device=dev)) % 4          # [n_inc, 3]
            po = torch.gather(inc_pos, 1, others).long()                             # [n_inc, 3]
            pk = inc_local_elem.long() | (a.long() << 16)
            for j in range(3):
                pk = pk | (po[:, j] << (18 + 8 * j))
            self.inc_pack = pk.contiguous()
            n_inc = int(a.shape[0])
            dpos_inc = inc_pos[torch.arange(n_inc, device=dev), a.long()].long()
            has = inc_per_row > 0
            first = torch.clamp(iptr[:-1], max=max(0, n_inc - 1))
            rdiag = torch.where(has, dpos_inc[first] if n_inc else torch.zeros_like(first), torch.zeros_like(first))
            self.rdiag = rdiag.to(torch.uint8).contiguous()
            max_deg = int(deg.max()) if N else 0
            if max_deg <= 32 and (not E or int(elems_per_part.max()) <= 32767):
                pk32 = inc_local_elem.long() | (a.long() << 15)
                for j in range(3):
                    pk32 = pk32 | (po[:, j] << (17 + 5 * j))
                self.inc_pack32 = pk32.to(torch.int64).to(torch.int32).contiguous()  # uint32 bit pattern
        self.indptr = indptr.contiguous()
        self.max_vtx = int(verts_per_part.max()) if E else 0
        self.max_slots = int(slots_per_part.max()) if N else 0
        self.max_rows = int(rows_per_part.max()) if N else 0
        self.max_elems = int(elems_per_part.max()) if E else 0
        self.max_deg = int(deg.max()) if N else 0
        self.n_pairs = int(pairs.shape[0])
        self.n_incidences = int(pi.shape[0])
        if int(iptr[-1]) >= 2**31 or self.n_pairs * B >= 2**31:
            raise NotImplementedError("mesh too large for 32-bit plan offsets")

    @property
    def redundancy(self) -> float:
        """Element computations per element (patch halo overhead)."""
        return self.n_pairs / max(1, self.n_elements)

    def to_struct(self) -> _lib.PatchPlan:
        s = _lib.PatchPlan()
        s.n_patches, s.n_elements, s.n_points, s.n_basis = self.n_patches, self.n_elements, self.n_points, self.n_basis
        for name in ("vptr", "vtx", "eptr", "elem", "econn", "rptr", "rows", "racc", "iptr",
                     "inc_elem", "inc_a", "inc_pos", "indptr"):
            setattr(s, name, getattr(self, name).data_ptr())
        s.inc_pack = 0 if self.inc_pack is None else self.inc_pack.data_ptr()
        s.inc_pack32 = 0 if self.inc_pack32 is None else self.inc_pack32.data_ptr()
        s.rdiag = 0 if self.rdiag is None else self.rdiag.data_ptr()
        s.max_vtx, s.max_slots, s.max_rows, s.max_elems = self.max_vtx, self.max_slots, self.max_rows, self.max_elems
        s.max_deg, s.pad1 = self.max_deg, 0
        return s

    def nbytes(self) -> int:
        return sum(getattr(self, n).numel() * getattr(self, n).element_size()
                   for n in ("vptr", "vtx", "eptr", "elem", "econn", "rptr", "rows", "racc", "iptr",
                             "inc_elem", "inc_a", "inc_pos"))
