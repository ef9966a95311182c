"""Slab decomposition of the solver's fields over ranks, and the all-to-all
transposes between z-slabs and y-slabs.

This is the one-rank-per-GPU form of the reference's 2DECOMP pencil
transposes (``transpose_x_to_y`` / ``transpose_y_to_z`` and back, called
from src/transeq.f90, src/navier.f90 and src/poisson.f90 around every y and
z line solve and FFT pass).  A field is a C-ordered (nz, ny, nx) array, x
fastest, as everywhere in this package.

* z-slabs: rank r holds the planes z in [zs[r], ze[r]) with all y and x, so
  x and y lines (compact solves, the x and y FFT passes) are local;
* y-slabs: rank r holds the rows y in [ys[r], ye[r]) with all z and x, so x
  and z lines are local;
* one all-to-all moves a field between the two: rank r sends to rank s the
  block z in [zs[r], ze[r]), y in [ys[s], ye[s]) (contiguous after packing),
  and places the block received from s at z in [zs[s], ze[s]).

A step sharded this way runs the x and y work on z-slabs, one transpose of
the fields to y-slabs for the z lines and the z FFT pass, and one back; the
only other exchange is the sum of the diagnostics (``allreduce_sum``).

Blocks are split as evenly as possible, the remainder going to the first
ranks; a rank may own no plane (more ranks than planes).  The module moves
data only, through ``torch.distributed.all_to_all_single``: host tensors on
the gloo backend, device tensors on NCCL.  Trailing dimensions after x are
carried along (e.g. a complex field viewed as (..., 2) reals).
"""


def block_range(n, size, rank):
    """[start, end) of rank's share of n items split over size ranks."""
    if n < 0 or size < 1 or not 0 <= rank < size:
        raise ValueError("block_range: n >= 0, size >= 1, 0 <= rank < size")
    base, extra = divmod(n, size)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


class Slabs:
    """Index maps of the z-slab and y-slab decompositions of an
    (nz, ny, nx) grid over `size` ranks, seen from `rank`."""

    def __init__(self, nx, ny, nz, rank, size):
        if min(nx, ny, nz) < 1:
            raise ValueError("Slabs: grid dimensions must be positive")
        self.nx, self.ny, self.nz = nx, ny, nz
        self.rank, self.size = rank, size
        self.zr = [block_range(nz, size, r) for r in range(size)]
        self.yr = [block_range(ny, size, r) for r in range(size)]

    @property
    def z_slab(self):
        """(start, end) of this rank's z planes."""
        return self.zr[self.rank]

    @property
    def y_slab(self):
        """(start, end) of this rank's y rows."""
        return self.yr[self.rank]

    def z_shape(self):
        z0, z1 = self.z_slab
        return (z1 - z0, self.ny, self.nx)

    def y_shape(self):
        y0, y1 = self.y_slab
        return (self.nz, y1 - y0, self.nx)

    def z_to_y(self, a, group=None):
        """This rank's z-slab (nzl, ny, nx, ...) -> its y-slab (nz, nyl, nx, ...)."""
        import torch
        import torch.distributed as dist
        rest = tuple(a.shape[3:])
        if tuple(a.shape[:3]) != self.z_shape():
            raise ValueError(f"z_to_y: expected a z-slab of shape {self.z_shape()}, got {tuple(a.shape[:3])}")
        nzl = a.shape[0]
        y0, y1 = self.y_slab
        inner = self.nx * _prod(rest)
        send = torch.cat([a[:, ys:ye].reshape(-1) for ys, ye in self.yr]) if self.size > 1 else a.reshape(-1)
        in_splits = [nzl * (ye - ys) * inner for ys, ye in self.yr]
        out_splits = [(ze - zs) * (y1 - y0) * inner for zs, ze in self.zr]
        recv = torch.empty(sum(out_splits), dtype=a.dtype, device=a.device)
        if self.size > 1:
            dist.all_to_all_single(recv, send.contiguous(), out_splits, in_splits, group=group)
        else:
            recv.copy_(send)
        out = torch.empty((self.nz, y1 - y0, self.nx) + rest, dtype=a.dtype, device=a.device)
        off = 0
        for (zs, ze), cnt in zip(self.zr, out_splits):
            out[zs:ze] = recv[off:off + cnt].view((ze - zs, y1 - y0, self.nx) + rest)
            off += cnt
        return out

    def y_to_z(self, b, group=None):
        """This rank's y-slab (nz, nyl, nx, ...) -> its z-slab (nzl, ny, nx, ...)."""
        import torch
        import torch.distributed as dist
        rest = tuple(b.shape[3:])
        if tuple(b.shape[:3]) != self.y_shape():
            raise ValueError(f"y_to_z: expected a y-slab of shape {self.y_shape()}, got {tuple(b.shape[:3])}")
        nyl = b.shape[1]
        z0, z1 = self.z_slab
        inner = self.nx * _prod(rest)
        send = torch.cat([b[zs:ze].reshape(-1) for zs, ze in self.zr]) if self.size > 1 else b.reshape(-1)
        in_splits = [(ze - zs) * nyl * inner for zs, ze in self.zr]
        out_splits = [(z1 - z0) * (ye - ys) * inner for ys, ye in self.yr]
        recv = torch.empty(sum(out_splits), dtype=b.dtype, device=b.device)
        if self.size > 1:
            dist.all_to_all_single(recv, send.contiguous(), out_splits, in_splits, group=group)
        else:
            recv.copy_(send)
        out = torch.empty((z1 - z0, self.ny, self.nx) + rest, dtype=b.dtype, device=b.device)
        off = 0
        for (ys, ye), cnt in zip(self.yr, out_splits):
            out[:, ys:ye] = recv[off:off + cnt].view((z1 - z0, ye - ys, self.nx) + rest)
            off += cnt
        return out


def allreduce_sum(x, group=None):
    """Sum of a host or device tensor over all ranks (diagnostics such as the
    kinetic energy of postprocess_tgv, src/Case-TGV.f90:189-477)."""
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(x, op=dist.ReduceOp.SUM, group=group)
    return x


def _prod(t):
    p = 1
    for v in t:
        p *= v
    return p
