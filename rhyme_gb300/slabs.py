"""One box decomposed into slabs along its outermost axis, one slab per GPU.

Each slab is a box of its own: the whole box's extent across the outermost
axis and its share of the rows along it, with two ghost rows on each side.
Its faces on that axis have the HALO boundary type, which the ghost fill
leaves alone, except the first slab's left face and the last slab's right
face when the whole box's face there is not periodic (those keep the box's
type). One step of the whole box (src/main.f90:109-134) becomes:

1. dt: each slab's CFL time step and the minimum over the slabs, which is
   the whole box's dt bit for bit (dt = RN(courant minval(dx) / max) falls
   as the maximum grows, so the minimum is the one at the largest maximum);
2. the ghost fill of each slab (its HALO faces untouched);
3. the halo exchange: each slab's first two interior rows go to the right
   ghost rows of its left neighbour, its last two interior rows to the left
   ghost rows of its right neighbour (the ends are neighbours when the box
   is periodic along the axis);
4. the solve of each slab.

The slabs' interiors then equal the whole box's interior after every step.
run_local() steps all slabs in one process (one GPU, or the CPU oracle);
run_rank() is one rank of a torch.distributed job (gloo or NCCL), the dt
minimum an all-reduce and the exchange point-to-point messages. The
operations on a slab come from an `ops` object: dt(s), fill(s),
get_rows(s, row0, n), set_rows(s, row0, rows), solve(s, dt), with
GpuOps (rhyme_gb300.gpu) here.
"""
import numpy as np

from .params import HALO, PERIODIC

GHOST = 2


def split_rows(n, parts):
    """Interior rows (start, count) of each slab, near-equal, count >= 2."""
    if parts < 1 or n < 2 * parts:
        raise ValueError("%d rows cannot make %d slabs of at least 2 rows" % (n, parts))
    base, extra = divmod(n, parts)
    out, start = [], 0
    for r in range(parts):
        c = base + (1 if r < extra else 0)
        out.append((start, c))
        start += c
    return out


def slab_cells(cells, start, count):
    """The slab's ghosted array (a copy): rows [start, start + count + 4) of
    the whole box's outermost axis (cells in the reference layout, shape
    (NCMP, rows, ...))."""
    return np.ascontiguousarray(cells[:, start:start + count + 2 * GHOST])


def slab_bc(bc, ndim, r, parts):
    """Boundary types of slab r of `parts`: HALO on the outermost axis'
    faces that border another slab."""
    out = list(bc) + [bc[-1]] * (6 - len(bc))
    if parts == 1:
        return out
    lo, hi = 2 * (ndim - 1), 2 * (ndim - 1) + 1
    periodic = bc[lo] == PERIODIC and bc[hi] == PERIODIC
    if r > 0 or periodic:
        out[lo] = HALO
    if r < parts - 1 or periodic:
        out[hi] = HALO
    return out


def neighbours(r, parts, periodic):
    """(left, right) slab of slab r, None where the box ends."""
    left = r - 1 if r > 0 else (parts - 1 if periodic and parts > 1 else None)
    right = r + 1 if r < parts - 1 else (0 if periodic and parts > 1 else None)
    return left, right


def run_local(slabs, counts, nsteps, ops, periodic):
    """nsteps steps of all slabs in this process; returns the dt trace."""
    parts = len(slabs)
    dts = []
    for _ in range(nsteps):
        dt = min(ops.dt(s) for s in slabs)
        for s in slabs:
            ops.fill(s)
        if parts > 1:
            firsts = [ops.get_rows(s, GHOST, GHOST) for s in slabs]
            lasts = [ops.get_rows(s, c, GHOST) for s, c in zip(slabs, counts)]
            for r in range(parts):
                left, right = neighbours(r, parts, periodic)
                if left is not None:
                    ops.set_rows(slabs[left], counts[left] + GHOST, firsts[r])
                if right is not None:
                    ops.set_rows(slabs[right], 0, lasts[r])
        for s in slabs:
            ops.solve(s, dt)
        dts.append(dt)
    return np.array(dts)


def run_rank(slab, count, nsteps, ops, periodic, rank, world, device=None):
    """nsteps steps of this rank's slab in a torch.distributed job of
    `world` ranks (slab r on rank r); returns the dt trace. The dt and the
    halo rows travel as tensors on `device`: by default the current CUDA
    device under NCCL (which carries only CUDA tensors), the CPU otherwise."""
    import torch
    import torch.distributed as dist
    if device is None:
        device = "cuda" if world > 1 and dist.get_backend() == "nccl" else "cpu"
    dts = []
    left, right = neighbours(rank, world, periodic)
    # rows that stay on the GPU: the library copies them straight into CUDA
    # tensors, which NCCL sends and receives (no host staging)
    on_device = str(device).startswith("cuda") and hasattr(ops, "rows_into")
    if on_device and world > 1:
        shape = ops.rows_shape(slab, GHOST)
        first, last, into_right, into_left = (torch.empty(shape, dtype=torch.float64, device=device)
                                              for _ in range(4))
    for _ in range(nsteps):
        if world > 1:
            t = torch.tensor([ops.dt(slab)], dtype=torch.float64, device=device)
            dist.all_reduce(t, op=dist.ReduceOp.MIN)
            dt = float(t.item())
        else:
            dt = ops.dt(slab)
        ops.fill(slab)
        if world > 1:
            if on_device:
                ops.rows_into(slab, GHOST, GHOST, first)
                ops.rows_into(slab, count, GHOST, last)
            else:
                first = torch.from_numpy(ops.get_rows(slab, GHOST, GHOST)).to(device)
                last = torch.from_numpy(ops.get_rows(slab, count, GHOST)).to(device)
                into_right = torch.empty_like(first)  # -> my right ghost rows
                into_left = torch.empty_like(last)    # -> my left ghost rows
            # two phases, rows travelling left then rows travelling right, so
            # that a pair of ranks (both neighbours of each other when two
            # ranks wrap around) has one message each way per phase: NCCL
            # matches messages by order, not by tag
            for send, to, recv, frm in ((first, left, into_right, right), (last, right, into_left, left)):
                reqs = []
                if to is not None:
                    reqs.append(dist.P2POp(dist.isend, send, to))
                if frm is not None:
                    reqs.append(dist.P2POp(dist.irecv, recv, frm))
                if reqs:
                    for q in dist.batch_isend_irecv(reqs):
                        q.wait()
            if on_device:
                # the receives ran on torch's stream; the library copies on its own
                torch.cuda.current_stream().synchronize()
                if left is not None:
                    ops.set_rows(slab, 0, into_left)
                if right is not None:
                    ops.set_rows(slab, count + GHOST, into_right)
            else:
                if left is not None:
                    ops.set_rows(slab, 0, into_left.cpu().numpy())
                if right is not None:
                    ops.set_rows(slab, count + GHOST, into_right.cpu().numpy())
        ops.solve(slab, dt)
        dts.append(dt)
    return np.array(dts)


class GpuOps:
    """Slab operations through the C-ABI (rhyme_gb300.gpu): a slab is
    (context, box)."""

    def __init__(self, dx):
        self.dx = dx

    def dt(self, s):
        ctx, box = s
        return ctx.cfl_time_step(box, self.dx)

    def fill(self, s):
        ctx, box = s
        ctx.set_boundaries(box)

    def get_rows(self, s, row0, n):
        ctx, box = s
        return ctx.get_rows(box, row0, n)

    def rows_shape(self, s, n):
        ctx, box = s
        return ctx.rows_shape(box, n)

    def rows_into(self, s, row0, n, out):
        """The rows into a CUDA tensor (device to device)."""
        ctx, box = s
        ctx.get_rows(box, row0, n, out=out)

    def set_rows(self, s, row0, rows):
        ctx, box = s
        ctx.set_rows(box, row0, rows)

    def solve(self, s, dt):
        ctx, box = s
        ctx.muscl_hancock_solve(box, self.dx, dt)
