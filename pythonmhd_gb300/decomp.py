"""Spatial domain decomposition of the 2D step over several GPUs (one block per rank).

The 2D grid is split into py x px blocks.  Each rank advances its block on its
own handle, on an *extended* block: the block plus a halo of ``halo`` cells on
every side that has a neighbour (every side of a periodic axis that is split;
no halo at an outflow edge of the whole grid, where the handle's own outflow
boundary is the true one).  One cycle:

1. the halo exchange: each side's ``halo`` strip of cells and faces comes from the
   neighbouring block's interior -- first along x for the block's rows, then along
   y over the full extended width, so the corner strips arrive too;
2. the global dt: each rank's CFL dt of its extended block (``Grid2D.cfl_dt``; the
   halo cells are copies of real cells), reduced with a MIN over ranks -- the dt
   of the whole grid bit for bit, since dt = cfl / max(speed) and a correctly
   rounded division is monotone (the reference reduces the maximum speed over the
   whole grid, Source/EvolveFunctions_MHD.py:472-475);
3. one cycle of the extended block with that dt (``Grid2D.advance_dt``).  The
   block's interior cells and faces depend only on inputs within the footprint of
   one cycle (``FOOTPRINT``: at most 4 cells away for PPM, measured by perturbing
   one cell), so with a halo wider than the footprint they come out exactly as in
   a run of the whole grid, and the halo's own, wrong, values are replaced by the
   next exchange.

The exchange is written as a list of copies between ranks (``halo_plan``), so the
same plan runs over ``torch.distributed`` point-to-point messages (NCCL between
GPUs, gloo on CPUs) or as direct copies inside one process.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

OUTFLOW, PERIODIC = 0, 1
# cells one cycle's output depends on, per reconstruction (0 first order, 1 PLM, 2 PPM):
# one perturbed cell changes cells and faces at most this far away after one cycle
FOOTPRINT = {0: 2, 1: 3, 2: 4}


def default_halo(recon):
    """Halo width: the footprint of one cycle plus one cell of margin."""
    return FOOTPRINT[recon] + 1


def _splits(n, parts):
    """Block edges of n cells in `parts` nearly equal blocks."""
    return [n * k // parts for k in range(parts + 1)]


@dataclass(frozen=True)
class Block:
    rank: int
    by: int                # block row / column in the py x px layout
    bx: int
    y0: int                # interior cells [y0, y1) x [x0, x1) of the whole grid
    y1: int
    x0: int
    x1: int
    hy: tuple              # halo cells below / above (0 at an outflow edge or an unsplit axis)
    hx: tuple              # halo cells left / right
    bcy: int               # boundary condition of the extended block's handle
    bcx: int

    @property
    def shape(self):
        """(ny, nx) of the extended block."""
        return (self.y1 - self.y0 + self.hy[0] + self.hy[1], self.x1 - self.x0 + self.hx[0] + self.hx[1])

    @property
    def interior(self):
        """Slices of the interior cells in the extended block."""
        ny, nx = self.shape
        return slice(self.hy[0], ny - self.hy[1]), slice(self.hx[0], nx - self.hx[1])


class Decomposition:
    """py x px blocks of an ny x nx grid with boundary conditions bcx, bcy (0 outflow,
    1 periodic); rank r holds block (r // px, r % px)."""

    def __init__(self, ny, nx, py, px, bcx=PERIODIC, bcy=PERIODIC, halo=5):
        if py < 1 or px < 1 or ny < py or nx < px:
            raise ValueError("more blocks than cells along an axis")
        self.ny, self.nx, self.py, self.px = int(ny), int(nx), int(py), int(px)
        self.bcx, self.bcy, self.halo = int(bcx), int(bcy), int(halo)
        self.ys, self.xs = _splits(ny, py), _splits(nx, px)
        for edges, n, p, bc in ((self.ys, ny, py, bcy), (self.xs, nx, px, bcx)):
            sizes = np.diff(edges)
            # a neighbour's strip must lie inside its interior, and a block must hold cells
            if p > 1 and sizes.min() < self.halo:
                raise ValueError(f"blocks of {sizes.min()} cells are thinner than the halo ({self.halo})")
        self.blocks = [self._block(r) for r in range(py * px)]

    @property
    def size(self):
        return self.py * self.px

    def _halo(self, k, p, bc):
        if p == 1:
            return (0, 0), bc                   # unsplit axis: the handle's own boundary condition
        lo = self.halo if (bc == PERIODIC or k > 0) else 0
        hi = self.halo if (bc == PERIODIC or k < p - 1) else 0
        return (lo, hi), OUTFLOW               # split axis: halos; the handle's edges are outflow

    def _block(self, r):
        by, bx = divmod(r, self.px)
        hy, bcy = self._halo(by, self.py, self.bcy)
        hx, bcx = self._halo(bx, self.px, self.bcx)
        return Block(r, by, bx, self.ys[by], self.ys[by + 1], self.xs[bx], self.xs[bx + 1], hy, hx, bcy, bcx)

    def neighbour(self, r, axis, step):
        """Rank of the block `step` (+-1) along axis (0 y, 1 x) from rank r, or None."""
        b = self.blocks[r]
        by, bx = b.by, b.bx
        if axis == 0:
            by += step
            if not 0 <= by < self.py:
                if self.bcy != PERIODIC:
                    return None
                by %= self.py
        else:
            bx += step
            if not 0 <= bx < self.px:
                if self.bcx != PERIODIC:
                    return None
                bx %= self.px
        return by * self.px + bx

    # -- whole grid <-> extended blocks ---------------------------------------
    def local_state(self, r, prim, cons, fbx=None, fby=None):
        """The extended block of rank r cut from a whole-grid state (halos included,
        wrapped across periodic edges): (prim, cons[, faceBx, faceBy])."""
        b = self.blocks[r]
        ny_e, nx_e = b.shape
        rows = np.mod(np.arange(b.y0 - b.hy[0], b.y0 - b.hy[0] + ny_e), self.ny)
        cols = np.mod(np.arange(b.x0 - b.hx[0], b.x0 - b.hx[0] + nx_e), self.nx)
        out = [np.ascontiguousarray(a[:, rows][:, :, cols]) for a in (prim, cons)]
        if fbx is not None:
            # face f of a periodic axis of n cells is face f mod n (face n duplicates face 0)
            fcols = np.arange(b.x0 - b.hx[0], b.x0 - b.hx[0] + nx_e + 1)
            fcols = np.mod(fcols, self.nx) if self.bcx == PERIODIC else fcols
            frows = np.arange(b.y0 - b.hy[0], b.y0 - b.hy[0] + ny_e + 1)
            frows = np.mod(frows, self.ny) if self.bcy == PERIODIC else frows
            out.append(np.ascontiguousarray(fbx[rows][:, fcols]))
            out.append(np.ascontiguousarray(fby[frows][:, cols]))
        return tuple(out)

    def assemble(self, locals_):
        """Whole-grid state from every rank's extended block (interiors and their faces;
        a face two blocks share is computed by both, equally)."""
        first = locals_[0]
        mhd = len(first) == 4
        nv = first[0].shape[0]
        prim = np.empty((nv, self.ny, self.nx))
        cons = np.empty_like(prim)
        fbx = np.empty((self.ny, self.nx + 1)) if mhd else None
        fby = np.empty((self.ny + 1, self.nx)) if mhd else None
        for b, st in zip(self.blocks, locals_):
            iy, ix = b.interior
            prim[:, b.y0:b.y1, b.x0:b.x1] = st[0][:, iy, ix]
            cons[:, b.y0:b.y1, b.x0:b.x1] = st[1][:, iy, ix]
            if mhd:
                fbx[b.y0:b.y1, b.x0:b.x1 + 1] = st[2][iy, ix.start:ix.stop + 1]
                fby[b.y0:b.y1 + 1, b.x0:b.x1] = st[3][iy.start:iy.stop + 1, ix]
        return (prim, cons, fbx, fby) if mhd else (prim, cons)


@dataclass(frozen=True)
class Copy:
    """One strip of one array moved from rank src to rank dst.  ``array``: 0 prim,
    1 cons, 2 faceBx, 3 faceBy; ``sel_src`` / ``sel_dst``: (row slice, column slice)
    in the two extended blocks (the leading variable axis of prim/cons is whole)."""
    src: int
    dst: int
    array: int
    sel_src: tuple
    sel_dst: tuple
    phase: int             # 0 along x, 1 along y (y copies read what x copies wrote)


def _strips(b_src, b_dst, axis, step, faces_normal, h):
    """Source and destination index ranges along `axis` for a strip that block b_dst
    receives from its neighbour b_src at `step` (+1: the neighbour is above / to the right)."""
    lo_s = b_src.hy[0] if axis == 0 else b_src.hx[0]
    n_s = (b_src.y1 - b_src.y0) if axis == 0 else (b_src.x1 - b_src.x0)
    lo_d = b_dst.hy[0] if axis == 0 else b_dst.hx[0]
    n_d = (b_dst.y1 - b_dst.y0) if axis == 0 else (b_dst.x1 - b_dst.x0)
    if step > 0:
        # dst's upper halo <- src's lowest interior cells (faces: skip the shared face)
        s0 = lo_s + (1 if faces_normal else 0)
        d0 = lo_d + n_d + (1 if faces_normal else 0)
    else:
        # dst's lower halo <- src's highest interior cells (faces: below the shared face)
        s0 = lo_s + n_s - h
        d0 = lo_d - h
    return slice(s0, s0 + h), slice(d0, d0 + h)


def halo_plan(dec: Decomposition, mhd=True):
    """Every copy of one halo exchange, phase 0 (x) before phase 1 (y)."""
    plan = []
    for phase, axis in ((0, 1), (1, 0)):
        for b in dec.blocks:
            halos = b.hy if axis == 0 else b.hx
            for side, step in ((0, -1), (1, +1)):
                h = halos[side]
                if h == 0:
                    continue
                src = dec.neighbour(b.rank, axis, step)
                if src is None:
                    continue
                bs = dec.blocks[src]
                ny_e, nx_e = b.shape
                ny_s, nx_s = bs.shape
                for arr in ((0, 1, 2, 3) if mhd else (0, 1)):
                    normal = (arr == 2 and axis == 1) or (arr == 3 and axis == 0)
                    a_s, a_d = _strips(bs, b, axis, step, normal, h)
                    if axis == 1:
                        # along x: the interior rows (faceBy: its interior face rows)
                        iy_s, iy_d = bs.interior[0], b.interior[0]
                        if arr == 3:
                            iy_s = slice(iy_s.start, iy_s.stop + 1)
                            iy_d = slice(iy_d.start, iy_d.stop + 1)
                        plan.append(Copy(src, b.rank, arr, (iy_s, a_s), (iy_d, a_d), phase))
                    else:
                        # along y: the full extended width (faceBx: one more column)
                        w_s = slice(0, nx_s + (1 if arr == 2 else 0))
                        w_d = slice(0, nx_e + (1 if arr == 2 else 0))
                        plan.append(Copy(src, b.rank, arr, (a_s, w_s), (a_d, w_d), phase))
    return plan


def _view(state, arr, sel):
    a = state[arr]
    return a[:, sel[0], sel[1]] if arr < 2 else a[sel[0], sel[1]]


def exchange_local(plan, states):
    """Run a halo exchange between blocks held in one process (NumPy arrays or torch
    tensors, indexable per rank)."""
    for phase in (0, 1):
        for c in plan:
            if c.phase == phase:
                dst = _view(states[c.dst], c.array, c.sel_dst)
                src = _view(states[c.src], c.array, c.sel_src)
                if hasattr(dst, "copy_"):
                    dst.copy_(src)
                else:
                    dst[...] = src


def exchange_dist(plan, rank, state, group=None):
    """This rank's part of a halo exchange over torch.distributed: for every copy it
    sends or receives, a contiguous buffer goes point to point (NCCL for CUDA tensors,
    gloo for CPU tensors); phase 1 starts after phase 0 has landed."""
    import torch
    import torch.distributed as dist
    for phase in (0, 1):
        ops, recvs = [], []
        for c in plan:
            if c.phase != phase:
                continue
            if c.src == rank and c.dst == rank:
                _view(state, c.array, c.sel_dst).copy_(_view(state, c.array, c.sel_src))
                continue
            if c.src == rank:
                buf = _view(state, c.array, c.sel_src).contiguous()
                ops.append(dist.P2POp(dist.isend, buf, c.dst, group))
            if c.dst == rank:
                buf = torch.empty_like(_view(state, c.array, c.sel_dst).contiguous())
                recvs.append((c, buf))
                ops.append(dist.P2POp(dist.irecv, buf, c.src, group))
        if ops:
            for req in dist.batch_isend_irecv(ops):
                req.wait()
        for c, buf in recvs:
            _view(state, c.array, c.sel_dst).copy_(buf)


def global_dt(local_dt, group=None, device=None):
    """MIN over ranks of the blocks' CFL dts (the dt of the whole grid)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(local_dt)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MIN, group=group)
    return float(t.item())


def clip_dt(t, dt, t_end):
    """The evolve loop's end-time clip (Source/EvolveFunctions_MHD.py:474-475)."""
    return t_end - t if t + dt > t_end else dt


def run_block(block, exchange, reduce_min, t0, t_end, cycle0, max_cycles, cfl):
    """The evolve loop of one rank's block (Source/EvolveFunctions_MHD.py:464-692):
    while t < t_end and cycle < max_cycles, exchange the halos, agree on the global
    dt and advance one cycle.  ``block`` holds the extended state (``block.state``)
    and provides ``cfl_dt(cfl)`` and ``step(t, t_end, cycle, dt) -> t``; ``exchange``
    fills the halos of ``block.state``; ``reduce_min`` is the MIN over ranks.  Every
    rank runs the same number of cycles with the same dts.  Returns (t, cycle)."""
    t, cyc = t0, cycle0
    while t < t_end and cyc < max_cycles:
        exchange(block.state)
        dt = reduce_min(block.cfl_dt(cfl))
        t = block.step(t, t_end, cyc, dt)
        cyc += 1
    return t, cyc


class DeviceBlock:
    """One rank's extended block on a GPU handle (``Grid2D``): the state lives in torch
    tensors on the device (the halo exchange reads and writes them), and each cycle
    is copied into the handle and back on the device."""

    def __init__(self, dec, rank, dx, dy, gamma, mhd=True, recon=2, entropy_fix=False, eps=0.5, min_d=1e-12,
                 min_p=1e-12, min_e=1e-12, arith="exact", device=None, state=None):
        import torch
        from .solver import Grid2D
        b = dec.blocks[rank]
        ny, nx = b.shape
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.grid = Grid2D(ny, nx, dx, dy, b.bcx, b.bcy, gamma, mhd=mhd, recon=recon, entropy_fix=entropy_fix,
                           eps=eps, min_d=min_d, min_p=min_p, min_e=min_e, arith=arith)
        self.state = tuple(torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=self.device)
                           for a in state)

    def cfl_dt(self, cfl):
        self.grid.upload_device(*self.state)
        return self.grid.cfl_dt(cfl)

    def step(self, t, t_end, cycle, dt):
        t_new = self.grid.advance_dt(t, t_end, cycle, dt)
        self.grid.download_device(0, *self.state)
        return t_new

    def close(self):
        self.grid.close()


def run_local(blocks, plan, t0, t_end, cycle0, max_cycles, cfl):
    """The decomposed loop with every rank's block in this process (ranks in lock step:
    exchange, MIN of the blocks' dts, one cycle each).  The same cycles and dts as
    ``run_block`` on separate ranks; used to check the decomposition on one GPU."""
    t, cyc = t0, cycle0
    while t < t_end and cyc < max_cycles:
        exchange_local(plan, [b.state for b in blocks])
        dt = min(b.cfl_dt(cfl) for b in blocks)
        ts = [b.step(t, t_end, cyc, dt) for b in blocks]
        t = ts[0]
        cyc += 1
    return t, cyc
