"""Box-slab decomposition of one system over ranks: the multi-GPU step.

Replaces python-bh/barneshut/implementations/multigpu.py (create_tree :264-294, summarize
:296-306, evaluate :308-310 with copy_nonresident_neighbors :166-196).  The reference gathers
every particle on the host each step and re-splits; here each rank keeps only the particles of
its own boxes and exchanges with the others through torch.distributed (point-to-point sends and
all-reduces, so the same code runs over gloo on CPU tensors and over NCCL on CUDA tensors).
Per step:

1. bounding box: all-reduce of the ranks' extents; every rank squares the same box and derives
   the same step (helpers/grid.py:10-26, base.py:233);
2. ownership: the boxes in x-major order split into `world` contiguous ranges of (nearly) equal
   box count, as np.array_split splits them (multigpu.py:287-294); particles whose box another
   rank owns move to that rank (x, y, m, vx, vy, pid);
3. summarize: each rank's leaf moments (M, Sx, Sy, Sxx, Sxy, Syy about each box origin, FP64) of
   its own boxes, summed over ranks into the whole grid's B x 6 moments -- every box is non-zero
   on one rank only, so the sum is exact (multigpu.py:149-155, 303-306);
4. halo: the (x, y, m) of a rank's particles in boxes within `reach` boxes (Chebyshev distance)
   of another rank's range go to that rank (multigpu.py:166-196 sends the 8 neighbours, reach
   1, which is the flat far field's near field; the opening-angle near field reaches further,
   halo_reach);
5. evaluate: the rank's own particles against its own and halo particles for the near field and
   the whole grid's moments for the far field, through an evaluator callable; then the tick
   (gpu/grid.py:159-174).

Within a box, particles are kept in particle-id order on every rank, so the sums each box and
each target accumulate run in the same order as on a single rank.
"""
import math

import numpy as np

FIELDS = 6  # x, y, m, vx, vy, pid (pid carried as float64, exact below 2**53)


def box_ranges(G, world):
    """Owned box range [b0, b1) of each rank: the G*G boxes in x-major order (box = gx * G + gy)
    split like np.array_split (the first B % world ranges one box longer)."""
    B = G * G
    q, r = divmod(B, world)
    out, b = [], 0
    for k in range(world):
        n = q + (1 if k < r else 0)
        out.append((b, b + n))
        b += n
    return out


def owner_of_boxes(boxes, ranges):
    """Rank owning each box index."""
    starts = np.array([r[0] for r in ranges], dtype=np.int64)
    return np.searchsorted(starts, np.asarray(boxes, dtype=np.int64), side="right") - 1


def square_box(mnx, mny, mxx, mxy, G):
    """The square bounding box of helpers/grid.py:10-26 from the extents: the shorter side's
    maximum moves out to the longer side's length; step = edge / G.  Returns (min_x, min_y,
    max_x, max_y, step) in the oracle's layout."""
    xe, ye = mxx - mnx, mxy - mny
    if xe > ye:
        mxy += xe - ye
    elif ye > xe:
        mxx += ye - xe
    return np.array([mnx, mny, mxx, mxy, (mxx - mnx) / G])


def box_keys(x, y, bb, G):
    """clip(floor((p - min) / step), 0, G - 1) per coordinate (sequential.py:32-34)."""
    kx = np.clip(np.floor((x - bb[0]) / bb[4]), 0, G - 1).astype(np.int64)
    ky = np.clip(np.floor((y - bb[1]) / bb[4]), 0, G - 1).astype(np.int64)
    return kx, ky


def halo_reach(theta, group_dim):
    """Boxes (Chebyshev distance from a target's box) that its near field can reach: 1 for the
    flat far field (theta <= 0, the 3 x 3 neighbourhood); in theta mode a near box is rejected
    for the target's group rectangle, so its centre of mass lies within 1/theta box edges of
    that rectangle -- floor(1/theta) + 1 boxes beyond it, one more for rounding -- and the
    rectangle reaches group_dim - 1 boxes past the target's box."""
    if theta <= 0:
        return 1
    return (group_dim - 1) + int(math.floor(1.0 / theta)) + 2


def halo_boxes(G, b0, b1, reach):
    """Boxes outside [b0, b1) within `reach` boxes (Chebyshev) of a box in it."""
    if b1 <= b0:
        return np.zeros(0, dtype=np.int64)
    own = np.arange(b0, b1, dtype=np.int64)
    gx, gy = own // G, own % G
    mask = np.zeros((G, G), dtype=bool)
    for ddx in range(-reach, reach + 1):
        xs = gx + ddx
        okx = (xs >= 0) & (xs < G)
        for ddy in range(-reach, reach + 1):
            ys = gy + ddy
            ok = okx & (ys >= 0) & (ys < G)
            mask[xs[ok], ys[ok]] = True
    flat = mask.ravel()
    flat[b0:b1] = False
    return np.flatnonzero(flat)


class SlabComm:
    """The collectives the slab step needs, over torch.distributed (gloo or NCCL).  Tensors live
    on `device` (CPU for gloo, the rank's GPU for NCCL)."""

    def __init__(self, device="cpu"):
        import torch
        import torch.distributed as dist

        self.torch, self.dist = torch, dist
        self.device = device
        self.rank = dist.get_rank()
        self.world = dist.get_world_size()

    def allreduce(self, arr, op):
        t = self.torch.as_tensor(np.ascontiguousarray(arr, dtype=np.float64), device=self.device)
        self.dist.all_reduce(t, op=op)
        return t.cpu().numpy()

    def extents(self, x, y):
        R = self.dist.ReduceOp
        if len(x):
            mn = np.array([x.min(), y.min()])
            mx = np.array([x.max(), y.max()])
        else:
            mn, mx = np.full(2, np.inf), np.full(2, -np.inf)
        return self.allreduce(mn, R.MIN), self.allreduce(mx, R.MAX)

    def sum(self, arr):
        return self.allreduce(arr, self.dist.ReduceOp.SUM)

    def exchange(self, parts):
        """parts[r]: (n_r, k) float64 rows for rank r.  Returns the rows every rank sent here,
        concatenated in rank order (this rank's own part in its place)."""
        torch, dist = self.torch, self.dist
        k = parts[self.rank].shape[1]
        cnt = torch.tensor([p.shape[0] for p in parts], dtype=torch.int64, device=self.device)
        allc = [torch.zeros_like(cnt) for _ in range(self.world)]
        dist.all_gather(allc, cnt)
        recv = [None] * self.world
        ops = []
        for r in range(self.world):
            if r == self.rank:
                continue
            n_in = int(allc[r][self.rank])
            recv[r] = torch.empty((n_in, k), dtype=torch.float64, device=self.device)
            if parts[r].shape[0]:
                ops.append(dist.P2POp(dist.isend, torch.as_tensor(np.ascontiguousarray(parts[r]),
                                                                  device=self.device), r))
            if n_in:
                ops.append(dist.P2POp(dist.irecv, recv[r], r))
        if ops:
            for w in dist.batch_isend_irecv(ops):
                w.wait()
        out = []
        for r in range(self.world):
            out.append(parts[r] if r == self.rank else recv[r].cpu().numpy())
        return np.concatenate(out, axis=0) if out else np.zeros((0, k))


class SlabSystem:
    """One rank's share of a system: the particles of its own boxes, state rows
    (x, y, m, vx, vy, pid) sorted by pid."""

    def __init__(self, state, G, comm, theta=0.5, group_dim=1):
        self.G = G
        self.comm = comm
        self.theta = theta
        self.group_dim = group_dim if theta > 0 else 1
        self.ranges = box_ranges(G, comm.world)
        self.state = np.asarray(state, dtype=np.float64).reshape(-1, FIELDS)
        self.reach = halo_reach(theta, self.group_dim)

    # -------------------------------------------------------------- create_tree
    def create_tree(self):
        """Bounding box over all ranks, every particle to the rank owning its box, then the
        near-field halo from the other ranks."""
        s = self.state
        mn, mx = self.comm.extents(s[:, 0], s[:, 1])
        self.extents = np.array([mn[0], mn[1], mx[0], mx[1]])
        self.bb = square_box(mn[0], mn[1], mx[0], mx[1], self.G)
        kx, ky = box_keys(s[:, 0], s[:, 1], self.bb, self.G)
        dest = owner_of_boxes(kx * self.G + ky, self.ranges)
        parts = [s[dest == r] for r in range(self.comm.world)]
        mine = self.comm.exchange(parts)
        self.state = mine[np.argsort(mine[:, 5], kind="stable")]
        kx, ky = box_keys(self.state[:, 0], self.state[:, 1], self.bb, self.G)
        self.box = kx * self.G + ky
        b0, b1 = self.ranges[self.comm.rank]
        assert np.all((self.box >= b0) & (self.box < b1)), "particle outside the rank's boxes"
        self.halo = self.exchange_halo()

    def exchange_halo(self):
        """(x, y, m) of the particles of the other ranks' boxes that this rank's near field
        reaches, in particle-id order."""
        world, rank = self.comm.world, self.comm.rank
        parts = []
        for r in range(world):
            if r == rank:
                parts.append(np.zeros((0, 4)))
                continue
            want = halo_boxes(self.G, *self.ranges[r], self.reach)
            sel = np.isin(self.box, want)
            s = self.state[sel]
            parts.append(np.column_stack([s[:, 0], s[:, 1], s[:, 2], s[:, 5]]))
        h = self.comm.exchange(parts)
        if len(h):
            h = h[np.argsort(h[:, 3], kind="stable")]
        return h[:, :3]

    def local_particles(self):
        """x, y, m of the rank's own particles followed by its halo."""
        s, h = self.state, self.halo
        return (np.concatenate([s[:, 0], h[:, 0]]), np.concatenate([s[:, 1], h[:, 1]]),
                np.concatenate([s[:, 2], h[:, 2]]))

    # ---------------------------------------------------------------- summarize
    def summarize(self, leaf_moments):
        """leaf_moments(x, y, m, G, bb) -> (G, G, 6) leaf moments of the local particles; the
        rank keeps those of its own boxes, and the whole grid's moments are their sum over
        ranks."""
        x, y, m = self.local_particles()
        local = np.array(leaf_moments(x, y, m, self.G, self.bb), dtype=np.float64).reshape(-1, 6)
        b0, b1 = self.ranges[self.comm.rank]
        local[:b0] = 0.0
        local[b1:] = 0.0
        self.leaf = self.comm.sum(local.reshape(-1)).reshape(self.G, self.G, 6)

    # ----------------------------------------------------------------- evaluate
    def evaluate(self, evaluator):
        """evaluator(x, y, m, targets, bb, leaf, extents) -> (ax, ay) over the local particles
        (own then halo) of which the rows `targets` (the own ones) are used."""
        x, y, m = self.local_particles()
        own = np.arange(len(self.state))
        ax, ay = evaluator(x, y, m, own, self.bb, self.leaf, self.extents)
        self.ax, self.ay = np.asarray(ax)[own], np.asarray(ay)[own]
        return self.ax, self.ay

    def timestep(self, dt):
        """v += a dt; x += v dt (gpu/grid.py:159-174)."""
        s = self.state
        s[:, 3] = s[:, 3] + self.ax * dt
        s[:, 4] = s[:, 4] + self.ay * dt
        s[:, 0] = s[:, 0] + s[:, 3] * dt
        s[:, 1] = s[:, 1] + s[:, 4] * dt


class PlanSlab:
    """The CUDA step on one rank's part of a system: a plan over the rank's own and halo
    particles whose grid is the whole system's (bh_set_grid) and whose far field comes from the
    whole grid's leaf moments (bh_set_leaf_moments).  `leaf_moments` (for SlabSystem.summarize)
    builds the plan and returns its leaf moments; the instance is then the evaluator."""

    def __init__(self, params, device="cuda"):
        self.params = params
        self.device = device
        self.plan = None

    def leaf_moments(self, x, y, m, G, bb):
        from . import native

        if self.plan is not None:
            self.plan.close()
        n = len(x)
        self.plan = native.Plan([n], [G], self.params, device=self.device)
        self.plan.set_grid(self._extents)
        z = np.zeros(n)
        self.plan.load(x, y, m, z, z)
        self.plan.create_tree()
        self.plan.summarize()
        return self.plan.leaf_moments().cpu().numpy()

    def bind(self, slab):
        """Take the whole system's extents of the step from `slab` (after its create_tree)."""
        self._extents = slab.extents
        return self

    def __call__(self, x, y, m, targets, bb, leaf, extents):
        self.plan.set_leaf_moments(leaf)
        self.plan.evaluate()
        o = self.plan.store()
        return o["ax"].cpu().numpy(), o["ay"].cpu().numpy()

    def close(self):
        if self.plan is not None:
            self.plan.close()
            self.plan = None
