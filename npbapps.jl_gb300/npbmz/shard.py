"""Zones of one BT-MZ / SP-MZ problem spread over several ranks, one GPU each.

The reference runs one MPI process per zone group: map_zones assigns zones to
processes (src/BT/setup_mpi.jl:123-433, SP: src/SP/setup_mpi.jl:125-435), and
exch_qbc moves the faces between zones of different processes with one MPI
message per face (exch_qbc_send / exch_qbc_recv, src/BT/exchange_qbc.jl:
145-465).  Here:

- `map_zones` restates the reference's mapping on the host;
- `ShardPlan` lists, for one rank, its zones (renumbered 0..n-1 in ascending
  global order, the reference's proc_zone_id order), their neighbour table
  with NPBMZ_REMOTE for faces owned by other ranks, and the faces it sends to
  and receives from each peer in one order both ends agree on;
- `exchange_faces` moves one step's faces with torch.distributed point-to-
  point operations (NCCL between GPUs, gloo on the CPU) between the packed
  buffers of the C ABI (npbmz_pack_faces / npbmz_unpack_faces);
- `ShardedProblem` runs the node loop: pack, exchange, unpack, then
  npbmz_step (the faces between the rank's own zones and adi), with the norms
  summed over ranks by one all-reduce of 10 doubles.

Side numbering follows include/npbmz.h: 0 west, 1 east, 2 south, 3 north.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

WEST, EAST, SOUTH, NORTH = range(4)
OPPOSITE = (EAST, WEST, NORTH, SOUTH)
REMOTE = -1


def map_zones(nranks, nx, ny, nz, nbr, x_zones, y_zones, bload=1):
    """Rank of every zone: the reference's map_zones (src/BT/setup_mpi.jl:
    123-270).  Zones are first ordered by size, largest first (a selection
    sort that keeps the first of equal sizes).  With |bload| <= 1 (the
    reference's call, src/BT/bt-driver.jl:87) a block split of the zone grid
    into n1 x n2 = nranks blocks is used when x_zones and y_zones divide
    evenly; otherwise, and for |bload| > 1, zones go one by one to the
    least-loaded rank, preferring among zones within 5 % of the next one's
    size the zone with the most face points shared with that rank.  The
    reference's later thread rebalancing has no counterpart: a rank is one
    GPU.  Returns an int array (rank per zone, 0-based)."""
    nzn = len(nx)
    if nranks < 1:
        raise ValueError("nranks must be >= 1")
    size = [float(nx[z]) * float(ny[z]) * float(nz[z]) for z in range(nzn)]
    order = list(range(nzn))
    for a in range(nzn - 1):
        best, cur = a, size[order[a]]
        for b in range(a + 1, nzn):
            if cur < size[order[b]]:
                best, cur = b, size[order[b]]
        if best != a:
            order[a], order[best] = order[best], order[a]
    rank_of = [-1] * nzn
    load = [0.0] * nranks
    if abs(bload) <= 1:
        np1 = np2 = 0
        work = y_zones % nranks
        n1, n2 = 1, nranks
        while n1 <= n2:
            if n1 * n2 == nranks:
                w = x_zones % n1 + y_zones % n2
                if w <= work:
                    work, np1, np2 = w, n1, n2
            n1 += 1
            n2 = nranks // n1
        if work == 0:
            bx, by = x_zones // np1, y_zones // np2
            for z in range(nzn):
                r = (z % x_zones) // bx + ((z // x_zones) // by) * np1
                rank_of[z] = r
            return np.array(rank_of, np.int32)
    x_size = [int(nx[i]) for i in range(x_zones)]
    y_size = [int(ny[j * x_zones]) for j in range(y_zones)]

    def comm_index(z, r):
        jz, iz = divmod(z, x_zones)
        c = 0
        if rank_of[nbr[4 * z + WEST]] == r:
            c += y_size[jz]
        if rank_of[nbr[4 * z + EAST]] == r:
            c += y_size[jz]
        if rank_of[nbr[4 * z + SOUTH]] == r:
            c += x_size[iz]
        if rank_of[nbr[4 * z + NORTH]] == r:
            c += x_size[iz]
        return c

    a = 0
    while a < nzn:
        r = 0
        for q in range(1, nranks):
            if load[r] > load[q]:
                r = q
        pick = order[a]
        if a < nzn - 1:
            best = comm_index(pick, r)
            for b in range(a + 1, nzn):
                z2 = order[b]
                if (size[order[a]] - size[z2]) / size[order[a]] > 0.05:
                    break
                if rank_of[z2] < 0:
                    c = comm_index(z2, r)
                    if c > best:
                        pick, best = z2, c
        rank_of[pick] = r
        load[r] += size[pick]
        while a < nzn and rank_of[order[a]] >= 0:
            a += 1
    return np.array(rank_of, np.int32)


def face_size(nx, ny, nz, side):
    """Doubles of one exchanged face: 5 (n-2)(nz-2), n = ny for west/east."""
    return 5 * ((ny if side < 2 else nx) - 2) * (nz - 2)


@dataclass
class ShardPlan:
    """One rank's share of a multi-zone problem and its face traffic."""

    rank: int
    zones: np.ndarray            # global ids of this rank's zones, ascending
    nbr: np.ndarray              # [4 * len(zones)]: local neighbour or REMOTE
    peers: list                  # ranks this rank exchanges faces with, ascending
    send_faces: dict = field(default_factory=dict)  # peer -> [(local zone, side)] in exchange order
    recv_faces: dict = field(default_factory=dict)
    send_span: dict = field(default_factory=dict)   # peer -> (offset, count) in doubles
    recv_span: dict = field(default_factory=dict)

    @property
    def send(self):
        """Every sent face, peer by peer: the list npbmz_face_plan takes."""
        return [f for peer in self.peers for f in self.send_faces.get(peer, [])]

    @property
    def recv(self):
        return [f for peer in self.peers for f in self.recv_faces.get(peer, [])]

    @property
    def send_count(self):
        return sum(c for _, c in self.send_span.values())

    @property
    def recv_count(self):
        return sum(c for _, c in self.recv_span.values())


def shard_plan(rank_of, rank, nx, ny, nz, nbr):
    """The plan of `rank` for the zone-to-rank map rank_of.

    A face travels from zone h (side t) on one rank to zone g = nbr[h][t] on
    another, arriving as g's ghost plane on side opposite(t).  Both ends order
    the faces they exchange with one peer by (g, g's side): the sender by the
    face's destination, the receiver by its own ghost plane."""
    rank_of = np.asarray(rank_of)
    zones = np.flatnonzero(rank_of == rank).astype(np.int32)
    local = {int(g): i for i, g in enumerate(zones)}
    lnbr = np.full(4 * len(zones), REMOTE, np.int32)
    sends, recvs = {}, {}
    for i, g in enumerate(zones):
        for s in range(4):
            o = int(nbr[4 * g + s])
            if rank_of[o] == rank:
                lnbr[4 * i + s] = local[o]
                continue
            peer = int(rank_of[o])
            recvs.setdefault(peer, []).append(((int(g), s), (i, s)))
            sends.setdefault(peer, []).append(((o, OPPOSITE[s]), (i, s)))
    peers = sorted(set(sends) | set(recvs))
    plan = ShardPlan(rank, zones, lnbr, peers)
    so = ro = 0
    for peer in peers:
        plan.send_faces[peer] = [f for _, f in sorted(sends.get(peer, []))]
        plan.recv_faces[peer] = [f for _, f in sorted(recvs.get(peer, []))]
        sc = sum(face_size(nx[zones[i]], ny[zones[i]], nz[zones[i]], s) for i, s in plan.send_faces[peer])
        rc = sum(face_size(nx[zones[i]], ny[zones[i]], nz[zones[i]], s) for i, s in plan.recv_faces[peer])
        plan.send_span[peer] = (so, sc)
        plan.recv_span[peer] = (ro, rc)
        so += sc
        ro += rc
    return plan


def exchange_faces(plan, send, recv, dist, group=None):
    """One step's face traffic: send[span(peer)] to each peer and recv[span(peer)]
    from it, as one batch of point-to-point operations (torch tensors: CUDA
    with NCCL, CPU with gloo).  The peers' ranks are ranks of `group`."""
    ops = []
    for peer in plan.peers:
        so, sc = plan.send_span[peer]
        ro, rc = plan.recv_span[peer]
        if sc:
            ops.append(dist.P2POp(dist.isend, send[so:so + sc], peer, group))
        if rc:
            ops.append(dist.P2POp(dist.irecv, recv[ro:ro + rc], peer, group))
    if ops:
        for w in dist.batch_isend_irecv(ops):
            w.wait()


class ShardedProblem:
    """One rank's zones of a BT-MZ / SP-MZ problem on its GPU (the current
    torch device), stepped in lockstep with the other ranks of `group`.

        rank_of = map_zones(world, nx, ny, nz, nbr, x_zones, y_zones)
        sp = ShardedProblem(geom, dt, flags, rank_of, rank, dist)
        sp.setup(ce); sp.step(n); xcr, xce = sp.verify()
    """

    def __init__(self, geom, dt, flags, rank_of, rank, dist, group=None):
        import torch

        import npbmz

        self.dist, self.group, self.torch = dist, group, torch
        self.global_geom = geom
        self.plan = shard_plan(rank_of, rank, geom.nx, geom.ny, geom.nz, geom.nbr)
        z = self.plan.zones
        local = npbmz.Geometry(geom.kind, geom.nx[z].copy(), geom.ny[z].copy(), geom.nz[z].copy(), self.plan.nbr,
                               geom.gx, geom.gy, geom.gz, geom.x_zones, geom.y_zones)
        self.problem = npbmz.Problem(local, dt, flags)
        self.stream = torch.cuda.current_stream()
        self.problem.set_stream(self.stream.cuda_stream)
        ns, nr = self.problem.face_plan(self.plan.send, self.plan.recv)
        assert ns == self.plan.send_count and nr == self.plan.recv_count
        self.send = torch.empty(max(ns, 1), dtype=torch.float64, device="cuda")
        self.recv = torch.empty(max(nr, 1), dtype=torch.float64, device="cuda")

    def setup(self, ce=None):
        self.problem.setup(ce)

    def _exchange(self):
        p = self.problem
        p.pack_faces(self.send.data_ptr())
        exchange_faces(self.plan, self.send, self.recv, self.dist, self.group)
        p.unpack_faces(self.recv.data_ptr())

    def step(self, nsteps=1, norms=False):
        """nsteps steps of the node loop; with norms, the per-step xcr / xce
        of the whole problem (summed over ranks), shape (nsteps, 2, 5)."""
        out = np.zeros((nsteps, 2, 5)) if norms else None
        for s in range(nsteps):
            self._exchange()
            if norms:
                out[s] = self.problem.step(1, norms=True)[0]
            else:
                self.problem.step(1)
        if norms:
            t = self.torch.tensor(out, dtype=self.torch.float64, device="cuda")
            self.dist.all_reduce(t, group=self.group)
            out = t.cpu().numpy()
        return out

    def verify(self):
        """verify's node part over all ranks' zones (sums over zones)."""
        xcr, xce = self.problem.verify()
        t = self.torch.tensor(np.concatenate([xcr, xce]), dtype=self.torch.float64, device="cuda")
        self.dist.all_reduce(t, group=self.group)
        v = t.cpu().numpy()
        return v[:5], v[5:]

    def close(self):
        self.problem.close()
