"""Zones of one problem over several ranks, on the CPU (no GPU).

- map_zones restates the reference's zone-to-process mapping
  (src/BT/setup_mpi.jl:123-270): the block split it takes when the zone grid
  divides evenly, and the size-sorted bin packing otherwise.
- shard_plan: every face between zones of different ranks is sent exactly
  once and received exactly once, in the same order at both ends, with equal
  sizes.
- Two gloo ranks (world size 2, 127.0.0.1) run the exchange of one step:
  each packs its faces, exchange_faces moves them, each unpacks them and
  copies the faces between its own zones.  The result is bit-for-bit the
  oracle's single-process exch_qbc on the same u.  The pack and unpack
  stand-ins here do on numpy arrays what npbmz_pack_faces and
  npbmz_unpack_faces do on the device (tests/test_gpu_shard.py checks those
  against the single-handle step).
"""
import os
import socket

import numpy as np
import pytest

from npbmz import shard

WEST, EAST, SOUTH, NORTH = range(4)


def geometry(oracle_mod, kind, cls):
    import npbmz

    niter, dt, ratio, xz, yz, gx, gy, gz = npbmz.CLASSES[kind][cls]
    nx, ny, nz, nbr = oracle_mod.zone_setup(npbmz.KINDS[kind], gx, gy, gz, xz, yz, ratio)
    return dict(kind=npbmz.KINDS[kind], nx=nx, ny=ny, nz=nz, nbr=nbr, gx=gx, gy=gy, gz=gz, xz=xz, yz=yz, dt=dt)


def test_map_zones_block_split_when_the_grid_divides(oracle_mod):
    """BT class C (16 x 16 zones) over 2 ranks: n1 x n2 = 1 x 2 leaves no
    remainder, so the reference splits the zone rows in halves."""
    g = geometry(oracle_mod, "BT", "C")
    r = shard.map_zones(2, g["nx"], g["ny"], g["nz"], g["nbr"], g["xz"], g["yz"])
    np.testing.assert_array_equal(r, [(z // 16) // 8 for z in range(256)])
    r4 = shard.map_zones(4, g["nx"], g["ny"], g["nz"], g["nbr"], g["xz"], g["yz"])
    # 2 x 2 blocks of 8 x 8 zones
    np.testing.assert_array_equal(r4, [(z % 16) // 8 + ((z // 16) // 8) * 2 for z in range(256)])


@pytest.mark.parametrize("nranks", [2, 3, 5, 8])
def test_map_zones_bin_packing_balances_the_points(oracle_mod, nranks):
    """bload = 2 (or a zone grid that does not divide): every zone gets a
    rank, and the largest rank carries at most 10 % more points than the
    mean on BT class C's geometric zones (area ratio 20.8)."""
    g = geometry(oracle_mod, "BT", "C")
    r = shard.map_zones(nranks, g["nx"], g["ny"], g["nz"], g["nbr"], g["xz"], g["yz"], bload=2)
    assert r.min() == 0 and r.max() == nranks - 1
    pts = g["nx"].astype(np.int64) * g["ny"] * g["nz"]
    load = np.bincount(r, weights=pts, minlength=nranks)
    assert load.max() <= 1.10 * load.mean(), load
    # the same map every time
    np.testing.assert_array_equal(r, shard.map_zones(nranks, g["nx"], g["ny"], g["nz"], g["nbr"], g["xz"], g["yz"],
                                                     bload=2))


def test_map_zones_falls_back_to_bin_packing(oracle_mod):
    """3 ranks cannot split a 4 x 4 zone grid into equal blocks: bin packing."""
    g = geometry(oracle_mod, "SP", "W")
    a = shard.map_zones(3, g["nx"], g["ny"], g["nz"], g["nbr"], g["xz"], g["yz"])
    b = shard.map_zones(3, g["nx"], g["ny"], g["nz"], g["nbr"], g["xz"], g["yz"], bload=2)
    np.testing.assert_array_equal(a, b)
    assert sorted(np.bincount(a)) == [5, 5, 6]


@pytest.mark.parametrize("kind,cls,nranks,bload", [("BT", "W", 2, 1), ("BT", "B", 3, 1), ("SP", "B", 4, 2),
                                                   ("BT", "C", 8, 2), ("BT", "S", 2, 2)])
def test_shard_plans_agree_at_both_ends(oracle_mod, kind, cls, nranks, bload):
    g = geometry(oracle_mod, kind, cls)
    r = shard.map_zones(nranks, g["nx"], g["ny"], g["nz"], g["nbr"], g["xz"], g["yz"], bload=bload)
    plans = [shard.shard_plan(r, q, g["nx"], g["ny"], g["nz"], g["nbr"]) for q in range(nranks)]
    remote_faces = 0
    for a in plans:
        assert len(a.zones) == int(np.sum(r == a.rank))
        for i, gz in enumerate(a.zones):
            for s in range(4):
                o = int(g["nbr"][4 * gz + s])
                if r[o] == a.rank:
                    assert a.zones[a.nbr[4 * i + s]] == o
                else:
                    assert a.nbr[4 * i + s] == shard.REMOTE
                    remote_faces += 1
        for peer in a.peers:
            b = plans[peer]
            assert a.rank in b.peers
            assert a.send_span[peer][1] == b.recv_span[a.rank][1]
            # the k-th face a sends to b arrives as the k-th face b receives from a
            dest = [(int(g["nbr"][4 * a.zones[i] + s]), shard.OPPOSITE[s]) for i, s in a.send_faces[peer]]
            assert dest == [(int(b.zones[i]), s) for i, s in b.recv_faces[a.rank]]
    assert sum(len(p.recv) for p in plans) == remote_faces == sum(len(p.send) for p in plans)


# ---- numpy stand-ins of the device pack / unpack (include/npbmz.h) ----------
def plane(u, side, ghost):
    """View of the face plane of a dense zone array u[5, nz, ny, nx]."""
    nz, ny, nx = u.shape[1:]
    if side == WEST:
        return u[:, 1:nz - 1, 1:ny - 1, 0 if ghost else 1]
    if side == EAST:
        return u[:, 1:nz - 1, 1:ny - 1, nx - 1 if ghost else nx - 2]
    if side == SOUTH:
        return u[:, 1:nz - 1, 0 if ghost else 1, 1:nx - 1]
    return u[:, 1:nz - 1, ny - 1 if ghost else ny - 2, 1:nx - 1]


def pack(us, faces):
    return np.concatenate([plane(us[i], s, False).reshape(-1) for i, s in faces]) if faces else np.zeros(0)


def unpack(us, faces, buf):
    pos = 0
    for i, s in faces:
        v = plane(us[i], s, True)
        v[...] = buf[pos:pos + v.size].reshape(v.shape)
        pos += v.size


def local_exchange(us, lnbr):
    for i in range(len(us)):
        for s in range(4):
            o = lnbr[4 * i + s]
            if o >= 0:
                plane(us[i], s, True)[...] = plane(us[o], shard.OPPOSITE[s], False)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, kind, cls, bload, q):
    try:
        import sys
        from pathlib import Path

        root = Path(__file__).resolve().parents[1]
        sys.path[:0] = [str(root), str(root / "npbapps.jl_gb300")]
        import torch
        import torch.distributed as dist

        import npbmz
        from oracle import oracle

        os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        dist.init_process_group("gloo", rank=rank, world_size=world)
        g = geometry(oracle, kind, cls)
        o = oracle.Oracle(g["kind"], g["nx"], g["ny"], g["nz"], g["nbr"], g["dt"], g["gx"], g["gy"], g["gz"], g["xz"],
                          g["yz"], npbmz.CE_REFERENCE)
        rng = np.random.default_rng(7)
        full = [o.get(0, z) * (1.0 + 0.01 * rng.standard_normal(o.get(0, z).shape)) for z in range(o.nzones)]
        for z in range(o.nzones):
            o.set(0, z, full[z])
        o.phase(5, -1)  # the oracle's exch_qbc over all zones
        want = [o.get(0, z) for z in range(o.nzones)]
        r = shard.map_zones(world, g["nx"], g["ny"], g["nz"], g["nbr"], g["xz"], g["yz"], bload=bload)
        plan = shard.shard_plan(r, rank, g["nx"], g["ny"], g["nz"], g["nbr"])
        us = [full[z].copy() for z in plan.zones]
        send = torch.from_numpy(pack(us, plan.send))
        recv = torch.zeros(plan.recv_count, dtype=torch.float64)
        assert send.numel() == plan.send_count
        dist.barrier()
        shard.exchange_faces(plan, send, recv, dist)
        unpack(us, plan.recv, recv.numpy())
        local_exchange(us, plan.nbr)
        for i, z in enumerate(plan.zones):
            np.testing.assert_array_equal(us[i], want[z], err_msg=f"rank {rank} zone {z}")
        dist.barrier()
        dist.destroy_process_group()
        q.put((rank, "ok", len(plan.zones), plan.send_count))
    except Exception as e:  # reported to the parent
        import traceback

        q.put((rank, "fail", traceback.format_exc(), 0))


@pytest.mark.parametrize("kind,cls,bload", [("BT", "W", 1), ("BT", "W", 2), ("SP", "W", 2), ("BT", "S", 1)])
def test_two_gloo_ranks_reproduce_exch_qbc(oracle_mod, kind, cls, bload):
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, kind, cls, bload, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
    for rank, status, info, sent in results:
        assert status == "ok", f"rank {rank}:\n{info}"
        assert sent > 0
