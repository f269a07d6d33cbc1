"""Zones of one problem split over several handles, on one GPU, through the C ABI.

Each "rank" is a handle holding only its zones (map_zones, shard_plan) with
NPBMZ_REMOTE faces.  A step packs every rank's faces (npbmz_pack_faces),
moves each peer's share into the receiver's buffer with a device copy (the
stand-in for NCCL send/recv; no kernel waits on another rank), unpacks them
(npbmz_unpack_faces) and steps every handle.  u must then be bit-for-bit the
single-handle run's, zone by zone, for the exact, FMA and mixed graph
variants, and the per-step norms summed over ranks must match the single
handle's to 1e-13 (summation order).  ShardedProblem itself runs as a
one-rank NCCL group against the plain handle.
"""
import os
import socket

import numpy as np
import pytest

import npbmz
from npbmz import shard

pytestmark = pytest.mark.gpu

NORM_REL = 1e-13


def geom_class(kind, cls):
    niter, dt, ratio, xz, yz, gx, gy, gz = npbmz.CLASSES[kind][cls]
    k = npbmz.KINDS[kind]
    nx, ny, nz, nbr = npbmz.zone_setup(k, gx, gy, gz, xz, yz, ratio)
    return npbmz.Geometry(k, nx, ny, nz, nbr, gx, gy, gz, xz, yz), dt


@pytest.mark.parametrize("kind,cls,nranks,bload", [("BT", "W", 2, 1), ("BT", "B", 3, 2), ("SP", "W", 3, 1),
                                                   ("SP", "B", 4, 2)])
@pytest.mark.parametrize("flags", [npbmz.EXACT, 0, npbmz.MIXED | npbmz.GRAPH], ids=["exact", "fma", "mixed-graph"])
def test_sharded_handles_match_the_single_handle(kind, cls, nranks, bload, flags):
    torch = pytest.importorskip("torch")
    geom, dt = geom_class(kind, cls)
    ce, _ = npbmz.seeded_coefficients(5, geom.nx, geom.ny, geom.nz, geom.gx, geom.gy, geom.gz, geom.x_zones,
                                      geom.y_zones)
    stream = torch.cuda.current_stream().cuda_stream
    full = npbmz.Problem(geom, dt, flags)
    full.set_stream(stream)
    full.setup(ce)
    rank_of = shard.map_zones(nranks, geom.nx, geom.ny, geom.nz, geom.nbr, geom.x_zones, geom.y_zones, bload=bload)
    plans, probs, sends, recvs = [], [], [], []
    for r in range(nranks):
        pl = shard.shard_plan(rank_of, r, geom.nx, geom.ny, geom.nz, geom.nbr)
        z = pl.zones
        g = npbmz.Geometry(geom.kind, geom.nx[z].copy(), geom.ny[z].copy(), geom.nz[z].copy(), pl.nbr, geom.gx,
                           geom.gy, geom.gz, geom.x_zones, geom.y_zones)
        p = npbmz.Problem(g, dt, flags)
        p.set_stream(stream)
        p.setup(ce)
        ns, nr = p.face_plan(pl.send, pl.recv)
        assert (ns, nr) == (pl.send_count, pl.recv_count)
        plans.append(pl)
        probs.append(p)
        sends.append(torch.empty(max(ns, 1), dtype=torch.float64, device="cuda"))
        recvs.append(torch.full((max(nr, 1),), float("nan"), dtype=torch.float64, device="cuda"))
    nsteps = 6
    want = full.step(nsteps, norms=True)
    got = np.zeros_like(want)
    for s in range(nsteps):
        for p, b in zip(probs, sends):
            p.pack_faces(b.data_ptr())
        for r, pl in enumerate(plans):
            for q in pl.peers:
                ro, rc = pl.recv_span[q]
                so, sc = plans[q].send_span[r]
                assert rc == sc
                recvs[r][ro:ro + rc].copy_(sends[q][so:so + sc])
        for p, b in zip(probs, recvs):
            p.unpack_faces(b.data_ptr())
        for p in probs:
            got[s] += p.step(1, norms=True)[0]
    np.testing.assert_allclose(got, want, rtol=NORM_REL, atol=0)
    for r, pl in enumerate(plans):
        for i, z in enumerate(pl.zones):
            np.testing.assert_array_equal(probs[r].download(npbmz.U, i), full.download(npbmz.U, int(z)),
                                          err_msg=f"rank {r} zone {z}")


def test_face_plan_rejects_a_face_that_is_not_remote():
    geom, dt = geom_class("BT", "S")
    p = npbmz.Problem(geom, dt, 0)
    with pytest.raises(npbmz.NpbmzError, match="not an NPBMZ_REMOTE face"):
        p.face_plan([], [(0, 0)])
    with pytest.raises(npbmz.NpbmzError, match="bad zone"):
        p.face_plan([(7, 0)], [])


def test_sharded_problem_on_a_one_rank_nccl_group():
    torch = pytest.importorskip("torch")
    import torch.distributed as dist

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    torch.cuda.set_device(0)
    dist.init_process_group("nccl", rank=0, world_size=1)
    try:
        geom, dt = geom_class("SP", "W")
        ce, _ = npbmz.seeded_coefficients(2, geom.nx, geom.ny, geom.nz, geom.gx, geom.gy, geom.gz, geom.x_zones,
                                          geom.y_zones)
        rank_of = shard.map_zones(1, geom.nx, geom.ny, geom.nz, geom.nbr, geom.x_zones, geom.y_zones)
        sp = shard.ShardedProblem(geom, dt, npbmz.MIXED | npbmz.GRAPH, rank_of, 0, dist)
        sp.setup(ce)
        a = sp.step(4, norms=True)
        p = npbmz.Problem(geom, dt, npbmz.MIXED | npbmz.GRAPH)
        p.setup(ce)
        b = p.step(4, norms=True)
        np.testing.assert_allclose(a, b, rtol=NORM_REL, atol=0)
        np.testing.assert_allclose(np.concatenate(sp.verify()), np.concatenate(p.verify()), rtol=NORM_REL, atol=0)
        sp.close()
    finally:
        dist.destroy_process_group()
