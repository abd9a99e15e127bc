"""Sharded extraction with a live process group: two processes (gloo), both
on GPU 0, each holding only its own point planes, run
shard.extract_sharded(..., dist=dist) end to end -- count, the all-gather of
(vertices, quads) totals, emit.  Their parts, concatenated in rank order,
must equal the whole volume's mesh bit for bit.  The ranks' kernels never
wait on each other: the only exchange is the host-side all-gather."""
import os
import socket
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _volume(kind):
    from framework_gb300 import fields
    if kind == "u16":
        return fields.value_noise_u16((150, 70, 261), base_period=16, seed=12, device="cuda"), 32768.0
    return fields.gaussian_blobs((140, 90, 300), seed=5, device="cuda"), 0.5


def _worker(rank, world, port, kind, out_dir):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import framework_gb300 as fg
    from framework_gb300 import shard
    torch.cuda.set_device(0)
    vol, iso = _volume(kind)
    nz = vol.shape[0]
    zb, ze = shard.shard_ranges(nz - 1, world)[rank]
    p0, p1 = shard.point_planes(nz, zb, ze)
    local = vol[p0:p1].clone()          # this rank holds only its planes
    del vol
    mn, mx = (-1.0, 0.5, 2.0), (3.0, 4.0, 11.0)
    with fg.Extractor(0) as ex:
        part = shard.extract_sharded(ex, local, nz, zb, ze, mn, mx, iso, triangles=True, dist=dist)
        torch.cuda.synchronize()
        np.savez(os.path.join(out_dir, "part%d.npz" % rank), vertices=part["vertices"].cpu().numpy(),
                 quads=part["quads"].cpu().numpy(), triangles=part["triangles"].cpu().numpy(),
                 offsets=np.array([part["vertex_offset"], part["quad_offset"], part["n_vertices_total"],
                                   part["n_quads_total"]], np.int64))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("kind", ["u16", "f32"])
def test_two_process_shards_equal_whole(extractor, tmp_path, kind):
    import torch
    import torch.multiprocessing as mp
    mp.spawn(_worker, args=(2, _free_port(), kind, str(tmp_path)), nprocs=2, join=True)
    vol, iso = _volume(kind)
    mn, mx = (-1.0, 0.5, 2.0), (3.0, 4.0, 11.0)
    nv, nq = extractor.extract_device(vol, mn, mx, iso)
    v = torch.empty((nv, 3), device="cuda")
    q = torch.empty((nq, 4), dtype=torch.int32, device="cuda")
    t = torch.empty((2 * nq, 3), dtype=torch.int32, device="cuda")
    extractor.extract_device(vol, mn, mx, iso, v, q, t)
    parts = [np.load(os.path.join(str(tmp_path), "part%d.npz" % r)) for r in range(2)]
    assert parts[0]["offsets"][0] == 0 and parts[1]["offsets"][0] == len(parts[0]["vertices"])
    assert all(int(p["offsets"][2]) == nv and int(p["offsets"][3]) == nq for p in parts)
    got_v = np.concatenate([p["vertices"] for p in parts])
    got_q = np.concatenate([p["quads"] for p in parts])
    got_t = np.concatenate([p["triangles"] for p in parts])
    assert np.array_equal(got_v.view(np.uint32), v.cpu().numpy().view(np.uint32))
    assert np.array_equal(got_q, q.cpu().numpy()) and np.array_equal(got_t, t.cpu().numpy())
