"""Sharded extraction of one volume across ranks, one GPU each.

The volume's cell planes are split into z ranges.  Every rank holds its range
plus a small halo of point planes (``point_planes``), counts its part
(``Extractor.shard_count``), and the ranks exchange their (vertices, quads)
totals: the one collective of the path, an all-gather of two integers per
rank.  An exclusive scan of the totals gives each rank the number of
vertices and quads before its part; ``Extractor.shard_emit`` then writes the
part with global vertex indices.  Concatenated in rank order the parts are
the unsharded mesh, bit for bit.
"""


def point_planes(nz, z_begin, z_end):
    """Point planes [p0, p1) a rank with cell planes [z_begin, z_end) of a
    volume with ``nz`` point planes must hold: one below its first cell plane
    (the 2B/3B test looks one cell down) and three above its last (the next
    rank's first cell plane, which its top quads reference, with that plane's
    2B/3B test)."""
    return (max(z_begin - 1, 0), min(z_end + 3, nz))


def shard_ranges(cells_z, world, align=32):
    """Balanced cell-plane ranges [z_begin, z_end) for ``world`` ranks, inner
    boundaries on multiples of ``align`` (so that deep bricks fit)."""
    if world < 1 or cells_z < 1:
        raise ValueError("need at least one rank and one cell plane")
    bounds = [0]
    for r in range(1, world):
        b = int(round(cells_z * r / world / align)) * align
        bounds.append(min(max(b, bounds[-1] + 1), cells_z - (world - r)))
    bounds.append(cells_z)
    return [(bounds[r], bounds[r + 1]) for r in range(world)]


def exclusive_offsets(totals, rank):
    """(vertex_offset, quad_offset) of ``rank`` from all ranks' (V, Q)."""
    return (sum(int(t[0]) for t in totals[:rank]), sum(int(t[1]) for t in totals[:rank]))


def exchange_totals(n_vertices, n_quads, dist=None, group=None):
    """All ranks' (vertices, quads) totals, in rank order (one all-gather;
    a single process without ``dist`` gets its own)."""
    if dist is None or not dist.is_initialized():
        return [(int(n_vertices), int(n_quads))]
    import torch
    device = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    mine = torch.tensor([int(n_vertices), int(n_quads)], dtype=torch.int64, device=device)
    parts = [torch.empty_like(mine) for _ in range(dist.get_world_size(group))]
    dist.all_gather(parts, mine, group=group)
    return [(int(p[0]), int(p[1])) for p in parts]


def extract_sharded(ex, local, nz, z_begin, z_end, xyz_min=None, xyz_max=None, iso=0.0, triangles=False,
                    dist=None, group=None):
    """This rank's part of the mesh of a sharded volume: a dict with the
    vertices, quads (global indices) and optional triangles as CUDA tensors,
    the part's offsets in the whole mesh, and the whole mesh's totals."""
    import torch
    nv, nq = ex.shard_count(local, nz, z_begin, z_end, xyz_min, xyz_max, iso)
    totals = exchange_totals(nv, nq, dist, group)
    rank = dist.get_rank(group) if dist is not None and dist.is_initialized() else 0
    voff, qoff = exclusive_offsets(totals, rank)
    dev = local.device
    v = torch.empty((max(nv, 1), 3), dtype=torch.float32, device=dev)
    q = torch.empty((max(nq, 1), 4), dtype=torch.int32, device=dev)
    t = torch.empty((max(2 * nq, 1), 3), dtype=torch.int32, device=dev) if triangles else None
    ex.shard_emit(voff, v, q, t)
    return {"vertices": v[:nv], "quads": q[:nq], "triangles": t[:2 * nq] if t is not None else None,
            "vertex_offset": voff, "quad_offset": qoff,
            "n_vertices_total": sum(a for a, _ in totals), "n_quads_total": sum(b for _, b in totals)}
