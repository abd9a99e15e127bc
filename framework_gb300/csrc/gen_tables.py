#!/usr/bin/env python3
"""Generate the Dual Marching Cubes lookup tables (``dmc_tables.inc``).

The reference ships its tables as literal arrays (DMC_CUDA/DMC_CUDA/src/dmc.cu:45-661).
Their content has to be identical here, because the table entries decide the
numbering of dual vertices inside a cell and therefore the vertex order and
every quad index of the output. Rather than carrying the literal arrays, this
script derives them from the geometry of the cube and records the only part
that is a pure convention (the numbering of the patches of a cell) as data:

* Cube conventions (dmc.cu:1109-1129 edge endpoints, :1018-1027 config bit i =
  ``v[i] < iso``; corner i sits at (i&1 ^ (i>>1)&1, (i>>1)&1, i>>2)).
* Patch structure.  The iso-surface inside a cell is a set of polygons whose
  boundary segments lie on the six faces.  On a face with two sign changes the
  two crossed edges are joined.  On an *ambiguous* face (corners alternate) two
  pairings are possible.  ``config_edge_lut1`` always joins the inside corners
  (bit 1, ``v < iso``), i.e. the segments cut off the outside corners.
  ``config_edge_lut2`` differs only for the 36 "2B/3B" configurations
  (dmc.cu:607-620): those with exactly one ambiguous face and two or three
  inside corners; there that face takes the other pairing.  The patches are the
  connected components of crossed edges under these joins.
* Patch numbering.  A patch's index m is its dual vertex index in the cell.
  For most configurations the patches are numbered in order of their lowest
  edge.  ``PATCH_ORDER`` lists the configurations that use another order, as the
  lowest edge of patch 0, 1, ...; this is the reference's convention and has to
  be matched for an identical vertex order.
* ``edge owner`` and ``ring`` tables follow dmc.cu:634-658: each edge belongs to
  exactly one cell (edges 6, 9, 10 of a cell are its own), and the four cells
  around an owned edge are visited in a fixed counter-clockwise order.

Run ``python gen_tables.py`` to rewrite ``dmc_tables.inc`` next to this file;
``python gen_tables.py --check`` exits non-zero if the file is stale.
"""
import hashlib
import os
import sys

CORNERS = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0),
           (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
EDGES = [(0, 1), (1, 2), (2, 3), (0, 3), (0, 4), (1, 5),
         (2, 6), (3, 7), (4, 5), (5, 6), (6, 7), (4, 7)]
# faces in the reference's numbering (dmc.cu:615-632): -z, -y, +x, +y, -x, +z,
# each listed as a closed loop of corners
FACES = [(0, 1, 2, 3), (0, 1, 5, 4), (1, 2, 6, 5), (2, 3, 7, 6), (0, 3, 7, 4), (4, 5, 6, 7)]
# neighbour direction checked for an ambiguous face: 0 +x, 1 -x, 2 +y, 3 -y, 4 +z, 5 -z
FACE_DIR = [5, 3, 0, 2, 1, 4]

# lowest edge of patch 0, 1, ... for configurations not numbered by lowest edge
PATCH_ORDER_LUT1 = {
    0x1a: (1, 0), 0x25: (2, 0), 0x3d: (6, 0), 0x3e: (6, 0), 0x53: (5, 1), 0x56: (5, 0),
    0x59: (7, 0), 0x5c: (7, 1), 0x5e: (0, 7, 5), 0x5f: (7, 5), 0x69: (4, 0), 0x6a: (1, 0),
    0x6b: (4, 1), 0x6d: (4, 0), 0x75: (2, 0), 0x78: (7, 2), 0x7a: (7, 0, 1), 0x7e: (7, 0),
    0x95: (2, 0), 0x97: (5, 2), 0x9e: (5, 0), 0xa3: (4, 1), 0xa5: (0, 2, 6, 4), 0xa6: (6, 0),
    0xa7: (2, 6, 4), 0xa9: (4, 0), 0xac: (6, 1), 0xaf: (6, 4), 0xb4: (6, 1), 0xb5: (6, 2, 0),
    0xba: (1, 0), 0xbd: (6, 0), 0xc3: (4, 1), 0xc5: (2, 0), 0xc7: (4, 2), 0xca: (1, 0),
    0xcb: (4, 1), 0xd2: (5, 0), 0xda: (1, 0, 5), 0xde: (5, 0), 0xe1: (4, 0), 0xe5: (2, 4, 0),
    0xe7: (4, 2), 0xfa: (1, 0),
}
# the same for the 36 2B/3B configurations under their alternative face pairing
PATCH_ORDER_LUT2_AMBIGUOUS = {
    0x05: (1, 0), 0x18: (4, 2), 0x21: (5, 0), 0x34: (4, 1), 0x38: (4, 2), 0x42: (6, 0),
    0x45: (1, 0), 0x50: (6, 4), 0x61: (5, 0), 0x68: (5, 2), 0x81: (7, 0), 0x8a: (2, 0),
    0x92: (4, 0), 0x94: (4, 1), 0xa0: (7, 5), 0xc1: (6, 0), 0xc2: (6, 0),
}

NO_VERTEX = 0xFF


def edge_index(a, b):
    return EDGES.index((min(a, b), max(a, b)))


def inside(config, corner):
    return (config >> corner) & 1


def ambiguous_faces(config):
    out = []
    for f, loop in enumerate(FACES):
        if all(inside(config, loop[i]) != inside(config, loop[(i + 1) % 4]) for i in range(4)):
            out.append(f)
    return out


def is_2b_3b(config):
    return len(ambiguous_faces(config)) == 1 and bin(config).count("1") in (2, 3)


def patches(config, flipped_face=None):
    """Connected components of crossed edges; returns list of edge lists."""
    parent = list(range(12))

    def find(x):
        while parent[x] != x:
            parent[x] = parent[parent[x]]
            x = parent[x]
        return x

    for f, loop in enumerate(FACES):
        fe = [edge_index(loop[i], loop[(i + 1) % 4]) for i in range(4)]
        crossed = [inside(config, loop[i]) != inside(config, loop[(i + 1) % 4]) for i in range(4)]
        if sum(crossed) == 2:
            a, b = [fe[i] for i in range(4) if crossed[i]]
            parent[find(a)] = find(b)
        elif sum(crossed) == 4:
            join_inside = f != flipped_face
            # a segment cuts off corner i when it joins the two face edges at i
            cut = [i for i in range(4) if inside(config, loop[i]) != join_inside]
            for i in cut:
                a, b = fe[(i - 1) % 4], fe[i]
                parent[find(a)] = find(b)
    groups = {}
    for e in range(12):
        a, b = EDGES[e]
        if inside(config, a) != inside(config, b):
            groups.setdefault(find(e), []).append(e)
    return list(groups.values())


def config_row(config, lut2):
    flipped = None
    order = PATCH_ORDER_LUT1
    if lut2 and is_2b_3b(config):
        flipped = ambiguous_faces(config)[0]
        order = PATCH_ORDER_LUT2_AMBIGUOUS
    groups = sorted(patches(config, flipped), key=min)
    if config in order:
        lowest = order[config]
        groups = [next(g for g in groups if min(g) == e) for e in lowest]
    row = [NO_VERTEX] * 12
    for m, g in enumerate(groups):
        for e in g:
            row[e] = m
    return row, len(groups)


def build():
    lut = [[], []]
    nv = [[], []]
    for which in (0, 1):
        for c in range(256):
            row, n = config_row(c, which == 1)
            lut[which].append(row)
            nv[which].append(n)
    amb_face = []
    for c in range(256):
        amb_face.append(ambiguous_faces(c)[0] if is_2b_3b(c) else NO_VERTEX)
    return lut, nv, amb_face


def render(lut, nv, amb_face):
    blob = bytes(v for which in (0, 1) for row in lut[which] for v in row)
    blob += bytes(nv[0]) + bytes(nv[1]) + bytes(amb_face)
    digest = hashlib.sha256(blob).hexdigest()
    out = ["/* Generated by gen_tables.py; do not edit by hand. */",
           "/* sha256 of (edge_lut1, edge_lut2, nvert_lut1, nvert_lut2, ambiguous_face): */",
           "#define DMC_TABLES_SHA256 \"%s\"" % digest, ""]

    def arr(name, vals, per_line):
        out.append("static const unsigned char %s[%d] = {" % (name, len(vals)))
        for i in range(0, len(vals), per_line):
            out.append("  " + ", ".join("%d" % v for v in vals[i:i + per_line]) + ",")
        out.append("};")

    arr("DMC_EDGE_LUT1", [v for row in lut[0] for v in row], 12)
    arr("DMC_EDGE_LUT2", [v for row in lut[1] for v in row], 12)
    arr("DMC_NVERT_LUT1", nv[0], 16)
    arr("DMC_NVERT_LUT2", nv[1], 16)
    out.append("/* face (0 -z,1 -y,2 +x,3 +y,4 -x,5 +z) of a 2B/3B configuration, 255 otherwise */")
    arr("DMC_AMBIGUOUS_FACE", amb_face, 16)
    out.append("/* neighbour direction per face: 0 +x,1 -x,2 +y,3 -y,4 +z,5 -z */")
    arr("DMC_FACE_DIR", FACE_DIR, 6)
    return "\n".join(out) + "\n", digest


def main():
    here = os.path.dirname(os.path.abspath(__file__))
    path = os.path.join(here, "dmc_tables.inc")
    text, digest = render(*build())
    if "--check" in sys.argv:
        cur = open(path).read() if os.path.exists(path) else ""
        if cur != text:
            print("dmc_tables.inc is stale")
            return 1
        print("ok", digest)
        return 0
    with open(path, "w") as f:
        f.write(text)
    print("wrote", path, digest)
    return 0


if __name__ == "__main__":
    sys.exit(main())
