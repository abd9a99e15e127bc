"""A second, pure-Python restatement of the reference's DMC pass for tiny
volumes (test infrastructure).  It reads the lookup tables produced by
framework_gb300/csrc/gen_tables.py and follows dmc.cu:2069-2208 with Python
ints and numpy float32 scalars, so the C oracle can be cross-checked on cases
small enough for pure-Python loops."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "framework_gb300", "csrc"))
import gen_tables  # noqa: E402

_LUT, _NV, _AMB = gen_tables.build()
CORNER = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
EDGE = gen_tables.EDGES
OWNER = {0: ((0, -1, -1), 10), 1: ((0, 0, -1), 9), 2: ((0, 0, -1), 10), 3: ((-1, 0, -1), 9),
         4: ((-1, -1, 0), 6), 5: ((0, -1, 0), 6), 6: ((0, 0, 0), 6), 7: ((-1, 0, 0), 6),
         8: ((0, -1, 0), 10), 9: ((0, 0, 0), 9), 10: ((0, 0, 0), 10), 11: ((-1, 0, 0), 9)}
RING = {6: [6, 7, 4, 5], 9: [9, 1, 3, 11], 10: [10, 8, 0, 2]}
F = np.float32


def extract(vol, iso, xyz_min=(0, 0, 0), xyz_max=None, num_smooth=0):
    vol = np.asarray(vol)
    nz, ny, nx = vol.shape
    cx, cy, cz = nx - 1, ny - 1, nz - 1
    if xyz_max is None:
        xyz_max = (nx - 1, ny - 1, nz - 1)
    mn = [F(v) for v in xyz_min]
    rng = [F(F(xyz_max[i]) - mn[i]) for i in range(3)]
    size = (cx, cy, cz)
    iso = F(iso)

    def val(x, y, z):
        return F(vol[z, y, x])

    def corners(x, y, z):
        return [val(x + a, y + b, z + c) for a, b, c in CORNER]

    def cfg(x, y, z):
        return sum(1 << i for i, v in enumerate(corners(x, y, z)) if v < iso)

    def coord(i, ax):
        return F(F(F(F(i) / F(size[ax])) * rng[ax]) + mn[ax])

    def bip(a, b):
        if a == b:
            return False
        lo, hi = min(a, b), max(a, b)
        return not ((lo < iso and hi < iso) or (lo > iso and hi > iso))

    def lerp(p0, p1, v0, v1):
        t = F(F(iso - v0) / F(v1 - v0))
        omt = F(F(1) - t)
        return [F(F(p0[c] * omt) + F(p1[c] * t)) for c in range(3)]

    cells = [(x, y, z) for z in range(cz) for y in range(cy) for x in range(cx)]
    active = {}
    order = []
    for (x, y, z) in cells:
        c = cfg(x, y, z)
        if c not in (0, 255):
            active[(x, y, z)] = dict(cfg=c)
            order.append((x, y, z))
    for key in order:
        x, y, z = key
        v = corners(x, y, z)
        info = 0
        for s, p0 in enumerate((2, 5, 7)):
            if bip(v[p0], v[6]):
                info |= 1 << s
                if v[p0] <= iso:
                    info |= 1 << (s + 3)
        r = active[key]
        r["info"] = info
        lut2 = False
        face = _AMB[r["cfg"]]
        if face != 255:
            d = gen_tables.FACE_DIR[face]
            off = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)][d]
            n = (x + off[0], y + off[1], z + off[2])
            if all(0 <= n[i] < size[i] for i in range(3)):
                lut2 = _AMB[active[n]["cfg"]] != 255
        r["lut2"] = lut2
        r["niso"] = _NV[1 if lut2 else 0][r["cfg"]]
        r["nv"] = r["niso"] + bin(info & 7).count("1")
    vb = 0
    for key in order:
        active[key]["vb"] = vb
        vb += active[key]["nv"]
    verts = [None] * vb
    for key in order:
        x, y, z = key
        r = active[key]
        v = corners(x, y, z)
        x0, x1, y0, y1, z0, z1 = coord(x, 0), coord(x + 1, 0), coord(y, 1), coord(y + 1, 1), coord(z, 2), coord(z + 1, 2)
        i = r["vb"] + r["niso"]
        if r["info"] & 1:
            verts[i] = lerp((x1, y1, z0), (x1, y1, z1), v[2], v[6]); i += 1
        if r["info"] & 2:
            verts[i] = lerp((x1, y0, z1), (x1, y1, z1), v[5], v[6]); i += 1
        if r["info"] & 4:
            verts[i] = lerp((x1, y1, z1), (x0, y1, z1), v[6], v[7]); i += 1

    def lut(r, e):
        return _LUT[1 if r["lut2"] else 0][r["cfg"]][e]

    def edge_vertex(r, e):
        s = {6: 0, 9: 1, 10: 2}[e]
        return r["vb"] + r["niso"] + bin(r["info"] & ((1 << s) - 1)).count("1")

    for key in order:
        x, y, z = key
        r = active[key]
        acc = {}
        for e in range(12):
            m = lut(r, e)
            if m == 255:
                continue
            off, oe = OWNER[e]
            o = (x + off[0], y + off[1], z + off[2])
            if min(o) < 0:
                continue
            src = verts[edge_vertex(active[o], oe)]
            if m not in acc:
                acc[m] = [list(src), 1]
            else:
                acc[m][0] = [F(acc[m][0][c] + src[c]) for c in range(3)]
                acc[m][1] += 1
        for m in range(r["niso"]):
            if m in acc:
                s, n = acc[m]
                verts[r["vb"] + m] = [F(s[c] / F(n)) for c in range(3)]
    quads = []
    quad_edge = []                      # (owner key, axis slot) of each quad
    for key in order:
        x, y, z = key
        r = active[key]
        for s, e in enumerate((6, 9, 10)):
            if not r["info"] & (1 << s):
                continue
            lim = {6: (x + 1 < cx and y + 1 < cy), 9: (x + 1 < cx and z + 1 < cz), 10: (y + 1 < cy and z + 1 < cz)}[e]
            if not lim:
                continue
            p0 = (2, 5, 7)[s]
            if ((r["cfg"] >> p0) & 1) == ((r["cfg"] >> 6) & 1):
                continue
            ccw = (r["info"] >> (s + 3)) & 1
            ks = [0, 1, 2, 3] if ccw else [0, 3, 2, 1]
            q = []
            for k in ks:
                re = RING[e][k]
                off, _ = OWNER[re]
                rc = (x - off[0], y - off[1], z - off[2])
                rr = active[rc]
                q.append(rr["vb"] + lut(rr, re))
            quads.append(q)
            quad_edge.append((key, s))
    for _ in range(num_smooth):
        _smooth_iteration(verts, quads, quad_edge, active, order, lut, edge_vertex, coord)
    V = np.array([v if v is not None else [np.nan] * 3 for v in verts], dtype=np.float32).reshape(-1, 3)
    return V, np.array(quads, dtype=np.uint32).reshape(-1, 4)


# ---- smoothing (dmc.cu:1710-1981): the arithmetic of oracle/dmc_oracle.c ----

def _cross_pos(l, m, r):
    dx1, dy1 = F(r[0] - m[0]), F(r[1] - m[1])
    dx2, dy2 = F(l[0] - m[0]), F(l[1] - m[1])
    return F(F(dx1 * dy2) - F(dx2 * dy1)) >= 0


def _corner_cos(l, m, r):
    ux, uy, vx, vy = F(l[0] - m[0]), F(l[1] - m[1]), F(r[0] - m[0]), F(r[1] - m[1])
    iu = F(F(1) / np.sqrt(F(F(ux * ux) + F(uy * uy))))
    iv = F(F(1) / np.sqrt(F(F(vx * vx) + F(vy * vy))))
    ux, uy, vx, vy = F(ux * iu), F(uy * iu), F(vx * iv), F(vy * iv)
    return F(F(ux * vx) + F(uy * vy))


def _inside(p0, p1, p2, pt):
    v0x, v0y = F(p1[0] - p0[0]), F(p1[1] - p0[1])
    v1x, v1y = F(p2[0] - p0[0]), F(p2[1] - p0[1])
    v2x, v2y = F(pt[0] - p0[0]), F(pt[1] - p0[1])
    d00 = F(F(v0x * v0x) + F(v0y * v0y))
    d10 = F(F(v1x * v0x) + F(v1y * v0y))
    d11 = F(F(v1x * v1x) + F(v1y * v1y))
    d20 = F(F(v2x * v0x) + F(v2y * v0y))
    d21 = F(F(v2x * v1x) + F(v2y * v1y))
    inv = F(F(1) / F(F(d00 * d11) - F(d10 * d10)))
    beta = F(F(F(d11 * d20) - F(d10 * d21)) * inv)
    gamma = F(F(F(d00 * d21) - F(d10 * d20)) * inv)
    alpha = F(F(F(1) - beta) - gamma)
    ok = float(beta) > -1e-4 and float(gamma) > -1e-4 and float(F(beta + gamma)) < 1.0 + 1e-4
    return ok, (alpha, beta, gamma)


def _smooth_iteration(verts, quads, quad_edge, active, order, lut, edge_vertex, coord):
    with np.errstate(all="ignore"):
        moved = []
        for q, (key, s) in zip(quads, quad_edge):
            ax, ay = (1 if s == 2 else 0), (1 if s == 0 else 2)
            P = [(verts[i][ax], verts[i][ay]) for i in q]
            pos = [_cross_pos(P[(i + 3) % 4], P[i], P[(i + 1) % 4]) for i in range(4)]
            npos = sum(pos)
            if npos == 2:
                continue
            if npos in (0, 4):
                cs = [_corner_cos(P[(i + 3) % 4], P[i], P[(i + 1) % 4]) for i in range(4)]
                split0 = 0
                for i in range(1, 4):
                    if cs[i] < cs[split0]:
                        split0 = i
            else:
                split0 = [i for i in range(4) if pos[i] == (npos == 1)][-1]
            split1 = (split0 + 2) % 4
            x, y, z = key
            x1, y1, z1 = coord(x + 1, 0), coord(y + 1, 1), coord(z + 1, 2)
            origin = (y1 if s == 2 else x1, y1 if s == 0 else z1)
            ok, w = _inside(P[split0], P[(split0 + 1) % 4], P[split1], origin)
            abc = (split0, (split0 + 1) % 4, split1)
            if not ok:
                ok, w = _inside(P[split1], P[(split1 + 1) % 4], P[split0], origin)
                abc = (split1, (split1 + 1) % 4, split0)
            if not ok:
                continue
            va, vb, vc = verts[q[abc[0]]], verts[q[abc[1]]], verts[q[abc[2]]]
            nv = [F(F(F(w[0] * va[k]) + F(w[1] * vb[k])) + F(w[2] * vc[k])) for k in range(3)]
            moved.append((edge_vertex(active[key], (6, 9, 10)[s]), nv))
        for i, nv in moved:
            verts[i] = nv
        for key in order:
            x, y, z = key
            r = active[key]
            acc = {}
            for e in range(12):
                m = lut(r, e)
                if m == 255:
                    continue
                off, oe = OWNER[e]
                o = (x + off[0], y + off[1], z + off[2])
                if min(o) < 0:
                    continue
                src = verts[edge_vertex(active[o], oe)]
                if m not in acc:
                    acc[m] = [list(src), 1]
                else:
                    acc[m][0] = [F(acc[m][0][c] + src[c]) for c in range(3)]
                    acc[m][1] += 1
            for m, (sm, n) in acc.items():
                if m < r["niso"]:
                    verts[r["vb"] + m] = [F(sm[c] / F(n)) for c in range(3)]
