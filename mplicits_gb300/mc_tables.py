"""Marching-cubes case tables, derived here from first principles.

The reference extracts its mesh with ``skimage.measure.marching_cubes``
(i3d/meshing.py:296-298, scikit-image 0.25.2, Lewiner method).  That library
is a third-party dependency that is not part of the reference tree, so this
module does not reproduce its tables.  It derives a classic marching-cubes
table (Lorensen & Cline 1987) with one fixed face-ambiguity rule, which makes
the extracted surface watertight:

* corner ``c`` (0..7) of the cell whose minimum grid point is (i, j, k) sits at
  ``(i + (c & 1), j + ((c >> 1) & 1), k + ((c >> 2) & 1))``;
* a corner is *inside* when its value is ``< iso`` (bit ``c`` of the case);
* edge ``e = 4 * axis + m`` joins corner ``c0`` (bit ``axis`` clear, the other
  two bits taken from ``m``) to ``c0 | (1 << axis)``;
* on a face with four crossing edges the two inside corners are cut off
  separately ("inside corners separated"), on every face, so neighbouring
  cells agree about the shared face;
* every face segment is directed so that, seen from outside the cube
  through that face, the inside corner lies on its right; the directed
  segments of the six faces chain into closed loops (so every triangle's
  right-hand normal points from the inside towards increasing values);
* each loop is fanned into triangles from an apex none of whose diagonals
  joins two points of one cube face, so no chord is shared with a
  neighbouring cell.

``python -m mplicits_gb300.mc_tables`` regenerates ``csrc/mc_tables.h``; a test
checks the committed header against this generator.
"""

from __future__ import annotations

import os

import numpy as np

AXES = 3


def corner_offset(c: int) -> tuple:
    return (c & 1, (c >> 1) & 1, (c >> 2) & 1)


def _edge_list():
    """12 edges as (axis, c0, c1) with e = 4 * axis + m."""
    edges = []
    for axis in range(3):
        others = [a for a in range(3) if a != axis]
        for m in range(4):
            c0 = 0
            if m & 1:
                c0 |= 1 << others[0]
            if m & 2:
                c0 |= 1 << others[1]
            edges.append((axis, c0, c0 | (1 << axis)))
    return edges


EDGES = _edge_list()


def _edge_index(ca: int, cb: int) -> int:
    lo, hi = min(ca, cb), max(ca, cb)
    for e, (_, c0, c1) in enumerate(EDGES):
        if c0 == lo and c1 == hi:
            return e
    raise ValueError((ca, cb))


def _faces():
    """Six faces: (four corners in cyclic order, outward normal)."""
    faces = []
    for axis in range(3):
        u, v = [a for a in range(3) if a != axis]
        for side in (0, 1):
            base = side << axis
            cyc = [base, base | (1 << u), base | (1 << u) | (1 << v), base | (1 << v)]
            n = np.zeros(3)
            n[axis] = 1.0 if side else -1.0
            faces.append((cyc, n))
    return faces


FACES = _faces()


def _edge_mid(e):
    _, c0, c1 = EDGES[e]
    p0 = np.array(corner_offset(c0), float)
    p1 = np.array(corner_offset(c1), float)
    return 0.5 * (p0 + p1)


def _directed(e_a, e_b, normal, inside_corner):
    """Orient the segment e_a -> e_b so that, seen from outside the cube
    through this face, the inside corner lies on its right."""
    pa, pb = _edge_mid(e_a), _edge_mid(e_b)
    left = np.cross(normal, pb - pa)
    c = np.array(corner_offset(inside_corner), float)
    s = float(np.dot(left, c - 0.5 * (pa + pb)))
    assert abs(s) > 1e-9
    return (e_a, e_b) if s < 0 else (e_b, e_a)


def _face_segments(case: int):
    """Directed segments (edge id -> edge id) on every face for one case."""
    segs = []
    for cyc, normal in FACES:
        inside = [(case >> c) & 1 for c in cyc]
        cross = []  # edge ids of the crossing boundary edges, in cycle order
        for t in range(4):
            if inside[t] != inside[(t + 1) % 4]:
                cross.append(_edge_index(cyc[t], cyc[(t + 1) % 4]))
        if len(cross) == 2:
            ins = next(cyc[t] for t in range(4) if inside[t])
            segs.append(_directed(cross[0], cross[1], normal, ins))
        elif len(cross) == 4:
            # Ambiguous face: cut off each inside corner on its own.  Corner t
            # is adjacent to boundary edges t-1 and t of the cycle.
            for t in range(4):
                if inside[t]:
                    e_prev = _edge_index(cyc[(t - 1) % 4], cyc[t])
                    e_next = _edge_index(cyc[t], cyc[(t + 1) % 4])
                    segs.append(_directed(e_prev, e_next, normal, cyc[t]))
    return segs


def _loops(segs):
    nxt = {}
    for a, b in segs:
        assert a not in nxt, (a, segs)
        nxt[a] = b
    assert sorted(nxt) == sorted(nxt.values())
    seen = set()
    loops = []
    for start in sorted(nxt):
        if start in seen:
            continue
        loop = [start]
        seen.add(start)
        cur = nxt[start]
        while cur != start:
            loop.append(cur)
            seen.add(cur)
            cur = nxt[cur]
        loops.append(loop)
    return loops


def _outward(e, case):
    """Unit vector along edge e from its inside corner to its outside corner."""
    axis, c0, c1 = EDGES[e]
    d = np.zeros(3)
    d[axis] = 1.0 if (case >> c0) & 1 else -1.0
    return d


def _edge_faces(e):
    _, c0, c1 = EDGES[e]
    return {fi for fi, (cyc, _) in enumerate(FACES) if c0 in cyc and c1 in cyc}


def _fan(loop, case):
    """Fan-triangulate a directed loop from an apex none of whose diagonals
    joins two points of one cube face (such a chord would be shared with the
    neighbouring cell and pinch the surface); among those apexes take the one
    whose triangles best keep the winding towards increasing values."""
    n = len(loop)
    best = None
    for a in range(n):
        rot = loop[a:] + loop[:a]
        if any(_edge_faces(rot[0]) & _edge_faces(rot[k]) for k in range(2, n - 1)):
            continue
        tris = [(rot[0], rot[t], rot[t + 1]) for t in range(1, n - 1)]
        score = 0
        for tri in tris:
            p = [_edge_mid(e) for e in tri]
            nrm = np.cross(p[1] - p[0], p[2] - p[0])
            score += float(np.dot(nrm, sum(_outward(e, case) for e in tri)) > 0)
        if best is None or score > best[0]:
            best = (score, tris)
    assert best is not None, (case, loop)
    return best[1]


def build_tables():
    """Return (tri_count[256], tri_edges[256][MAX*3]) with -1 padding."""
    cases = []
    for case in range(256):
        tris = []
        for loop in _loops(_face_segments(case)):
            tris.extend(_fan(loop, case))
        cases.append(tris)
    max_tris = max(len(t) for t in cases)
    count = np.array([len(t) for t in cases], np.int32)
    table = -np.ones((256, max_tris * 3), np.int32)
    for case, tris in enumerate(cases):
        flat = [e for tri in tris for e in tri]
        table[case, : len(flat)] = flat
    return count, table


def edge_table():
    """(axis, corner0 offset, corner1 offset) per edge as an int array [12, 7]."""
    out = np.zeros((12, 7), np.int32)
    for e, (axis, c0, c1) in enumerate(EDGES):
        out[e] = (axis, *corner_offset(c0), *corner_offset(c1))
    return out


def render_header() -> str:
    count, table = build_tables()
    max_tris = table.shape[1] // 3
    lines = [
        "// Generated by mplicits_gb300/mc_tables.py -- do not edit by hand.",
        "// Marching-cubes tables: corner c at (c&1, (c>>1)&1, (c>>2)&1) along",
        "// array axes (0,1,2); case bit c set when value[c] < iso; edge",
        "// e = 4*axis + m; triangles wound towards increasing values.",
        "#pragma once",
        f"#define MPL_MC_MAX_TRIS {max_tris}",
        "static const unsigned char MPL_MC_TRI_COUNT[256] = {",
    ]
    for r in range(0, 256, 32):
        lines.append("  " + ", ".join(str(int(v)) for v in count[r:r + 32]) + ",")
    lines.append("};")
    lines.append(f"static const signed char MPL_MC_TRI_EDGES[256][{max_tris * 3}] = {{")
    for case in range(256):
        lines.append("  {" + ", ".join(str(int(v)) for v in table[case]) + "},")
    lines.append("};")
    et = edge_table()
    lines.append("// per edge: axis, corner0 (d0,d1,d2), corner1 (d0,d1,d2)")
    lines.append("static const signed char MPL_MC_EDGE[12][7] = {")
    for e in range(12):
        lines.append("  {" + ", ".join(str(int(v)) for v in et[e]) + "},")
    lines.append("};")
    return "\n".join(lines) + "\n"


HEADER_PATH = os.path.join(os.path.dirname(__file__), "csrc", "mc_tables.h")


def ambiguity_classes():
    """Per case (0..255): (face, interior).  ``face``: some face of the cell
    has its two inside corners on one diagonal and its two outside corners on
    the other (four crossing edges), the configuration where this table's
    fixed rule ("inside corners separated") and a face test such as the
    asymptotic decider of Lewiner et al. 2003 (scikit-image's method) can
    choose different segment pairs.  ``interior``: no face is ambiguous but
    the two inside (or the two outside) corners are the ends of a body
    diagonal, the case where Lewiner's interior test may join them with a
    tube instead of two separate triangles.  Every other case has one
    topology; two tables can then still triangulate a loop of four or more
    vertices differently, which changes faces but not the surface's
    vertices or its connectivity."""
    out = []
    for case in range(256):
        ins = [(case >> c) & 1 for c in range(8)]
        face = any(ins[cyc[0]] == ins[cyc[2]] and ins[cyc[1]] == ins[cyc[3]] and
                   ins[cyc[0]] != ins[cyc[1]] for cyc, _ in _faces())
        n_in = sum(ins)
        pair = None
        if n_in == 2:
            pair = [c for c in range(8) if ins[c]]
        elif n_in == 6:
            pair = [c for c in range(8) if not ins[c]]
        interior = (not face) and pair is not None and (pair[0] ^ pair[1]) == 7
        out.append((face, interior))
    return out


if __name__ == "__main__":
    with open(HEADER_PATH, "w") as f:
        f.write(render_header())
    c, t = build_tables()
    print("max triangles per case:", t.shape[1] // 3, "total:", int(c.sum()))
