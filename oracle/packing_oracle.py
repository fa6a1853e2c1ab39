"""CPU oracle of the incircle packing (TEST INFRASTRUCTURE: only tests/ and bench.py's CPU
baseline use it; the product path is pg_pack_incenters on the GPU).

A numpy restatement of the reference's get_incenter_mesh_loc (exp_dict.py:1072-1313) after its
mesher:
  element_circles   triangles exp_dict.py:1087-1125, tetrahedra :1127-1172 (same operations in
                    the same order, so results are bit-identical to the reference's numpy code)
  node_elements     get_nbd_vertex_elem, exp_dict.py:71-86
  plain_nodal       modify_nodal_circles = False, exp_dict.py:1280-1296
  maximin_nodal     modify_nodal_circles = True, exp_dict.py:1186-1278: the per-node GEKKO model
                    (same constraints, box and initial guess), at the local maximum defined below.

Pinned against tests/golden/pack*.npz, which make_packing_golden.py produced by running the
reference's own get_incenter_mesh_loc with its mesher replaced by the test mesh and GEKKO replaced
by a recorder that hands the same model to scipy's SLSQP (gekko is not installed): element and
plain nodal circles are bit-identical; maximin circles agree where both solvers reach the same
local maximum of the reference's model.
"""
import math

import numpy as np


def element_circles(pos, T):
    """Incenters [m, dim] and inradii [m, 1] of the elements."""
    if pos.shape[1] == 2:
        v_a, v_b, v_c = pos[T[:, 0]], pos[T[:, 1]], pos[T[:, 2]]
        ab, ac, bc = v_b - v_a, v_c - v_a, v_c - v_b
        l_a = np.sqrt(np.sum(bc ** 2, axis=1))[:, None]
        l_b = np.sqrt(np.sum(ac ** 2, axis=1))[:, None]
        l_c = np.sqrt(np.sum(ab ** 2, axis=1))[:, None]
        sum_l = l_a + l_b + l_c
        incenter = (l_a * v_a + l_b * v_b + l_c * v_c) / sum_l
        area = 0.25 * np.sqrt(sum_l * (l_a - l_b + l_c) * (l_b - l_c + l_a) * (l_c - l_a + l_b))
        return incenter, 2 * area / sum_l
    p = [pos[T[:, k]] for k in range(4)]
    x1, y1, z1 = p[0].T
    x2, y2, z2 = p[1].T
    x3, y3, z3 = p[2].T
    x4, y4, z4 = p[3].T
    vol = np.abs(1 / 6 * ((x4 - x1) * ((y2 - y1) * (z3 - z1) - (z2 - z1) * (y3 - y1)) +
                          (y4 - y1) * ((z2 - z1) * (x3 - x1) - (x2 - x1) * (z3 - z1)) +
                          (z4 - z1) * ((x2 - x1) * (y3 - y1) - (y2 - y1) * (x3 - x1))))
    alpha = (vol * 6)[:, None]

    def face(a, b, c):
        # doubled area of face (a, b, c) from the three 2x2 minors
        xa, ya, za = a.T
        xb, yb, zb = b.T
        xc, yc, zc = c.T
        return np.sqrt(((xa - xc) * (ya - yb) - (xa - xb) * (ya - yc)) ** 2 +
                       ((xa - xc) * (za - zb) - (xa - xb) * (za - zc)) ** 2 +
                       ((ya - yc) * (za - zb) - (ya - yb) * (za - zc)) ** 2)

    s123, s124, s134, s234 = face(p[0], p[1], p[2]), face(p[0], p[1], p[3]), face(p[0], p[2], p[3]), face(p[1], p[2], p[3])
    denom = (s123 + s124 + s134 + s234)[:, None]
    numer = np.zeros((len(denom), 3))
    for c in range(3):
        numer[:, c] = s234 * p[0][:, c] + s134 * p[1][:, c] + s124 * p[2][:, c] + s123 * p[3][:, c]
    return numer / denom, alpha / denom


def node_elements(T, n_nodes):
    """Elements around every node, ascending (np.where(T == i)[0])."""
    rows = [[] for _ in range(n_nodes)]
    for e, tri in enumerate(T):
        for v in tri:
            rows[int(v)].append(e)
    return rows


def plain_nodal(pos, incenter, rad, nbd, bdry):
    """Interior nodes: centre = node, radius = min_k |incenter_k - node| - r_k."""
    bset = set(int(b) for b in bdry)
    cen, rr = [], []
    for i in range(len(pos)):
        if i in bset:
            continue
        e = nbd[i]
        rr.append(np.amin(np.sqrt(np.sum((incenter[e] - pos[i]) ** 2, axis=1)) - rad[e].transpose()))
        cen.append(pos[i])
    return np.array(cen).reshape(-1, pos.shape[1]), np.array(rr).reshape(-1, 1)


# ---- maximin nodal circles ------------------------------------------------------------------------
# The reference builds, per node, the GEKKO model max Z s.t. Z <= |x - c_k| - r_k (the node's element
# incircles), Z <= |u x (x - e1)| / |u| (boundary nodes with gen_bdry: the lines of their boundary
# edges), x in the box of the incircle centres (plus the node for boundary nodes), started from the
# node (interior) or the mean of the centres and the node (boundary), and solves it with a local
# solver (APOPT). The model has several local maxima around many nodes; the one defined here -- and
# computed on the GPU -- is the local maximum that steepest ascent of the minimum over the
# constraints reaches from that initial guess, made exact by solving the three constraints tight
# there. The functions below restate the GPU kernel operation for operation (IEEE double, no fused
# multiply-add), so its results are reproduced bit for bit.

def _mm_value(M, x, y):
    m = math.inf
    for cx, cy, cr in zip(M["cx"], M["cy"], M["cr"]):
        m = min(m, math.sqrt((x - cx) * (x - cx) + (y - cy) * (y - cy)) - cr)
    for ax, ay, ab in zip(M["ax"], M["ay"], M["ab"]):
        m = min(m, abs(ax * x + ay * y + ab))
    return m


def _clamp(v, lo, hi):
    return min(max(v, lo), hi)


def _min_norm(gx, gy):
    bx, by, bn = 0.0, 0.0, math.inf
    n = len(gx)
    for i in range(n):
        n2 = gx[i] * gx[i] + gy[i] * gy[i]
        if n2 < bn:
            bn, bx, by = n2, gx[i], gy[i]
        for j in range(i + 1, n):
            dx, dy = gx[j] - gx[i], gy[j] - gy[i]
            dd = dx * dx + dy * dy
            if dd <= 0.0:
                continue
            t = _clamp(-(gx[i] * dx + gy[i] * dy) / dd, 0.0, 1.0)
            px, py = gx[i] + t * dx, gy[i] + t * dy
            p2 = px * px + py * py
            if p2 < bn:
                bn, bx, by = p2, px, py
    for i in range(n):
        if bx * (gx[i] - bx) + by * (gy[i] - by) < -1e-12:
            return 0.0, 0.0
    return bx, by


def _ascent(M):
    lo, hi = M["lo"], M["hi"]
    x, y = _clamp(0.0, lo[0], hi[0]), _clamp(0.0, lo[1], hi[1])
    fx = _mm_value(M, x, y)
    step = 0.25
    it = 0
    while it < 6000 and step > 1e-7:  # within reach of the exact solve (pg_pack.cu, same bound)
        it += 1
        gx, gy = [], []
        for cx, cy, cr in zip(M["cx"], M["cy"], M["cr"]):
            dx, dy = x - cx, y - cy
            d = math.sqrt(dx * dx + dy * dy)
            if d - cr <= fx + step and d > 0.0:
                gx.append(dx / d)
                gy.append(dy / d)
        for ax, ay, ab in zip(M["ax"], M["ay"], M["ab"]):
            s = ax * x + ay * y + ab
            if abs(s) <= fx + step:
                sg = -1.0 if s < 0.0 else 1.0
                gx.append(sg * ax)
                gy.append(sg * ay)
        dx, dy = _min_norm(gx, gy) if gx else (0.0, 0.0)
        if (x <= lo[0] and dx < 0.0) or (x >= hi[0] and dx > 0.0):
            dx = 0.0
        if (y <= lo[1] and dy < 0.0) or (y >= hi[1] and dy > 0.0):
            dy = 0.0
        nd = math.sqrt(dx * dx + dy * dy)
        if nd < 1e-12:
            step *= 0.5
            continue
        s = 0.5 * step / nd
        nx, ny = _clamp(x + s * dx, lo[0], hi[0]), _clamp(y + s * dy, lo[1], hi[1])
        fn = _mm_value(M, nx, ny)
        if fn > fx:
            x, y, fx = nx, ny, fn
            step = min(step * 1.5, 0.25)
        else:
            step *= 0.5
    return x, y, fx, step


def _det3(A):
    return (A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) - A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]) +
            A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]))


def _solve_triple(M, P):
    """Points where the three pieces are tight: piece = (kind, idx, sign, val), kind 0 circle,
    1 line (sign = side), 2 box face (sign = axis, val = coordinate)."""
    circ = [p[1] for p in P if p[0] == 0]
    R, rhs = [], []
    for kind, idx, sign, val in P:
        if kind == 1:
            R.append([sign * M["ax"][idx], sign * M["ay"][idx], -1.0])
            rhs.append(-sign * M["ab"][idx])
        elif kind == 2:
            a = int(sign)
            R.append([1.0 if a == 0 else 0.0, 1.0 if a == 1 else 0.0, 0.0])
            rhs.append(val)
    if not circ:
        det = _det3(R)
        if abs(det) < 1e-14:
            return []
        sol = []
        for c in range(3):
            A = [[rhs[i] if j == c else R[i][j] for j in range(3)] for i in range(3)]
            sol.append(_det3(A) / det)
        return [tuple(sol)]
    c1 = circ[0]
    p1x, p1y, r1 = M["cx"][c1], M["cy"][c1], M["cr"][c1]
    for cj in circ[1:]:
        pjx, pjy, rj = M["cx"][cj], M["cy"][cj], M["cr"][cj]
        R.append([2.0 * (pjx - p1x), 2.0 * (pjy - p1y), 2.0 * (rj - r1)])
        rhs.append((pjx * pjx + pjy * pjy - rj * rj) - (p1x * p1x + p1y * p1y - r1 * r1))
    Dx = R[0][1] * R[1][2] - R[0][2] * R[1][1]
    Dy = R[0][2] * R[1][0] - R[0][0] * R[1][2]
    Dz = R[0][0] * R[1][1] - R[0][1] * R[1][0]
    g00 = R[0][0] * R[0][0] + R[0][1] * R[0][1] + R[0][2] * R[0][2]
    g01 = R[0][0] * R[1][0] + R[0][1] * R[1][1] + R[0][2] * R[1][2]
    g11 = R[1][0] * R[1][0] + R[1][1] * R[1][1] + R[1][2] * R[1][2]
    gd = g00 * g11 - g01 * g01
    if Dx * Dx + Dy * Dy + Dz * Dz < 1e-24 or abs(gd) < 1e-24:
        return []
    u0, u1 = (g11 * rhs[0] - g01 * rhs[1]) / gd, (g00 * rhs[1] - g01 * rhs[0]) / gd
    q0x, q0y, q0z = u0 * R[0][0] + u1 * R[1][0], u0 * R[0][1] + u1 * R[1][1], u0 * R[0][2] + u1 * R[1][2]
    ex, ey, ez = q0x - p1x, q0y - p1y, q0z + r1
    a = Dx * Dx + Dy * Dy - Dz * Dz
    b = 2.0 * (ex * Dx + ey * Dy - ez * Dz)
    c = ex * ex + ey * ey - ez * ez
    ts = []
    if abs(a) < 1e-14:
        if abs(b) < 1e-300:
            return []
        ts.append(-c / b)
    else:
        disc = b * b - 4.0 * a * c
        if disc < 0.0:
            if disc < -1e-12 * (b * b + abs(4.0 * a * c)):
                return []
            disc = 0.0
        q = -0.5 * (b + math.copysign(math.sqrt(disc), b))
        ts.append(q / a)
        if q != 0.0:
            ts.append(c / q)
    out = []
    for t in ts:
        zx, zy, zz = q0x + t * Dx, q0y + t * Dy, q0z + t * Dz
        if all(zz + M["cr"][cj] >= -1e-12 for cj in circ):
            out.append((zx, zy, zz))
    return out


def maximin_node(pos, i, elems, incenter, rad, lines, boundary):
    """Centre, radius and whether the exact solve succeeded for node i. elems: the node's elements
    (ascending); lines: (e1, e2) endpoints of its boundary edges (ascending edge index)."""
    nx, ny = float(pos[i][0]), float(pos[i][1])
    lo, hi = [math.inf, math.inf], [-math.inf, -math.inf]
    sx = sy = 0.0
    for t in elems:
        px, py = float(incenter[t][0]), float(incenter[t][1])
        lo = [min(lo[0], px), min(lo[1], py)]
        hi = [max(hi[0], px), max(hi[1], py)]
        sx += px
        sy += py
    x0, y0 = nx, ny
    if boundary:
        lo = [min(lo[0], nx), min(lo[1], ny)]
        hi = [max(hi[0], nx), max(hi[1], ny)]
        x0 = (sx + nx) / float(len(elems) + 1)
        y0 = (sy + ny) / float(len(elems) + 1)
    L = max(max(hi[0] - lo[0], hi[1] - lo[1]), 1e-300)
    iL = 1.0 / L
    M = {"cx": [(float(incenter[t][0]) - x0) * iL for t in elems],
         "cy": [(float(incenter[t][1]) - y0) * iL for t in elems],
         "cr": [float(rad[t][0]) * iL for t in elems], "ax": [], "ay": [], "ab": []}
    if boundary:
        for e1, e2 in lines:
            e1x, e1y = float(e1[0]), float(e1[1])
            ux, uy = float(e2[0]) - e1x, float(e2[1]) - e1y
            un = math.sqrt(ux * ux + uy * uy)
            if not un > 0.0:
                continue
            ax, ay = -uy / un, ux / un
            M["ax"].append(ax)
            M["ay"].append(ay)
            M["ab"].append((ax * (x0 - e1x) + ay * (y0 - e1y)) * iL)
    M["lo"] = [(lo[0] - x0) * iL, (lo[1] - y0) * iL]
    M["hi"] = [(hi[0] - x0) * iL, (hi[1] - y0) * iL]
    x, y, fx, step = _ascent(M)
    near = max(1e-6, 8.0 * step)
    S = []
    for k in range(len(M["cx"])):
        v = math.sqrt((x - M["cx"][k]) * (x - M["cx"][k]) + (y - M["cy"][k]) * (y - M["cy"][k])) - M["cr"][k]
        if v <= fx + near and len(S) < PS_MAX:
            S.append((0, k, 0.0, 0.0))
    for l in range(len(M["ax"])):
        s = M["ax"][l] * x + M["ay"][l] * y + M["ab"][l]
        if abs(s) <= fx + near and len(S) < PS_MAX:
            S.append((1, l, -1.0 if s < 0.0 else 1.0, 0.0))
    for a in range(2):
        w = x if a == 0 else y
        if w - M["lo"][a] <= near and len(S) < PS_MAX:
            S.append((2, a, float(a), M["lo"][a]))
        if M["hi"][a] - w <= near and len(S) < PS_MAX:
            S.append((2, a, float(a), M["hi"][a]))
    bx, by, bf, bd = x, y, fx, math.inf
    for p in range(len(S)):
        for q in range(p + 1, len(S)):
            for r in range(q + 1, len(S)):
                T3 = (S[p], S[q], S[r])
                boxes = [t for t in T3 if t[0] == 2]
                axes = 0
                for t in boxes:
                    axes |= 1 << int(t[2])
                if len(boxes) == 3 or (len(boxes) == 2 and axes != 3):
                    continue
                for qx, qy, qz in _solve_triple(M, T3):
                    tol = 1e-11
                    if qx < M["lo"][0] - tol or qx > M["hi"][0] + tol or qy < M["lo"][1] - tol or qy > M["hi"][1] + tol:
                        continue
                    cx, cy = _clamp(qx, M["lo"][0], M["hi"][0]), _clamp(qy, M["lo"][1], M["hi"][1])
                    v = _mm_value(M, cx, cy)
                    if len(boxes) < 2 and abs(v - qz) > 1e-9:
                        continue
                    if v < fx - 1e-12:
                        continue
                    d = (cx - x) * (cx - x) + (cy - y) * (cy - y)
                    if d < bd:
                        bd, bx, by, bf = d, cx, cy, v
    return (x0 + bx * L, y0 + by * L), bf * L, bd != math.inf


PS_MAX = 12


def maximin_nodal(pos, incenter, rad, nbd, bdry, bdry_edges, gen_bdry):
    """Interior nodes (and boundary nodes with gen_bdry) in node order: (centres, radii, solved)."""
    bset = set(int(b) for b in bdry)
    node_edges = [[] for _ in range(len(pos))]
    for k, (a, b) in enumerate(np.asarray(bdry_edges, np.int64).reshape(-1, 2)):
        node_edges[int(a)].append(k)
        node_edges[int(b)].append(k)
    cen, rr, ok = [], [], []
    for i in range(len(pos)):
        boundary = i in bset
        if boundary and not gen_bdry:
            continue
        lines = [(pos[bdry_edges[k][0]], pos[bdry_edges[k][1]]) for k in sorted(node_edges[i])] if boundary else []
        c, r, good = maximin_node(pos, i, sorted(nbd[i]), incenter, rad, lines, boundary)
        cen.append(c)
        rr.append(r)
        ok.append(good)
    return np.array(cen).reshape(-1, 2), np.array(rr).reshape(-1, 1), np.array(ok, bool)


def incenter_mesh_loc(pos, T, bdry_nodes, bdry_edges, modify_nodal_circles, gen_bdry):
    """Element circles followed by the nodal circles: (incenter [k, dim], radius [k, 1], ok)."""
    inc, rad = element_circles(pos, T)
    nbd = node_elements(T, len(pos))
    if modify_nodal_circles:
        c, r, ok = maximin_nodal(pos, inc, rad, nbd, bdry_nodes, bdry_edges, gen_bdry)
    else:
        c, r = plain_nodal(pos, inc, rad, nbd, bdry_nodes)
        ok = np.ones(len(r), bool)
    return np.append(inc, c, axis=0), np.append(rad, r, axis=0), ok
