"""Small hand-built configurations (N = 2..8) that put rod pairs in every
branch of the reference's segment-distance routine, spherocyl_dist
(v25/functions.cpp:89-489), at segment distances inside the WCA range:

* the nine (s, t) regions of non-parallel, non-intersecting axis lines
  (:277-445);
* axis lines that intersect (:127-276): each of the four closest end-point
  pairs (im = 0..3), each with its three outcomes -- the far end projects
  onto the other segment ('s'), the near end does ('t'), or neither ('end');
* parallel rods (:447-486): no unique closest pair (sentinel -1e6, the
  two-particle case documented at :1489-1494), and end to end in the four
  combinations (sentinels -1e10, -2e10, -3e10, -4e10; force_sc tests -3e10
  twice, :1526,1529, so the -4e10 pair keeps lever arms of order 4e10).

Pairs are placed around anchors of a 24^3 box, one anchor crossing a
periodic face, so pairs of one system do not interact; a few systems add a
free rod, a bundle of three parallel rods or a rod with four partners, so
one particle sums several pairs.  Non-parallel pairs are turned by a seeded
rotation; parallel ones only by signed permutations, which keep them
exactly parallel (the -4e10 torque multiplies o_i x o_j, zero only then).

branch() restates, for the tests, only which branch the reference takes.
"""
import itertools
import math

import numpy as np

BOX = 24.0
ANCHORS = np.array([[6.0, 6.0, 6.0], [18.0, 18.0, 6.0], [18.0, 6.0, 18.0], [6.0, 18.0, 23.5]])
LONE = np.array([0.5, 12.5, 12.5])

X, Y, Z = np.eye(3)


def _perp(z0, xs, h, flip=False, lB=2.0):
    """Rod A (length 2) on the z axis; rod B along +x (or -x), its centre at
    height z0, lateral offset h along y, shifted xs along x."""
    return (np.array([[0.0, 0.0, 0.0], [xs, h, z0]]), np.array([Z, -X if flip else X]), np.array([2.0, lB]))


def _par(dx, dz, flip=False, lB=2.0, dy=0.0):
    """Both rods along z (B along -z if flip), B's centre at (dx, dy, dz)."""
    return (np.array([[0.0, 0.0, 0.0], [dx, dy, dz]]), np.array([Z, -Z if flip else Z]), np.array([2.0, lB]))


# name -> (positions relative to the anchor, rod axes, lengths); the name
# says which branch the pair is built for
PAIRS = {
    # non-parallel, lines apart: regions of (s, t), v25/functions.cpp:280-284
    "region5": _perp(0.2, 0.0, 0.9),
    "region2": _perp(1.5, 0.0, 0.9),
    "region8": _perp(-1.5, 0.0, 0.9),
    "region6": _perp(0.1, -1.5, 0.9),
    "region4": _perp(-0.1, 1.5, 0.9, lB=2.5),
    "region3": _perp(1.5, -1.5, 0.35),
    "region1": _perp(1.5, 1.5, 0.35),
    "region7": _perp(-1.5, 1.5, 0.35),
    "region9": _perp(-1.5, -2.0, 0.35, lB=3.0),
    # axis lines that cross: closest end points A head/tail x B head/tail
    "intersect0-s": _perp(0.3, -1.9, 0.0),
    "intersect0-t": _perp(1.9, -0.5, 0.0),
    "intersect0-end": _perp(1.6, -1.6, 0.0),
    "intersect1-s": _perp(0.3, 1.9, 0.0),
    "intersect1-t": _perp(1.9, 0.5, 0.0),
    "intersect1-end": _perp(1.6, 1.6, 0.0),
    "intersect2-s": _perp(-0.3, -1.9, 0.0),
    "intersect2-t": _perp(-1.9, -0.5, 0.0),
    "intersect2-end": _perp(-1.6, -1.6, 0.0),
    "intersect3-s": _perp(-0.3, 1.9, 0.0),
    "intersect3-t": _perp(-1.9, 0.5, 0.0, lB=2.5),
    "intersect3-end": _perp(-1.6, 1.6, 0.0),
    # parallel
    "parallel-documented": _par(1.1, 0.0, dy=0.25, lB=3.0),  # v25/functions.cpp:1489-1494, beyond 2^(1/6)
    "parallel-none": _par(1.0, 0.3, dy=0.25, lB=3.0),
    "parallel++": _par(0.2, 2.9),
    "parallel--": _par(0.2, -2.9),
    "parallel+-": _par(0.2, 2.9, flip=True),
    "parallel-+": _par(0.2, -2.9, flip=True),
}

# systems: lists of pairs (+ 'lone' for a free rod, or a whole cluster)
SYSTEMS = [
    ["parallel-+"],
    ["parallel-documented"],
    ["region5", "lone"],
    ["region2", "region8"],
    ["region6", "region4", "lone"],
    ["region1", "region3", "region7"],
    ["region9", "parallel-none", "parallel++", "lone"],
    ["parallel--", "parallel+-", "intersect0-s", "intersect0-t"],
    ["intersect0-end", "intersect1-s", "intersect1-t", "intersect1-end"],
    ["intersect2-s", "intersect2-t", "intersect2-end", "intersect3-s"],
    ["intersect3-t", "intersect3-end"],
    ["bundle"],
    ["star", "region5"],
]


def _cluster(name):
    if name == "bundle":  # three parallel rods, each pair side by side
        return (np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.3], [0.5, 0.95, -0.2]]), np.array([Z, Z, Z]),
                np.array([2.0, 2.0, 2.5]))
    if name == "star":  # a rod with four partners: two across it, one off each end
        return (np.array([[0.0, 0.0, 0.0], [0.0, 0.9, 0.5], [0.3, -0.9, -0.5], [0.2, 0.0, 2.9], [0.2, 0.0, -2.9]]),
                np.array([Z, X, -X, Z, Z]), np.array([2.0, 2.0, 2.0, 2.0, 2.0]))
    raise KeyError(name)


def frame(u):
    """A rotation whose third row (the rod axis) is u; exact for unit u on an axis."""
    u = np.asarray(u, dtype=np.float64)
    k = int(np.argmin(np.abs(u)))
    a = np.zeros(3)
    a[k] = 1.0
    e1 = np.cross(a, u)
    e1 = e1 / np.sqrt(e1 @ e1)
    e2 = np.cross(u, e1)
    return np.stack([e1, e2, u])


def _signed_perms():
    out = []
    for p in itertools.permutations(range(3)):
        for sg in itertools.product((1.0, -1.0), repeat=3):
            R = np.zeros((3, 3))
            for i in range(3):
                R[i, p[i]] = sg[i]
            if np.linalg.det(R) > 0:
                out.append(R)
    return out


def _rotation(rng, exact):
    if exact:
        P = _signed_perms()
        return P[int(rng.integers(len(P)))]
    q, r = np.linalg.qr(rng.normal(size=(3, 3)))
    q = q * np.sign(np.diag(r))
    return q if np.linalg.det(q) > 0 else -q


def build(seed=0):
    """The systems: a list of dicts r, O, length, dia, box and the pairs
    placed in it, pairs = [(name, index of its first rod, rods)]."""
    rng = np.random.default_rng(seed)
    out = []
    for members in SYSTEMS:
        r, O, ln, pairs = [], [], [], []
        for k, name in enumerate(members):
            if name == "lone":
                r.append(LONE.copy())
                O.append(frame(np.array([1.0, 2.0, 3.0]) / math.sqrt(14.0)))
                ln.append(2.0)
                continue
            rel, ax, lens = PAIRS[name] if name in PAIRS else _cluster(name)
            exact = name.startswith("parallel") or name in ("bundle", "star")
            R = _rotation(rng, exact)
            pairs.append((name, len(r), len(rel)))
            for q in range(len(rel)):
                r.append(np.mod(ANCHORS[k] + R @ rel[q], BOX))
                O.append(frame(R @ ax[q]))
                ln.append(float(lens[q]))
        n = len(r)
        assert 2 <= n <= 8
        out.append(dict(members=members, pairs=pairs, r=np.array(r), O=np.array(O), length=np.array(ln),
                        dia=np.ones(n), box=np.full(3, BOX)))
    return out


def _dot(u, v):
    return u[0] * v[0] + u[1] * v[1] + u[2] * v[2]


def _mi(v, L):
    return [v[a] - L[a] * math.floor(v[a] / L[a] + 0.5) for a in range(3)]


def branch(c, i, j):
    """Which branch spherocyl_dist (v25/functions.cpp:89-489) takes for
    particle i against particle j of configuration c, in its own FP64
    expressions: 'regionK', 'intersectIM-{s,t,end}' or 'parallel{none,++,--,+-,-+}'."""
    L = [float(x) for x in c["box"]]
    ri, rj = [float(x) for x in c["r"][i]], [float(x) for x in c["r"][j]]
    oA, oB = [float(x) for x in c["O"][i][2]], [float(x) for x in c["O"][j][2]]
    lA, lB = float(c["length"][i]), float(c["length"][j])
    rAB = _mi([ri[a] - rj[a] for a in range(3)], L)
    doto, dotrA, dotrB = _dot(oA, oB), _dot(rAB, oA), _dot(rAB, oB)
    a, b, cc = lA * lA, doto * lA * lB, lB * lB
    d = dotrA * lA - a / 2 + b / 2
    e = dotrB * lB + cc / 2 - b / 2
    det = a * cc - b * b
    s, t = b * e - cc * d, a * e - b * d
    if det > 1.e-12:
        s0, t0 = s / det, t / det
        dis = [rAB[k] + (s0 - 0.5) * lA * oA[k] - (t0 - 0.5) * lB * oB[k] for k in range(3)]
        if _dot(dis, dis) < 1.e-12:
            pp = [[ri[k] + lA * oA[k] / 2 for k in range(3)], [ri[k] - lA * oA[k] / 2 for k in range(3)],
                  [rj[k] + lB * oB[k] / 2 for k in range(3)], [rj[k] - lB * oB[k] / 2 for k in range(3)]]
            dd = [_dot(v, v) for v in (_mi([pp[0][k] - pp[2][k] for k in range(3)], L),
                                       _mi([pp[0][k] - pp[3][k] for k in range(3)], L),
                                       _mi([pp[1][k] - pp[2][k] for k in range(3)], L),
                                       _mi([pp[1][k] - pp[3][k] for k in range(3)], L))]
            im, mind = 0, 1.e6
            for k in range(4):
                if dd[k] < mind:
                    im, mind = k, dd[k]
            far = 2 if im in (0, 2) else 3  # the end of B whose projection onto A is tried first
            sv = _dot(_mi([pp[1][k] - pp[far][k] for k in range(3)], L), oA) / -lA
            if 0 <= sv <= 1:
                return f"intersect{im}-s"
            near = 0 if im in (0, 1) else 1  # then A's end projected onto B
            tv = _dot(_mi([pp[3][k] - pp[near][k] for k in range(3)], L), oB) / -lB
            return f"intersect{im}-" + ("t" if 0 <= tv <= 1 else "end")
        if s >= 0:
            if s <= det:
                reg = (5 if t <= det else 6) if t >= 0 else 4
            else:
                reg = (2 if t <= det else 3) if t >= 0 else 1
        else:
            reg = (8 if t <= det else 9) if t >= 0 else 7
        return f"region{reg}"
    if abs(dotrA) < (lA + lB) / 2:
        return "parallel-none"
    if doto > 0:
        p = [rAB[k] + lA * oA[k] / 2 + lB * oB[k] / 2 for k in range(3)]
        m = [rAB[k] - lA * oA[k] / 2 - lB * oB[k] / 2 for k in range(3)]
        return "parallel--" if _dot(m, m) < _dot(p, p) else "parallel++"
    p = [rAB[k] + lA * oA[k] / 2 - lB * oB[k] / 2 for k in range(3)]
    m = [rAB[k] - lA * oA[k] / 2 + lB * oB[k] / 2 for k in range(3)]
    return "parallel-+" if _dot(m, m) < _dot(p, p) else "parallel+-"


ALL_BRANCHES = ({f"region{k}" for k in range(1, 10)}
                | {f"intersect{im}-{x}" for im in range(4) for x in ("s", "t", "end")}
                | {"parallel-none", "parallel++", "parallel--", "parallel+-", "parallel-+"})
