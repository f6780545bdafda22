"""TEST INFRASTRUCTURE: the picture mdsc_render draws, restated in numpy (FP64),
for small images.  The reference's own viewer (v25/graphic.cpp) needs an
OpenGL display, which this machine does not have; this restatement follows
the same scene description (v25/graphic.cpp:183-330,405-415,612-692) and is
the checker for the GPU ray caster -- parity with the GL pixels themselves
is unpinned."""
from __future__ import annotations

import math

import numpy as np

TONE = (1.0, 0.4, 0.6, 0.2, 0.8)


def camera(width, height, theta, phi, dist, ref, shift):
    usr = dist * np.array([math.sin(theta) * math.cos(phi), math.sin(theta) * math.sin(phi), math.cos(theta)])
    ref = np.asarray(ref, dtype=np.float64)
    view = usr - ref
    vn, un = np.linalg.norm(view), np.linalg.norm(usr)
    eye = usr + un * view / vn - np.asarray(shift, dtype=np.float64)
    fwd = -view / vn
    wu = np.array([0.0, 1.0, 0.0]) if abs(fwd[2]) > 0.999999 else np.array([0.0, 0.0, 1.0])
    right = np.cross(fwd, wu)
    right /= np.linalg.norm(right)
    up = np.cross(right, fwd)
    tan_half = math.tan(math.pi / 6)
    pix = 2.0 * (vn + un) * tan_half / height
    light = usr / un if un > 0 else np.array([0.0, 0.0, 1.0])
    return eye, fwd, right, up, tan_half, pix, light


def capsules(r, O, length, dia, species, dip, box, pix, dipoles=True, draw_box=True):
    """(a, b, radius, kind, tone, ex, flat colour) of every capsule."""
    caps = []
    for i in range(len(r)):
        u = O[i][2]
        h = 0.5 * length[i]
        caps.append((r[i] - h * u, r[i] + h * u, 0.5 * dia[i], 0, TONE[species[i] % 5], O[i][0], None))
        if dipoles:
            for w in np.asarray(dip[i]).reshape(-1, 5):
                if w[4] == 0.0:
                    continue
                p = r[i] + w[0] * O[i][2]
                d = O[i].T @ w[1:4]
                mlt = 1.5 * 0.5 * dia[i]
                caps.append((p - mlt * d, p, pix, 1, -1.0, None, (0.0, 0.0, 1.0)))
                caps.append((p, p + mlt * d, pix, 1, -1.0, None, (1.0, 0.0, 0.0)))
    if draw_box:
        h = 0.5 * np.asarray(box, dtype=np.float64)
        for axis in range(3):
            o1, o2 = (axis + 1) % 3, (axis + 2) % 3
            for corner in range(4):
                a = np.zeros(3)
                b = np.zeros(3)
                a[axis], b[axis] = -h[axis], h[axis]
                a[o1] = b[o1] = h[o1] if corner & 1 else -h[o1]
                a[o2] = b[o2] = h[o2] if corner & 2 else -h[o2]
                caps.append((a, b, 0.5 * pix, 1, -1.0, None, (0.6, 0.3, 0.3)))
    return caps


def hit(o, d, a, b, rad):
    """Distances along the unit rays d (n, 3) from o to the capsule, or -1."""
    ba, oa = b - a, o - a
    baba = ba @ ba
    bard, baoa = d @ ba, oa @ ba
    rdoa, oaoa = d @ oa, oa @ oa
    qa = baba - bard * bard
    qb = baba * rdoa - baoa * bard
    qc = baba * oaoa - baoa * baoa - rad * rad * baba
    t = np.full(len(d), -1.0)
    disc = qb * qb - qa * qc
    ok = (qa > 1e-12 * baba) & (disc >= 0)
    tc = np.where(ok, (-qb - np.sqrt(np.where(ok, disc, 0.0))) / np.where(ok, qa, 1.0), -1.0)
    y = baoa + tc * bard
    body = ok & (tc > 0) & (y > 0) & (y < baba)
    t[body] = tc[body]
    best = np.full(len(d), -1.0)
    for c in (a, b):
        oc = o - c
        hb = d @ oc
        hc = oc @ oc - rad * rad
        dd = hb * hb - hc
        ts = np.where(dd >= 0, -hb - np.sqrt(np.maximum(dd, 0.0)), -1.0)
        take = (ts > 0) & ((best < 0) | (ts < best))
        best[take] = ts[take]
    return np.where(body, t, best)


def render(width, height, r, O, length, dia, species, dip, box, theta=0.1, phi=0.0, dist=15.0, ref=(0, 0, 0),
           shift=(0, 0, 0), dipoles=True, draw_box=True):
    eye, fwd, right, up, tan_half, pix, light = camera(width, height, theta, phi, dist, ref, shift)
    ys, xs = np.mgrid[0:height, 0:width]
    sx = (2.0 * (xs + 0.5) / width - 1.0) * tan_half * width / height
    sy = (1.0 - 2.0 * (ys + 0.5) / height) * tan_half
    d = fwd[None, None, :] + sx[..., None] * right + sy[..., None] * up
    d = (d / np.linalg.norm(d, axis=-1, keepdims=True)).reshape(-1, 3)
    caps = capsules(r, O, length, dia, species, dip, box, pix, dipoles, draw_box)
    tmin = np.full(len(d), np.inf)
    idx = np.full(len(d), -1)
    for k, (a, b, rad, *_rest) in enumerate(caps):
        t = hit(eye, d, a, b, rad)
        take = (t > 0) & (t < tmin)
        tmin[take] = t[take]
        idx[take] = k
    col = np.ones((len(d), 3))
    for k in np.unique(idx[idx >= 0]):
        a, b, rad, kind, tone, ex, flat = caps[k]
        m = idx == k
        if kind == 1:
            col[m] = flat
            continue
        p = eye + tmin[m, None] * d[m]
        ba = b - a
        s = np.clip(((p - a) @ ba) / (ba @ ba), 0.0, 1.0)
        nv = (p - a - s[:, None] * ba) / rad
        u = ba / np.linalg.norm(ba)
        base = np.full((m.sum(), 3), tone)
        cap = s >= 1.0
        z = nv @ u
        base[cap & (z > 0.8)] = (0.0, 0.0, 1.0)
        bodyp = (s > 0.0) & (s < 1.0)
        ey = np.cross(u, ex)
        phi_ = np.arctan2(nv @ ey, nv @ ex)
        facet = math.pi / 6
        wr = np.maximum(0.0, 1.0 - np.abs(phi_) / facet)
        wg = np.maximum(0.0, 1.0 - np.abs(phi_ - math.pi / 2) / facet)
        wt = 1.0 - wr - wg
        stripes = np.stack([wt * tone + wr, wt * tone + wg, wt * tone], axis=-1)
        base[bodyp] = stripes[bodyp]
        shade = 0.5 + 0.7 * np.maximum(0.0, nv @ light)
        col[m] = np.minimum(1.0, base * shade[:, None])
    return np.rint(255.0 * np.clip(col, 0.0, 1.0)).astype(np.uint8).reshape(height, width, 3)
