"""The headless picture (mdsc_render, mdspherocyl_gb300/render.py) against
the numpy restatement of the viewer's scene (oracle/render_np.py).  The
reference's OpenGL viewer itself cannot run here (no display), so the pixels
are checked against the restatement: all but the silhouette and colour-edge
pixels equal, where FP32 and FP64 may round a ray differently."""
import os
import tempfile

import numpy as np
import pytest

from conftest import ROOT
from mdspherocyl_gb300 import files as F
from mdspherocyl_gb300 import lib as L
from mdspherocyl_gb300.driver import layout
from oracle import render_np

RUN = os.path.join(ROOT, "tests", "golden", "run_v25", "init")


def _one_rod():
    """A rod along +x whose body x and y axes point 45 degrees away from +z,
    so that from above the camera sees neither meridian."""
    c = np.sqrt(0.5)
    O = np.array([[[0.0, c, c], [0.0, -c, c], [1.0, 0.0, 0.0]]])
    return np.zeros((1, 3)), O


def test_restatement_draws_the_scene():
    """One rod along x: seen from above, the grey body in the middle on
    white; seen from the +x side at a slant, its blue tip."""
    r, O = _one_rod()
    args = (r, O, np.array([4.0]), np.array([1.0]), [1], [np.zeros((0, 5))])  # species 1: grey 0.4
    img = render_np.render(64, 64, *args, box=(8.0, 8.0, 8.0), theta=1e-6, dist=4.0, draw_box=False)
    assert img.shape == (64, 64, 3)
    assert tuple(img[2, 2]) == (255, 255, 255)
    c = img[32, 32].astype(int)
    assert c[0] == c[1] == c[2] == round(255 * 0.4 * 1.2)  # the grey body, lit head-on
    side = render_np.render(64, 64, *args, box=(8.0, 8.0, 8.0), theta=1.0, phi=0.0, dist=4.0, draw_box=False)
    blue = (side[..., 2] > 150) & (side[..., 0] < 60) & (side[..., 1] < 60)
    assert blue.sum() > 10
    with tempfile.TemporaryDirectory() as d:
        L.write_ppm(os.path.join(d, "a.ppm"), img)
        assert np.array_equal(L.read_ppm(os.path.join(d, "a.ppm")), img)


def _run_state():
    p = F.read_input(os.path.join(RUN, "input.txt"))
    length, dia, mass, dip, nd, nd_part = layout(p)
    c = F.read_conf(os.path.join(RUN, "conf.dat"), p.n_part, nd_part)
    species = np.repeat(np.arange(p.n_comp), p.n_part)
    return p, length, dia, mass, dip, nd, c, species


def _close(a, b, frac=0.02, tol=3):
    diff = np.abs(a.astype(int) - b.astype(int)).max(axis=-1)
    return (diff > tol).mean() <= frac, (diff > tol).mean()


@pytest.mark.gpu
@pytest.mark.parametrize("view", [dict(theta=0.1, phi=0.0, dist=15.0),
                                  dict(theta=1.1, phi=0.7, dist=20.0, ref=(2.0, -1.0, 0.5)),
                                  dict(theta=0.6, phi=2.0, dist=6.0, dipoles=False, box=False)])
def test_gpu_picture_matches_the_restatement(view):
    from mdspherocyl_gb300.systems import SystemSpec, SystemState

    p, length, dia, mass, dip, nd, c, species = _run_state()
    spec = SystemSpec(n=p.n_total, box=c["box"], alpha=p.alpha, K_max=1, ksq_max=0)
    st = SystemState(c["r"], c["p"], c["O"], c["l"], length, dia, mass, dip)
    W, H = 160, 120
    with L.Batch([spec], None, descs=[L.desc_from_spec(spec, nd)]) as bt:
        bt.upload(0, st)
        bt.set_species(0, p.n_part)
        img = bt.render(0, width=W, height=H, **view)
    want = render_np.render(W, H, c["r"], c["O"], length, dia, species, dip, c["box"],
                            theta=view["theta"], phi=view["phi"], dist=view["dist"], ref=view.get("ref", (0, 0, 0)),
                            dipoles=view.get("dipoles", True), draw_box=view.get("box", True))
    ok, frac = _close(img, want)
    assert ok, frac
    assert (img != 255).any()  # something was drawn


@pytest.mark.gpu
def test_render_run_directory_and_options():
    from mdspherocyl_gb300.render import main, render_run

    with tempfile.TemporaryDirectory() as d:
        assert main([RUN, os.path.join(d, "c.ppm"), "--size", "96", "64", "--dist", "30"]) == 0
        img = L.read_ppm(os.path.join(d, "c.ppm"))
        assert img.shape == (64, 96, 3) and (img != 255).any()
    plain = render_run(RUN, width=64, height=64, dist=30.0)
    imgs = render_run(RUN, width=64, height=64, dist=30.0, images=True)
    none = render_run(RUN, width=64, height=64, dist=30.0, cluster=10 ** 6, box=False)
    assert (none == 255).all()  # no particle carries that label
    assert (imgs != 255).sum() >= (plain != 255).sum()  # images add rods
