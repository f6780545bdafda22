"""A picture of a run directory's conf.dat, without a display.

    python -m mdspherocyl_gb300.render <run-directory> <out.ppm> [--theta T] [--phi P] [--dist D]
        [--ref X Y Z] [--size W H] [--images] [--no-dipoles] [--no-box] [--cluster C] [--device N]

The reference looks at its configurations with an SDL/OpenGL viewer
(v25/graphic.cpp) that reads input.txt and conf.dat; this draws the same
scene with the library's ray caster (mdsc_render) into a PPM file.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

from . import files as F
from . import lib as L
from .driver import layout
from .systems import SystemSpec, SystemState


def render_run(workdir: str, device: int = 0, **view):
    """The picture of workdir's conf.dat (species and shapes from input.txt)."""
    p = F.read_input(os.path.join(workdir, "input.txt"))
    length, dia, mass, dip, nd, nd_part = layout(p)
    c = F.read_conf(os.path.join(workdir, "conf.dat"), p.n_part, nd_part)
    box = c["box"]
    spec = SystemSpec(n=p.n_total, box=box, alpha=p.alpha, K_max=1, ksq_max=0, dt=p.Dt)
    st = SystemState(c["r"], c["p"], c["O"], c["l"], length, dia, mass, dip)
    with L.Batch([spec], None, device=device, descs=[L.desc_from_spec(spec, nd)]) as bt:
        bt.upload(0, st, clust=c["clust"].astype(np.int32))
        if p.n_comp > 1:
            bt.set_species(0, p.n_part)
        return bt.render(0, **view)


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("workdir")
    ap.add_argument("out")
    ap.add_argument("--theta", type=float, default=0.1)
    ap.add_argument("--phi", type=float, default=0.0)
    ap.add_argument("--dist", type=float, default=15.0)
    ap.add_argument("--ref", type=float, nargs=3, default=(0.0, 0.0, 0.0))
    ap.add_argument("--size", type=int, nargs=2, default=(480, 480))
    ap.add_argument("--images", action="store_true")
    ap.add_argument("--no-dipoles", action="store_true")
    ap.add_argument("--no-box", action="store_true")
    ap.add_argument("--cluster", type=int, default=-1)
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args(argv)
    img = render_run(a.workdir, a.device, width=a.size[0], height=a.size[1], theta=a.theta, phi=a.phi,
                     dist=a.dist, ref=a.ref, dipoles=not a.no_dipoles, images=a.images, box=not a.no_box,
                     cluster=a.cluster)
    L.write_ppm(a.out, img)
    return 0


if __name__ == "__main__":
    sys.exit(main())
