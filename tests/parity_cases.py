"""Shared parity cases: (model, box, camera) groups at oracle-friendly sizes."""
from __future__ import annotations

import numpy as np

from gaussmle_gb300 import simulate
from gaussmle_gb300.models import (AstigmaticXYZNB, GaussianXYNB, GaussianXYNBS,
                                   GaussianXYNBSXSY)
from gaussmle_gb300.constraints import default_constraints

# The parity bar and the comparison live with the oracle (oracle/parity.py):
# positions, sigmas and z within 1e-3, N and bg within 1e-4 relative, CRLB
# within 1e-3 relative, identical convergence flags.
from oracle.parity import TOL_POS, TOL_REL_CRLB, TOL_REL_NBG, compare  # noqa: E402,F401

CASES = [
    # name, model, box, camera, n
    ("xynb-11-poisson", 0, 11, 0, 3000),
    ("xynb-7-poisson", 0, 7, 0, 2000),
    ("xynb-5-poisson", 0, 5, 0, 1000),
    ("xynbs-13-scmos-adu", 1, 13, 2, 2000),
    ("xynbs-9-scmos-var", 1, 9, 1, 2000),
    ("xynbsxsy-13-scmos-adu", 2, 13, 2, 2000),
    ("xynbsxsy-11-poisson", 2, 11, 0, 2000),
    ("astig-15-poisson", 3, 15, 0, 2000),
    ("astig-15-scmos-adu", 3, 15, 2, 1000),
    ("xynb-15-scmos-adu", 0, 15, 2, 1000),
]


def make_case(name, model, box, camera, n, seed=None, sensor=256):
    rng = np.random.Generator(np.random.Philox(seed if seed is not None else 4242 + box + 17 * model))
    maps = simulate.scmos_maps(rng, sensor, sensor) if camera else None
    if model == 3:
        psf = AstigmaticXYZNB(1.3, 1.3, 0.05, 0.05, 0.3, 0.3, 50.0, 100.0)
        cons = simulate.ASTIG_WIDE
        x, y, N, bg = simulate._xy_n_bg(rng, n, box, 1000, 10000, 2, 30)
        truth = np.stack([x, y, rng.uniform(-400, 400, n), N, bg], 1)
    else:
        psf = {0: GaussianXYNB(1.3), 1: GaussianXYNBS(), 2: GaussianXYNBSXSY()}[model]
        cons = default_constraints(psf, 11)
        x, y, N, bg = simulate._xy_n_bg(rng, n, box)
        cols = [x, y, N, bg]
        if model == 1:
            cols.append(rng.uniform(1.0, 1.8, n))
        if model == 2:
            cols += [rng.uniform(1.0, 2.0, n), rng.uniform(1.0, 2.0, n)]
        truth = np.stack(cols, 1)
    truth = truth.astype(np.float32)
    if camera:
        xc, yc = simulate.random_corners(rng, n, box, sensor, sensor)
        data = simulate.scmos_rois(rng, psf, truth, box, maps, xc, yc)
        if camera == 1:  # variance-only: data converted to e- on the host
            var, gain, off = maps
            rows = (yc[:, None, None] - 1) + np.arange(box)[None, None, :]
            cols_ = (xc[:, None, None] - 1) + np.arange(box)[None, :, None]
            g = gain[rows, cols_]
            o = off[rows, cols_]
            adu_c = np.ascontiguousarray(data.transpose(2, 1, 0))
            e = ((adu_c - o) * g).astype(np.float32)
            data = e.transpose(2, 1, 0)
    else:
        xc = yc = np.ones(n, np.int32)
        data = simulate.poisson_rois(rng, psf, truth, box)
    return simulate.Workload(name, psf, box, camera, cons, np.asfortranarray(data), xc, yc,
                             truth, maps=maps)


def oracle_desc(O, w, iterations=20):
    c = w.constraints
    return O.make_desc(w.psf.model_id, w.box, iterations, w.camera, w.psf.psf_vector(),
                       c.lower, c.upper, c.max_step)
