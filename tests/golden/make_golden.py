"""Generate the golden fixtures under tests/golden/.

1. astig_theory_crlb.npz - the reference's own first-principles Fisher / CRLB
   derivation for the astigmatic PSF, dev/astig_theory/compute_theoretical_crlb.jl,
   restated in float64 with its parameters (sigma0 1.3 px, Ax 0.05, Ay -0.05,
   Bx 0.01, By -0.01, gamma 200, d 500, 15x15 box, x 8.3, y 8.2, N 2000,
   bg 1, z on 50 points of [-600, 600]).  It is independent of GaussLib:
   PSF, derivatives and the Fisher sum are written out from the mathematics,
   so it checks the oracle's derivative and CRLB code.  (The script evaluates
   erf with Abramowitz-Stegun 7.1.26, |error| <= 1.5e-7; scipy's erf is used
   here, so agreement is expected to a few 1e-6 relative.)
2. oracle_<case>.npz - small seeded inputs for every (model, camera) and the
   FP32 oracle's outputs: regression fixtures for the oracle and the GPU.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from math import pi, sqrt
from pathlib import Path

import numpy as np
from scipy.special import erf

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "gaussmle.jl_gb300"))
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

# parameters of dev/astig_theory/compute_theoretical_crlb.jl
THEORY = dict(sigma0=1.3, Ax=0.05, Ay=-0.05, Bx=0.01, By=-0.01, gamma=200.0, d=500.0,
              box=15, x=8.3, y=8.2, N=2000.0, bg=1.0)


def theory_crlb(z: float, p=THEORY) -> np.ndarray:
    """CRLB [x, y, z, N, bg] of the Poisson Fisher matrix at z (float64)."""
    s0, g, d, box = p["sigma0"], p["gamma"], p["d"], p["box"]

    def alpha(zs, A, B):
        u = zs / d
        return 1 + u ** 2 + A * u ** 3 + B * u ** 4

    def dalpha(zs, A, B):
        return (2 / d ** 2) * zs + (3 * A / d ** 3) * zs ** 2 + (4 * B / d ** 4) * zs ** 3

    def sigma(gam, A, B):
        return s0 * sqrt(alpha(z - gam, A, B))

    def dsigma(gam, A, B):
        zs = z - gam
        return s0 / (2 * sqrt(alpha(zs, A, B))) * dalpha(zs, A, B)

    sx, sy = sigma(g, p["Ax"], p["Bx"]), sigma(-g, p["Ay"], p["By"])
    dsx, dsy = dsigma(g, p["Ax"], p["Bx"]), dsigma(-g, p["Ay"], p["By"])
    t = np.arange(1, box + 1, dtype=np.float64)

    def phi(mu, s):
        return 0.5 * (erf((t - mu + 0.5) / (sqrt(2) * s)) - erf((t - mu - 0.5) / (sqrt(2) * s)))

    def dphi_dmu(mu, s):
        u, lo = (t - mu + 0.5) / s, (t - mu - 0.5) / s
        return (np.exp(-0.5 * u * u) - np.exp(-0.5 * lo * lo)) / (sqrt(2 * pi) * s)

    def dphi_ds(mu, s):
        u, lo = (t - mu + 0.5) / s, (t - mu - 0.5) / s
        return -(u * np.exp(-0.5 * u * u) - lo * np.exp(-0.5 * lo * lo)) / (sqrt(2 * pi) * s)

    N, bg = p["N"], p["bg"]
    px, py = phi(p["x"], sx), phi(p["y"], sy)          # first index pairs with x
    dpx, dpy = dphi_dmu(p["x"], sx), dphi_dmu(p["y"], sy)
    spx, spy = dphi_ds(p["x"], sx), dphi_ds(p["y"], sy)
    P = np.outer
    mu = bg + N * P(px, py)
    der = [N * P(dpx, py), N * P(px, dpy), N * (P(spx, py) * dsx + P(px, spy) * dsy),
           P(px, py), np.ones_like(mu)]
    F = np.array([[np.sum(a * b / mu) for b in der] for a in der])
    F += 1e-10 * np.abs(F).max() * np.eye(5)
    return np.sqrt(np.maximum(np.diag(np.linalg.inv(F)), 0))


def make_theory():
    zs = np.linspace(-600, 600, 50)
    crlb = np.array([theory_crlb(z) for z in zs])
    psf = np.array([THEORY["sigma0"], THEORY["sigma0"], THEORY["Ax"], THEORY["Ay"],
                    THEORY["Bx"], THEORY["By"], THEORY["gamma"], THEORY["d"]], np.float32)
    theta = np.array([[THEORY["x"], THEORY["y"], z, THEORY["N"], THEORY["bg"]] for z in zs])
    np.savez(HERE / "astig_theory_crlb.npz", z=zs, crlb=crlb, psf=psf, theta=theta,
             box=THEORY["box"])


GOLDEN_CASES = [("xynb-11-poisson", 0, 11, 0, 96), ("xynbs-13-scmos-adu", 1, 13, 2, 96),
                ("xynbsxsy-11-scmos-var", 2, 11, 1, 96), ("astig-15-poisson", 3, 15, 0, 96),
                ("xynb-7-poisson", 0, 7, 0, 64)]


def make_oracle_fixtures():
    from oracle import oracle as O
    from parity_cases import make_case, oracle_desc
    for name, model, box, cam, n in GOLDEN_CASES:
        w = make_case(name, model, box, cam, n, seed=777 + model, sensor=64)
        r = O.fit(oracle_desc(O, w), w.data, w.x_corners, w.y_corners, w.maps, "f32")
        maps = w.maps if w.maps is not None else (np.zeros((1, 1), np.float32),) * 3
        np.savez_compressed(HERE / f"oracle_{name}.npz", data=np.asfortranarray(w.data),
                            xc=w.x_corners, yc=w.y_corners, var=maps[0], gain=maps[1],
                            offset=maps[2], model=model, box=box, camera=cam,
                            psf=w.psf.psf_vector(), lower=w.constraints.lower,
                            upper=w.constraints.upper, max_step=w.constraints.max_step,
                            params=r["params"], crlb=r["crlb"], llr=r["llr"], flags=r["flags"])


if __name__ == "__main__":
    make_theory()
    make_oracle_fixtures()
    print("wrote", sorted(p.name for p in HERE.glob("*.npz")))
