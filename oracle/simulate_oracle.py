"""CPU restatement of the device ROI generator (gmle_simulate_device).

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker of the device
generator.  The product path never uses it.

The reference simulator (src/simulator.jl:228-307, `_generate_single_roi!`)
draws, per pixel (i, j) of a ROI, Poisson(mu) photo-electrons with
mu = bg + N psf_x(j) psf_y(i) (`_evaluate_psf_pixel`, src/simulator.jl:
312-346), and for an sCMOS camera adds Normal(0, readnoise) and converts to
ADU, total / gain + offset.  Its random streams (Julia's default RNG and
Distributions.jl's Poisson sampler) cannot be reproduced, so the device
generator defines its own, restated here draw for draw:

* random numbers: Philox4x32-10 (Salmon, Moraes, Dror and Shaw, "Parallel
  random numbers: as easy as 1, 2, 3", SC 2011), key = the 64-bit seed,
  counter = (pixel index p, ROI index low word, high word, block r); a
  32-bit word w gives the uniform (w + 0.5) / 2^32 in float64 or
  ((w >> 8) + 0.5) / 2^24 in float32, both exact;
* Poisson(lam): lam < 10 by inversion in float32 (sequential search of the
  CDF from exp(-lam)); lam >= 10 by Hormann's transformed rejection with
  squeeze in float64 (PTRS; W. Hormann, "The transformed rejection method
  for generating Poisson random variables", Insurance: Mathematics and
  Economics 12, 1993) in float32, but for the exact acceptance test at
  lam >= 64, in float64, with ln k! from a table below 10 and the Stirling
  series above; uniforms taken in order from blocks r = 0, 1, 2, ...;
  lam <= 0 gives 0 as in the reference;
* read noise: Box-Muller in float32, z = sqrt(-2 ln u1) cos(2 pi u2) from the
  first two words of block r = 0xFFFF, times sqrt(var);
* mu in float32 from erf-integrated 1-D Gaussians (src/gausslib/
  baselibrary.jl:8-14, with the astigmatic widths sigma0 sqrt(alpha(z -+
  gamma)), baselibrary.jl:75-83), then float32 arithmetic for the camera:
  (count + z sqrt(var)) / gain + offset.
Maps are indexed like the fitting kernel, row = y (the reference simulator
indexes its maps transposed, src/simulator.jl:292-304).
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf

M0, M1 = 0xD2511F53, 0xCD9E8D57
W0, W1 = 0x9E3779B9, 0xBB67AE85
MASK = 0xFFFFFFFF
NOISE_BLOCK = 0xFFFF


def philox4x32_10(ctr, key):
    """Philox4x32-10 of counters ctr (..., 4) uint32 with keys key (..., 2)."""
    c = [np.asarray(ctr[..., i], np.uint64) for i in range(4)]
    k0 = np.asarray(key[..., 0], np.uint64)
    k1 = np.asarray(key[..., 1], np.uint64)
    for _ in range(10):
        p0 = np.uint64(M0) * c[0]
        p1 = np.uint64(M1) * c[2]
        hi0, lo0 = p0 >> np.uint64(32), p0 & np.uint64(MASK)
        hi1, lo1 = p1 >> np.uint64(32), p1 & np.uint64(MASK)
        c = [hi1 ^ c[1] ^ k0, lo1, hi0 ^ c[3] ^ k1, lo0]
        k0 = (k0 + np.uint64(W0)) & np.uint64(MASK)
        k1 = (k1 + np.uint64(W1)) & np.uint64(MASK)
    return np.stack([x.astype(np.uint32) for x in c], axis=-1)


class _Stream:
    """The uniforms of one pixel: blocks r = 0, 1, ... of its counter."""

    def __init__(self, seed: int, roi: int, pixel: int):
        self.key = np.array([seed & MASK, (seed >> 32) & MASK], np.uint32)
        self.base = [pixel & MASK, roi & MASK, (roi >> 32) & MASK]
        self.r, self.words, self.i = 0, None, 4

    def block(self, r: int) -> np.ndarray:
        return philox4x32_10(np.array(self.base + [r], np.uint32), self.key)

    def word(self) -> int:
        if self.i == 4:
            self.words, self.i = self.block(self.r), 0
            self.r += 1
        w = int(self.words[self.i])
        self.i += 1
        return w

    def uniform(self) -> float:
        return (self.word() + 0.5) * 2.0 ** -32

    def uniform_f(self) -> np.float32:
        return np.float32((self.word() >> 8) + 0.5) * np.float32(2.0 ** -24)


_LOG_FACT = [0.0, 0.0, 0.6931471805599453, 1.791759469228055, 3.1780538303479458,
             4.787491742782046, 6.579251212010101, 8.525161361065415, 10.60460290274525,
             12.801827480081469]


def log_factorial(k, t):
    """ln k! in type t (float32 or float64): a table below 10, else the
    Stirling series (k + 1/2) ln(k + 1) - (k + 1) + ln(2 pi)/2 + 1/(12 (k + 1))
    - 1/(360 (k + 1)^3)."""
    if k < 10:
        return t(_LOG_FACT[int(k)])
    x = t(k) + t(1.0)
    rx = t(1.0) / x
    c = (t(0.0833333333) if t is np.float32 else t(0.083333333333333333),
         t(0.00277777778) if t is np.float32 else t(0.0027777777777777778),
         t(0.918938533) if t is np.float32 else t(0.9189385332046728))
    corr = rx * (c[0] - (rx * rx) * c[1])
    return (((t(k) + t(0.5)) * np.log(x)) - x + c[2]) + corr


def poisson(lam: float, s: _Stream) -> int:
    """One Poisson(lam) draw from the stream (inversion / PTRS)."""
    if not lam > 0.0:
        return 0
    if lam < 10.0:
        lf = np.float32(lam)
        u = s.uniform_f()
        p = np.exp(-lf)
        f = p
        k = 0
        while u > f and k < 1000:
            k += 1
            p = np.float32(p * np.float32(lf / np.float32(k)))
            f = np.float32(f + p)
        return k
    f32 = np.float32
    lf = f32(lam)
    slam = np.sqrt(lf)
    b = f32(0.931) + f32(2.53) * slam
    a = f32(-0.059) + f32(0.02483) * b
    invalpha = f32(1.1239) + f32(1.1328) / (b - f32(3.4))
    vr = f32(0.9277) - f32(3.6224) / (b - f32(2.0))
    ld = float(lf)
    loglam = np.log(ld) if lf >= f32(64.0) else 0.0
    loglamf = np.log(lf)
    for _ in range(10000):
        u = s.uniform_f() - f32(0.5)
        v = s.uniform_f()
        us = f32(0.5) - abs(u)
        k = np.floor(((f32(2.0) * a) / us + b) * u + lf + f32(0.43))
        if us >= f32(0.07) and v <= vr:
            return int(k)
        if k < 0 or (us < f32(0.013) and v > us):
            continue
        if lf < f32(64.0):
            lhs = (np.log(v) + np.log(invalpha)) - np.log(a / (us * us) + b)
            rhs = (-lf + k * loglamf) - log_factorial(k, f32)
        else:
            usd, kd = float(us), float(k)
            lhs = (np.log(float(v)) + np.log(float(invalpha))) - np.log(float(a) / (usd * usd) + float(b))
            rhs = (-ld + kd * loglam) - log_factorial(kd, np.float64)
        if lhs <= rhs:
            return int(k)
    return int(np.floor(np.float32(lam)))


def expectation64(model: int, psf, theta: np.ndarray, box: int) -> np.ndarray:
    """(box, box) float64 expectation of one ROI, [row i, column j]."""
    t = np.asarray(theta, np.float64)
    psf = np.asarray(psf, np.float64)
    if model == 3:
        x, y, z, n, bg = t[:5]
        sx0, sy0, ax, ay, bx, by, gam, d = psf[:8]
        def width(s0, u, a, b):
            # alpha = 1 + u^2 + A u^3 + B u^4 as explicit products, left to right
            u2 = u * u
            return s0 * np.sqrt(((1.0 + u2) + a * (u2 * u)) + b * (u2 * u2))
        sx = width(sx0, (z - gam) / d, ax, bx)
        sy = width(sy0, (z + gam) / d, ay, by)
    else:
        x, y, n, bg = t[:4]
        sx = sy = psf[0] if model == 0 else t[4]
        if model == 2:
            sy = t[5]
    idx = np.arange(1, box + 1, dtype=np.float64)

    def axis(c, s):
        k = 1.0 / (np.sqrt(2.0) * s)
        return 0.5 * (erf(((idx - c) + 0.5) * k) - erf(((idx - c) - 0.5) * k))
    # mu[i, j] = bg + N (psf_y[i] psf_x[j])
    return bg + n * np.outer(axis(y, sy), axis(x, sx))


def expectation32(model: int, psf, theta: np.ndarray, box: int) -> np.ndarray:
    """The generator's (box, box) float32 expectation of one ROI, [row i,
    column j]: expectation64's formula in float32, each operation rounded."""
    f = np.float32
    t = np.asarray(theta, np.float32)
    psf = np.asarray(psf, np.float32)
    if model == 3:
        x, y, z, n, bg = t[:5]
        sx0, sy0, ax, ay, bx, by, gam, d = psf[:8]

        def width(s0, u, a, b):
            u2 = u * u
            return s0 * np.sqrt(((f(1.0) + u2) + a * (u2 * u)) + b * (u2 * u2))
        sx = width(sx0, (z - gam) / d, ax, bx)
        sy = width(sy0, (z + gam) / d, ay, by)
    else:
        x, y, n, bg = t[:4]
        sx = sy = psf[0] if model == 0 else t[4]
        if model == 2:
            sy = t[5]
    idx = np.arange(1, box + 1, dtype=np.float32)

    def axis(c, s):
        k = f(1.0) / (f(1.41421356) * s)
        lo = erf(((idx - c) - f(0.5)) * k).astype(np.float32)
        hi = erf(((idx - c) + f(0.5)) * k).astype(np.float32)
        return (f(0.5) * (hi - lo)).astype(np.float32)
    return (bg + n * np.outer(axis(y, sy), axis(x, sx)).astype(np.float32)).astype(np.float32)


def simulate(model: int, box: int, camera: int, psf, truth: np.ndarray, seed: int,
             maps=None, xc=None, yc=None) -> np.ndarray:
    """(box, box, n) float32 ROIs, as the device generator writes them.
    truth is (n, P); maps (var, gain, offset) are (ny, nx) arrays indexed
    [row = y, column = x]; corners 1-based."""
    n = truth.shape[0]
    out = np.empty((box, box, n), np.float32, order="F")
    for k in range(n):
        mu = expectation32(model, psf, truth[k], box)
        for j in range(box):
            for i in range(box):
                p = i + box * j
                s = _Stream(seed, k, p)
                cnt = poisson(float(mu[i, j]), s)
                if camera == 0:
                    out[i, j, k] = np.float32(cnt)
                    continue
                var, gain, off = (m[yc[k] - 1 + i, xc[k] - 1 + j] for m in maps)
                w = s.block(NOISE_BLOCK)
                f32 = np.float32
                u1 = f32((int(w[0]) >> 8) + 0.5) * f32(2.0 ** -24)
                u2 = f32((int(w[1]) >> 8) + 0.5) * f32(2.0 ** -24)
                z = np.sqrt(f32(-2.0) * np.log(u1)) * np.cos(f32(6.28318530717958648) * u2)
                tot = np.float32(cnt) + z * np.sqrt(np.float32(var))
                out[i, j, k] = tot if camera == 1 else tot / np.float32(gain) + np.float32(off)
    return out
