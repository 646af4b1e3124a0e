"""The CPU restatement of the device ROI generator (oracle/simulate_oracle.py):
its Philox4x32-10 against the published known-answer vectors, and its Poisson
sampler (inversion below lam = 10, PTRS above) against the Poisson law."""
import numpy as np
import pytest

from oracle import simulate_oracle as S

# Known-answer vectors of Philox4x32-10 published with the Random123 library
# (counter words, key words -> output words).
KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF), (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,expect", KAT)
def test_philox_known_answers(ctr, key, expect):
    out = S.philox4x32_10(np.array(ctr, np.uint32), np.array(key, np.uint32))
    assert tuple(int(x) for x in out) == expect


@pytest.mark.parametrize("lam", [0.3, 3.0, 9.7, 10.2, 45.0, 800.0])
def test_poisson_sampler_follows_the_poisson_law(lam):
    """Mean, variance and a chi-square test of the histogram against the pmf."""
    from scipy import stats
    n = 4000
    draws = np.array([S.poisson(lam, S._Stream(77, k, 5)) for k in range(n)])
    se = np.sqrt(lam / n)
    assert abs(draws.mean() - lam) < 5 * se
    assert abs(draws.var() / lam - 1) < 5 * np.sqrt(2.0 / n) + 0.02
    lo, hi = int(stats.poisson.ppf(1e-3, lam)), int(stats.poisson.ppf(1 - 1e-3, lam))
    edges = np.arange(lo, hi + 2) - 0.5
    obs, _ = np.histogram(np.clip(draws, lo, hi), edges)
    pmf = stats.poisson.pmf(np.arange(lo, hi + 1), lam)
    pmf[0] += stats.poisson.cdf(lo - 1, lam)
    pmf[-1] += stats.poisson.sf(hi, lam)
    exp = n * pmf
    keep = exp >= 5  # pool the sparse tails
    o = np.append(obs[keep], obs[~keep].sum())
    e = np.append(exp[keep], exp[~keep].sum())
    if e[-1] == 0:
        o, e = o[:-1], e[:-1]
    chi2 = ((o - e) ** 2 / e).sum()
    assert stats.chi2.sf(chi2, len(o) - 1) > 1e-4


def test_stream_is_counter_based():
    """A pixel's draws depend only on (seed, ROI, pixel)."""
    a = [S._Stream(5, 123, 7).uniform() for _ in range(3)]
    b = [S._Stream(5, 123, 7).uniform() for _ in range(3)]
    c = S._Stream(6, 123, 7).uniform()
    assert a == b and c != a[0]
