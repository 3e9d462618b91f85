"""Distribution tests of the random streams, in the reference's chi-squared form.

The reference tests its generators by binning draws and comparing bin counts with their
expectations through a reduced chi-squared (Old/tests/rand_test.hpp:17-30): a binomial test
of the {0,1} integer stream (100 tosses per trial, binned by |#zeros - 50|, :46-68), 100
uniform bins of the double stream (:70-82), a log-normal(0, 0.25) histogram truncated at 2
(:84-104) and unit length of the sphere stream (:106-117). The same statistics are applied
here to

  * the oracle's restatement of the reference's three MT19937 generators, at the reference's
    sample sizes, and
  * the counter-based Philox stream that every sweep kernel draws from: the 23-bit uniforms
    that the Metropolis test and the sphere proposal use, their joint distribution across
    the four words of one draw, across consecutive sweeps of one site and across chains.

The reference bounds the reduced chi-squared (0.9 < chi2/dof < 1.3 or 1.8); that band's false
failure rate depends on the number of bins. These tests bound the two-sided tail probability
of the chi-squared statistic instead (1e-4 on either side), after merging the bins whose
expectation is below 5, and also report the reduced value. Seeds are fixed, so the results
are deterministic.
"""
import math

import numpy as np
import pytest
from scipy import stats as S

from oracle import oracle as O

P_LO = 1e-4


def chi2_check(count, expect, what):
    """Merges low-expectation bins, then bounds the chi-squared tail probability on both sides."""
    count = np.asarray(count, float)
    expect = np.asarray(expect, float)
    assert abs(count.sum() - expect.sum()) <= 1e-6 * count.sum(), (what, count.sum(), expect.sum())
    keep = expect >= 5
    c = np.append(count[keep], count[~keep].sum())
    e = np.append(expect[keep], expect[~keep].sum())
    if e[-1] < 5:        # fold a small remainder into the smallest kept bin
        j = int(np.argmin(e[:-1]))
        c[j] += c[-1]
        e[j] += e[-1]
        c, e = c[:-1], e[:-1]
    x2 = float(((c - e) ** 2 / e).sum())
    dof = len(c) - 1
    p = S.chi2.sf(x2, dof)
    assert P_LO < p < 1 - P_LO, "%s: chi2/dof = %.3f over %d dof, p = %.2e" % (what, x2 / dof, dof, p)
    return x2 / dof


def test_int_stream_binomial():
    """1e6 trials of 100 {0,1} draws; P(|#0 - 50| = k) = C(100, 50+k) 2^-100 (x2 for k > 0)."""
    r = O.Rng(11, 12, 13)
    ntoss, ntrial, chunk = 100, 1_000_000, 100_000
    counts = np.zeros(ntoss // 2 + 1)
    for _ in range(ntrial // chunk):
        zeros = (r.fill("int2", ntoss * chunk).reshape(chunk, ntoss) == 0).sum(1)
        counts += np.bincount(np.abs(zeros - ntoss // 2), minlength=len(counts))
    k = np.arange(len(counts))
    expect = np.array([math.comb(ntoss, ntoss // 2 + int(i)) for i in k], float) * 2.0 ** -ntoss
    expect[1:] *= 2
    chi2_check(counts, expect * ntrial, "int2 binomial")


def test_double_stream_uniform():
    """1e8 draws of the double stream in 100 equal bins."""
    r = O.Rng(11, 12, 13)
    nbin, chunk = 100, 10_000_000
    counts = np.zeros(nbin)
    for _ in range(10):
        u = r.fill("uniform", chunk)
        assert u.min() >= 0 and u.max() < 1
        counts += np.bincount((u * nbin).astype(np.int64), minlength=nbin)
    chi2_check(counts, np.full(nbin, 1e8 / nbin), "uniform")


def test_lognormal_histogram():
    """1e6 log-normal(0, 0.25) draws below 2 in bins of width 0.02 against the CDF."""
    r = O.Rng(11, 12, 13)
    x = r.fill("lognormal", 1_100_000, 0.0, 0.25)
    assert np.all(x > 0)
    x = x[x < 2.0][:1_000_000]
    assert len(x) == 1_000_000
    nbin = 100
    counts = np.bincount((x * (nbin / 2.0)).astype(np.int64), minlength=nbin)
    edges = np.arange(nbin + 1) * (2.0 / nbin)
    cdf = S.norm.cdf(np.log(np.maximum(edges, 1e-300)) / 0.25)
    cdf[0] = 0.0
    expect = np.diff(cdf) / cdf[-1] * len(x)
    chi2_check(counts, expect, "lognormal")
    assert abs(np.log(x).mean()) < 5e-3


def test_sphere_stream_unit_and_uniform():
    """1e6 directions: unit length, z uniform on (-1,1), azimuth uniform, (z, phi) jointly uniform."""
    r = O.Rng(11, 12, 20)
    v = r.fill("dir3d", 1_000_000)
    assert np.abs((v * v).sum(1) - 1).max() < 1e-12
    zb = np.minimum(((v[:, 2] + 1) * 10).astype(np.int64), 19)
    pb = np.minimum(((np.arctan2(v[:, 1], v[:, 0]) + np.pi) / (2 * np.pi) * 20).astype(np.int64), 19)
    n = len(v)
    chi2_check(np.bincount(zb, minlength=20), np.full(20, n / 20), "dir3d z")
    chi2_check(np.bincount(pb, minlength=20), np.full(20, n / 20), "dir3d phi")
    chi2_check(np.bincount(zb * 20 + pb, minlength=400), np.full(400, n / 400), "dir3d (z, phi)")


# ---------------------------------------------------------------------------------------------
# The sweep kernels' Philox stream
# ---------------------------------------------------------------------------------------------

SEED = 0x5EED1234ABCD


def u01f(w):
    """The kernels' uniform: (top 23 bits + 1/2) 2^-23, in (0, 1)."""
    return ((w >> 9).astype(np.float64) + 0.5) * 2.0 ** -23


@pytest.fixture(scope="module")
def sweep_words():
    return O.philox_boxes(SEED, 3, 17, 1 << 22)


def test_philox_words_uniform(sweep_words):
    """Each of the four words of a draw: 100 equal bins of its 23-bit uniform, and bit 31."""
    n = len(sweep_words)
    for k in range(4):
        u = u01f(sweep_words[:, k])
        assert u.min() > 0 and u.max() < 1
        chi2_check(np.bincount((u * 100).astype(np.int64), minlength=100), np.full(100, n / 100),
                   "philox word %d" % k)
        ones = int((sweep_words[:, k] >> 31).sum())
        assert abs(ones - n / 2) < 4.5 * math.sqrt(n / 4), (k, ones)    # the Ising proposal bit


@pytest.mark.parametrize("a,b", [(0, 1), (0, 2), (1, 2), (2, 3)])
def test_philox_word_pairs_independent(sweep_words, a, b):
    """Joint 32 x 32 histogram of two words of one draw (proposal z and phi, acceptance u)."""
    ia = (u01f(sweep_words[:, a]) * 32).astype(np.int64)
    ib = (u01f(sweep_words[:, b]) * 32).astype(np.int64)
    n = len(sweep_words)
    chi2_check(np.bincount(ia * 32 + ib, minlength=1024), np.full(1024, n / 1024), "words %d,%d" % (a, b))


def test_philox_consecutive_sweeps_and_chains_independent():
    """The same site in consecutive sweeps, and in neighbouring chains, draws independent words."""
    n = 1 << 20
    base = O.philox_boxes(SEED, 3, 17, n)
    for other, what in ((O.philox_boxes(SEED, 3, 18, n), "sweep+1"),
                        (O.philox_boxes(SEED, 4, 17, n), "chain+1"),
                        (O.philox_boxes(SEED, 3, 17, n, stream=2), "mask stream")):
        ia = (u01f(base[:, 2]) * 32).astype(np.int64)
        ib = (u01f(other[:, 2]) * 32).astype(np.int64)
        chi2_check(np.bincount(ia * 32 + ib, minlength=1024), np.full(1024, n / 1024), what)
        assert abs(np.corrcoef(u01f(base[:, 0]), u01f(other[:, 0]))[0, 1]) < 5 / math.sqrt(n)


def test_sphere_proposal_uniform_on_the_sphere(sweep_words):
    """The kernels' proposal (z = 2u0 - 1, phi = pi (2u1 - 1)) covers S^2 uniformly: z and phi
    equal-area bins, jointly, and the mean direction is zero."""
    z = 2 * u01f(sweep_words[:, 0]) - 1
    phi = np.pi * (2 * u01f(sweep_words[:, 1]) - 1)
    rxy = np.sqrt(np.maximum(0, 1 - z * z))
    v = np.stack([rxy * np.cos(phi), rxy * np.sin(phi), z], 1)
    n = len(v)
    assert np.all(np.abs(v.mean(0)) < 5 / math.sqrt(3 * n))
    zb = np.minimum(((z + 1) * 10).astype(np.int64), 19)
    pb = np.minimum(((phi + np.pi) / (2 * np.pi) * 20).astype(np.int64), 19)
    chi2_check(np.bincount(zb * 20 + pb, minlength=400), np.full(400, n / 400), "proposal (z, phi)")
    # second moments of a uniform direction: <x^2> = <y^2> = <z^2> = 1/3
    assert np.all(np.abs((v * v).mean(0) - 1 / 3) < 5 * math.sqrt(4 / 45 / n))


def test_metropolis_acceptance_rate():
    """P(u < exp(-b dE)) from the acceptance word equals exp(-b dE) within binomial error."""
    n = 1 << 21
    u = u01f(O.philox_boxes(SEED, 7, 1, n)[:, 2])
    for x in (0.05, 0.5, 1.0, 2.0, 4.0, 8.0):
        p = math.exp(-x)
        acc = int((np.log(u) < -x).sum())
        assert abs(acc - n * p) < 5 * math.sqrt(n * p * (1 - p)) + 1, (x, acc / n, p)
