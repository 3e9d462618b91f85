"""The learned start's equilibrium bookkeeping on the CPU (no GPU): the sweeps-to-equilibrium
test on synthetic relaxation curves, its two tolerances and its time axis, and the reference
statistics of long-chain samples."""
import numpy as np

from nanomagmc_gb300 import warmstart as W


def _ref(mean=(-1.0, 0.5, 10.0), sd=(0.01, 0.01, 2.0)):
    return {k: (mean[i], sd[i], sd[i] / 4) for i, k in enumerate("EMQ")}


def _rel(E, M, Q, t=None):
    return W.Relaxation(np.asarray(E, float), np.asarray(M, float), np.asarray(Q, float),
                        None if t is None else np.asarray(t))


def test_equilibrated_series_passes_at_once_with_the_spread():
    ref = _ref()
    n = 40
    rng = np.random.default_rng(1)
    # a 16-chain mean in equilibrium: spread sd / 4 around the mean
    E = -1.0 + rng.normal(0, 0.01 / 4, n)
    M = 0.5 + rng.normal(0, 0.01 / 4, n)
    Q = 10.0 + rng.normal(0, 2.0 / 4, n)
    assert W.sweeps_to_equilibrium(_rel(E, M, Q), ref, 16, every=10) == 0
    # the sigma-of-the-mean test on a series whose means sit 1.5 of those sigmas away: never
    off = _rel(E * 0 - 1.0 + 1.5 * 0.01 / 4, M * 0 + 0.5, Q * 0 + 10.0)
    assert W.sweeps_to_equilibrium(off, ref, 16, every=10, tol="mean") is None
    assert W.sweeps_to_equilibrium(off, ref, 16, every=10, tol="spread") == 0


def test_relaxing_series_and_time_axis():
    ref = _ref()
    t = np.array(list(range(0, 11)) + list(range(20, 101, 10)))
    E = -1.0 + 0.5 * np.exp(-t / 3.0)            # within 0.01 from t = 12 on
    M = np.full(len(t), 0.5)
    Q = np.full(len(t), 10.0)
    rel = _rel(E, M, Q, t)
    # the first measurement of five consecutive ones inside the band is t = 20
    assert W.sweeps_to_equilibrium(rel, ref, 16, every=10) == 20
    # without a time axis the index times `every` is the answer
    assert W.sweeps_to_equilibrium(_rel(E, M, Q), ref, 16, every=10) == 110
    # a series that leaves the band again within five measurements starts over after the exit
    E2 = E.copy()
    E2[13] = -0.9                                # t = 40
    assert W.sweeps_to_equilibrium(_rel(E2, M, Q, t), ref, 16) == 50


def test_reference_stats_of_samples():
    rng = np.random.default_rng(2)
    v = np.stack([rng.normal(-1.0, 0.01, (400, 16)), rng.normal(0.5, 0.02, (400, 16)),
                  rng.normal(10.0, 2.0, (400, 16))], -1)
    ref = W.reference_stats(v)
    for i, k in enumerate("EMQ"):
        mean, sd, se = ref[k]
        assert abs(mean - v[..., i].mean()) < 1e-12
        assert abs(sd - v[..., i].std(ddof=1)) < 1e-12
        # standard error of the grand mean from the 16 per-chain averages
        m = v[..., i].mean(0)
        assert abs(se - m.std(ddof=1) / 4) < 1e-12
