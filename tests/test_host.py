"""Host-side behaviour of libnmmc without a GPU: input keys and error codes
(Old/lib/param_read.cpp), list loading, the interaction reader, protocol plans
(Old/lib/protocol.cpp), particle shapes and sizes, and the binning statistics."""
import ctypes as C
import os

import numpy as np
import pytest

from nanomagmc_gb300 import _lib as L
from nanomagmc_gb300.sampler import interactions_file, load_lists, read_input, read_interactions
from oracle import oracle as O

INPUT = """ISDISTRIB 1
MEANSIZE 20
SIZEDEV 5
BOLTZMANN 1
ISPERIO 0
LATTSHAPE w
WEIBULLFACT 3
NLATTS 4
NSAMPS 10
EQSWEEPS 200
SAMPSWEEPS 5
EXCHANGE 1
DMISTREN 0.5
TEMPNAME t.dat
FIELDNAME h.dat
INTERACTIONS 2d_nn_interfacial.dat
PROTOCOL 1
ISISING 0
"""


def write_input(tmp_path, text=INPUT, T="1.5 1.0 0.5", H="0 0.5 1"):
    (tmp_path / "Temps").mkdir(exist_ok=True)
    (tmp_path / "Fields").mkdir(exist_ok=True)
    (tmp_path / "Temps" / "t.dat").write_text(T)
    (tmp_path / "Fields" / "h.dat").write_text(H)
    p = tmp_path / "INPUT.dat"
    p.write_text(text)
    return str(p)


def test_read_input_keys(tmp_path):
    o = read_input(write_input(tmp_path))
    assert o.is_ising == 0 and o.distrib == 1 and o.shape_code == b"w"
    assert o.amean == 20 and o.asd == 5 and o.beta_w == 3
    assert o.edge_size == (20 + 2 * 5) * 3          # param_read.cpp:62
    assert o.n_latts == 4 and o.n_samp == 10 and o.eq_sweeps == 200 and o.samp_sweeps == 5
    assert o.J == 1 and o.K == 0.5 and o.protocol == 1 and o.is_perio == 0
    assert o.int_file == b"2d_nn_interfacial.dat"
    # AtoLn (functions.cpp:56-62)
    av, am2 = 25.0, 400.0
    assert o.lmean == pytest.approx(np.log(am2 / np.sqrt(av + am2)))
    assert o.lsd == pytest.approx(np.sqrt(np.log(1 + av / am2)))


def test_square_edge_and_first_match_wins(tmp_path):
    text = INPUT.replace("ISDISTRIB 1", "ISDISTRIB 0\nSIZE 24").replace("LATTSHAPE w", "LATTSHAPE s")
    text += "SIZE 99\n"
    o = read_input(write_input(tmp_path, text))
    assert o.edge_size == 24 and o.amean == 24


@pytest.mark.parametrize("key", ["ISISING", "EXCHANGE", "LATTSHAPE", "NLATTS", "PROTOCOL", "INTERACTIONS"])
def test_missing_key_is_105(tmp_path, key):
    text = "\n".join(l for l in INPUT.splitlines() if not l.startswith(key + " "))
    with pytest.raises(L.NmmcError) as e:
        read_input(write_input(tmp_path, text))
    assert e.value.code == 105 and key in str(e.value)


def test_missing_file_is_105(tmp_path):
    with pytest.raises(L.NmmcError) as e:
        read_input(str(tmp_path / "nope.dat"))
    assert e.value.code == 105


def test_load_lists_float_storage(tmp_path):
    o = read_input(write_input(tmp_path, T="2.6 2.55 0.1"))
    T, H = load_lists(o, str(tmp_path))
    assert np.array_equal(T, np.float32([2.6, 2.55, 0.1]).astype(float))
    assert np.array_equal(H, [0, 0.5, 1])


def test_interaction_reader_matches_oracle():
    for name, dim in [("3d_nn_bloch.dat", 3), ("2d_nn_interfacial.dat", 2), ("2d_nn.dat", 2)]:
        it = read_interactions(interactions_file(name), dim, 1.5, 0.3)
        off, J, D = O.read_interactions(interactions_file(name), dim, 1.5, 0.3)
        assert it.n == len(J)
        for r in range(it.n):
            assert list(it.offset[r]) == list(off[r])
            assert it.J[r] == J[r]
            assert list(it.D[r]) == list(D[r])


def test_3d_file_read_as_2d_desynchronises_like_the_reference():
    """A 2-D read of the 7-column file takes 2 ints per record (field_type.cpp:54-59)."""
    it = read_interactions(interactions_file("3d_nn_bloch.dat"), 2, 1.0, 1.0)
    off, J, D = O.read_interactions(interactions_file("3d_nn_bloch.dat"), 2, 1.0, 1.0)
    assert it.n == len(J) and it.n != 6


def plan(proto, nH=3, nT=4):
    out = [C.c_int() for _ in range(7)]
    rc = L.load().nmmc_protocol_plan(proto, nH, nT, *[C.byref(x) for x in out])
    return rc, [x.value for x in out]


def test_protocol_plans():
    assert plan(1) == (0, [0, 0, 3, 1, 0, 4, 1])      # v1 = H forward, v2 = T forward
    assert plan(2) == (0, [1, 0, 4, 1, 0, 3, 1])      # v1 = T, v2 = H
    assert plan(4) == (0, [1, 0, 4, 1, 2, -1, -1])    # v2 = H reversed (protocol.cpp:44-54)
    assert plan(3)[0] == 207 and plan(7)[0] == 207


def shape_mask(shape, edge, size, wbeta, seed, lattice):
    dim = 3 if shape in "cCxX" else 2
    m = np.zeros(edge ** dim, np.uint8)
    n, s, s4 = C.c_int(), C.c_int(), C.c_int()
    L.check(L.load().nmmc_shape_mask(shape.encode(), edge, size, wbeta, seed, lattice,
                                     m.ctypes.data_as(C.c_void_p), C.byref(n), C.byref(s), C.byref(s4)))
    return m, (n.value, s.value, s4.value)


@pytest.mark.parametrize("shape,edge,size", [("w", 45, 10.0), ("w", 31, 7.5), ("x", 15, 4.0)])
def test_weibull_masks_match_oracle(shape, edge, size):
    dim = 3 if shape == "x" else 2
    jf = "3d_nn_bloch.dat" if dim == 3 else "2d_nn.dat"
    off, J, D = O.read_interactions(interactions_file(jf), dim, 1.0, 0.0)
    for lattice in range(3):
        m, counts = shape_mask(shape, edge, size, 3.0, 1234, lattice)
        o = O.Lattice.create(dim, edge, False, False, shape, off, J, D, size=size, wbeta=3.0,
                             seed=1234, chain=lattice)
        locs = o.locs()
        box = locs[:, 0] + edge * (locs[:, 1] + edge * locs[:, 2])
        ref = np.zeros_like(m)
        ref[box] = 1
        assert np.array_equal(m, ref)
        assert counts == (o.n, o.snum, o.s4num)


def test_weibull_mean_filled_sites():
    """Expected filled sites of a 2-D Weibull disc with beta = 3: 2 pi (a r0)^2 Gamma(2/3)/3."""
    from math import gamma, pi
    a = 20.0
    r0 = 1 / gamma(1 + 1 / 3)
    expect = 2 * pi * (a * r0) ** 2 * gamma(2 / 3) / 3
    n = [shape_mask("w", 90, a, 3.0, 99, k)[1][0] for k in range(20)]
    assert abs(np.mean(n) - expect) < 0.02 * expect


def test_chain_count_limit_refused_before_device_work():
    """A context holds at most NMMC_MAX_CHAINS chains (the launches put the chain list on
    grid.y); one more is refused with 300 before any device call, so also without a GPU."""
    from nanomagmc_gb300.sampler import Sampler, make_options
    inter = read_interactions(interactions_file("2d_nn.dat"), 2)
    with pytest.raises(L.NmmcError) as e:
        Sampler(make_options("s", edge=4), inter, T=np.ones(L.MAX_CHAINS + 1))
    assert e.value.code == 300
    assert "at most 65535" in str(e.value)


def test_bad_shape_is_103():
    m = np.zeros(100, np.uint8)
    rc = L.load().nmmc_shape_mask(b"q", 10, 1.0, 3.0, 0, 0, m.ctypes.data_as(C.c_void_p), None, None, None)
    assert rc == 103


def test_lognormal_sizes():
    am, asd = 20.0, 5.0
    av, am2 = asd ** 2, am ** 2
    lm, ls = np.log(am2 / np.sqrt(av + am2)), np.sqrt(np.log(1 + av / am2))
    s = np.array([L.load().nmmc_lognormal_size(7, k, lm, ls) for k in range(20000)])
    assert abs(s.mean() - am) < 0.2 and abs(s.std() - asd) < 0.2


def binning(x):
    m, e, t = C.c_double(), C.c_double(), C.c_double()
    x = np.ascontiguousarray(x, float)
    L.check(L.load().nmmc_binning(x.ctypes.data_as(C.c_void_p), len(x), C.byref(m), C.byref(e), C.byref(t)))
    return m.value, e.value, t.value


def test_binning_white_noise_and_ar1():
    rng = np.random.default_rng(0)
    x = rng.normal(size=1 << 14)
    m, e, t = binning(x)
    assert abs(e - 1 / np.sqrt(len(x))) < 0.25 / np.sqrt(len(x)) and t < 1.0
    # AR(1) with phi = 0.9: tau_int = (1+phi)/(2(1-phi)) = 9.5
    y = np.zeros(1 << 16)
    for i in range(1, len(y)):
        y[i] = 0.9 * y[i - 1] + rng.normal()
    m, e, t = binning(y)
    assert 6 < t < 13
