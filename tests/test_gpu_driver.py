"""The protocol driver (nmmc_run, the program of Old/lib/main.cpp) on a small input:
output arrays with the shapes of Old/lib/output.cpp:161-249, /Complete flags, resume."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from nanomagmc_gb300 import _lib as L
from nanomagmc_gb300.build import RUN

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

INPUT = """ISISING {ising}
EXCHANGE 1
DMISTREN {dmi}
ISDISTRIB {distrib}
SIZE 8
MEANSIZE 6
SIZEDEV 1.5
LATTSHAPE {shape}
WEIBULLFACT 3
NLATTS 2
BOLTZMANN 1
ISPERIO {perio}
SAMPSWEEPS 2
EQSWEEPS 10
NSAMPS 5
TEMPNAME t.dat
FIELDNAME h.dat
PROTOCOL {proto}
INTERACTIONS {jfile}
"""


def workdir(tmp_path, **kw):
    (tmp_path / "Temps").mkdir()
    (tmp_path / "Fields").mkdir()
    (tmp_path / "Js").mkdir()
    (tmp_path / "Temps" / "t.dat").write_text("1.5 1.0 0.5\n")
    (tmp_path / "Fields" / "h.dat").write_text("0.0 0.4\n")
    shutil.copy(os.path.join(ROOT, "data", "Js", kw["jfile"]), tmp_path / "Js" / kw["jfile"])
    (tmp_path / "INPUT.dat").write_text(INPUT.format(**kw))
    return tmp_path


def run(wd, out, seed=3):
    lib = L.load()
    return lib.nmmc_run(str(wd / "INPUT.dat").encode(), str(wd).encode(), str(out).encode(), seed, 0)


@pytest.mark.parametrize("proto", [1, 2, 4])
def test_heisenberg_protocols(tmp_path, proto):
    wd = workdir(tmp_path, ising=0, dmi=0.5, distrib=0, shape="s", perio=1, proto=proto,
                 jfile="2d_nn_interfacial.dat")
    out = tmp_path / "Output"
    assert run(wd, out) == 0
    nH, nT, NS, NL = 2, 3, 5, 2
    for name in ("mags", "energies", "sub_mags", "sub4_mags", "mag_xs", "mag_ys", "mag_zs",
                 "sub_mag_xs", "sub4_mag_zs"):
        a = np.load(out / (name + ".npy"))
        assert a.shape == (nH, nT, NS * NL) and a.dtype == np.float32
        assert np.all(np.isfinite(a)) and np.any(a != 0)
    q = np.load(out / "top_chars.npy")
    assert q.shape == (nH, nT, 1, NS * NL)
    m = np.load(out / "mags.npy")
    mx, my, mz = (np.load(out / (n + ".npy")) for n in ("mag_xs", "mag_ys", "mag_zs"))
    assert np.allclose(m, np.sqrt(mx ** 2 + my ** 2 + mz ** 2), rtol=1e-5, atol=1e-4)
    assert np.all(np.abs(m) <= 64 + 1e-3)
    nv1 = nH if proto == 1 else nT
    assert np.array_equal(np.load(out / "complete.npy"), np.ones((nv1, NL), np.int32))
    assert np.allclose(np.load(out / "Ts.npy"), [1.5, 1.0, 0.5])
    # /Av_Latt and /Sing_Latt of lattice 0 at every (T, H) point (x slowest, 3 components)
    for t in range(nT):
        for h in range(nH):
            av = np.load(out / "Av_Latt" / ("T_%d-H_%d.npy" % (t, h)))
            sg = np.load(out / "Sing_Latt" / ("T_%d-H_%d.npy" % (t, h)))
            assert av.shape == sg.shape == (8, 8, 3) and av.dtype == np.float32
            assert np.allclose(np.linalg.norm(sg, axis=-1), 1, atol=1e-5)   # unit spins
            assert np.all(np.linalg.norm(av, axis=-1) <= NS + 1e-4)         # sum of NS samples
            assert np.any(np.linalg.norm(av, axis=-1) > 1.5)
    # a rerun finds every (v1, lattice) complete and leaves the samples untouched
    before = np.load(out / "energies.npy")
    assert run(wd, out) == 0
    assert np.array_equal(np.load(out / "energies.npy"), before)


def test_ising_weibull_distrib(tmp_path):
    wd = workdir(tmp_path, ising=1, dmi=0.0, distrib=1, shape="w", perio=0, proto=1, jfile="2d_nn.dat")
    out = tmp_path / "Output"
    assert run(wd, out) == 0
    e = np.load(out / "energies.npy")
    assert e.shape == (2, 3, 10) and np.all(np.isfinite(e))
    assert not os.path.exists(out / "top_chars.npy")     # Ising / distributed sizes: no Q
    assert not os.path.exists(out / "mag_xs.npy")


def test_cli_and_error_codes(tmp_path):
    wd = workdir(tmp_path, ising=0, dmi=0.5, distrib=0, shape="s", perio=1, proto=3,
                 jfile="2d_nn_interfacial.dat")
    r = subprocess.run([RUN, "INPUT.dat", "out"], cwd=wd, capture_output=True, text=True)
    assert r.returncode == 207 % 256 and "protocol" in r.stderr.lower()
    (wd / "INPUT.dat").write_text(INPUT.format(ising=0, dmi=0.5, distrib=0, shape="s", perio=1, proto=1,
                                               jfile="2d_nn_interfacial.dat").replace("LATTSHAPE s", "LATTSHAPE q"))
    r = subprocess.run([RUN, "INPUT.dat", "out"], cwd=wd, capture_output=True, text=True)
    assert r.returncode == 103
    (wd / "INPUT.dat").write_text(INPUT.format(ising=0, dmi=0.5, distrib=0, shape="s", perio=1, proto=1,
                                               jfile="2d_nn_interfacial.dat"))
    r = subprocess.run([RUN, "INPUT.dat", "out"], cwd=wd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert os.path.exists(wd / "out" / "energies.npy")


def test_partial_resume_recomputes_only_unfinished_pairs(tmp_path):
    """A run whose /Complete flags mark one (v1, lattice) pair unfinished redoes only that
    pair: the base chains are rebuilt deterministically and the pair's inner chain walks the
    same Philox counters again, so its samples return (to FP32 rounding: other chains share
    its kernel launches) and every other sample is left untouched. Arrays of another run's
    shape are ignored and the whole run is redone."""
    wd = workdir(tmp_path, ising=0, dmi=0.5, distrib=0, shape="s", perio=1, proto=1,
                 jfile="2d_nn_interfacial.dat")
    out = tmp_path / "Output"
    assert run(wd, out) == 0
    names = ("energies", "mags", "mag_zs", "sub4_mags")
    full = {n: np.load(out / (n + ".npy")) for n in names}
    NS = 5
    comp = np.load(out / "complete.npy")
    assert comp.shape == (2, 2)           # protocol 1: v1 = field (2 values) x 2 lattices
    comp[1, 0] = 0
    np.save(out / "complete.npy", comp)
    blk = np.zeros(full["energies"].shape, bool)
    blk[1, :, 0:NS] = True                # v1 = 1, lattice 0: all temperatures, its NS samples
    for n in names:
        a = full[n].copy()
        a[blk] = 0.0
        np.save(out / (n + ".npy"), a)
    assert run(wd, out) == 0
    assert np.array_equal(np.load(out / "complete.npy"), np.ones((2, 2), np.int32))
    for n in names:
        got = np.load(out / (n + ".npy"))
        assert np.array_equal(got[~blk], full[n][~blk]), n
        assert np.allclose(got[blk], full[n][blk], rtol=1e-5, atol=1e-4), (n, np.abs(got[blk] - full[n][blk]).max())
    # a sample array of another shape: flags are not trusted, everything is recomputed
    np.save(out / "energies.npy", np.zeros((3, 3), np.float32))
    assert run(wd, out) == 0
    e = np.load(out / "energies.npy")
    assert e.shape == full["energies"].shape
    assert np.allclose(e, full["energies"], rtol=1e-5, atol=1e-4)


# ---- output slots against an analytic model ------------------------------------------------
# With EXCHANGE 0 and DMISTREN 0 every spin feels only the field, so each sample's
# magnetisation along the field has a closed-form mean at its own (H, T) point: N L(H/T) for
# Heisenberg spins (Langevin, <s_z> = coth x - 1/x) and N tanh(H/T) for Ising spins. A sample
# written to the wrong [H, T] slot, or a lattice's samples to another lattice's block, moves
# the slot's mean by many standard errors.
ZEEMAN_TS, ZEEMAN_HS = [2.0, 1.0, 0.5], [0.0, 0.3, 0.9, 0.6]


def langevin(x):
    x = np.asarray(x, float)
    out = np.zeros_like(x)
    nz = np.abs(x) > 1e-6
    out[nz] = 1.0 / np.tanh(x[nz]) - 1.0 / x[nz]
    return out


def zeeman_workdir(tmp_path, ising, shape, perio, proto, jfile, nlatts, nsamp):
    (tmp_path / "Temps").mkdir()
    (tmp_path / "Fields").mkdir()
    (tmp_path / "Js").mkdir()
    (tmp_path / "Temps" / "t.dat").write_text(" ".join(map(str, ZEEMAN_TS)) + "\n")
    (tmp_path / "Fields" / "h.dat").write_text(" ".join(map(str, ZEEMAN_HS)) + "\n")
    shutil.copy(os.path.join(ROOT, "data", "Js", jfile), tmp_path / "Js" / jfile)
    text = (INPUT.format(ising=ising, dmi=0, distrib=0, shape=shape, perio=perio, proto=proto, jfile=jfile)
            .replace("EXCHANGE 1", "EXCHANGE 0").replace("NLATTS 2", "NLATTS %d" % nlatts)
            .replace("NSAMPS 5", "NSAMPS %d" % nsamp))
    (tmp_path / "INPUT.dat").write_text(text)
    return tmp_path


def lattice_sites(wd, seed, nlatts):
    """Filled sites of each lattice, from the options nmmc_run reads and the same shape draw."""
    lib = L.load()
    opt = L.Options()
    L.check(lib.nmmc_read_input(str(wd / "INPUT.dat").encode(), C.byref(opt)))
    edge = int(opt.edge_size)
    dim = 3 if opt.shape_code in b"cCxX" else 2
    mask = np.zeros(edge ** dim, np.uint8)
    out = []
    for k in range(nlatts):
        num = C.c_int()
        L.check(lib.nmmc_shape_mask(opt.shape_code, edge, opt.amean, opt.beta_w, seed, k,
                                    mask.ctypes.data_as(C.c_void_p), C.byref(num), None, None))
        out.append(num.value)
    return np.array(out)


@pytest.mark.parametrize("proto", [1, 2, 4])
@pytest.mark.parametrize("kind", ["heisenberg", "ising"])
def test_protocol_slots_match_their_points(tmp_path, proto, kind):
    from scipy.stats import norm

    from stats import binned_error
    ising = kind == "ising"
    nl, ns, seed = 3, 400, 3
    if ising:
        wd = zeeman_workdir(tmp_path, 1, "s", 1, proto, "2d_nn.dat", nl, ns)
    else:   # Weibull grains: every lattice its own number of filled sites
        wd = zeeman_workdir(tmp_path, 0, "w", 0, proto, "2d_nn_interfacial.dat", nl, ns)
    out = tmp_path / "Output"
    assert run(wd, out, seed=seed) == 0
    nsites = lattice_sites(wd, seed, nl)
    if not ising:
        assert len(set(nsites)) == nl, nsites            # the blocks are distinguishable
    # the lists in file order; /Complete is [v1, lattice] with v1 = H for protocol 1, T otherwise
    assert np.allclose(np.load(out / "Ts.npy"), ZEEMAN_TS) and np.allclose(np.load(out / "Hs.npy"), ZEEMAN_HS)
    nv1 = len(ZEEMAN_HS) if proto == 1 else len(ZEEMAN_TS)
    assert np.array_equal(np.load(out / "complete.npy"), np.ones((nv1, nl), np.int32))
    e = np.load(out / "energies.npy").astype(np.float64)
    # the magnetisation along the field: mag_zs (Heisenberg); from E = -H M (Ising, whose
    # mags.npy holds |M|), so the zero-field column has no signed value there
    mz = e * 0.0 if ising else np.load(out / "mag_zs.npy").astype(np.float64)
    assert e.shape == (len(ZEEMAN_HS), len(ZEEMAN_TS), ns * nl)
    # 3 sigma for the family of slots compared (two-sided tail 0.0027 split over the slots)
    nslots = (len(ZEEMAN_HS) - int(ising)) * len(ZEEMAN_TS) * nl
    zmax = norm.isf(0.0027 / 2 / nslots)
    worst = 0.0
    for hi, H in enumerate(ZEEMAN_HS):
        if ising and H == 0.0:
            continue
        for ti, T in enumerate(ZEEMAN_TS):
            per = np.tanh(H / T) if ising else float(langevin(H / T))
            for k in range(nl):
                sl = slice(k * ns, (k + 1) * ns)
                blk = -e[hi, ti, sl] / H if ising else mz[hi, ti, sl]
                if not ising:   # Zeeman energy of the same samples (FP32 storage)
                    assert np.allclose(e[hi, ti, sl], -H * blk, rtol=1e-5, atol=1e-3)
                mean, err = blk.mean(), binned_error(blk)
                dev = abs(mean - nsites[k] * per) / err
                worst = max(worst, dev)
                assert dev <= zmax, (kind, proto, H, T, k, mean, nsites[k] * per, err, zmax)
    print("largest slot deviation: %.2f sigma (bound %.2f for %d slots)" % (worst, zmax, nslots))
