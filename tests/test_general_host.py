"""Host side of general interaction tables (no GPU): the reader keeps every record in file
order beyond the old 64-record limit, and every colouring nmmc_colouring returns is a valid
parallel update order (no two sites of one colour class interact through any coupling record,
and the period divides a periodic edge)."""
import ctypes as C
import itertools

import numpy as np
import pytest

from nanomagmc_gb300 import _lib as L
from nanomagmc_gb300.sampler import interactions_file, read_interactions

from general_tables import coupling_offsets, write_table


def colouring(inter, dim, edge, periodic, ising=False):
    out = (C.c_int * 5)()
    L.check(L.load().nmmc_colouring(dim, edge, int(periodic), int(ising), C.byref(inter), out))
    return list(out)


def colour_of(col, x, y, z):
    kind, q, p, b, c = col
    if kind == 1:
        return (x + b * y + c * z) % q
    return x % p + p * (y % p) + p * p * (z % p)


def check_valid(col, offsets, dim, edge, periodic):
    kind, q, p, b, c = col
    assert kind in (1, 2) and 2 <= q <= 4096
    if periodic:
        assert edge % p == 0
    rng = range(edge)
    for x, y, z in itertools.product(rng, rng, rng if dim == 3 else [0]):
        ci = colour_of(col, x, y, z)
        assert 0 <= ci < q
        for o in offsets:
            t = [x + o[0], y + o[1], z + o[2]]
            if periodic:
                t = [v % edge for v in t[:dim]] + t[dim:]
            elif any(v < 0 or v >= edge for v in t[:dim]):
                continue
            if tuple(t) == (x, y, z):
                continue                       # self: skipped, as the reference skips i == j
            assert colour_of(col, *t) != ci, (col, (x, y, z), o)


def test_nearest_neighbour_tables_keep_the_checkerboard():
    for name, dim in (("2d_nn_interfacial.dat", 2), ("3d_nn_bloch.dat", 3), ("2d_nn.dat", 2)):
        inter = read_interactions(interactions_file(name), dim, 1.0, 0.5)
        assert colouring(inter, dim, 16, True) == [0, 2, 2, 1, 1]


CASES = [("2d_j1j2", 2, 12, True), ("2d_j1j2", 2, 9, False), ("2d_j1j3", 2, 12, True), ("2d_j1j3", 2, 11, False),
         ("3d_j1j2", 3, 8, True), ("3d_j1j2", 3, 7, False), ("2d_long", 2, 20, True), ("2d_long", 2, 24, False),
         ("2d_long", 2, 8, True)]


@pytest.mark.parametrize("name,dim,edge,periodic", CASES)
def test_colouring_is_a_valid_parallel_order(tmp_path, name, dim, edge, periodic):
    inter = read_interactions(write_table(str(tmp_path), name), dim, 1.0, 1.0)
    col = colouring(inter, dim, edge, periodic)
    check_valid(col, coupling_offsets(name), dim, edge, periodic)


def test_colouring_counts_only_coupling_records(tmp_path):
    # with DMISTREN = 0 and EXCHANGE = 0 nothing couples: the checkerboard stays
    path = write_table(str(tmp_path), "2d_j1j2")
    assert colouring(read_interactions(path, 2, 0.0, 0.0), 2, 12, True)[0] == 0
    # Ising ignores D: the J2 records still make the table general
    assert colouring(read_interactions(path, 2, 1.0, 0.0), 2, 12, True, ising=True)[0] in (1, 2)


def test_reader_keeps_more_than_64_records_in_file_order(tmp_path):
    path = write_table(str(tmp_path), "2d_long")
    inter = read_interactions(path, 2, 2.0, 1.0)
    rec = np.loadtxt(path)
    assert inter.n == len(rec) == 80
    off = np.array([[inter.offset[k][0], inter.offset[k][1]] for k in range(inter.n)])
    assert np.array_equal(off, rec[:, :2].astype(int))
    assert np.allclose([inter.J[k] for k in range(inter.n)], 2.0 * rec[:, 2], rtol=1e-15, atol=0)
    assert inter.n <= L.MAX_OFFSETS == 2048


def test_reader_accepts_the_maximum_table_and_refuses_a_larger_one(tmp_path):
    """NMMC_MAX_OFFSETS records load in file order; one more is refused with
    NMMC_ERR_UNSUPPORTED instead of being truncated."""
    rng = np.random.default_rng(2)
    n = L.MAX_OFFSETS
    rec = np.column_stack([rng.integers(-40, 41, size=(n + 1, 2)), rng.normal(size=(n + 1, 4))])
    full = tmp_path / "max.dat"
    np.savetxt(full, rec[:n], fmt=["%d", "%d", "%.17g", "%.17g", "%.17g", "%.17g"])
    inter = read_interactions(str(full), 2, 1.0, 1.0)
    assert inter.n == n
    assert [inter.offset[n - 1][0], inter.offset[n - 1][1]] == [int(rec[n - 1, 0]), int(rec[n - 1, 1])]
    assert inter.J[n - 1] == rec[n - 1, 2]
    over = tmp_path / "over.dat"
    np.savetxt(over, rec, fmt=["%d", "%d", "%.17g", "%.17g", "%.17g", "%.17g"])
    with pytest.raises(L.NmmcError) as e:
        read_interactions(str(over), 2, 1.0, 1.0)
    assert e.value.code == L.ERR_UNSUPPORTED
