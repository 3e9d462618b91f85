"""Interaction tables beyond the axis nearest neighbours, written in the reference's Js/
record format (d offset ints, J, Dx, Dy, Dz per record; Old/lib/field_type.cpp:49-71)."""
import os

import numpy as np

# nearest-neighbour records with interfacial DMI D = z x r (the 2d_nn_interfacial.dat values)
_NN2 = [((1, 0), 1.0, (0, 1, 0)), ((-1, 0), 1.0, (0, -1, 0)),
        ((0, 1), 1.0, (-1, 0, 0)), ((0, -1), 1.0, (1, 0, 0))]
_NN3 = [((1, 0, 0), 1.0, (1, 0, 0)), ((-1, 0, 0), 1.0, (-1, 0, 0)), ((0, 1, 0), 1.0, (0, 1, 0)),
        ((0, -1, 0), 1.0, (0, -1, 0)), ((0, 0, 1), 1.0, (0, 0, 1)), ((0, 0, -1), 1.0, (0, 0, -1))]


def _records(name):
    if name == "2d_j1j2":      # J1 + interfacial DMI, antiferromagnetic next-nearest (diagonal) J2
        return _NN2 + [((dx, dy), -0.3, (0, 0, 0)) for dx in (1, -1) for dy in (1, -1)]
    if name == "2d_j1j3":      # J1 + third neighbours (+-2 on an axis) with half the DMI
        return _NN2 + [((2 * o[0], 2 * o[1]), 0.25, tuple(0.5 * d for d in D)) for o, _, D in _NN2]
    if name == "3d_j1j2":      # bulk DMI J1 + the 12 face-diagonal J2
        rec = list(_NN3)
        for a in range(3):
            for b in range(a + 1, 3):
                for sa in (1, -1):
                    for sb in (1, -1):
                        o = [0, 0, 0]
                        o[a], o[b] = sa, sb
                        rec.append((tuple(o), 0.1, (0, 0, 0)))
        return rec
    if name == "2d_long":      # every offset within radius 5, J = exp(-|r|) / 2 (80 records)
        rec = []
        for dx in range(-5, 6):
            for dy in range(-5, 6):
                r2 = dx * dx + dy * dy
                if 0 < r2 <= 25:
                    rec.append(((dx, dy), 0.5 * float(np.exp(-np.sqrt(r2))), (0, 0, 0)))
        return rec
    raise ValueError(name)


def write_table(directory, name):
    """Writes the named table to directory/name.dat and returns the path."""
    path = os.path.join(directory, name + ".dat")
    with open(path, "w") as f:
        for off, J, D in _records(name):
            f.write(" ".join(str(v) for v in off) + " %.17g %.17g %.17g %.17g\n" % (J, *D))
    return path


def coupling_offsets(name, ising=False):
    """Offsets of the records that couple sites (nonzero J, or nonzero D on Heisenberg)."""
    out = []
    for off, J, D in _records(name):
        if J != 0 or (not ising and any(d != 0 for d in D)):
            out.append(tuple(off) + (0,) * (3 - len(off)))
    return out
