"""The exact finite-lattice Ising energy used by the GPU statistics test is pinned here:
Kaufman's formula against full enumeration (3x3, 4x4) and against Onsager's infinite lattice."""
import numpy as np
import pytest

from onsager import TC, energy_per_site_brute, energy_per_site_torus, onsager_energy


@pytest.mark.parametrize("L", [3, 4])
@pytest.mark.parametrize("T", [1.0, 2.0, TC, 3.0, 5.0])
def test_kaufman_matches_enumeration(L, T):
    assert energy_per_site_torus(T, L) == pytest.approx(energy_per_site_brute(T, L), abs=1e-6)


@pytest.mark.parametrize("T", [1.5, 2.0, 2.6, 3.5])
def test_large_torus_approaches_onsager(T):
    pytest.importorskip("scipy")
    assert energy_per_site_torus(T, 256) == pytest.approx(onsager_energy(T), abs=1e-4)
