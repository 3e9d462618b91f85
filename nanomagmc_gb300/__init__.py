"""GB300-native Metropolis spin-lattice sampler with NanoMagMC's semantics.

The product is the CUDA library ``_build/libnmmc.so`` behind the C ABI of
``include/nmmc.h``; this package binds it for Python callers (``sampler``) and holds its
build recipe (``build``).
"""
from .sampler import Sampler, State, make_options, read_input, load_lists, read_interactions, interactions_file  # noqa: F401
