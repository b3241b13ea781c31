"""GB300-native Dirac-Coulomb-Breit Fock build for BERTHA (host side).

The compute path is libberthagpu.so (CUDA, sm_103a) behind the C ABI of
include/bertha_gpu.h; this package only describes the basis, reads decks and
calls the library.
"""
from ._lib import BerthaGPUError, HMLT, SHAPE, lib  # noqa: F401
from .build import build  # noqa: F401
from .deck import (Basis, atom_basis, batched_atoms, c6h6_basis, density,  # noqa: F401
                   geometric, h2o_basis, make_basis, read_deck, shape_isym, tlf_basis,
                   tlf_small_basis)
from .fock import FockBatch, FockBuilder  # noqa: F401
