"""GB300-native Hubbard exact diagonalisation: the Siro-Harju spin-split
matvec and the device-resident Lanczos solver it drives, behind the
reference's H_TBq / Hubbard / Lanczos operator surface.

The compute path is the compiled C-ABI library ``_lib/libedgb300.so``
(hand-written sm_103a CUDA); this package only binds it.
"""
from ._capi import EdError, load  # noqa: F401
from .hubbard import (H_TBq, Hubbard, Lanczos, basis_rank, basis_unrank, binom,  # noqa: F401
                      lanczos_batch, lanczos_multi, random_vector, tridiag_lowest)
from . import hubbard  # noqa: F401
from . import lattices  # noqa: F401

__all__ = ["EdError", "load", "H_TBq", "Hubbard", "Lanczos", "basis_rank", "basis_unrank", "binom",
           "lanczos_batch", "lanczos_multi", "random_vector", "tridiag_lowest", "lattices"]
