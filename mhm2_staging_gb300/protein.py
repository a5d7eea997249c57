"""Protein alphabet for mhsw_align_protein: the 24 letters of the reference's protein
kernels' 24 x 24 matrices (src/adept-sw/kernel.cpp:510-899 take a scoring matrix and a
91-entry ASCII encoding) and the encoding that maps them to 0..23."""
from __future__ import annotations

import numpy as np

PROTEIN_LETTERS = "ARNDCQEGHILKMFPSTWYVBZX*"


def protein_encoding() -> np.ndarray:
    """91-entry ASCII encoding: the letters above to 0..23, every other byte below 91 to
    22 ('X')."""
    enc = np.full(91, PROTEIN_LETTERS.index("X"), dtype=np.int16)
    for k, ch in enumerate(PROTEIN_LETTERS):
        enc[ord(ch)] = k
    return enc
