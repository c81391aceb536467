"""XT3D: the NPF formulation with the full hydraulic conductivity tensor
(src/Model/ModelUtilities/Xt3dInterface.f90, Xt3dAlgorithm.f90).

The device computes the XT3D terms (gbsln_create_tensor); this module gives
the matrix pattern they need: with XT3D each row holds the cell, its
neighbours and the neighbours of its neighbours (xt3d_ac,
Xt3dInterface.f90:124-189), the diagonal first and the rest ascending as
the solution's sparse matrix sorts them (Sparse.f90:217-239).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp


def xt3d_pattern(ia, ja) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """(sia, sja, idxglo): the XT3D solution pattern of the connectivity
    ia/ja (0-based, diagonal first) and the position in it of each of the
    connectivity's entries."""
    ia = np.asarray(ia, np.int64)
    ja = np.asarray(ja, np.int64)
    n = ia.size - 1
    a = sp.csr_matrix((np.ones(ja.size, np.int8), ja, ia), shape=(n, n))
    a2 = (a @ a).tocsr()
    a2 = (a2 + a).tocsr()
    a2.sum_duplicates()
    a2.sort_indices()
    rows = np.repeat(np.arange(n), np.diff(a2.indptr))
    cols = a2.indices.astype(np.int64)
    # the diagonal first, the rest ascending
    order = np.lexsort((cols, cols != rows, rows))
    sja = cols[order]
    sia = a2.indptr.astype(np.int64)
    key = rows[order] * n + sja
    srt = np.argsort(key, kind="stable")
    rown = np.repeat(np.arange(n), np.diff(ia))
    idxglo = srt[np.searchsorted(key[srt], rown * n + ja)]
    return sia.astype(np.int32), sja.astype(np.int32), idxglo.astype(np.int32)
