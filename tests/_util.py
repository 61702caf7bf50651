"""Helpers shared by the tests."""
import hashlib

import numpy as np


def digest(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u4").tobytes()).hexdigest()


def csr_digest(off, col, wt) -> str:
    h = hashlib.sha256()
    for a in (off, col, wt):
        h.update(np.ascontiguousarray(a, dtype="<u4").tobytes())
    return h.hexdigest()


def expand_to_split(dist_orig, parent_node):
    """Distances over split ids: every piece holds its parent's value."""
    return np.asarray(dist_orig)[np.asarray(parent_node)]
