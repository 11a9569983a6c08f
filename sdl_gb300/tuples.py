"""Digests and multiset arithmetic of object lists (hit-index tuples).

The reference identifies an object by the idx of its hits (``isIdxMatched``,
``Hit.cc:175-182``, ``MiniDoublet.cc:686-693``, ``Segment.cc:868-875``) and its
stage loops can produce the same tuple twice (a connection list with a
repeated module), so two object lists are equal when they are equal as
multisets of tuples.  Large lists (millions of rows per batch) are compared
through one 64-bit hash per row:

* :func:`row_hashes` -- a splitmix64-style mix folded over the row's int32
  values, seeded by the row width;
* :func:`multiset_digest` -- the sum of the row hashes mod 2^64, which does not
  depend on row order (the CPU checker computes the same value per event);
* :func:`multiset_intersection` -- the size of the multiset intersection of
  two lists (the track-candidate recall of a pruned chain against the plain
  one is ``|pruned & plain| / |plain|``).
"""
from __future__ import annotations

import numpy as np

_G = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_S30, _S27, _S31 = np.uint64(30), np.uint64(27), np.uint64(31)


def _mix(z: np.ndarray) -> np.ndarray:
    z = z + _G
    z = (z ^ (z >> _S30)) * _M1
    z = (z ^ (z >> _S27)) * _M2
    return z ^ (z >> _S31)


def row_hashes(t: np.ndarray) -> np.ndarray:
    """One uint64 per row of an (n, w) int32 tuple array."""
    t = np.asarray(t)
    if t.ndim != 2:
        raise ValueError("expected an (n, width) array")
    n, w = t.shape
    h = np.full(n, np.uint64(w), dtype=np.uint64)
    for c in range(w):
        h = _mix(h ^ t[:, c].astype(np.uint32).astype(np.uint64))
    return h


def multiset_digest(t: np.ndarray) -> int:
    """Order-independent digest of a tuple multiset (sum of row hashes mod 2^64)."""
    return int(np.sum(row_hashes(t), dtype=np.uint64)) if len(t) else 0


def multiset_intersection(a: np.ndarray, b: np.ndarray) -> int:
    """Number of rows the two tuple multisets share (with multiplicity)."""
    if len(a) == 0 or len(b) == 0:
        return 0
    ua, ca = np.unique(row_hashes(a), return_counts=True)
    ub, cb = np.unique(row_hashes(b), return_counts=True)
    _, ia, ib = np.intersect1d(ua, ub, assume_unique=True, return_indices=True)
    return int(np.minimum(ca[ia], cb[ib]).sum())


def split_by_event(t: np.ndarray, counts: np.ndarray) -> list:
    """Rows of a batch-wide object list (events in order) split per event."""
    return np.split(t, np.cumsum(np.asarray(counts, dtype=np.int64))[:-1]) if len(counts) else []
