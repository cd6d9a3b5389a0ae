"""Decoding of the xform pick tables in a prepared parameter block (the
layout of RFK_OFF_ALIAS / RFK_OFF_CALIAS in rfk_iterate.cuh): after the reals,
padded to an even offset, nx (threshold, alias) pairs, then with chaos one
such table per previous xform."""
import numpy as np


def alias_distribution(block: np.ndarray, size_reals: int, nx: int, row: int | None = None) -> np.ndarray:
    """Pick probabilities of the base table (row None) or of chaos row `row`:
    entry i keeps i with probability min(threshold, 1), else takes its alias;
    each entry is drawn with probability 1 / nx."""
    off = (size_reals + 1) // 2 * 2 + (0 if row is None else 2 * nx * (1 + row))
    tbl = np.ascontiguousarray(block[off:off + 2 * nx], dtype=np.float32)
    thr = np.clip(tbl[0::2].astype(np.float64), 0.0, 1.0)
    alias = tbl[1::2].view(np.int32)
    assert np.all((alias >= 0) & (alias < nx)), alias
    p = np.zeros(nx)
    np.add.at(p, np.arange(nx), thr / nx)
    np.add.at(p, alias, (1.0 - thr) / nx)
    return p
