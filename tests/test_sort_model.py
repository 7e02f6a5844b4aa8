"""A CPU model of the chunked counting sort of ``csrc/sort.cu`` (no GPU).

The kernels' index arithmetic restated with numpy on the same chunk sizes:
per chunk, each live particle gets (entry, rank) from the chunk's cell table,
packed as ``(rank << table_bits) | entry``; each entry reserves its run below
the cell's remaining count (``old = count[c]; count[c] -= m``) and gets a place
in the chunk's output order; the output order is packed as
``(entry << 11) | staged index``; a particle's destination is
``first[entry] + (j - place[entry])``.  The test checks that the result is a
permutation of the live particles sorted by key, that counts return to zero
and that every packed value fits its field, for scrambled, nearly sorted and
partly removed inputs, with a partial last chunk.
"""
from __future__ import annotations

import numpy as np
import pytest

DEAD = 0xFFFFFFFF
IDX_BITS = 11


def chunk_sort(keys, nkeys, chunk, table_bits, rng):
    n = len(keys)
    live = keys != DEAD
    count = np.bincount(keys[live], minlength=nkeys).astype(np.int64)
    offset = np.concatenate([[0], np.cumsum(count)])
    total = int(offset[-1])
    out = np.full(n, -1, dtype=np.int64)
    chunks = list(range(0, n, chunk))
    rng.shuffle(chunks)  # chunks reserve in any order (blocks race)
    for base in chunks:
        idx = np.arange(base, min(base + chunk, n))
        k = keys[idx]
        sel = k != DEAD
        table = {}
        er = np.full(len(idx), DEAD, dtype=np.int64)
        for s in np.flatnonzero(sel):
            c = int(k[s])
            e = table.setdefault(c, [len(table), 0])
            r = e[1]
            e[1] += 1
            er[s] = (r << table_bits) | e[0]
            assert er[s] < 2 ** 32 and e[0] < 2 ** table_bits
        assert len(table) * 2 <= 2 ** table_bits  # the table stays at most half full
        place, first, at = {}, {}, 0
        for c, (ent, m) in table.items():
            old = int(count[c])
            count[c] -= m
            assert count[c] >= 0
            first[ent] = int(offset[c]) + old - m
            place[ent] = at
            at += m
        perm = np.full(at, -1, dtype=np.int64)
        for s in np.flatnonzero(sel):
            ent, r = int(er[s]) & (2 ** table_bits - 1), int(er[s]) >> table_bits
            j = place[ent] + r
            perm[j] = (ent << IDX_BITS) | int(s)
            assert s < 2 ** IDX_BITS
        assert (perm >= 0).all()
        for j in range(at):
            ent, s = int(perm[j]) >> IDX_BITS, int(perm[j]) & (2 ** IDX_BITS - 1)
            d = first[ent] + (j - place[ent])
            assert 0 <= d < total and out[d] == -1
            out[d] = idx[s]
    assert (count == 0).all()
    return out[:total], total


@pytest.mark.parametrize("layout", ["scrambled", "nearly_sorted", "removed"])
def test_chunked_counting_sort_model(layout):
    rng = np.random.default_rng(3)
    nkeys, n = 4000, 20000 + 517  # a partial last chunk
    if layout == "scrambled":
        keys = rng.integers(0, nkeys, n)
    else:
        keys = np.sort(rng.integers(0, nkeys, n))
        keys = np.clip(keys + rng.integers(-3, 4, n), 0, nkeys - 1)  # drift since the last sort
    keys = keys.astype(np.int64)
    if layout == "removed":
        keys[rng.random(n) < 0.1] = DEAD
    for chunk, table_bits in ((2048, 12), (1536, 12)):  # count kernel, scatter kernel
        out, total = chunk_sort(keys.copy(), nkeys, chunk, table_bits, rng)
        assert total == int((keys != DEAD).sum())
        assert np.array_equal(np.sort(out), np.flatnonzero(keys != DEAD))  # every live particle once
        assert (np.diff(keys[out]) >= 0).all()  # sorted by key
