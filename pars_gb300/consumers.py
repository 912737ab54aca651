"""Stage-2 consumers of a structural index: random access (cf. structural_cursor,
include/pars/model/cursor.hpp:16-45) and a streaming replay (cf. replay,
include/pars/model/visit.hpp:34-48).  Both are format-agnostic: they know byte
offsets and partners, nothing about JSON or CSV.  They take the arrays a scan
returns (host copies: DeviceResult.to_numpy(), HostResult, a batch document)."""
from __future__ import annotations

import numpy as np

_WS = b" \t\n\r"


class StructuralCursor:
    """Random access to token i: its offset, byte, partner index and the run of
    non-structural bytes before it."""

    def __init__(self, base, pos, pair=None):
        self.base = memoryview(np.ascontiguousarray(base, dtype=np.uint8)).cast("B")
        self.pos = np.asarray(pos, dtype=np.int64)
        self.pair = None if pair is None else np.asarray(pair, dtype=np.int64)
        self.n = int(self.pos.size)

    def valid(self, i: int) -> bool:
        return 0 <= i < self.n

    def off(self, i: int) -> int:
        return int(self.pos[i])

    def ch(self, i: int) -> str:
        return chr(self.base[int(self.pos[i])])

    def match_index(self, i: int) -> int:
        return int(self.pair[i]) if self.pair is not None else -1

    def gap_begin(self, i: int) -> int:
        return int(self.pos[i - 1]) + 1 if i else 0

    def gap_end(self, i: int) -> int:
        return int(self.pos[i])

    def gap(self, i: int) -> bytes:
        return bytes(self.base[self.gap_begin(i):self.gap_end(i)])


def trim(s: bytes) -> bytes:
    """ASCII whitespace trimmed from both ends."""
    return s.strip(_WS)


def replay(base, n: int, pos, pair, visitor) -> None:
    """Visits the document in order: visitor.scalar(begin, end) for every run of
    non-structural bytes, visitor.symbol(offset, char, partner_offset or -1) for
    every structural byte."""
    b = memoryview(np.ascontiguousarray(base, dtype=np.uint8)).cast("B")
    pos = np.asarray(pos, dtype=np.int64)
    prev = 0
    for i in range(pos.size):
        p = int(pos[i])
        if p > prev:
            visitor.scalar(prev, p)
        match = int(pos[pair[i]]) if (pair is not None and pair[i] >= 0) else -1
        visitor.symbol(p, chr(b[p]), match)
        prev = p + 1
    if n > prev:
        visitor.scalar(prev, n)
