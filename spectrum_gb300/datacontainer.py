"""Positional parameter blobs in the reference's DataContainer byte layout.

Every plugin of the reference is set up from a ``DataContainer``: a sequence of records, each a
one-byte payload size followed by the payload (common/data_container.cc:139-224). ``Insert`` of a
``std::vector`` stores the vector's bytes as one record. The plugin's ``Setup*`` reads the records
back in a fixed order (e.g. src/background_base.cc:342-346).

This module writes exactly those bytes, so a blob built here can be handed to the C ABI
(``spx_add_plugin``) or to the reference itself. Python has no static types, so the record type
is chosen by the method: ``double``, ``int``, ``bool``, ``vec`` (GeoVector, 3 doubles),
``mi`` (MultiIndex, 3 ints), ``mat`` (GeoMatrix, 9 doubles), ``ints`` (std::vector<int>).
"""
from __future__ import annotations

import struct
from typing import Iterable, Sequence


class DataContainer:
    """Builder and reader of reference-format parameter blobs."""

    def __init__(self) -> None:
        self._records: list[bytes] = []

    # -- reference API names ------------------------------------------------------------------
    def Clear(self) -> None:  # noqa: N802 (reference method name)
        self._records.clear()

    def size(self) -> int:
        """Number of records (``DataContainer::size``)."""
        return len(self._records)

    def length(self) -> int:
        """Total byte length (``DataContainer::length``)."""
        return sum(len(r) + 1 for r in self._records)

    def data(self) -> bytes:
        """The blob (``DataContainer::data``)."""
        out = bytearray()
        for r in self._records:
            if len(r) > 255:
                raise ValueError("a DataContainer record holds at most 255 bytes")
            out.append(len(r))
            out += r
        return bytes(out)

    # -- typed inserts ------------------------------------------------------------------------
    def _add(self, payload: bytes) -> "DataContainer":
        if len(payload) > 255:
            raise ValueError("a DataContainer record holds at most 255 bytes")
        self._records.append(payload)
        return self

    def double(self, v: float) -> "DataContainer":
        return self._add(struct.pack("<d", float(v)))

    def int(self, v: int) -> "DataContainer":
        return self._add(struct.pack("<i", int(v)))

    def bool(self, v: bool) -> "DataContainer":
        return self._add(struct.pack("<?", bool(v)))

    def vec(self, v: Sequence[float]) -> "DataContainer":
        if len(v) != 3:
            raise ValueError("GeoVector needs 3 components")
        return self._add(struct.pack("<3d", *map(float, v)))

    def mi(self, v: Sequence[int]) -> "DataContainer":
        if len(v) != 3:
            raise ValueError("MultiIndex needs 3 components")
        return self._add(struct.pack("<3i", *map(int, v)))

    def mat(self, rows: Sequence[Sequence[float]]) -> "DataContainer":
        flat = [float(x) for row in rows for x in row]
        if len(flat) != 9:
            raise ValueError("GeoMatrix needs 3x3 components")
        return self._add(struct.pack("<9d", *flat))

    def ints(self, v: Iterable[int]) -> "DataContainer":
        v = list(v)
        return self._add(struct.pack("<%di" % len(v), *map(int, v)))


def read_records(blob: bytes) -> list[bytes]:
    """Split a blob into its record payloads (inverse of ``DataContainer.data``)."""
    out = []
    pos = 0
    while pos < len(blob):
        n = blob[pos]
        if pos + 1 + n > len(blob):
            raise ValueError("truncated DataContainer blob")
        out.append(blob[pos + 1:pos + 1 + n])
        pos += 1 + n
    return out
