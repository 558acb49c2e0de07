"""The reference's distribution dump files, read on the host.

One file holds one distribution, in the layout DistributionTemplated::Dump writes
(src/distribution_templated.cc:394-425), native little-endian:

    u32 name length, the class name
    1 byte of Specie (a class with static members only: sizeof is 1)
    u32 records and u32 bytes of the parameter container, then the container's bytes
    i32 n_events, i32 counts[bins], the per-bin sums (double, GeoVector or GeoMatrix: 1, 3 or 9 doubles)
    u32 n, GeoVector values_record[n]; u32 m, the per-bin type weights_record[m]

The number of bins is not stored; it follows from the container's first record, n_bins, with
every dimension below one counted as one (src/distribution_templated.cc:98-116). The C ABI writes
and reads these files (spx_dump_distribution, spx_restore_distribution); this module lets host
code and tests read them without a device.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass

import numpy as np

#: doubles per bin of the reference's distribution classes (DistributionTemplated<double|GeoVector|GeoMatrix>)
CLASS_WIDTH = {"DistributionPositionCumulativeOrder1": 3, "DistributionPositionCumulativeOrder2": 9}


@dataclass
class DistroDump:
    class_name: str
    specie: int
    n_records: int
    container: bytes
    n_events: int
    counts: np.ndarray          # int32[bins]
    sums: np.ndarray            # float64[bins, width]
    values_record: np.ndarray   # float64[n, 3]
    weights_record: np.ndarray  # float64[m, width]

    @property
    def n_bins(self) -> tuple[int, int, int]:
        return container_bins(self.container)


def container_bins(container: bytes) -> tuple[int, int, int]:
    """n_bins of a DistributionTemplated container: its first record, a MultiIndex of three ints."""
    if len(container) < 13 or container[0] != 12:
        raise ValueError("the container does not start with a MultiIndex record")
    nb = struct.unpack_from("<3i", container, 1)
    return tuple(max(n, 1) for n in nb)


def read(data: bytes | str, width: int | None = None) -> DistroDump:
    """Parse one dump file (a path or its bytes). ``width`` overrides the class-name lookup."""
    if isinstance(data, str):
        with open(data, "rb") as f:
            data = f.read()
    pos = 0

    def take(n: int) -> bytes:
        nonlocal pos
        if pos + n > len(data):
            raise ValueError("dump file is truncated")
        out = data[pos:pos + n]
        pos += n
        return out

    (name_len,) = struct.unpack("<I", take(4))
    name = take(name_len).decode()
    specie = take(1)[0]
    n_records, length = struct.unpack("<2I", take(8))
    container = take(length)
    w = width if width is not None else CLASS_WIDTH.get(name, 1)
    nb = container_bins(container)
    bins = nb[0] * nb[1] * nb[2]
    (n_events,) = struct.unpack("<i", take(4))
    counts = np.frombuffer(take(4 * bins), dtype="<i4").copy()
    sums = np.frombuffer(take(8 * bins * w), dtype="<f8").reshape(bins, w).copy()
    (n_val,) = struct.unpack("<I", take(4))
    values = np.frombuffer(take(24 * n_val), dtype="<f8").reshape(n_val, 3).copy()
    (n_wgt,) = struct.unpack("<I", take(4))
    weights = np.frombuffer(take(8 * w * n_wgt), dtype="<f8").reshape(n_wgt, w).copy()
    if pos != len(data):
        raise ValueError(f"{len(data) - pos} bytes after the record arrays")
    return DistroDump(name, specie, n_records, bytes(container), n_events, counts, sums, values, weights)
