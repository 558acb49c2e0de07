"""The reference's text output of a distribution: DistributionTemplated::Print1D, Print2D and
PrintRecords (src/distribution_templated.cc:472-686), which SimulationMaster::PrintDistro1D,
PrintDistro2D and PrintRecords call (src/simulation.cc:856-886).

The files are written as the reference's ``std::ofstream`` writes them: a comment line with the
event (or record) count and an empty line, then one row per bin (or record) of columns 20 characters
wide, each number in the stream's default notation (printf ``%g``) at 10 significant digits, or at the
stream's default 6 in PrintRecords, which sets no precision.
Print1D collapses the other two dimensions of the histogram, Print2D the remaining one, summing the
counts and the per-bin sums in the reference's loop order; a row holds the bin centre (the
log-centre of a logarithmic axis), the mean and the sum of the weights (1, 3 or 9 numbers each,
by the distribution's width), and the count. With ``phys_units`` every value is multiplied by the
container's unit_val and every weight by its unit_distro, as the reference does.
"""
from __future__ import annotations

import math
import struct
from dataclasses import dataclass

import numpy as np

from .datacontainer import read_records


@dataclass
class DistroHeader:
    """The DistributionTemplated part of a distribution's parameter container
    (SetupDistribution, src/distribution_templated.cc:92-137)."""
    n_bins: tuple[int, int, int]   # each below one counted as one
    limits0: tuple[float, float, float]
    bin_size: tuple[float, float, float]
    log_bins: tuple[int, int, int]
    unit_distro: tuple[float, ...]  # width values (a double, GeoVector or row-major GeoMatrix)
    unit_val: tuple[float, float, float]
    width: int

    @classmethod
    def from_container(cls, blob: bytes, width: int) -> "DistroHeader":
        rec = read_records(blob)
        n_bins = struct.unpack("<3i", rec[0])
        minval = struct.unpack("<3d", rec[1])
        maxval = struct.unpack("<3d", rec[2])
        log_bins = struct.unpack("<3i", rec[3])
        unit_distro = struct.unpack(f"<{width}d", rec[5])
        unit_val = struct.unpack("<3d", rec[6])
        nb = tuple(max(n, 1) for n in n_bins)
        lo, size = [], []
        for k in range(3):
            a, b = (math.log10(minval[k]), math.log10(maxval[k])) if log_bins[k] else (minval[k], maxval[k])
            lo.append(a)
            size.append((b - a) / nb[k])
        return cls(nb, tuple(lo), tuple(size), log_bins, unit_distro, unit_val, width)

    def bin_cent(self, ijk: int, b: int) -> float:
        """DistributionBase::BinCent (src/distribution_base.hh:267-272)."""
        if b < 0 or b >= self.n_bins[ijk]:
            return 0.0
        x = self.limits0[ijk] + (b + 0.5) * self.bin_size[ijk]
        return math.pow(10.0, x) if self.log_bins[ijk] else x


def _num(x: float, prec: int = 10) -> str:
    if x != x:  # the C library prints the sign of a NaN
        return f"{'-nan' if math.copysign(1.0, x) < 0 else 'nan':>20}"
    return f"{x:20.{prec}g}"


def _sum_distro_cols(h: DistroHeader, n: int, s: list[float], phys_units: bool) -> str:
    """PrintSumDistro (src/distribution_templated.cc:472-535): mean and sum of the weights."""
    if h.width == 1:
        u = h.unit_distro[0] if phys_units else 1.0
        return _num((s[0] / n if n else 0.0) * u) + _num(s[0] * u)
    if not n:
        return _num(0.0) * (2 * h.width)
    if phys_units:
        return "".join(_num(s[i] / n * h.unit_distro[i]) for i in range(h.width)) + \
            "".join(_num(s[i] * h.unit_distro[i]) for i in range(h.width))
    return "".join(_num(s[i] / n) for i in range(h.width)) + "".join(_num(s[i]) for i in range(h.width))


def _lin(h: DistroHeader, b) -> int:
    return (b[0] * h.n_bins[1] + b[1]) * h.n_bins[2] + b[2]


def format_1d(h: DistroHeader, counts, sums, n_events: int, ijk: int, phys_units: bool = False) -> str | None:
    """DistributionTemplated::Print1D (src/distribution_templated.cc:546-579); None for an axis out of
    range (the reference then writes nothing)."""
    if ijk < 0 or ijk >= 3:
        return None
    sums = np.asarray(sums, dtype=np.float64).reshape(len(counts), h.width)
    i1, i2 = (ijk + 1) % 3, (ijk + 2) % 3
    out = [f"# Total number of events: {n_events}\n\n"]
    b = [0, 0, 0]
    for b0 in range(h.n_bins[ijk]):
        b[ijk] = b0
        n = 0
        s = [0.0] * h.width
        for b1 in range(h.n_bins[i1]):
            b[i1] = b1
            for b2 in range(h.n_bins[i2]):
                b[i2] = b2
                k = _lin(h, b)
                n += int(counts[k])
                for w in range(h.width):
                    s[w] += float(sums[k, w])
        out.append(_num(h.bin_cent(ijk, b0) * (h.unit_val[ijk] if phys_units else 1.0)) +
                   _sum_distro_cols(h, n, s, phys_units) + f"{n:20d}\n")
    return "".join(out)


def format_2d(h: DistroHeader, counts, sums, n_events: int, ijk1: int, ijk2: int,
              phys_units: bool = False) -> str | None:
    """DistributionTemplated::Print2D (src/distribution_templated.cc:591-632): Print1D for equal axes."""
    if not (0 <= ijk1 < 3 and 0 <= ijk2 < 3):
        return None
    if ijk1 == ijk2:
        return format_1d(h, counts, sums, n_events, ijk1, phys_units)
    ijk = ({0, 1, 2} - {ijk1, ijk2}).pop()
    sums = np.asarray(sums, dtype=np.float64).reshape(len(counts), h.width)
    out = [f"# Total number of events: {n_events}\n\n"]
    b = [0, 0, 0]
    for b1 in range(h.n_bins[ijk1]):
        b[ijk1] = b1
        for b2 in range(h.n_bins[ijk2]):
            b[ijk2] = b2
            n = 0
            s = [0.0] * h.width
            for b0 in range(h.n_bins[ijk]):
                b[ijk] = b0
                k = _lin(h, b)
                n += int(counts[k])
                for w in range(h.width):
                    s[w] += float(sums[k, w])
            out.append(_num(h.bin_cent(ijk1, b1) * (h.unit_val[ijk1] if phys_units else 1.0)) +
                       _num(h.bin_cent(ijk2, b2) * (h.unit_val[ijk2] if phys_units else 1.0)) +
                       _sum_distro_cols(h, n, s, phys_units) + f"{n:20d}\n")
    return "".join(out)


def format_records(h: DistroHeader, values, weights, phys_units: bool = False) -> str:
    """DistributionTemplated::PrintRecords (src/distribution_templated.cc:673-682) with PrintWeight
    (:643-666): per record its three values and its weight(s)."""
    values = np.asarray(values, dtype=np.float64).reshape(-1, 3)
    weights = np.asarray(weights, dtype=np.float64).reshape(len(values), h.width)
    out = [f"# Total number of records: {len(values)}\n\n"]
    for v, w in zip(values, weights):
        row = "".join(_num(float(v[j]) * (h.unit_val[j] if phys_units else 1.0), 6) for j in range(3))
        row += "".join(_num(float(w[i]) * (h.unit_distro[i] if phys_units else 1.0), 6) for i in range(h.width))
        out.append(row + "\n")
    return "".join(out)


def _write(path: str, text: str | None) -> None:
    if text is not None:
        with open(path, "w") as f:
            f.write(text)


def print_1d(path: str, h: DistroHeader, counts, sums, n_events: int, ijk: int, phys_units: bool = False) -> None:
    _write(path, format_1d(h, counts, sums, n_events, ijk, phys_units))


def print_2d(path: str, h: DistroHeader, counts, sums, n_events: int, ijk1: int, ijk2: int,
             phys_units: bool = False) -> None:
    _write(path, format_2d(h, counts, sums, n_events, ijk1, ijk2, phys_units))


def print_records(path: str, h: DistroHeader, values, weights, phys_units: bool = False) -> None:
    _write(path, format_records(h, values, weights, phys_units))
