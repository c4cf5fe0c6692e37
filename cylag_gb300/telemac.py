"""TELEMAC results as field sets (the readers behind
EulerianFieldSet.from_telemac2d / from_telemac3d,
cylag/core/eulerian_field_set.pyx:316-484, and read_cli,
cylag/geom/read_cli.pyx:24-93).

The reference reads result files through TELEMAC's own Python tools
(``data_manip.extraction.telemac_file.TelemacFile``), which are not part of
CyLag.  This module reads the Selafin format directly with numpy, following
TELEMAC's published file layout: Fortran sequential records (a 4-byte
big-endian length before and after each record) holding

* an 80-character title, ending in "SERAFIN " (FP32 values) or
  "SERAFIND" (FP64 values);
* NBV1, NBV2, then NBV1 + NBV2 variable records of 32 characters (name,
  unit);
* IPARAM (10 integers; IPARAM(7) is the number of planes of a 3D file,
  IPARAM(10) = 1 announces a 6-integer date record);
* NELEM, NPOIN, NDP, 1; the connectivity IKLE (1-based); IPOBO; X; Y;
* per time step: the time, then one record of NPOIN values per variable.

3D files store prisms (NDP = 6) over NPLAN planes of the 2D mesh; node
``plane * npoin2 + i`` is 2D node i on that plane, which is CyLag's layer
layout.  ``write_selafin`` writes the same layout (test data, synthetic
cases).
"""
from __future__ import annotations

import numpy as np

BND_WALL_REF = 0
MAX_NUMBER_OF_OPEN_BND = 30


def _records(buf):
    """Splits a Fortran sequential big-endian file into its records."""
    out, pos, n = [], 0, len(buf)
    while pos < n:
        if pos + 4 > n:
            raise ValueError("truncated Selafin record marker")
        ln = int(np.frombuffer(buf, ">i4", 1, pos)[0])
        start, end = pos + 4, pos + 4 + ln
        if end + 4 > n or int(np.frombuffer(buf, ">i4", 1, end)[0]) != ln:
            raise ValueError("inconsistent Selafin record length")
        out.append(buf[start:end])
        pos = end + 4
    return out


class SelafinFile:
    """A TELEMAC-2D/3D result file: ``times``, ``varnames``, the 2D mesh
    (``x``, ``y``, ``ikle2`` 0-based, ``npoin2``), ``nplan`` and
    ``get_data_value(name, k)`` (the values of one variable at record k,
    npoin2 * nplan of them), as TELEMAC's TelemacFile offers them."""

    def __init__(self, file_name):
        with open(file_name, "rb") as f:
            rec = _records(f.read())
        if len(rec) < 10:
            raise ValueError(f"{file_name}: not a Selafin file")
        self.title = rec[0].decode("latin-1")
        self.double = self.title[72:80].strip().upper() == "SERAFIND"
        fdt = ">f8" if self.double else ">f4"
        nbv1, nbv2 = (int(v) for v in np.frombuffer(rec[1], ">i4", 2))
        k = 2
        self.varnames, self.varunits = [], []
        for _ in range(nbv1 + nbv2):
            s = rec[k].decode("latin-1")
            self.varnames.append(s[:16].strip())
            self.varunits.append(s[16:32].strip())
            k += 1
        self.nbv1 = nbv1
        self.iparam = np.frombuffer(rec[k], ">i4", 10).astype(np.int64)
        k += 1
        if self.iparam[9] == 1:
            self.date = np.frombuffer(rec[k], ">i4", 6).astype(np.int64)
            k += 1
        nelem, npoin, ndp, _ = (int(v) for v in np.frombuffer(rec[k], ">i4", 4))
        k += 1
        self.ikle3 = np.frombuffer(rec[k], ">i4", nelem * ndp).reshape(nelem, ndp).astype(
            np.int32) - 1
        k += 1
        self.ipobo = np.frombuffer(rec[k], ">i4", npoin).astype(np.int32)
        k += 1
        x = np.frombuffer(rec[k], fdt, npoin).astype(np.float64)
        y = np.frombuffer(rec[k + 1], fdt, npoin).astype(np.float64)
        k += 2
        self.nplan = int(self.iparam[6]) if self.iparam[6] > 1 else 1
        self.npoin3, self.nelem3, self.ndp = npoin, nelem, ndp
        self.npoin2 = npoin // self.nplan
        if self.nplan > 1:
            if ndp != 6:
                raise ValueError("3D Selafin file without prisms")
            nelem2 = nelem // (self.nplan - 1)
            self.ikle2 = np.ascontiguousarray(self.ikle3[:nelem2, :3])
        else:
            self.ikle2 = self.ikle3
        self.x = np.ascontiguousarray(x[:self.npoin2])
        self.y = np.ascontiguousarray(y[:self.npoin2])
        nv = nbv1 + nbv2
        steps = rec[k:]
        if len(steps) % (nv + 1):
            raise ValueError("incomplete Selafin time record")
        self.ntimestep = len(steps) // (nv + 1)
        self.times = np.array([float(np.frombuffer(steps[t * (nv + 1)], fdt, 1)[0])
                               for t in range(self.ntimestep)])
        self._steps = steps
        self._fdt = fdt
        self._nv = nv

    def get_data_value(self, name, k):
        j = self.varnames.index(name)
        r = self._steps[k * (self._nv + 1) + 1 + j]
        return np.frombuffer(r, self._fdt, self.npoin3).astype(np.float64)


def _record(f, payload):
    n = np.array([len(payload)], ">i4").tobytes()
    f.write(n + payload + n)


def write_selafin(file_name, x, y, ikle2, times, variables, names, units=None, nplan=1,
                  double=False, title="CYLAG GB300 SYNTHETIC RESULTS"):
    """Writes a Selafin file: the 2D mesh (x, y, 0-based ikle2), ``nplan``
    planes (3D: prisms between consecutive planes), ``variables[t][v]``
    arrays of npoin2 * nplan values."""
    fdt = ">f8" if double else ">f4"
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    ikle2 = np.asarray(ikle2, dtype=np.int64)
    npoin2, nelem2 = len(x), len(ikle2)
    units = units or [""] * len(names)
    if nplan > 1:
        prisms = [np.hstack([ikle2 + p * npoin2, ikle2 + (p + 1) * npoin2])
                  for p in range(nplan - 1)]
        ikle, ndp = np.vstack(prisms), 6
        xx, yy = np.tile(x, nplan), np.tile(y, nplan)
    else:
        ikle, ndp = ikle2, 3
        xx, yy = x, y
    npoin = npoin2 * nplan
    iparam = np.zeros(10, ">i4")
    iparam[0] = 1
    if nplan > 1:
        iparam[6] = nplan
    with open(file_name, "wb") as f:
        t = title.ljust(72)[:72] + ("SERAFIND" if double else "SERAFIN ")
        _record(f, t.encode("latin-1"))
        _record(f, np.array([len(names), 0], ">i4").tobytes())
        for nm, un in zip(names, units):
            _record(f, (nm.ljust(16)[:16] + un.ljust(16)[:16]).encode("latin-1"))
        _record(f, iparam.tobytes())
        _record(f, np.array([len(ikle), npoin, ndp, 1], ">i4").tobytes())
        _record(f, (ikle + 1).astype(">i4").tobytes())
        _record(f, np.zeros(npoin, ">i4").tobytes())
        _record(f, xx.astype(fdt).tobytes())
        _record(f, yy.astype(fdt).tobytes())
        for ti, vals in zip(times, variables):
            _record(f, np.array([ti], fdt).tobytes())
            for v in vals:
                _record(f, np.asarray(v, dtype=np.float64).astype(fdt).tobytes())


def read_cli(file_name, vertex_id_column=11):
    """read_cli.pyx:24-93: (boundary_points [m, 2] = (vertex id, label),
    number of open boundaries).  A line "2 2 2 ..." is a wall point (label
    0); every other run of consecutive lines is a new open boundary (labels
    1, 2, ...); an open boundary cut by the file's start and end takes the
    first one's label."""
    points, new_boundary, count = [], False, 0
    with open(file_name) as f:
        for line in f:
            if count > MAX_NUMBER_OF_OPEN_BND:
                raise ValueError(f"Exceeding maximum number of open boundary (= "
                                 f"{MAX_NUMBER_OF_OPEN_BND})")
            w = line.split()
            if not w:
                continue
            if int(w[0]) == 2 and int(w[1]) == 2 and int(w[2]) == 2:
                label, new_boundary = BND_WALL_REF, False
            else:
                if not new_boundary:
                    count += 1
                label, new_boundary = count, True
            points.append([int(w[vertex_id_column]) - 1, label])
    if count > MAX_NUMBER_OF_OPEN_BND:
        raise ValueError(f"Exceeding maximum number of open boundary (= {MAX_NUMBER_OF_OPEN_BND})")
    bp = np.asarray(points).astype(np.int32)
    nb = bp.shape[0]
    if bp[0, 1] != BND_WALL_REF and bp[nb - 1, 1] != BND_WALL_REF:
        last = bp[nb - 1, 1]
        bp[bp[:, 1] == last, 1] = bp[0, 1]
    return bp, count
