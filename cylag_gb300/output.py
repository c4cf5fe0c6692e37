"""Particle snapshots (cylag/io/write_particles.pyx:17-91): the file
header, and one block per snapshot in CyLag's text format and/or one VTK
file per snapshot, formatted natively (``cg_snapshot_txt`` /
``cg_snapshot_vtk``).

A snapshot copies the particle arrays to the host once, between two GPU
calls, and hands the formatting to a writer thread, so the next steps run
while the previous snapshot is written.  Writes keep their order.
"""
from __future__ import annotations

import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from . import _lib


def prepare_output(pset, outputdir="particles", output_file_format="txt",
                   output_file_name="particles", model=1):
    """write_particles.pyx:17-50: output folder and the text header."""
    os.makedirs(outputdir, exist_ok=True)
    if output_file_format in ("txt", "all"):
        with open(os.path.join(outputdir, output_file_name + ".txt"), "w") as f:
            f.write("cylag particles result file\n")
            f.write("Variables: Tags, Xp, Yp, Zp, Up, Vp, Wp, ")
            if model >= 2:
                f.write("Us, Vs, Ws, ")
            if pset.additional_velocity:
                f.write("Ua, Va, Wa, ")
            if pset.additional_force:
                f.write("Fax, Fay, Faz, ")
            if pset.diameter_distribution != "monodisperse":
                f.write("dp, ")
            if pset.compute_depth:
                f.write("depth, ")
            f.write("\n")


def _ptr(a):
    return None if a is None else a.ctypes.data


def write_snapshot(arrays, dim, model, time, iteration, outputdir, file_name, fmt):
    """write_particles.pyx:52-91 on host copies of the particle arrays
    (``arrays``: tri, tag, position, velocity, fluid_velocity_seen,
    diameter or None, and optionally depth or None)."""
    L = _lib.load()
    tri, tag, pos, vel, fvs, diam = arrays[:6]
    depth = arrays[6] if len(arrays) > 6 else None
    n = len(tri)
    args = (int(dim), int(model), float(time), int(iteration), n, _ptr(tri), _ptr(tag),
            _ptr(pos), _ptr(vel), _ptr(fvs), _ptr(diam), _ptr(depth))
    if fmt in ("vtk", "all"):
        path = os.path.join(outputdir, f"{file_name}_{iteration}.vtk").encode()
        if L.cg_snapshot_vtk(path, *args) != 0:
            raise OSError(f"cannot write {path.decode()}")
    if fmt in ("txt", "all"):
        path = os.path.join(outputdir, file_name + ".txt").encode()
        if L.cg_snapshot_txt(path, *args) != 0:
            raise OSError(f"cannot write {path.decode()}")


class SnapshotWriter:
    """Ordered background writes of snapshots taken from a particle set."""

    def __init__(self, params, model):
        self.p = params
        self.model = model
        self._ex = ThreadPoolExecutor(max_workers=1, thread_name_prefix="cylag-snapshots")
        self._pending = []

    def take(self, pset, time, iteration):
        c = np.ascontiguousarray
        arrays = (c(pset.tri), c(pset.tag), c(pset.position), c(pset.velocity),
                  c(pset.fluid_velocity_seen) if self.model >= 2 else None,
                  None if pset.diameter_distribution == "monodisperse" else c(pset.diameter),
                  c(pset.depth) if pset.compute_depth else None)
        p = self.p
        self._pending.append(self._ex.submit(write_snapshot, arrays, pset.dim, self.model, time,
                                             iteration, p.output_rep, p.output_file_name,
                                             p.output_file_format))
        for f in [f for f in self._pending if f.done()]:
            f.result()   # re-raises a failed write
        self._pending = [f for f in self._pending if not f.done()]

    def wait(self):
        for f in self._pending:
            f.result()
        self._pending = []

    def close(self):
        self.wait()
        self._ex.shutdown(wait=True)
