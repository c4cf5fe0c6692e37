"""Statistics files of a run (cylag/io/write_statistics.pyx,
cylag/io/write_particles.pyx:339-388), in the reference's formats:

* ``<output_rep>/<bnd_statistics_file_name>_<j>.txt``: particles leaving
  through open boundary j per step;
* ``<output_rep>/<control_sections_file_name>_<c>.txt``: particles crossing
  control section c per step;
* ``<output_rep>/<stranding_output_file_name>.txt``: stranded positions.

The counts come from the GPU step; these functions only format them.
"""
from __future__ import annotations

import os

import numpy as np


def prepare_secstats_output(bnd_statistics=False, nopen=0, outputdir="particles",
                            bnd_file_name="bnd_stats", cs_statistics=False, ncsec=0,
                            cs_file_name="cs_stats"):
    """write_statistics.pyx:24-54: (over)writes the headers."""
    os.makedirs(outputdir, exist_ok=True)
    heads = []
    if bnd_statistics:
        heads += [(bnd_file_name, j, "cylag boundary statistics file") for j in range(1, nopen + 1)]
    if cs_statistics:
        heads += [(cs_file_name, j, "cylag control section file") for j in range(1, ncsec + 1)]
    for name, j, title in heads:
        with open(os.path.join(outputdir, f"{name}_{j}.txt"), "w") as f:
            f.write(title + "\n")
            f.write("Variables: Time, Npart")
            f.write("\n")


def write_secstats_buffer(times, data, nsteps, nsec, outputdir, bnd_file_name):
    """write_statistics.pyx:73-107: appends one line per buffered step."""
    data = np.asarray(data)
    for j in range(1, nsec + 1):
        with open(os.path.join(outputdir, f"{bnd_file_name}_{j}.txt"), "a") as f:
            for k in range(nsteps):
                f.write("{:.8f}, ".format(float(times[k])))
                f.write("{:16d}  ".format(int(data[k, j - 1])))
                f.write("\n")


def write_stranded_particles_txt_2d(outputdir, file_name, stranded_positions, stranded_count):
    """write_particles.pyx:339-388 (one process): the stranded positions."""
    if stranded_count <= 0:
        return
    os.makedirs(outputdir, exist_ok=True)
    fileout = os.path.join(outputdir, file_name + ".txt")
    if os.path.isfile(fileout):
        os.remove(fileout)
    with open(fileout, "w") as f:
        f.write("cylag stranded particles file\n")
        f.write("Variables: Xp, Yp, Zp\n")
        for i in range(stranded_count):
            x, y, z = (float(v) for v in stranded_positions[i, :3])
            f.write("{:.16e}, ".format(x))
            f.write("{:.16e}, ".format(y))
            f.write("{:.16e}\n".format(z))
