"""Import-time stand-in for h5py, used only when the reference CyLag build is
imported as a test oracle.  The reference imports h5py at module top
(cylag/core/eulerian_field_set.pyx:21) but the per-particle step never touches
HDF5; any real use raises."""


def string_dtype(*args, **kwargs):
    return object


class File:
    def __init__(self, *args, **kwargs):
        raise RuntimeError("h5py is not available in the oracle environment")
