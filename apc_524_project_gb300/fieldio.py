"""Reader of the field time series emoo_write_fields leaves in a directory.

The files hold the data of the reference's Hdf5IO output (one 4-D dataset
per field over the physical points, dims [nx][ny][nz][time], point
coordinates as attributes x, y, z, and a time dataset) as raw little-endian
doubles: time.f64, <name>.f64 (snapshot after snapshot, each [nx][ny][nz] in
C order) and <name>.xyz (x, y, z coordinate vectors)."""
import os

import numpy as np

NAMES = ("Ex", "Ey", "Ez", "Bx", "By", "Bz", "Jx", "Jy", "Jz", "rho")


def read_fields(d, n):
    """Returns (time[nt], {name: (data [nx, ny, nz, nt], (x, y, z))}) for the
    fields present in directory d of a grid of n = (nx, ny, nz) cells, data
    indexed like the reference's datasets."""
    t = np.fromfile(os.path.join(d, "time.f64"), dtype="<f8")
    out = {}
    for name in NAMES:
        p = os.path.join(d, name + ".f64")
        if not os.path.exists(p):
            continue
        raw = np.fromfile(p, dtype="<f8")
        if raw.size != len(t) * n[0] * n[1] * n[2]:
            raise ValueError(f"{name}: {raw.size} values for {len(t)} snapshots of {n}")
        data = np.moveaxis(raw.reshape(len(t), n[0], n[1], n[2]), 0, 3)
        xyz = np.fromfile(os.path.join(d, name + ".xyz"), dtype="<f8")
        x, y, z = np.split(xyz, [n[0], n[0] + n[1]])
        out[name] = (data, (x, y, z))
    return t, out
