"""PCTD version-0 proton history files (reader and writer).

Layout, as read by count_histories_v0 and read_data_chunk_v02
(src/pCT_Reconstruction_Data_Segments.cu:997-1097, 1769-1933), little endian:

    char[4]  "PCTD"
    int32    version id (0)
    int32    number of histories N
    float32  projection angle [deg]
    float32  beam energy [MeV]
    int32    generation date, int32 pre-process date (Unix time)
    int32 n + n bytes   phantom name
    int32 n + n bytes   data source
    int32 n + n bytes   prepared by
    float32[N] x 13     t0 t1 t2 t3, v0 v1 v2 v3, u0 u1 u2 u3, WEPL   (mm)

One file per gantry angle, named <dir>/<folder>/projection_<angle:03d>.bin,
where angle = int(file_index * GANTRY_ANGLE_INTERVAL) (.cu:1807-1813).  The
reader maps the header angle to the gantry angle as (int(angle) + 270) % 360
(.cu:1921); the writer stores (gantry + 90) % 360 so the round trip lands on
the intended gantry angle.
"""
import os
import struct

import numpy as np

FIELDS = ["t0", "t1", "t2", "t3", "v0", "v1", "v2", "v3", "u0", "u1", "u2", "u3", "wepl"]
MAGIC = b"PCTD"


def file_name(directory, folder, gantry_angle, base="projection", ext=".bin"):
    return os.path.join(directory, folder, "%s_%03d%s" % (base, gantry_angle, ext))


def write_file(path, arrays13, projection_angle, beam_energy=200.0, phantom_name=b"synthetic",
               data_source=b"pct_gb300 generator", prepared_by=b"pct_gb300"):
    """Writes one PCTD v0 file; arrays13 is a (13, N) float32 array in mm."""
    a = np.ascontiguousarray(arrays13, dtype="<f4")
    if a.ndim != 2 or a.shape[0] != 13:
        raise ValueError("expected a (13, N) array")
    n = a.shape[1]
    with open(path, "wb") as f:
        f.write(MAGIC)
        f.write(struct.pack("<ii", 0, n))
        f.write(struct.pack("<ff", float(projection_angle), float(beam_energy)))
        f.write(struct.pack("<ii", 0, 0))
        for s in (phantom_name, data_source, prepared_by):
            f.write(struct.pack("<i", len(s)))
            f.write(s)
        f.write(a.tobytes())


def read_file(path):
    """Returns (arrays13 (13, N) float32 in mm, projection_angle, beam_energy)."""
    with open(path, "rb") as f:
        data = f.read()
    if len(data) < 36 or data[:4] != MAGIC:
        raise ValueError("%s: not a PCTD file" % path)
    version, n = struct.unpack_from("<ii", data, 4)
    if version != 0:
        raise ValueError("%s: PCTD version %d is not supported" % (path, version))
    if n < 0:
        raise ValueError("%s: negative history count" % path)
    angle, energy = struct.unpack_from("<ff", data, 12)
    off = 28
    for _ in range(3):
        if off + 4 > len(data):
            raise ValueError("%s: truncated header" % path)
        (ln,) = struct.unpack_from("<i", data, off)
        if ln < 0 or off + 4 + ln > len(data):
            raise ValueError("%s: bad string length" % path)
        off += 4 + ln
    need = 13 * 4 * n
    if off + need > len(data):
        raise ValueError("%s: truncated history data (%d of %d bytes)" % (path, len(data) - off, need))
    arrays = np.frombuffer(data, dtype="<f4", count=13 * n, offset=off).reshape(13, n).copy()
    return arrays, angle, energy


def write_scan(directory, folder, arrays13, projection_angle, num_angles, gantry_angle_interval):
    """Splits an angle-major history set into one file per gantry angle."""
    os.makedirs(os.path.join(directory, folder), exist_ok=True)
    proj = np.asarray(projection_angle, dtype=np.float32)
    gantry = (proj.astype(np.int64) + 270) % 360
    paths = []
    for k in range(num_angles):
        g = int(k * gantry_angle_interval)
        sel = np.nonzero(gantry == g)[0]
        p = file_name(directory, folder, g)
        write_file(p, arrays13[:, sel], (g + 90) % 360)
        paths.append(p)
    return paths


def read_scan(directory, folder, num_angles, gantry_angle_interval):
    """Reads every angle file in order; returns ((13, N) arrays, per-history projection angle)."""
    parts, angles = [], []
    for k in range(num_angles):
        a, ang, _ = read_file(file_name(directory, folder, int(k * gantry_angle_interval)))
        parts.append(a)
        angles.append(np.full(a.shape[1], ang, dtype=np.float32))
    return np.concatenate(parts, axis=1), np.concatenate(angles)
