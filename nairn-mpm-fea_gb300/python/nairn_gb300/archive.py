"""Reader and writer for NairnMPM binary particle archives.

Format (NairnMPM/src/System/ArchiveData.cpp:464-490 header, 721-1506 records,
CalcArchiveSize :255-430): a 64-byte header "ver6", the MPMArchiveOrder and crack
order strings, the dimension character, then one fixed-size record per particle.
Record: int element (1-based), double mass, short material (1-based) + 2 pad
bytes, angles (3D: z,y,x degrees; 2D: z angle, thickness), position, original
position, then optional items in archive-order sequence.  Stress is written as
Cauchy stress, rho*sp (ArchiveData.cpp:888-900).
"""
from __future__ import annotations

import numpy as np

HEADER_LENGTH = 64

# archive-order indices (NairnMPM/src/System/ArchiveData.hpp:22-32)
ARCH_ByteOrder, ARCH_Defaults = 0, 1
(ARCH_Velocity, ARCH_Stress, ARCH_Strain, ARCH_PlasticStrain, ARCH_OldOrigPosition,
 ARCH_WorkEnergy, ARCH_DeltaTemp, ARCH_PlasticEnergy, ARCH_ver2Empty, ARCH_ShearComponents,
 ARCH_StrainEnergy, ARCH_History, ARCH_Concentration, ARCH_HeatEnergy, ARCH_ElementCrossings,
 ARCH_RotStrain) = range(2, 18)


def _dtype(order: str, three_d: bool) -> np.dtype:
    vec = 3 if three_d else 2
    ten = 6 if three_d else 4
    f = [("elem", "<i4"), ("mass", "<f8"), ("mat", "<i2"), ("pad", "<i2")]
    if three_d:
        f += [("anglez", "<f8"), ("angley", "<f8"), ("anglex", "<f8")]
    else:
        f += [("anglez", "<f8"), ("thick", "<f8")]
    f += [("pos", "<f8", (vec,)), ("origpos", "<f8", (vec,))]

    def on(i):
        return len(order) > i and order[i] == "Y"

    if on(ARCH_Velocity):
        f.append(("vel", "<f8", (vec,)))
    if on(ARCH_Stress):
        f.append(("stress", "<f8", (ten,)))
    if on(ARCH_Strain):
        f.append(("strain", "<f8", (ten,)))
    if on(ARCH_PlasticStrain):
        f.append(("plastic", "<f8", (ten,)))
    if on(ARCH_WorkEnergy):
        f.append(("work", "<f8"))
    if on(ARCH_DeltaTemp):
        f.append(("dtemp", "<f8"))
    if on(ARCH_PlasticEnergy):
        f.append(("plastE", "<f8"))
    if on(ARCH_ShearComponents):
        f.append(("shear", "<f8", (2,)))
    if on(ARCH_StrainEnergy):
        f.append(("strainE", "<f8"))
    if on(ARCH_History):
        f.append(("hist1", "<f8"))
    if on(ARCH_Concentration):
        f.append(("conc", "<f8", (1 + vec,)))
    if on(ARCH_HeatEnergy):
        f.append(("heatE", "<f8"))
    if on(ARCH_ElementCrossings):
        f.append(("crossings", "<i4"))
    if on(ARCH_Strain):  # ARCH_RotStrain follows ARCH_Strain (CalcArchiveSize)
        f.append(("angle0", "<f8", (3 if three_d else 1,)))
    return np.dtype(f)


def read_archive(path: str) -> dict:
    """Return a dict of numpy arrays (one row per particle) plus 'time_ms'."""
    with open(path, "rb") as fh:
        raw = fh.read()
    hdr = raw[:HEADER_LENGTH]
    if hdr[:4] != b"ver6":
        raise ValueError(f"{path}: not a ver6 NairnMPM archive")
    n_mpm = hdr[4]
    order = hdr[5:5 + n_mpm].decode("ascii")
    k = 5 + n_mpm
    n_crack = hdr[k]
    k += 1 + n_crack
    three_d = chr(hdr[k]) == "3"
    k += 2  # dimension, structured flag
    time_ms = float(np.frombuffer(hdr[k:k + 4], "<f4")[0])
    if order[0] != "i":
        raise ValueError("big-endian archives are not supported")
    dt = _dtype(order, three_d)
    rec = dt.itemsize
    body = raw[HEADER_LENGTH:]
    # crack records can make records longer than the particle record
    n = len(body) // rec
    arr = np.frombuffer(body[:n * rec], dtype=dt)
    out = {name: np.array(arr[name]) for name in dt.names if name != "pad"}
    out["time_ms"] = time_ms
    out["three_d"] = three_d
    out["order"] = order
    return out
