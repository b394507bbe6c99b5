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


ARCH_MAXMPMITEMS = 25


def normalize_order(order: str) -> str:
    """ArchiveData::CalcArchiveSize (ArchiveData.cpp:266-283): pad to the
    known items with 'N', defaults on, retired items off, RotStrain = Strain."""
    o = list(order if len(order) >= 2 else "mY")
    o += ["N"] * (ARCH_MAXMPMITEMS - len(o))
    o = o[:ARCH_MAXMPMITEMS]
    o[ARCH_Defaults] = "Y"
    o[ARCH_OldOrigPosition] = "N"
    o[ARCH_ver2Empty] = "N"
    o[ARCH_RotStrain] = o[ARCH_Strain]
    return "".join(o)


def record_dtype(order: str, three_d: bool) -> np.dtype:
    """The particle record of an (unnormalized) MPMArchiveOrder string."""
    return _dtype(normalize_order(order), three_d)


def write_archive(path: str, order: str, three_d: bool, time_ms: float, records: bytes,
                  crack_order: str = "iYNNNNN", structured: bool = True) -> None:
    """A ver6 archive: the 64-byte header of ArchiveData::SetArchiveHeader
    (ArchiveData.cpp:464-486) followed by the particle records."""
    mo = normalize_order(order)
    hdr = bytearray(HEADER_LENGTH)
    k = 0
    for chunk in (b"ver6", bytes([len(mo)]), mo.encode("ascii"), bytes([len(crack_order)]),
                  crack_order.encode("ascii"), b"3" if three_d else b"2", b"1" if structured else b"0"):
        hdr[k:k + len(chunk)] = chunk
        k += len(chunk)
    hdr[k:k + 4] = np.float32(time_ms).tobytes()
    with open(path, "wb") as fh:
        fh.write(bytes(hdr))
        fh.write(records)


def pack_records(p: dict, materials, order: str, three_d: bool, thickness: float = 1.0) -> bytes:
    """CPU restatement of ArchiveData::ArchiveResults' particle records
    (ArchiveData.cpp:807-1100) from a particle-state dict: the checker of the
    device packer (mpmgpu_archive_records), same arithmetic in the same order."""
    mo = normalize_order(order)
    dt = _dtype(mo, three_d)
    n = p["x"].shape[0]
    rec = np.zeros(n, dtype=dt)
    mat = p["mat"]
    rho0 = np.array([m["rho"] * 0.001 for m in materials])[mat]
    mtype = np.array([m["type"] for m in materials])[mat]
    rec["elem"] = p["elem"] + 1
    rec["mass"] = p["mass"]
    rec["mat"] = mat + 1
    # GetRotationZ/Y/XInDegrees with zero initial angles (MPMBase.cpp:601-622)
    rec["anglez"] = 180. * (0. - 0.5 * p["wxy"]) / np.pi
    if three_d:
        rec["angley"] = 180. * (0. + 0.5 * p["wxz"]) / np.pi
        rec["anglex"] = 180. * (0. - 0.5 * p["wyz"]) / np.pi
        axes = ("x", "y", "z")
    else:
        rec["thick"] = thickness
        axes = ("x", "y")
    rec["pos"] = np.stack([p[a] for a in axes], 1)
    rec["origpos"] = np.stack([p[a + "0"] for a in axes], 1)

    def on(i):
        return mo[i] == "Y"

    if on(ARCH_Velocity):
        rec["vel"] = np.stack([p["v" + a] for a in axes], 1)
    if on(ARCH_Stress):
        rho = rho0 / np.where(mtype == 28, p["hist0"], 1.)
        P = np.where(mtype == 1, 0., p["pressure"])
        cols = [rho * (p["sxx"] - P), rho * (p["syy"] - P), rho * (p["szz"] - P), rho * p["sxy"]]
        if three_d:
            cols += [rho * p["sxz"], rho * p["syz"]]
        rec["stress"] = np.stack(cols, 1)
    tens = ("xx", "yy", "zz", "xy", "xz", "yz") if three_d else ("xx", "yy", "zz", "xy")
    if on(ARCH_Strain):
        rec["strain"] = np.stack([p["e" + t] for t in tens], 1)
    if on(ARCH_PlasticStrain):
        rec["plastic"] = np.stack([p["p" + t] for t in tens], 1)
    if on(ARCH_WorkEnergy):
        rec["work"] = 1.e-9 * p["mass"] * p["work"]
    if on(ARCH_PlasticEnergy):
        rec["plastE"] = 1.e-9 * p["mass"] * p["plast"]
    if on(ARCH_ShearComponents):
        rec["shear"] = np.stack([0.5 * (p["exy"] - p["wxy"]), 0.5 * (p["exy"] + p["wxy"])], 1)
    if on(ARCH_StrainEnergy):
        rec["strainE"] = 1.e-9 * p["mass"] * p["work"]
    if on(ARCH_History):
        rec["hist1"] = p["hist0"]
    return rec.tobytes()
