"""Archive output: the particle records of a NairnMPM archive
(ArchiveData::ArchiveResults) packed on the device.  On the CPU: the record
layout and its size rules, the refusals, and a write/read round trip.  On the
GPU: the packed records equal the CPU restatement's bit for bit, and an
archive written from them matches the reference's own final archives of every
golden case."""
import ctypes as C
import os
import tempfile

import numpy as np
import pytest

from conftest import contact_tolerance, golden_cases, load_golden, model_for, rel_l2

ORDER = "iYYYYYNYNYNNNYNNNN"  # the golden archives' MPMArchiveOrder


@pytest.mark.parametrize("order", [ORDER, "iY", "iYYNNNNNNNNYYNYNNN", "iYNYNYNYNYNYNYNNNN"])
@pytest.mark.parametrize("dim", [2, 3])
def test_record_size_matches_layout(order, dim, gpu_lib):
    from nairn_gb300 import archive
    gpu_lib.mpmgpu_archive_record_size.restype = C.c_int64
    n = gpu_lib.mpmgpu_archive_record_size(dim, order.encode())
    assert n == archive.record_dtype(order, dim == 3).itemsize


@pytest.mark.parametrize("order", ["iYNNNNNNYNNNNNNNNN",  # temperature
                                   "iYNNNNNNNNNNNNNYNN",  # heat energy
                                   "iYNNNNNNNNNNNNNNYN",  # element crossings
                                   "iYNNNNNNNNNNNNNNNNY",  # damage normal
                                   "iYNNNNNNNNNNN\x03NNNN",  # history values 1 and 2
                                   "mYYNNNNNNNNNNNNNNN"])  # big-endian
def test_unheld_items_are_refused(order, gpu_lib):
    gpu_lib.mpmgpu_archive_record_size.restype = C.c_int64
    assert gpu_lib.mpmgpu_archive_record_size(3, order.encode()) == -2  # -MPMGPU_ERR_UNSUPPORTED


def test_write_read_round_trip():
    from nairn_gb300 import archive, model
    m = model.taylor_3d(radius=1.0, length=2.0, cell=0.5, steps=1)
    recs = archive.pack_records(m.particles, m.materials, ORDER, True)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "t.0")
        archive.write_archive(path, ORDER, True, 12.5, recs)
        a = archive.read_archive(path)
    assert a["three_d"] and abs(a["time_ms"] - 12.5) < 1e-6
    assert a["order"] == archive.normalize_order(ORDER)
    assert np.array_equal(a["elem"], m.particles["elem"] + 1)
    assert np.array_equal(a["pos"][:, 2], m.particles["z"])
    assert np.array_equal(a["mat"], m.particles["mat"] + 1)


@pytest.mark.parametrize("case", golden_cases())
def test_packer_matches_reference_archives(case):
    """The CPU restatement of the record, applied to the oracle's final state,
    reproduces the reference's own final archive of every golden case."""
    import oracle_lib
    from nairn_gb300 import abi, archive
    meta, g = load_golden(case)
    m = model_for(meta)
    p = abi.copy_particles(m.particles)
    # one thread: the reference's summation order (some contact runs are chaotic)
    oracle_lib.run(m, p, meta["steps"], nthreads=1)
    three_d = m.grid.dim == 3
    rec = np.frombuffer(archive.pack_records(p, m.materials, ORDER, three_d), archive.record_dtype(ORDER, three_d))
    for k in ("elem", "mass", "mat", "origpos"):
        assert np.array_equal(rec[k], g["final_" + k]), k
    for k in ("pos", "vel", "stress", "strain", "plastic", "work", "plastE", "hist1"):
        ref = g["final_" + k]
        if np.abs(ref).max() == 0.:
            assert np.abs(rec[k]).max() == 0., k
        else:
            assert rel_l2(rec[k], ref) <= 1e-12, (k, rel_l2(rec[k], ref))


@pytest.mark.gpu
@pytest.mark.parametrize("case", golden_cases())
def test_device_archive_matches_reference_archive(case, gpu_lib):
    from nairn_gb300 import archive
    from nairn_gb300.gpu import GpuRun
    meta, g = load_golden(case)
    m = model_for(meta)
    r = GpuRun(m)
    r.upload(m.particles)
    r.step(meta["steps"])
    recs = r.archive_records(ORDER)
    state = r.download(m.particles)
    r.close()
    three_d = m.grid.dim == 3
    # bit for bit the CPU restatement of the record on the same state
    assert recs == archive.pack_records(state, m.materials, ORDER, three_d)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "out.1")
        archive.write_archive(path, ORDER, three_d, 0., recs)
        a = archive.read_archive(path)
    for k in ("elem", "mass", "mat", "origpos"):
        assert np.array_equal(a[k], g["final_" + k]), k
    ctol = contact_tolerance(case, m, 1e-10)
    chaotic = ctol["vel"] > 1e-10
    for k in ("pos", "vel", "stress", "strain", "plastic", "work", "plastE", "hist1"):
        if np.abs(g["final_" + k]).max() == 0.:
            assert np.abs(a[k]).max() == 0., k
            continue
        # a run chaotic in the reference itself: its own sensitivity bounds the
        # archived quantities (energies and history follow stress and strain)
        tol = ctol.get(k, max(ctol["stress"], ctol["strain"]) if chaotic else 1e-10)
        assert rel_l2(a[k], g["final_" + k]) <= tol, (k, rel_l2(a[k], g["final_" + k]), tol)


@pytest.mark.gpu
@pytest.mark.parametrize("pinned", [True, False])
def test_async_archives_equal_the_synchronous_ones(pinned, gpu_lib):
    """Archives taken without waiting (mpmgpu_archive_records_async) while
    later steps run hold the state at the point they were requested: the
    same bytes as a synchronous archive of a second run stopped there (both
    runs with deterministic node sums).  Three archives in a row also check
    that each waits for the one before."""
    from nairn_gb300 import model
    from nairn_gb300.gpu import GpuRun, pin, unpin
    gpu_lib.mpmgpu_archive_record_size.restype = C.c_int64
    m = model.contact_3d(plate=(8, 8, 3), block=(3, 3, 2), block_x0=1.0, block_y0=1.5, steps=30)
    rec = int(gpu_lib.mpmgpu_archive_record_size(3, ORDER.encode()))
    at = (5, 12, 20)
    bufs = [np.zeros(m.n * rec, dtype=np.uint8) for _ in at]
    held = pin({str(k): b for k, b in enumerate(bufs)}) if pinned else []
    r = GpuRun(m, p2g=1)
    r.upload(m.particles)
    done = 0
    for k, buf in zip(at, bufs):
        r.step(k - done)
        done = k
        r.archive_records_async(ORDER, buf)
    r.step(m.nsteps - done)
    r.archive_wait()
    r.close()
    s = GpuRun(m, p2g=1)
    s.upload(m.particles)
    done = 0
    for k, buf in zip(at, bufs):
        s.step(k - done)
        done = k
        assert buf.tobytes() == s.archive_records(ORDER), k
    s.close()
    unpin(held)
