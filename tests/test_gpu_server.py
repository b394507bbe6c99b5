"""Serving loop (mpmgpu_server_*): requests arriving while others run are
admitted as run slots and memory free up, run together with 2D and 3D work
overlapping, and each result is the one the run gives alone (the CPU oracle,
at the mode's tolerance)."""
import time

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-10
TOL_MIXED = 1e-5


def requests(count, seed, nmin=300, nmax=2500, smin=10, smax=40):
    from nairn_gb300 import model
    ps = model.serve_request_params(count, seed=seed, nmin=nmin, nmax=nmax, smin=smin, smax=smax)
    return model.serve_models(ps)


def oracle(m):
    import oracle_lib
    from nairn_gb300 import abi
    ref = abi.copy_particles(m.particles)
    oracle_lib.run(m, ref, m.nsteps, nthreads=4)
    return ref


def check(out, ref, dim, tol, what):
    keys = ("x", "y", "vx", "vy", "sxx", "syy", "sxy") + (("z", "vz", "szz", "sxz", "syz") if dim == 3 else ())
    for k in keys:
        e = rel_l2(out[k], ref[k])
        assert e <= tol, (what, k, e)
    assert np.array_equal(out["elem"], ref["elem"]), what


def server(precision=0, budget=512 << 20, **kw):
    from nairn_gb300 import model
    from nairn_gb300.gpu import GpuServer
    return GpuServer(model.USAVG, model.SHAPE_UGIMP, precision, hbm_budget_bytes=budget, **kw)


@pytest.mark.parametrize("precision,tol", [(0, TOL), (1, TOL_MIXED)])
def test_each_result_is_the_run_alone(precision, tol, gpu_lib):
    """Staggered 2D and 3D arrivals; every result matches the oracle."""
    from nairn_gb300 import abi
    ms = requests(8, seed=precision + 1)
    s = server(precision, steps_per_round=4)
    ids = []
    for k, m in enumerate(ms):
        ids.append(s.submit(m))
        if k == 3:
            time.sleep(0.05)  # the second half arrives while the first runs
    s.drain(600)
    for rid, m in zip(ids, ms):
        info = s.poll(rid)
        assert info["state"] == abi.REQ_DONE and info["steps_done"] == m.nsteps, info
        check(s.result(rid), oracle(m), m.grid.dim, tol, m.name)
        s.release(rid)
    st = s.stats()
    assert st["completed"] == len(ms) and st["failed"] == 0
    assert st["particle_steps"] == sum(m.n * m.nsteps for m in ms)
    s.close()


def test_admission_waits_for_memory(gpu_lib):
    """With a budget that holds only a few runs at once, the rest queue and
    are admitted as earlier runs finish; results are unchanged."""
    from nairn_gb300 import abi
    ms = requests(10, seed=7, nmin=2000, nmax=3000, smin=20, smax=30)
    s = server(0, budget=24 << 20, frac_3d=0.5, steps_per_round=5)
    ids = [s.submit(m) for m in ms]
    s.drain(600)
    waits = []
    for rid, m in zip(ids, ms):
        info = s.poll(rid)
        assert info["state"] == abi.REQ_DONE, (m.name, info)
        waits.append(info["queue_ms"])
        check(s.result(rid), oracle(m), m.grid.dim, TOL, m.name)
    assert max(waits) > 0.
    s.close()


def test_oversized_and_failing_requests_are_confined(gpu_lib):
    from nairn_gb300 import abi
    ms = requests(3, seed=5)
    s = server(0, budget=16 << 20, frac_3d=0.5)
    from nairn_gb300 import model
    big = model.block_2d(ncx=200, ncy=150, steps=5)  # 120,000 particles: more than the 2D share holds
    bad = {k: np.array(v, copy=True) for k, v in ms[0].particles.items()}
    bad["vx"][0] = -1.e9
    r_big = s.submit(big)
    r_bad = s.submit(ms[0], particles=bad)
    r_ok = [s.submit(m) for m in ms[1:]]
    s.drain(600)
    assert s.poll(r_big)["state"] == abi.REQ_FAILED and s.poll(r_big)["status"] == 4  # OOM
    assert s.poll(r_bad)["state"] == abi.REQ_FAILED and s.poll(r_bad)["status"] == 6  # LEFT_GRID
    assert s.wait(r_bad, 1.0) == 6
    for rid, m in zip(r_ok, ms[1:]):
        assert s.poll(rid)["state"] == abi.REQ_DONE
        check(s.result(rid), oracle(m), m.grid.dim, TOL, m.name)
    s.close()


def test_wait_times_out_and_release_needs_completion(gpu_lib):
    from nairn_gb300.gpu import GpuError
    from nairn_gb300 import model
    m = model.block_3d(ncx=12, ncy=12, ncz=12, steps=3000)
    s = server(1)
    rid = s.submit(m)
    assert s.wait(rid, 0.0) == 8  # MPMGPU_ERR_TIMEOUT
    with pytest.raises(GpuError, match="BUSY"):
        s.release(rid)
    assert s.wait(rid, 600) == 0
    s.release(rid)
    s.close()


def test_resident_cap_serialises_runs(gpu_lib):
    """With a resident-particle cap below any request, runs go one at a time
    (least work first once queued); results are unchanged."""
    from nairn_gb300 import abi
    ms = requests(5, seed=31, smin=10, smax=20)
    s = server(0, max_resident_particles=1, order="least_work")
    t0 = time.perf_counter()
    ids, sub = [], []
    for m in ms:
        sub.append(1e3 * (time.perf_counter() - t0))
        ids.append(s.submit(m))
    s.drain(600)
    spans = []
    for rid, m, ts in zip(ids, ms, sub):
        info = s.poll(rid)
        assert info["state"] == abi.REQ_DONE
        spans.append((ts + info["queue_ms"], ts + info["total_ms"]))
        check(s.result(rid), oracle(m), m.grid.dim, TOL, m.name)
    spans.sort()
    for (a0, a1), (b0, b1) in zip(spans, spans[1:]):
        assert b0 >= a1 - 1.0, spans  # no two runs resident at once (1 ms clock slack)
    s.close()


def test_deadline_order_runs_every_request(gpu_lib):
    """The deadline order (online step-time model, slowdown bound 1.5) with a
    burst of requests: every request completes with the oracle's result, and
    the server's step-time model has been fitted from its rounds."""
    from nairn_gb300 import abi
    ms = requests(10, seed=41)
    s = server(0, steps_per_round=4, order="deadline", slowdown_target=1.5)
    ids = [s.submit(m) for m in ms]
    s.drain(600)
    for rid, m in zip(ids, ms):
        info = s.poll(rid)
        assert info["state"] == abi.REQ_DONE and info["steps_done"] == m.nsteps, info
        check(s.result(rid), oracle(m), m.grid.dim, TOL, m.name)
    st = s.stats()
    assert st["completed"] == len(ms) and st["failed"] == 0 and st["rounds"] > 0
    s.close()


def test_bad_server_orders_are_refused(gpu_lib):
    from nairn_gb300.gpu import GpuError
    for kw in (dict(order="deadline", slowdown_target=0.5),):
        with pytest.raises(GpuError):
            server(0, **kw)


@pytest.mark.parametrize("precision,tol", [(0, TOL), (1, TOL_MIXED)])
def test_served_contact_runs(precision, tol, gpu_lib):
    """3D two-material contact requests (lCPDI, Coulomb friction) served
    together, arriving in two waves; each result is the oracle's."""
    from nairn_gb300 import model, abi
    from nairn_gb300.gpu import GpuServer
    ms = model.contact_models(6, seed=9, nmin=1500, nmax=6000, steps=20)
    for k, m in enumerate(ms):
        m.nsteps = 12 + 4 * k
    s = GpuServer(model.USAVG, model.SHAPE_LCPDI, precision, hbm_budget_bytes=512 << 20, frac_3d=1.0,
                  steps_per_round=5, max_fields=2, nodes_per_particle=3.0)
    ids = [s.submit(m) for m in ms[:3]]
    time.sleep(0.05)
    ids += [s.submit(m) for m in ms[3:]]
    s.drain(600)
    for rid, m in zip(ids, ms):
        info = s.poll(rid)
        assert info["state"] == abi.REQ_DONE and info["steps_done"] == m.nsteps, info
        check(s.result(rid), oracle(m), 3, tol, m.name)
    s.close()


def test_served_fmpm_runs(gpu_lib):
    """Requests under FMPM(2) on every second step, served together: each
    result is the oracle's (each request counts its steps from admission)."""
    from nairn_gb300 import model, abi
    from nairn_gb300.gpu import GpuServer
    ms = [model.cantilever_2d(nx=8 + 2 * k, ny=3 + k, steps=20 + 5 * k, xpic=(2, 1, 2)) for k in range(3)]
    s = GpuServer(model.USAVG, model.SHAPE_UGIMP, 0, hbm_budget_bytes=256 << 20, frac_3d=0.0, steps_per_round=3,
                  xpic=(2, 1, 2))
    ids = [s.submit(m) for m in ms]
    s.drain(600)
    for rid, m in zip(ids, ms):
        info = s.poll(rid)
        assert info["state"] == abi.REQ_DONE and info["steps_done"] == m.nsteps, info
        check(s.result(rid), oracle(m), 2, TOL, m.name)
    s.close()
