"""Host side of the batch API (no GPU): argument checks made before any device
call, the memory estimate the serving admission uses, and the seeded run
population of the 512-run batch."""
import ctypes as C

import numpy as np


def test_batch_create_rejects_bad_options_without_gpu_work(gpu_lib):
    from nairn_gb300 import abi, model
    base = dict(np=model.PLANE_STRAIN, method=model.USAVG, shape=model.SHAPE_UGIMP, precision=1, sort_interval=1,
                block=0, max_runs=4, max_materials=4, max_particles=1000, max_nodes=1000, fraction_usf=0.5)
    for bad, status in ((dict(shape=7), 2), (dict(max_fields=9), 2), (dict(np=11), 2), (dict(precision=3), 2),
                        (dict(max_runs=0), 1), (dict(max_particles=-5), 1), (dict(block=96), 1)):
        o = abi.MpmGpuBatchOptions(**{**base, **bad})
        h = C.c_void_p()
        assert gpu_lib.mpmgpu_batch_create(C.byref(o), C.byref(h)) == status, bad
        assert not h.value
        assert gpu_lib.mpmgpu_batch_last_error(None)


def test_batch_bytes_grows_with_capacity(gpu_lib):
    from nairn_gb300 import abi, model
    o = abi.MpmGpuBatchOptions(model.PLANE_STRAIN, model.USAVG, model.SHAPE_UGIMP, 1, 1, 0, 512, 512,
                               1_000_000, 500_000, 0.5)
    b1 = gpu_lib.mpmgpu_batch_bytes(C.byref(o))
    o.max_particles = 2_000_000
    b2 = gpu_lib.mpmgpu_batch_bytes(C.byref(o))
    # two arena buffers of 42 doubles + 4 ints per particle, plus sort keys
    assert b2 - b1 >= 1_000_000 * 2 * (42 * 8 + 4 * 4)
    assert b1 < 1_000_000 * 750 + 500_000 * 250  # about 730 B per particle slot, 217 B per node
    # two material fields: 26 double and 12 float columns per node and field
    o.max_particles, o.max_fields = 1_000_000, 2
    b3 = gpu_lib.mpmgpu_batch_bytes(C.byref(o))
    assert b3 - b1 == 500_000 * (2 * (26 * 8 + 12 * 4 + 1) - (19 * 8 + 12 * 4 + 1))
    # lCPDI corner scratch: 4 corners x (element + 6 doubles) per particle in 2D
    o.shape = model.SHAPE_LCPDI
    assert gpu_lib.mpmgpu_batch_bytes(C.byref(o)) - b3 == 1_000_000 * 4 * (4 + 6 * 8)


def test_batch_population_is_seeded_and_matches_the_spec():
    from nairn_gb300 import model
    a = model.batch_run_params(512, seed=2024)
    b = model.batch_run_params(512, seed=2024)
    assert a == b
    n = np.array([p["ncx"] * p["ncy"] * p["ppc_side"] ** 2 for p in a])
    assert n.min() >= 1800 and n.max() <= 210000
    assert 15e6 < n.sum() < 30e6  # log-uniform 2k-200k: mean about 43k
    types = [p["mat"]["type"] for p in a]
    assert 200 < types.count(model.MAT_PLASTIC) < 312
    E = np.array([p["mat"]["E"] for p in a])
    assert E.min() >= 100. and E.max() <= 200000.
    for p in a:
        if p["mat"]["type"] == model.MAT_PLASTIC:
            assert 0.001 * p["mat"]["E"] <= p["mat"]["yield_"] <= 0.01 * p["mat"]["E"]
        amp = np.abs(np.array(p["vel"])[[0, 1, 3, 4]]).sum()
        assert 99. <= amp <= 10001.


def test_block_model_is_consistent():
    from nairn_gb300 import model
    m = model.block_2d(ncx=10, ncy=4, fixed_left=True, vel=(100., 50., 0.3, -20., 10., 1.0))
    assert m.n == 10 * 4 * 4
    g = m.grid
    # every particle lies in its element
    col = m.particles["elem"] % g.nx
    row = m.particles["elem"] // g.nx
    assert np.all((g.xnodes[col] <= m.particles["x"]) & (m.particles["x"] < g.xnodes[col + 1]))
    assert np.all((g.ynodes[row] <= m.particles["y"]) & (m.particles["y"] < g.ynodes[row + 1]))
    assert len(m.bcs) == 2 * 5 and set(m.bcs["dir"]) == {1, 2}


def test_server_create_rejects_bad_options_without_gpu_work(gpu_lib):
    from nairn_gb300 import abi, model
    for budget, runs, frac in ((0, 8, 0.5), (1 << 30, 0, 0.5), (1 << 30, 8, 1.5)):
        o = abi.MpmGpuServerOptions(model.USAVG, model.SHAPE_UGIMP, 1, runs, 10, 1, 1, 0, budget, frac, 0.5, 0.5)
        h = C.c_void_p()
        assert gpu_lib.mpmgpu_server_create(C.byref(o), C.byref(h)) == 1
        assert not h.value and gpu_lib.mpmgpu_server_last_error(None)


def test_served_stream_is_seeded_and_matches_the_spec():
    from nairn_gb300 import model
    ps = model.serve_request_params(200, seed=77)
    assert ps == model.serve_request_params(200, seed=77)
    t = np.array([p[0] for p in ps])
    assert np.all(np.diff(t) > 0) and 6. < t[-1] < 14.  # Poisson, 20 per second
    dims = [p[1] for p in ps]
    assert 70 < dims.count(3) < 130
    n = np.array([kw["ncx"] * kw["ncy"] * (kw["ncz"] * 8 if d == 3 else 4) for _, d, kw in ps])
    assert n.min() >= 9000 and n.max() <= 2.2e6 and 2e5 < n.mean() < 6e5
    steps = np.array([kw["steps"] for _, _, kw in ps])
    assert steps.min() >= 200 and steps.max() <= 2000


def test_block_3d_model_is_consistent():
    from nairn_gb300 import model
    m = model.block_3d(ncx=4, ncy=3, ncz=5, fixed_base=True)
    assert m.n == 4 * 3 * 5 * 8
    g = m.grid
    e = m.particles["elem"]
    col, row, lay = e % g.nx, (e // g.nx) % g.ny, e // (g.nx * g.ny)
    for c, ax, nodes in ((col, "x", g.xnodes), (row, "y", g.ynodes), (lay, "z", g.znodes)):
        assert np.all((nodes[c] <= m.particles[ax]) & (m.particles[ax] < nodes[c + 1]))
    assert len(m.bcs) == (g.nx + 1) * (g.ny + 1) and set(m.bcs["dir"]) == {4}


def test_contact_population_is_seeded_and_matches_the_spec():
    from nairn_gb300 import model
    a = model.contact_run_params(64, seed=303)
    assert a == model.contact_run_params(64, seed=303)
    ms = model.contact_models(6, seed=303, nmin=20000, nmax=60000)
    for m in ms:
        assert m.options["shape"] == model.SHAPE_LCPDI and m.options["nfields"] == 2
        assert 15000 < m.n < 75000
        mats = m.materials
        assert mats[0]["type"] == model.MAT_ISO and mats[1]["type"] == model.MAT_NEOHOOKEAN
        assert m.extra["contact"]["friction"] == 0.3
        # the block lies on the plate, inside it in x and y
        blk = m.particles["mat"] == 1
        plate = ~blk
        assert blk.any() and plate.any()
        assert m.particles["x"][blk].max() <= m.particles["x"][plate].max()
        assert m.particles["z"][blk].min() >= m.particles["z"][plate].max()
