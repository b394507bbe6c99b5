"""Shared test helpers.  GPU tests are marked ``gpu``; everything else runs on CPU."""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "nairn-mpm-fea_gb300", "python"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def golden_cases():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))


def load_golden(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(d["meta"]))
    return meta, {k: d[k] for k in d.files if k != "meta"}


def view_for(p, m):
    """archive_view with each particle's material density and type."""
    rho = np.array([q["rho"] for q in m.materials])[p["mat"]]
    typ = np.array([q["type"] for q in m.materials])[p["mat"]]
    return archive_view(p, m.grid.dim, rho, typ)


def model_for(meta):
    from nairn_gb300 import model
    return getattr(model, meta["generator"])(**meta["kwargs"])


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def regression_sensitivity(m, steps):
    """How far the reference's own result moves (relative L2 per quantity)
    when the initial velocities are perturbed by 1e-9 relative: regression
    contact normals decide contact from point-cloud supports that sit near
    zero separation, so such a run is chaotic -- the oracle, which matches the
    reference to 1e-13, shows it."""
    import oracle_lib
    from nairn_gb300 import abi
    outs = []
    for eps in (0., 1e-9):
        p = abi.copy_particles(m.particles)
        rng = np.random.default_rng(1)
        for k in ("vx", "vy"):
            p[k] = p[k] * (1. + eps * rng.standard_normal(p[k].shape))
        oracle_lib.run(m, p, steps, nthreads=4)
        outs.append(view_for(p, m))
    return {k: rel_l2(outs[1][k], outs[0][k]) for k in ("pos", "vel", "stress", "strain")}


_SENSITIVITY = {}


def contact_sensitivity(case):
    """How far the reference's own result (the oracle, which matches it to
    1e-13) moves, per quantity (relative L2), when every initial velocity
    component is perturbed by 1e-9 relative -- the largest move over three
    seeded perturbations, for golden case `case`."""
    if case not in _SENSITIVITY:
        import oracle_lib
        from nairn_gb300 import abi
        meta, _ = load_golden(case)
        m = model_for(meta)
        keys = ("pos", "vel", "stress", "strain", "plastic", "hist1")

        def final(seed):
            p = abi.copy_particles(m.particles)
            if seed:
                rng = np.random.default_rng(seed)
                for k in ("vx", "vy", "vz"):
                    p[k] = p[k] * (1. + 1e-9 * rng.standard_normal(p[k].shape))
            oracle_lib.run(m, p, meta["steps"], nthreads=1)
            return view_for(p, m)

        base = final(0)
        moves = [final(seed) for seed in (1, 2, 3)]
        _SENSITIVITY[case] = {k: max(rel_l2(q[k], base[k]) for q in moves) for k in keys}
    return _SENSITIVITY[case]


def contact_tolerance(case, m, tol):
    """Per-quantity tolerance for golden case `case`: tol, except for a contact
    run that is chaotic in the reference itself -- contact and stick/slip
    decisions that sit on near-zero separations, so that a 1e-9 perturbation
    of the input moves the result by more than 1e-6 -- which is held to twice
    that movement (any other summation order moves it as much)."""
    keys = ("pos", "vel", "stress", "strain", "plastic", "hist1")
    if not (m.extra and m.extra.get("contact")):
        return {k: tol for k in keys}
    sens = contact_sensitivity(case)
    if sens["vel"] <= 1e-6:
        return {k: tol for k in keys}
    return {k: max(tol, 2. * sens[k]) for k in keys}


def archive_view(p, dim, rho_gcc, mat_type=1):
    """Particle dict -> the quantities a NairnMPM archive stores (ArchiveData.cpp:807-930).
    The stress is (s - P) rho0 / J, with J the relative volume: 1 for the
    small-strain materials, history 0 for Neohookean (type 28).  rho_gcc and
    mat_type may be per-particle arrays (several materials)."""
    P = p["pressure"]
    rho = np.asarray(rho_gcc, dtype=np.float64) * 1e-3
    neo = np.asarray(mat_type) == 28
    if rho.ndim:
        rho = (rho / np.where(neo, p["hist0"], 1.0))[:, None]
    elif neo.any():
        rho = rho / p["hist0"][:, None]
    if dim == 2:
        pos = np.stack([p["x"], p["y"]], 1)
        vel = np.stack([p["vx"], p["vy"]], 1)
        st = np.stack([p["sxx"] - P, p["syy"] - P, p["szz"] - P, p["sxy"]], 1) * rho
        ep = np.stack([p["exx"], p["eyy"], p["ezz"], p["exy"]], 1)
        pl = np.stack([p["pxx"], p["pyy"], p["pzz"], p["pxy"]], 1)
    else:
        pos = np.stack([p["x"], p["y"], p["z"]], 1)
        vel = np.stack([p["vx"], p["vy"], p["vz"]], 1)
        st = np.stack([p["sxx"] - P, p["syy"] - P, p["szz"] - P, p["sxy"], p["sxz"], p["syz"]], 1) * rho
        ep = np.stack([p["exx"], p["eyy"], p["ezz"], p["exy"], p["exz"], p["eyz"]], 1)
        pl = np.stack([p["pxx"], p["pyy"], p["pzz"], p["pxy"], p["pxz"], p["pyz"]], 1)
    return dict(pos=pos, vel=vel, stress=st, strain=ep, plastic=pl, hist1=p["hist0"], elem=p["elem"] + 1)


@pytest.fixture(scope="session")
def gpu_lib():
    import __graft_entry__ as g  # noqa: F401
    sys.path.insert(0, ROOT)
    import __graft_entry__
    __graft_entry__.build_library()
    from nairn_gb300 import gpu
    return gpu.lib()
