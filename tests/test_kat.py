"""Known-answer tests of the step's physics, on the CPU oracle and on the GPU
path (both transfer precisions and the deterministic node sums):

- a uniform translation is exact: every shape-function option reproduces the
  constant field, so velocities do not change, positions move by v t and no
  stress appears (partition of unity, gradients summing to zero);
- J2 radial return never leaves the yield surface: after every update the
  deviatoric stress satisfies |s| <= sqrt(2/3) (sigma_y + Ep alpha);
- a Neo-Hookean body at rest (F = I) stays free of stress;
- the cell of a particle on a cell face is the one the reference's truncated
  index gives (half-open cells, MeshInfo::FindElementFromPoint).
"""
import math

import numpy as np
import pytest


SHAPES = ("Classic", "uGIMP", "lCPDI")
# (dim, shape) pairs: every shape in 2D and 3D, and qCPDI, which exists in 2D only
SHAPE_DIMS = [(d, s) for d in (2, 3) for s in SHAPES] + [(2, "qCPDI")]
V0 = (1500., -700., 400.)  # mm/s


def oracle_run(m, steps, particles=None):
    import oracle_lib
    from nairn_gb300 import abi
    p = abi.copy_particles(particles if particles is not None else m.particles)
    oracle_lib.run(m, p, steps, nthreads=2)
    return p


def gpu_run(m, steps, particles=None, **kw):
    from nairn_gb300.gpu import GpuRun
    r = GpuRun(m, **kw)
    p = particles if particles is not None else m.particles
    r.upload(p)
    r.step(steps)
    out = r.download(p)
    r.close()
    return out


def translation_model(dim, gimp, method=None, steps=12):
    from nairn_gb300 import model
    kw = {} if method is None else {"method": method}
    if dim == 2:
        return model.block_2d(ncx=8, ncy=5, vel=(V0[0], 0., 0., V0[1], 0., 0.), gimp=gimp, steps=steps, **kw)
    return model.block_3d(ncx=5, ncy=4, ncz=4, vel=(V0[0], 0., 0., V0[1], 0., 0., V0[2], 0., 0.), gimp=gimp,
                          steps=steps, **kw)


def deformation_model(dim, gimp, steps=12):
    """The same body with a velocity field of the same amplitude that deforms it."""
    from nairn_gb300 import model
    if dim == 2:
        return model.block_2d(ncx=8, ncy=5, vel=(0., V0[0], 0.3, 0., V0[1], 1.1), gimp=gimp, steps=steps)
    return model.block_3d(ncx=5, ncy=4, ncz=4, vel=(0., V0[0], 0.3, 0., V0[1], 1.1, 0., V0[2], 0.7), gimp=gimp,
                          steps=steps)


STRESS = ("sxx", "syy", "szz", "sxy", "sxz", "syz")


def check_translation(m, out, ref_stress, tol_v, tol_s):
    dim = m.grid.dim
    t = m.nsteps * m.options["timestep"]
    p0 = m.particles
    for a, (k, kx) in enumerate((("vx", "x"), ("vy", "y"), ("vz", "z"))[:dim]):
        assert np.max(np.abs(out[k] - V0[a])) <= tol_v * abs(V0[a]), k
        assert np.max(np.abs(out[kx] - (p0[kx] + V0[a] * t))) <= tol_v * abs(V0[a]) * t + 1e-12, kx
    smax = max(np.max(np.abs(out[k])) for k in STRESS)
    sref = max(np.max(np.abs(ref_stress[k])) for k in STRESS)
    assert sref > 0. and smax <= tol_s * sref, (smax, sref)


@pytest.mark.parametrize("dim,gimp", SHAPE_DIMS)
def test_oracle_uniform_translation(dim, gimp):
    m = translation_model(dim, gimp)
    out = oracle_run(m, m.nsteps)
    dm = deformation_model(dim, gimp)
    check_translation(m, out, oracle_run(dm, dm.nsteps), 1e-12, 1e-9)


@pytest.mark.gpu
@pytest.mark.parametrize("dim,gimp", SHAPE_DIMS)
@pytest.mark.parametrize("precision,p2g,tol_v,tol_s", [(0, 0, 1e-12, 1e-9), (1, 0, 1e-7, 1e-5),
                                                       (0, 1, 1e-12, 1e-9)])
def test_gpu_uniform_translation(dim, gimp, precision, p2g, tol_v, tol_s, gpu_lib):
    from nairn_gb300 import model
    for method in (model.USAVG, model.USL):
        m = translation_model(dim, gimp, method=method)
        out = gpu_run(m, m.nsteps, precision=precision, p2g=p2g)
        dm = deformation_model(dim, gimp)
        check_translation(m, out, gpu_run(dm, dm.nsteps, precision=precision, p2g=p2g), tol_v, tol_s)


def yield_ratio(m, out):
    """|s| / (sqrt(2/3) (sigma_y + Ep alpha)) per particle, in the specific
    units the particle stress is stored in (stress / rho)."""
    mat = m.materials[0]
    rho = mat["rho"] * 1e-3  # g/mm^3, the reference's Legacy density
    # IsoPlasticity's reduced yield stress and LinearHardening's slope (MPa -> Legacy units, per density)
    ys, ep = mat["yield_"] * 1e6 / rho, mat["Ep"] * 1e6 / rho
    sxx, syy, szz = out["sxx"], out["syy"], out["szz"]
    smag = np.sqrt(sxx ** 2 + syy ** 2 + szz ** 2 + 2. * (out["sxy"] ** 2 + out["sxz"] ** 2 + out["syz"] ** 2))
    return smag / (math.sqrt(2. / 3.) * (ys + ep * out["hist0"]))


def taylor():
    from nairn_gb300 import model
    return model.taylor_3d(radius=1.5, length=3.0, cell=0.5, steps=60)


def test_oracle_radial_return_stays_on_yield_surface():
    m = taylor()
    out = oracle_run(m, m.nsteps)
    r = yield_ratio(m, out)
    assert np.max(r) <= 1. + 1e-9
    assert np.sum(out["hist0"] > 0.) > 10 and np.max(r) > 0.999  # particles did yield


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_gpu_radial_return_stays_on_yield_surface(precision, gpu_lib):
    m = taylor()
    out = gpu_run(m, m.nsteps, precision=precision)
    r = yield_ratio(m, out)
    assert np.max(r) <= 1. + 1e-9
    assert np.sum(out["hist0"] > 0.) > 10 and np.max(r) > 0.999


def neo_at_rest(dim):
    from nairn_gb300 import model
    # E and nu of the same G and K set the time step
    neo = dict(type=model.MAT_NEOHOOKEAN, field=0, rho=1.1, E=28.125, nu=0.40625, yield_=0., Ep=0., G=10.,
               K=50., UJOption=0)
    if dim == 2:
        m = model.block_2d(ncx=6, ncy=4, vel=(0., 0., 0., 0., 0., 0.), mat=neo, steps=10)
    else:
        m = model.block_3d(ncx=4, ncy=4, ncz=3, vel=(0.,) * 9, mat=neo, steps=10)
    model._initial_material_state(m.particles, m.materials[0])
    return m


def check_at_rest(out):
    for k in STRESS + ("pressure", "vx", "vy", "vz"):
        assert np.max(np.abs(out[k])) <= 1e-12, k
    assert np.max(np.abs(out["hist0"] - 1.)) <= 1e-14  # J


@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_neohookean_at_rest(dim):
    m = neo_at_rest(dim)
    check_at_rest(oracle_run(m, m.nsteps))


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("precision", [0, 1])
def test_gpu_neohookean_at_rest(dim, precision, gpu_lib):
    m = neo_at_rest(dim)
    check_at_rest(gpu_run(m, m.nsteps, precision=precision))


def on_faces():
    """A body at rest with every 7th particle moved onto the right face of
    its cell, still recorded in that cell (where the point is a member of the
    closed cell); after one step it belongs to the cell on the right, as the
    half-open cells of the reference put it, and the others stay."""
    from nairn_gb300 import model, abi
    m = model.block_2d(ncx=8, ncy=4, vel=(0., 0., 0., 0., 0., 0.), gimp="Classic", steps=1)
    p = abi.copy_particles(m.particles)
    g = m.grid
    sel = np.arange(m.n) % 7 == 3
    col = p["elem"] % g.nx
    p["x"][sel] = g.xnodes[col[sel] + 1]
    expect = p["elem"].copy()
    expect[sel] = (p["elem"][sel] // g.nx) * g.nx + np.floor((p["x"][sel] - g.xmin) / g.dx).astype(np.int32)
    assert np.all(expect[sel] == p["elem"][sel] + 1)
    return m, p, expect


def test_oracle_cell_index_on_faces():
    m, p, expect = on_faces()
    out = oracle_run(m, 1, particles=p)
    assert np.array_equal(out["elem"], expect)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_gpu_cell_index_on_faces(precision, gpu_lib):
    m, p, expect = on_faces()
    out = gpu_run(m, 1, particles=p, precision=precision)
    assert np.array_equal(out["elem"], expect)
