"""Host-side model construction for the synthetic workloads.

Builds the structured grid, the material points and the nodal velocity
conditions the same way NairnMPM's input stage does for the XML produced by
``inputs.py``, so the GPU step and the CPU oracle start from the state the
reference starts from:

  grid        MPMReadHandler::grid()            NairnMPM/src/Read_MPM/Generators.cpp:1675-1990
  particles   MPMReadHandler::MPMPts()          Generators.cpp:1423-1545
              ElementBase::MPMPoints()          NairnMPM/src/Elements/MoreMPMElementBase.cpp:348-440
  mass        NairnMPM::PreliminaryParticleCalcs NairnMPM/src/NairnMPM_Class/NairnMPM.cpp:589-730
  velocity BC DisBC on BCLine/BCBox             Generators.cpp:822-1010, ShapeController::nextNode

All arrays are numpy; ``abi.py`` turns them into the C ABI structs.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

PLANE_STRAIN, THREED = 10, 12
USF, USAVG, USL = 0, 2, 3
SHAPE_LINEAR, SHAPE_UGIMP, SHAPE_BGIMP, SHAPE_BSPLINE, SHAPE_LCPDI, SHAPE_QCPDI = 0, 1, 5, 6, 10, 11
MAT_ISO, MAT_PLASTIC, MAT_NEOHOOKEAN, MAT_RIGID = 1, 9, 28, 35

PARTICLE_FIELDS = ("x", "y", "z", "vx", "vy", "vz", "x0", "y0", "z0", "mass", "lpx", "lpy", "lpz",
                   "exx", "eyy", "ezz", "exy", "exz", "eyz", "wxy", "wxz", "wyz",
                   "sxx", "syy", "szz", "sxy", "sxz", "syz", "pressure",
                   "pxx", "pyy", "pzz", "pxy", "pxz", "pyz", "hist0", "hist1", "work", "plast")


@dataclass
class Grid:
    dim: int
    nx: int
    ny: int
    nz: int
    xmin: float
    ymin: float
    zmin: float
    dx: float
    dy: float
    dz: float
    thickness: float
    xnodes: np.ndarray
    ynodes: np.ndarray
    znodes: np.ndarray | None

    @property
    def nnodes(self) -> int:
        n = (self.nx + 1) * (self.ny + 1)
        return n * (self.nz + 1) if self.dim == 3 else n

    @property
    def nelems(self) -> int:
        return self.nx * self.ny * (self.nz if self.dim == 3 else 1)


@dataclass
class Model:
    grid: Grid
    particles: dict
    materials: list
    bcs: np.ndarray
    options: dict
    nsteps: int
    name: str = ""
    extra: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.particles["x"].shape[0])


BC_DTYPE = np.dtype([("node", "<i4"), ("dir", "<i4"), ("value", "<f8"), ("ftime", "<f8")])


def _axis(vmin: float, vmax: float, cell: float):
    """One axis of MPMReadHandler::grid() for a regular grid with cellsize set:
    round the max up to a grid line, add one border cell each side, then
    points vmin + i*delta."""
    n = int((vmax - vmin) / cell)
    newmax = vmin + n * cell
    if newmax < vmax:
        vmax = newmax + cell
        n += 1
    c = (vmax - vmin) / float(n)
    n += 2
    vmin -= c
    vmax += c
    delta = (vmax - vmin) / float(n)
    pts = vmin + np.arange(n + 1, dtype=np.float64) * delta
    return n, vmin, vmax, delta, pts


def make_grid(dim: int, xlim, ylim, zlim, cell: float, thickness: float = 1.0) -> Grid:
    nx, x0, x1, gx, xp = _axis(xlim[0], xlim[1], cell)
    ny, y0, y1, gy, yp = _axis(ylim[0], ylim[1], cell)
    if dim == 3:
        nz, z0, z1, gz, zp = _axis(zlim[0], zlim[1], cell)
        zmin = z0
    else:
        nz, gz, zp, zmin = 0, 0.0, None, thickness
    return Grid(dim, nx, ny, nz, x0, y0, zmin, gx, gy, gz, thickness, xp, yp, zp)


def _element_points(g: Grid, ppc_side: int):
    """Positions (nelems*ppe, 3) and element index of every candidate point, in
    the order MPMPts visits them (element-major, then ElementBase::MPMPoints
    order: z, then y, then x)."""
    n = ppc_side
    gap = 1. / float(n)
    vals = np.array([-1. + (2. * j + 1.) * gap for j in range(n)])
    if g.dim == 2:
        xi = np.array([(vals[j], vals[i], 0.) for i in range(n) for j in range(n)])
    else:
        xi = np.array([(vals[j], vals[ii], vals[i]) for i in range(n) for ii in range(n) for j in range(n)])
    ne = g.nelems
    e = np.arange(ne)
    col = e % g.nx
    row = (e // g.nx) % g.ny
    x0, x1 = g.xnodes[col], g.xnodes[col + 1]
    y0, y1 = g.ynodes[row], g.ynodes[row + 1]
    npp = xi.shape[0]
    pos = np.zeros((ne, npp, 3))
    if g.dim == 2:
        # Sum over element nodes (FourNodeIsoparam node order) of x_i * N_i
        # with N_i = 4*((1+xii*x)/4)*((1+eti*y)/4) (FourNodeIsoparam.cpp:71-87)
        xii = (-1., 1., 1., -1.)
        eti = (-1., -1., 1., 1.)
        nx_ = (x0, x1, x1, x0)
        ny_ = (y0, y0, y1, y1)
        for k in range(npp):
            px = np.zeros(ne)
            py = np.zeros(ne)
            for i in range(4):
                t1 = (1. + xii[i] * xi[k, 0]) / 4.
                t2 = (1. + eti[i] * xi[k, 1]) / 4.
                f = 4. * t1 * t2
                px = px + nx_[i] * f
                py = py + ny_[i] * f
            pos[:, k, 0] = px
            pos[:, k, 1] = py
    else:
        zr = e // (g.nx * g.ny)
        z0, z1 = g.znodes[zr], g.znodes[zr + 1]
        xii = (-1., 1., 1., -1., -1., 1., 1., -1.)
        eti = (-1., -1., 1., 1., -1., -1., 1., 1.)
        zti = (-1., -1., -1., -1., 1., 1., 1., 1.)
        nx_ = (x0, x1, x1, x0, x0, x1, x1, x0)
        ny_ = (y0, y0, y1, y1, y0, y0, y1, y1)
        nz_ = (z0, z0, z0, z0, z1, z1, z1, z1)
        # EightNodeIsoparamBrick::ShapeFunction (9-argument form): t1*t2*t3/8
        for k in range(npp):
            px = np.zeros(ne)
            py = np.zeros(ne)
            pz = np.zeros(ne)
            for i in range(8):
                t1 = (1. + xii[i] * xi[k, 0])
                t2 = (1. + eti[i] * xi[k, 1])
                t3 = (1. + zti[i] * xi[k, 2])
                f = t1 * t2 * t3 / 8.
                px = px + nx_[i] * f
                py = py + ny_[i] * f
                pz = pz + nz_[i] * f
            pos[:, k, 0] = px
            pos[:, k, 1] = py
            pos[:, k, 2] = pz
    elem = np.repeat(e, npp)
    return pos.reshape(-1, 3), elem


def _new_particles(pos, elem, g: Grid, ppc_side: int, rho_gcc: float, thick: float):
    n = pos.shape[0]
    p = {k: np.zeros(n) for k in PARTICLE_FIELDS}
    p["x"][:] = pos[:, 0]
    p["y"][:] = pos[:, 1]
    p["z"][:] = pos[:, 2]
    p["x0"][:] = pos[:, 0]
    p["y0"][:] = pos[:, 1]
    p["z0"][:] = pos[:, 2]
    lp = 1. / float(ppc_side)
    p["lpx"][:] = lp
    p["lpy"][:] = lp
    p["lpz"][:] = lp if g.dim == 3 else 1.
    col = elem % g.nx
    row = (elem // g.nx) % g.ny
    dxe = g.xnodes[col + 1] - g.xnodes[col]
    dye = g.ynodes[row + 1] - g.ynodes[row]
    psx = dxe * (0.5 * lp)
    psy = dye * (0.5 * lp)
    rho = rho_gcc * 0.001
    if g.dim == 3:
        zr = elem // (g.nx * g.ny)
        dze = g.znodes[zr + 1] - g.znodes[zr]
        psz = dze * (0.5 * lp)
        vol = 8. * psx * psy * psz
    else:
        vol = 4. * psx * psy * thick
    p["mass"][:] = rho * vol
    p["mat"] = np.zeros(n, dtype=np.int32)
    p["elem"] = elem.astype(np.int32)
    return p


GIMP_NAMES = {"Classic": SHAPE_LINEAR, "Dirac": SHAPE_LINEAR, "uGIMP": SHAPE_UGIMP, "GIMP": SHAPE_UGIMP,
              "B2SPLINE": SHAPE_BSPLINE, "B2GIMP": SHAPE_BGIMP,
              "lCPDI": SHAPE_LCPDI, "CPDI": SHAPE_LCPDI, "qCPDI": SHAPE_QCPDI}


def _material(mat_type, rho, E=0., nu=0., yield_=0., Ep=0., G=0., K=0., uj=0):
    return dict(type=mat_type, field=0, rho=rho, E=E if mat_type != MAT_NEOHOOKEAN else 0.,
                nu=nu if mat_type != MAT_NEOHOOKEAN else 0., yield_=yield_ if mat_type == MAT_PLASTIC else 0.,
                Ep=Ep if mat_type == MAT_PLASTIC else 0., G=G if mat_type == MAT_NEOHOOKEAN else 0.,
                K=K if mat_type == MAT_NEOHOOKEAN else 0., UJOption=uj if mat_type == MAT_NEOHOOKEAN else 0)


def _initial_material_state(p, mat):
    """MaterialBase::SetInitialParticleState / InitHistoryData of the material
    for all particles of p (one body): hyperelastic B = I in the plastic-strain
    slot (HyperElastic.cpp:45-53), Neohookean history J = Jres = 1
    (Neohookean.cpp:151-156)."""
    if mat["type"] == MAT_NEOHOOKEAN:
        for k in ("pxx", "pyy", "pzz", "hist0", "hist1"):
            p[k][:] = 1.


def _xpic_options(opts: dict, xpic) -> None:
    """PeriodicXPIC settings (inputs.xpic_xml): xpic = (order, fmpm, period)."""
    if xpic:
        order, fmpm, period = xpic
        opts.update(xpic_order=int(order), xpic_fmpm=1 if fmpm else 0, xpic_period=int(period))


def cantilever_2d(nx=100, ny=20, cell=1.0, ppc_side=2, E=1000., nu=0.33, rho=1.0, v0=1000.,
                  steps=1000, cfl=0.4, gimp="uGIMP", method=USAVG, margin_cells=4, mat_type=MAT_ISO,
                  G=0., K=0., uj=0, inc_terms=0, xpic=None, **_ignored) -> Model:
    """Model of inputs.cantilever_2d (same arguments)."""
    from . import inputs
    shape = GIMP_NAMES[gimp]
    L, H, m = nx * cell, ny * cell, margin_cells * cell
    g = make_grid(2, (-m, L + m), (-m, H + m), None, cell, 1.0)
    pos, elem = _element_points(g, ppc_side)
    inside = (pos[:, 0] <= L) & (pos[:, 0] >= 0.) & (pos[:, 1] <= H) & (pos[:, 1] >= 0.)
    p = _new_particles(pos[inside], elem[inside], g, ppc_side, rho, 1.0)
    # <vel0Y> expression v0*sin(pi*x/(2*L)) (Expression.cpp evaluates left to right)
    p["vy"][:] = v0 * np.sin(math.pi * p["x"] / (2. * L))
    mats = [_material(mat_type, rho, E=E, nu=nu, G=G, K=K, uj=uj)]
    _initial_material_state(p, mats[0])
    # BCLine x=0 from y=-cell/2 to H+cell/2 (LineController::ContainsPoint with the
    # 2D tolerance test); node order is increasing node number, one DisBC at a time
    nn = g.nnodes
    ids = np.arange(1, nn + 1)
    ndx = g.xnodes[(ids - 1) % (g.nx + 1)]
    ndy = g.ynodes[(ids - 1) // (g.nx + 1)]
    on = _line_contains(ndx, ndy, 0., -0.5 * cell, 0., H + 0.5 * cell, 0.01)
    nodes = ids[on]
    bcs = np.zeros(2 * nodes.size, dtype=BC_DTYPE)
    bcs["node"][:nodes.size] = nodes
    bcs["dir"][:nodes.size] = 1
    bcs["node"][nodes.size:] = nodes
    bcs["dir"][nodes.size:] = 2
    c = inputs.wave_speed(mat_type, rho, E=E, nu=nu, G=G, K=K)
    dt = inputs.cfl_timestep(g.dx, c, cfl)  # MeshInfo::GetMinCellDimension: grid.x for square grids
    opts = dict(np=PLANE_STRAIN, method=method, shape=shape, timestep=dt, fraction_usf=0.5,
                inc_defgrad_terms=inc_terms if inc_terms > 0 else 2, nfields=1)
    _xpic_options(opts, xpic)
    return Model(g, p, mats, bcs, opts, steps, name=f"cantilever_2d_{nx}x{ny}")


def _line_contains(x, y, x1, y1, x2, y2, tol):
    """LineController::ContainsPoint, 2D branch (Common/Read_XML/LineController.cpp:33-66)."""
    distSq = (x2 - x1) * (x2 - x1) + (y2 - y1) * (y2 - y1)
    dtol = math.sqrt(distSq) * tol
    dx, dy = x2 - x1, y2 - y1
    px, py = x - x1, y - y1
    ypr = -dy * px + dx * py
    xpr = dx * px + dy * py
    return (ypr <= dtol) & (ypr >= -dtol) & (xpr >= 0.) & (xpr <= distSq)


def taylor_3d(radius=5.0, length=25.0, cell=0.25, ppc_side=2, v0=-200000., E=200000., nu=0.3,
              yield_=300., Ep=2000., rho=7.8, steps=2000, cfl=0.5, gimp="uGIMP", method=USAVG,
              lateral_margin=None, mat_type=MAT_PLASTIC, G=0., K=0., uj=0, inc_terms=0, xpic=None, **_ignored) -> Model:
    """Model of inputs.taylor_3d (same arguments)."""
    from . import inputs
    shape = GIMP_NAMES[gimp]
    lm = lateral_margin if lateral_margin is not None else max(4 * cell, 0.8 * radius)
    xr = radius + lm
    g = make_grid(3, (-xr, xr), (-xr, xr), (-4 * cell, length + 4 * cell), cell)
    pos, elem = _element_points(g, ppc_side)
    # BoxController::ContainsPoint, cylinder along z (BoxController.cpp:47-98)
    xmin, xmax, ymin, ymax, zmin, zmax = -radius, radius, -radius, radius, 0., length
    xmid, ymid = (xmin + xmax) / 2., (ymin + ymax) / 2.
    a2 = (xmax - xmid) ** 2
    b2 = (ymax - ymid) ** 2
    z = pos[:, 2]
    dz = zmax - zmin
    R = (zmax - z + 1. * (z - zmin)) / dz
    ddx = pos[:, 0] - xmid
    ddy = pos[:, 1] - ymid
    inside = (z <= zmax) & (z >= zmin) & ((ddx * ddx / a2 + ddy * ddy / b2) <= R * R)
    p = _new_particles(pos[inside], elem[inside], g, ppc_side, rho, 1.0)
    p["vz"][:] = v0
    mats = [_material(mat_type, rho, E=E, nu=nu, yield_=yield_, Ep=Ep, G=G, K=K, uj=uj)]
    _initial_material_state(p, mats[0])
    nn = g.nnodes
    ids = np.arange(1, nn + 1)
    plane = (g.nx + 1) * (g.ny + 1)
    ndx = g.xnodes[(ids - 1) % (g.nx + 1)]
    ndy = g.ynodes[((ids - 1) % plane) // (g.nx + 1)]
    ndz = g.znodes[(ids - 1) // plane]
    bx = (-xr - cell, xr + cell, -xr - cell, xr + cell, -0.01 * cell, 0.01 * cell)
    on = (ndx <= bx[1]) & (ndx >= bx[0]) & (ndy <= bx[3]) & (ndy >= bx[2]) & (ndz <= bx[5]) & (ndz >= bx[4])
    nodes = ids[on]
    bcs = np.zeros(nodes.size, dtype=BC_DTYPE)
    bcs["node"] = nodes
    bcs["dir"] = 4
    c = inputs.wave_speed(mat_type, rho, E=E, nu=nu, G=G, K=K)
    dt = inputs.cfl_timestep(g.dx, c, cfl)  # cubic grid: grid.x
    opts = dict(np=THREED, method=method, shape=shape, timestep=dt, fraction_usf=0.5,
                inc_defgrad_terms=inc_terms if inc_terms > 0 else 1, nfields=1)
    _xpic_options(opts, xpic)
    return Model(g, p, mats, bcs, opts, steps, name=f"taylor_3d_r{radius}_c{cell}")


def block_2d(ncx=40, ncy=20, cell=1.0, ppc_side=2, mat=None, vel=(1000., 0., 0., 0., 0., 0.),
             fixed_left=False, steps=500, cfl=0.4, gimp="uGIMP", method=USAVG, margin_cells=4,
             name="block_2d", **_ignored) -> Model:
    """2D plane-strain rectangle of ncx x ncy cells (ppc_side^2 points per cell)
    with the initial velocity field

        vx = a0 + a1*sin(pi*x/L + phx),   vy = b0 + b1*sin(pi*y/H + phy)

    given as vel = (a0, a1, phx, b0, b1, phy) in mm/s and radians; optionally the
    left edge (x = 0) held at zero velocity in x and y, as in cantilever_2d.
    `mat` is one material dict (default: the cantilever's elastic material)."""
    from . import inputs
    shape = GIMP_NAMES[gimp]
    L, H, m = ncx * cell, ncy * cell, margin_cells * cell
    g = make_grid(2, (-m, L + m), (-m, H + m), None, cell, 1.0)
    pos, elem = _element_points(g, ppc_side)
    inside = (pos[:, 0] <= L) & (pos[:, 0] >= 0.) & (pos[:, 1] <= H) & (pos[:, 1] >= 0.)
    mat = dict(mat) if mat is not None else dict(type=MAT_ISO, field=0, rho=1.0, E=1000., nu=0.33, yield_=0.,
                                                 Ep=0., G=0., K=0., UJOption=0)
    p = _new_particles(pos[inside], elem[inside], g, ppc_side, mat["rho"], 1.0)
    a0, a1, phx, b0, b1, phy = vel
    p["vx"][:] = a0 + a1 * np.sin(math.pi * p["x"] / L + phx)
    p["vy"][:] = b0 + b1 * np.sin(math.pi * p["y"] / H + phy)
    bcs = np.zeros(0, dtype=BC_DTYPE)
    if fixed_left:
        nn = g.nnodes
        ids = np.arange(1, nn + 1)
        ndx = g.xnodes[(ids - 1) % (g.nx + 1)]
        ndy = g.ynodes[(ids - 1) // (g.nx + 1)]
        nodes = ids[_line_contains(ndx, ndy, 0., -0.5 * cell, 0., H + 0.5 * cell, 0.01)]
        bcs = np.zeros(2 * nodes.size, dtype=BC_DTYPE)
        bcs["node"][:nodes.size] = nodes
        bcs["dir"][:nodes.size] = 1
        bcs["node"][nodes.size:] = nodes
        bcs["dir"][nodes.size:] = 2
    c = inputs.iso_wave_speed(mat["E"], mat["nu"], mat["rho"])
    dt = inputs.cfl_timestep(g.dx, c, cfl)
    opts = dict(np=PLANE_STRAIN, method=method, shape=shape, timestep=dt, fraction_usf=0.5,
                inc_defgrad_terms=2, nfields=1)
    return Model(g, p, [mat], bcs, opts, steps, name=name)


def batch_run_params(count=512, seed=2024, nmin=2000, nmax=200000, steps=500, cell=1.0, ppc_side=2, cfl=0.4):
    """Seeded parameters of a batch of independent 2D runs (keyword dicts for
    block_2d): particle counts log-uniform in [nmin, nmax]; block aspect
    log-uniform in [1, 4]; 50/50 linear elastic (type 1) or von Mises with
    linear hardening (type 9), E log-uniform 0.1-200 GPa, nu uniform 0.2-0.45,
    yield uniform 0.1-1 % of E, tangent modulus uniform 0.1-5 % of E, density
    uniform 1-8 g/cm^3; velocity field amplitude uniform 0.1-10 m/s; every
    other run with its left edge held.  The grid margin covers the largest
    displacement the amplitude allows over the run's steps."""
    from . import inputs
    rng = np.random.default_rng(seed)
    out = []
    ppc = ppc_side * ppc_side
    for k in range(count):
        n = math.exp(rng.uniform(math.log(nmin), math.log(nmax)))
        aspect = math.exp(rng.uniform(0., math.log(4.)))
        cells = max(n / ppc, 9.)
        ncy = max(3, int(round(math.sqrt(cells / aspect))))
        ncx = max(3, int(round(cells / ncy)))
        E = math.exp(rng.uniform(math.log(100.), math.log(200000.)))  # MPa: 0.1-200 GPa
        nu = rng.uniform(0.2, 0.45)
        rho = rng.uniform(1., 8.)
        plastic = rng.uniform() < 0.5
        mat = dict(type=MAT_PLASTIC if plastic else MAT_ISO, field=0, rho=rho, E=E, nu=nu,
                   yield_=rng.uniform(0.001, 0.01) * E if plastic else 0., Ep=rng.uniform(0.001, 0.05) * E if plastic else 0.,
                   G=0., K=0., UJOption=0)
        amp = 1000. * rng.uniform(0.1, 10.)  # mm/s
        w = rng.uniform(-1., 1., 4)
        w = w / np.abs(w).sum()
        vel = (amp * w[0], amp * w[1], rng.uniform(0., 2. * math.pi), amp * w[2], amp * w[3],
               rng.uniform(0., 2. * math.pi))
        dt = inputs.cfl_timestep(cell, inputs.iso_wave_speed(E, nu, rho), cfl)
        travel = amp * dt * steps / cell
        out.append(dict(ncx=ncx, ncy=ncy, cell=cell, ppc_side=ppc_side, mat=mat, vel=vel, fixed_left=(k % 2 == 1),
                        steps=steps, cfl=cfl, margin_cells=3 + int(math.ceil(travel)), name=f"batch{seed}_{k}"))
    return out


def batch_models(count=512, seed=2024, **kw) -> list:
    """The Models of batch_run_params (same arguments)."""
    return [block_2d(**p) for p in batch_run_params(count=count, seed=seed, **kw)]


def block_3d(ncx=8, ncy=8, ncz=8, cell=1.0, ppc_side=2, mat=None, vel=(0., 0., 0., 0., -1000., 0., 0., 0., 0.),
             fixed_base=False, steps=500, cfl=0.5, gimp="uGIMP", method=USAVG, margin_cells=4,
             name="block_3d", **_ignored) -> Model:
    """3D box of ncx x ncy x ncz cells (ppc_side^3 points per cell) with the
    initial velocity field

        vx = a0 + a1*sin(pi*z/Lz + pa),  vy = b0 + b1*sin(pi*x/Lx + pb),  vz = c0 + c1*sin(pi*y/Ly + pc)

    given as vel = (a0, a1, pa, b0, b1, pb, c0, c1, pc); optionally the base
    plane z = 0 held at zero z velocity (a rigid wall, as in taylor_3d)."""
    from . import inputs
    shape = GIMP_NAMES[gimp]
    Lx, Ly, Lz, m = ncx * cell, ncy * cell, ncz * cell, margin_cells * cell
    g = make_grid(3, (-m, Lx + m), (-m, Ly + m), (-m, Lz + m), cell)
    pos, elem = _element_points(g, ppc_side)
    inside = ((pos[:, 0] <= Lx) & (pos[:, 0] >= 0.) & (pos[:, 1] <= Ly) & (pos[:, 1] >= 0.)
              & (pos[:, 2] <= Lz) & (pos[:, 2] >= 0.))
    mat = dict(mat) if mat is not None else dict(type=MAT_ISO, field=0, rho=1.0, E=1000., nu=0.33, yield_=0.,
                                                 Ep=0., G=0., K=0., UJOption=0)
    p = _new_particles(pos[inside], elem[inside], g, ppc_side, mat["rho"], 1.0)
    a0, a1, pa, b0, b1, pb, c0, c1, pc = vel
    p["vx"][:] = a0 + a1 * np.sin(math.pi * p["z"] / Lz + pa)
    p["vy"][:] = b0 + b1 * np.sin(math.pi * p["x"] / Lx + pb)
    p["vz"][:] = c0 + c1 * np.sin(math.pi * p["y"] / Ly + pc)
    bcs = np.zeros(0, dtype=BC_DTYPE)
    if fixed_base:
        ids = np.arange(1, g.nnodes + 1)
        plane = (g.nx + 1) * (g.ny + 1)
        ndz = g.znodes[(ids - 1) // plane]
        nodes = ids[(ndz <= 0.01 * cell) & (ndz >= -0.01 * cell)]
        bcs = np.zeros(nodes.size, dtype=BC_DTYPE)
        bcs["node"] = nodes
        bcs["dir"] = 4
    c = inputs.iso_wave_speed(mat["E"], mat["nu"], mat["rho"])
    dt = inputs.cfl_timestep(g.dx, c, cfl)
    opts = dict(np=THREED, method=method, shape=shape, timestep=dt, fraction_usf=0.5,
                inc_defgrad_terms=1, nfields=1)
    return Model(g, p, [mat], bcs, opts, steps, name=name)


def _random_material(rng):
    """Material of the batched and served populations: 50/50 linear elastic or
    von Mises with linear hardening, E log-uniform 0.1-200 GPa, nu 0.2-0.45,
    yield 0.1-1 % of E, tangent modulus 0.1-5 % of E, density 1-8 g/cm^3."""
    E = math.exp(rng.uniform(math.log(100.), math.log(200000.)))
    nu = rng.uniform(0.2, 0.45)
    rho = rng.uniform(1., 8.)
    plastic = rng.uniform() < 0.5
    return dict(type=MAT_PLASTIC if plastic else MAT_ISO, field=0, rho=rho, E=E, nu=nu,
                yield_=rng.uniform(0.001, 0.01) * E if plastic else 0.,
                Ep=rng.uniform(0.001, 0.05) * E if plastic else 0., G=0., K=0., UJOption=0)


def serve_request_params(count=200, seed=77, rate=20.0, nmin=10000, nmax=2000000, smin=200, smax=2000,
                         cell=1.0, ppc_side=2):
    """Seeded request stream of independent runs: Poisson arrivals at `rate`
    per second, 50/50 2D plane strain or 3D, particle counts log-uniform in
    [nmin, nmax], step counts uniform in [smin, smax], materials as the batched
    population, velocity amplitude 0.1-10 m/s.  Returns (arrival_s, dim,
    kwargs of block_2d / block_3d) per request."""
    from . import inputs
    rng = np.random.default_rng(seed)
    t = 0.
    out = []
    for k in range(count):
        t += rng.exponential(1. / rate)
        dim = 3 if rng.uniform() < 0.5 else 2
        n = math.exp(rng.uniform(math.log(nmin), math.log(nmax)))
        steps = int(rng.integers(smin, smax + 1))
        mat = _random_material(rng)
        amp = 1000. * rng.uniform(0.1, 10.)
        dt = inputs.cfl_timestep(cell, inputs.iso_wave_speed(mat["E"], mat["nu"], mat["rho"]), 0.4 if dim == 2 else 0.5)
        margin = 3 + int(math.ceil(amp * dt * steps / cell))
        if dim == 2:
            cells = max(n / ppc_side ** 2, 9.)
            aspect = math.exp(rng.uniform(0., math.log(4.)))
            ncy = max(3, int(round(math.sqrt(cells / aspect))))
            ncx = max(3, int(round(cells / ncy)))
            w = rng.uniform(-1., 1., 4)
            w = w / np.abs(w).sum()
            vel = (amp * w[0], amp * w[1], rng.uniform(0., 2. * math.pi), amp * w[2], amp * w[3],
                   rng.uniform(0., 2. * math.pi))
            kw = dict(ncx=ncx, ncy=ncy, cell=cell, ppc_side=ppc_side, mat=mat, vel=vel, fixed_left=(k % 2 == 1),
                      steps=steps, cfl=0.4, margin_cells=margin, name=f"req{seed}_{k}_2d")
        else:
            cells = max(n / ppc_side ** 3, 27.)
            side = cells ** (1. / 3.)
            ncx = max(3, int(round(side * math.exp(rng.uniform(-0.3, 0.3)))))
            ncy = max(3, int(round(side * math.exp(rng.uniform(-0.3, 0.3)))))
            ncz = max(3, int(round(cells / (ncx * ncy))))
            w = rng.uniform(-1., 1., 6)
            w = w / np.abs(w).sum()
            vel = (amp * w[0], amp * w[1], rng.uniform(0., 2. * math.pi), amp * w[2], amp * w[3],
                   rng.uniform(0., 2. * math.pi), amp * w[4], amp * w[5], rng.uniform(0., 2. * math.pi))
            kw = dict(ncx=ncx, ncy=ncy, ncz=ncz, cell=cell, ppc_side=ppc_side, mat=mat, vel=vel,
                      fixed_base=(k % 2 == 1), steps=steps, cfl=0.5, margin_cells=margin, name=f"req{seed}_{k}_3d")
        out.append((t, dim, kw))
    return out


def serve_models(params) -> list:
    """Models of serve_request_params entries."""
    return [block_3d(**kw) if dim == 3 else block_2d(**kw) for _, dim, kw in params]


def _body_particles(g, pos, elem, inside, ppc_side, mat, mat_index, vel, thick=1.0):
    """Particles of one <Body> (MPMReadHandler::MPMPts): the candidate points
    inside its shape, in element order, with the body's material and velocity."""
    p = _new_particles(pos[inside], elem[inside], g, ppc_side, mat["rho"], thick)
    p["mat"][:] = mat_index
    for k, v in zip(("vx", "vy", "vz"), vel):
        p[k][:] = v
    _initial_material_state(p, mat)
    return p


def _concat(parts):
    return {k: np.concatenate([q[k] for q in parts]) for k in parts[0]}


def _contact_options(normals, friction):
    # MpmGpuContact: displacement-based separation (contact_cutoff < 0)
    return dict(enabled=1, normals=int(normals), friction=float(friction), contact_cutoff=-1., rigid_gradient_bias=1.)


def _mat_from(d, default):
    d = dict(default if d is None else d)
    t = d.pop("mat_type")
    return _material(t, d["rho"], E=d.get("E", 0.), nu=d.get("nu", 0.), yield_=d.get("yield_", 0.),
                     Ep=d.get("Ep", 0.), G=d.get("G", 0.), K=d.get("K", 0.), uj=d.get("uj", 0))


def contact_2d(plate=(20, 4), block=(6, 4), block_x0=5.0, gap=0.0, cell=1.0, ppc_side=2, v=(2000., -2000.),
               plate_mat=None, block_mat=None, friction=0.3, normals=2, steps=200, cfl=0.4, gimp="uGIMP",
               method=USAVG, margin_cells=4, inc_terms=0, xpic=None, **_ignored) -> Model:
    """Model of inputs.contact_2d (same arguments): plate in material field 0,
    block in field 1, multimaterial contact on."""
    from . import inputs
    shape = GIMP_NAMES[gimp]
    pm = _mat_from(plate_mat, dict(mat_type=MAT_ISO, rho=2.7, E=70000., nu=0.33))
    bm = _mat_from(block_mat, dict(mat_type=MAT_NEOHOOKEAN, rho=1.1, G=10., K=50.))
    pm["field"], bm["field"] = 0, 1
    Lp, Hp = plate[0] * cell, plate[1] * cell
    Lb, Hb = block[0] * cell, block[1] * cell
    y0 = Hp + gap
    m = margin_cells * cell
    g = make_grid(2, (-m, Lp + m), (-m, y0 + Hb + m), None, cell, 1.0)
    pos, elem = _element_points(g, ppc_side)
    x, y = pos[:, 0], pos[:, 1]
    in_p = (x <= Lp) & (x >= 0.) & (y <= Hp) & (y >= 0.)
    in_b = (x <= block_x0 + Lb) & (x >= block_x0) & (y <= y0 + Hb) & (y >= y0) & ~in_p
    p = _concat([_body_particles(g, pos, elem, in_p, ppc_side, pm, 0, (0., 0., 0.)),
                 _body_particles(g, pos, elem, in_b, ppc_side, bm, 1, (v[0], v[1], 0.))])
    ids = np.arange(1, g.nnodes + 1)
    ndx = g.xnodes[(ids - 1) % (g.nx + 1)]
    ndy = g.ynodes[(ids - 1) // (g.nx + 1)]
    nodes = ids[_line_contains(ndx, ndy, -0.5 * cell, 0., Lp + 0.5 * cell, 0., 0.01)]
    bcs = np.zeros(2 * nodes.size, dtype=BC_DTYPE)
    bcs["node"][:nodes.size] = nodes
    bcs["dir"][:nodes.size] = 1
    bcs["node"][nodes.size:] = nodes
    bcs["dir"][nodes.size:] = 2
    c = max(inputs.wave_speed(q["type"], q["rho"], E=q["E"], nu=q["nu"], G=q["G"], K=q["K"]) for q in (pm, bm))
    dt = inputs.cfl_timestep(g.dx, c, cfl)
    opts = dict(np=PLANE_STRAIN, method=method, shape=shape, timestep=dt, fraction_usf=0.5,
                inc_defgrad_terms=inc_terms if inc_terms > 0 else 2, nfields=2)
    _xpic_options(opts, xpic)
    return Model(g, p, [pm, bm], bcs, opts, steps, name="contact_2d",
                 extra={"contact": _contact_options(normals, friction)})


def contact_3d(plate=(12, 12, 3), block=(4, 4, 3), block_x0=4.0, block_y0=4.0, gap=0.0, cell=0.5, ppc_side=2,
               v=(4000., 0., -4000.), plate_mat=None, block_mat=None, friction=0.3, normals=2, steps=100, cfl=0.5,
               gimp="lCPDI", method=USAVG, margin_cells=4, inc_terms=0, xpic=None, **_ignored) -> Model:
    """Model of inputs.contact_3d (same arguments)."""
    from . import inputs
    shape = GIMP_NAMES[gimp]
    pm = _mat_from(plate_mat, dict(mat_type=MAT_ISO, rho=2.7, E=70000., nu=0.33))
    bm = _mat_from(block_mat, dict(mat_type=MAT_NEOHOOKEAN, rho=1.1, G=10., K=50.))
    pm["field"], bm["field"] = 0, 1
    Lx, Ly, Hp = plate[0] * cell, plate[1] * cell, plate[2] * cell
    bx, by, bz = block[0] * cell, block[1] * cell, block[2] * cell
    z0 = Hp + gap
    m = margin_cells * cell
    g = make_grid(3, (-m, Lx + m), (-m, Ly + m), (-m, z0 + bz + m), cell)
    pos, elem = _element_points(g, ppc_side)
    x, y, z = pos[:, 0], pos[:, 1], pos[:, 2]
    in_p = (x <= Lx) & (x >= 0.) & (y <= Ly) & (y >= 0.) & (z <= Hp) & (z >= 0.)
    in_b = ((x <= block_x0 + bx) & (x >= block_x0) & (y <= block_y0 + by) & (y >= block_y0) & (z <= z0 + bz)
            & (z >= z0) & ~in_p)
    p = _concat([_body_particles(g, pos, elem, in_p, ppc_side, pm, 0, (0., 0., 0.)),
                 _body_particles(g, pos, elem, in_b, ppc_side, bm, 1, v)])
    ids = np.arange(1, g.nnodes + 1)
    plane = (g.nx + 1) * (g.ny + 1)
    ndx = g.xnodes[(ids - 1) % (g.nx + 1)]
    ndy = g.ynodes[((ids - 1) % plane) // (g.nx + 1)]
    ndz = g.znodes[(ids - 1) // plane]
    bx0, bx1, by0, by1 = -m - cell, Lx + m + cell, -m - cell, Ly + m + cell
    on = (ndx <= bx1) & (ndx >= bx0) & (ndy <= by1) & (ndy >= by0) & (ndz <= 0.01 * cell) & (ndz >= -0.01 * cell)
    nodes = ids[on]
    bcs = np.zeros(3 * nodes.size, dtype=BC_DTYPE)
    for k, d in enumerate((1, 2, 4)):
        bcs["node"][k * nodes.size:(k + 1) * nodes.size] = nodes
        bcs["dir"][k * nodes.size:(k + 1) * nodes.size] = d
    c = max(inputs.wave_speed(q["type"], q["rho"], E=q["E"], nu=q["nu"], G=q["G"], K=q["K"]) for q in (pm, bm))
    dt = inputs.cfl_timestep(g.dx, c, cfl)
    opts = dict(np=THREED, method=method, shape=shape, timestep=dt, fraction_usf=0.5,
                inc_defgrad_terms=inc_terms if inc_terms > 0 else 1, nfields=2)
    _xpic_options(opts, xpic)
    return Model(g, p, [pm, bm], bcs, opts, steps, name="contact_3d",
                 extra={"contact": _contact_options(normals, friction)})


def contact_run_params(count=64, seed=303, nmin=20000, nmax=500000, steps=100, cell=0.5, ppc_side=2,
                       friction=0.3, normals=2, gimp="lCPDI"):
    """Seeded population of independent 3D two-material contact runs of the
    contact_3d form (Neo-Hookean block G 10 MPa, K 50 MPa, rho 1.1 pressed and
    sliding on a linear elastic plate 70 GPa, 0.33, rho 2.7, Coulomb friction,
    lCPDI, 0.5 mm cells, 8 points per cell): particle counts log-uniform in
    [nmin, nmax]; plate aspect log-uniform in [0.7, 1.4]; plate 3-6 cells
    thick; block a third of the plate's width and depth, 2-4 cells tall,
    placed at a random in-plate position; pressing speed uniform 2-6 m/s,
    sliding speed uniform 0-6 m/s in a random direction."""
    rng = np.random.default_rng(seed)
    per_cell = ppc_side ** 3
    out = []
    for k in range(count):
        n = math.exp(rng.uniform(math.log(nmin), math.log(nmax)))
        pz = int(rng.integers(3, 7))
        bzc = int(rng.integers(2, 5))
        aspect = math.exp(rng.uniform(math.log(0.7), math.log(1.4)))
        # plate cells px*py*pz plus block cells (px/3)(py/3)bzc make n / per_cell
        area = max(n / per_cell / (pz + bzc / 9.), 36.)
        px = max(6, int(round(math.sqrt(area * aspect))))
        py = max(6, int(round(area / px)))
        bxc, byc = max(2, px // 3), max(2, py // 3)
        bx0 = cell * int(rng.integers(0, px - bxc + 1))
        by0 = cell * int(rng.integers(0, py - byc + 1))
        press = 1000. * rng.uniform(2., 6.)
        slide = 1000. * rng.uniform(0., 6.)
        ang = rng.uniform(0., 2. * math.pi)
        out.append(dict(plate=(px, py, pz), block=(bxc, byc, bzc), block_x0=bx0, block_y0=by0, cell=cell,
                        ppc_side=ppc_side, v=(slide * math.cos(ang), slide * math.sin(ang), -press),
                        friction=friction, normals=normals, steps=steps, gimp=gimp, name=f"contact{seed}_{k}"))
    return out


def contact_models(count=64, seed=303, **kw) -> list:
    """The Models of contact_run_params (same arguments)."""
    out = []
    for p in contact_run_params(count=count, seed=seed, **kw):
        name = p.pop("name")
        m = contact_3d(**p)
        m.name = name
        out.append(m)
    return out


# A rigid contact material (RigidMaterial, type 35): rho = 1 g/mm^3 in the
# reference's units, so each particle's mass is its volume in mm^3 (1000 g/cm^3
# here, which _new_particles scales by 1e-3 to exactly 1).
RIGID_RHO_GCC = 1000.


def _rigid_material():
    return dict(type=MAT_RIGID, field=0, rho=RIGID_RHO_GCC, E=0., nu=0., yield_=0., Ep=0., G=0., K=0., UJOption=0)


def rigid_contact_2d(plate=(20, 4), indenter=(6, 3), indenter_x0=7.0, gap=0.5, cell=1.0, ppc_side=2,
                     v=(0., -2000.), plate_mat=None, friction=0.3, normals=2, steps=150, cfl=0.4, gimp="uGIMP",
                     method=USAVG, margin_cells=4, inc_terms=0, **_ignored) -> Model:
    """Model of inputs.rigid_contact_2d (same arguments): elastic plate in
    material field 0 (base held), rigid indenter in field 1 moving at v."""
    from . import inputs
    shape = GIMP_NAMES[gimp]
    pm = _mat_from(plate_mat, dict(mat_type=MAT_ISO, rho=2.7, E=70000., nu=0.33))
    rm = _rigid_material()
    pm["field"], rm["field"] = 0, 1
    Lp, Hp = plate[0] * cell, plate[1] * cell
    Li, Hi = indenter[0] * cell, indenter[1] * cell
    y0 = Hp + gap
    m = margin_cells * cell
    g = make_grid(2, (-m, Lp + m), (-m, y0 + Hi + m), None, cell, 1.0)
    pos, elem = _element_points(g, ppc_side)
    x, y = pos[:, 0], pos[:, 1]
    in_p = (x <= Lp) & (x >= 0.) & (y <= Hp) & (y >= 0.)
    in_i = (x <= indenter_x0 + Li) & (x >= indenter_x0) & (y <= y0 + Hi) & (y >= y0) & ~in_p
    p = _concat([_body_particles(g, pos, elem, in_p, ppc_side, pm, 0, (0., 0., 0.)),
                 _body_particles(g, pos, elem, in_i, ppc_side, rm, 1, (v[0], v[1], 0.))])
    ids = np.arange(1, g.nnodes + 1)
    ndx = g.xnodes[(ids - 1) % (g.nx + 1)]
    ndy = g.ynodes[(ids - 1) // (g.nx + 1)]
    nodes = ids[_line_contains(ndx, ndy, -0.5 * cell, 0., Lp + 0.5 * cell, 0., 0.01)]
    bcs = np.zeros(2 * nodes.size, dtype=BC_DTYPE)
    bcs["node"][:nodes.size] = nodes
    bcs["dir"][:nodes.size] = 1
    bcs["node"][nodes.size:] = nodes
    bcs["dir"][nodes.size:] = 2
    c = inputs.wave_speed(pm["type"], pm["rho"], E=pm["E"], nu=pm["nu"], G=pm["G"], K=pm["K"])
    dt = inputs.cfl_timestep(g.dx, c, cfl)
    opts = dict(np=PLANE_STRAIN, method=method, shape=shape, timestep=dt, fraction_usf=0.5,
                inc_defgrad_terms=inc_terms if inc_terms > 0 else 2, nfields=2)
    return Model(g, p, [pm, rm], bcs, opts, steps, name="rigid_contact_2d",
                 extra={"contact": _contact_options(normals, friction)})


def rigid_taylor_3d(radius=1.0, length=2.0, cell=0.5, ppc_side=2, v0=-200000., E=200000., nu=0.3, yield_=300.,
                    Ep=2000., rho=7.8, slab_cells=2, vx0=0., friction=0.0, normals=2, steps=40, cfl=0.5, gimp="uGIMP",
                    method=USAVG, inc_terms=0, **_ignored) -> Model:
    """Model of inputs.rigid_taylor_3d (same arguments): the bar in material
    field 0, the stationary rigid slab (z in [-slab_cells*cell, 0]) in field 1,
    no grid velocity conditions."""
    from . import inputs
    shape = GIMP_NAMES[gimp]
    lm = max(4 * cell, 0.8 * radius)
    xr = radius + lm
    zs = slab_cells * cell
    g = make_grid(3, (-xr, xr), (-xr, xr), (-zs - 4 * cell, length + 4 * cell), cell)
    pos, elem = _element_points(g, ppc_side)
    # BoxController::ContainsPoint, cylinder along z (BoxController.cpp:47-98)
    xmin, xmax, ymin, ymax, zmin, zmax = -radius, radius, -radius, radius, 0., length
    xmid, ymid = (xmin + xmax) / 2., (ymin + ymax) / 2.
    a2 = (xmax - xmid) ** 2
    b2 = (ymax - ymid) ** 2
    x, y, z = pos[:, 0], pos[:, 1], pos[:, 2]
    R = (zmax - z + 1. * (z - zmin)) / (zmax - zmin)
    ddx, ddy = x - xmid, y - ymid
    in_bar = (z <= zmax) & (z >= zmin) & ((ddx * ddx / a2 + ddy * ddy / b2) <= R * R)
    in_slab = ((x <= xr - cell) & (x >= -xr + cell) & (y <= xr - cell) & (y >= -xr + cell) & (z <= 0.)
               & (z >= -zs) & ~in_bar)
    bm = _material(MAT_PLASTIC, rho, E=E, nu=nu, yield_=yield_, Ep=Ep)
    rm = _rigid_material()
    bm["field"], rm["field"] = 0, 1
    p = _concat([_body_particles(g, pos, elem, in_bar, ppc_side, bm, 0, (vx0, 0., v0)),
                 _body_particles(g, pos, elem, in_slab, ppc_side, rm, 1, (0., 0., 0.))])
    bcs = np.zeros(0, dtype=BC_DTYPE)
    c = inputs.wave_speed(MAT_PLASTIC, rho, E=E, nu=nu)
    dt = inputs.cfl_timestep(g.dx, c, cfl)
    opts = dict(np=THREED, method=method, shape=shape, timestep=dt, fraction_usf=0.5,
                inc_defgrad_terms=inc_terms if inc_terms > 0 else 1, nfields=2)
    return Model(g, p, [bm, rm], bcs, opts, steps, name=f"rigid_taylor_3d_r{radius}_c{cell}",
                 extra={"contact": _contact_options(normals, friction)})
