"""Seeded synthetic NairnMPM XML inputs for the explicit-step workloads.

The files use only the reference's own input vocabulary (NairnMPM/input/NairnMPM.dtd;
handlers in NairnMPM/src/Read_MPM/MPMReadHandler.cpp and Generators.cpp), so the
same file runs through the reference NairnMPM and through this project's host
reader.  Units are NairnMPM "Legacy" units: mm, g/cm^3, MPa, mm/s, ms.

Workloads (sizes are parameters so tests can run small copies):
  cantilever_2d  -- 2D plane-strain elastic cantilever, uGIMP, USAVG
  taylor_3d      -- 3D von Mises (linear hardening) Taylor bar onto a rigid wall
"""
from __future__ import annotations

import math

# IsotropicMat::WaveSpeed (NairnMPM/src/Materials/MoreIsotropicMat.cpp:388-395)
# evaluated in the reference's units: G in Pa, rho in g/mm^3 -> mm/s.


def iso_wave_speed(E_mpa: float, nu: float, rho_gcc: float) -> float:
    E = E_mpa * 1.e6
    G = E / (2. * (1. + nu))
    rho = rho_gcc * 0.001
    return math.sqrt(2. * G * (1. - nu) / (rho * (1. - 2. * nu)))


def neo_wave_speed(G_mpa: float, K_mpa: float, rho_gcc: float) -> float:
    """Neohookean::WaveSpeed (NairnMPM/src/Materials/Neohookean.cpp:359), mm/s."""
    return math.sqrt((K_mpa * 1.e6 + 4. * G_mpa * 1.e6 / 3.) / (rho_gcc * 0.001))


def wave_speed(mat_type: int, rho: float, E: float = 0., nu: float = 0., G: float = 0., K: float = 0.) -> float:
    return neo_wave_speed(G, K, rho) if mat_type == 28 else iso_wave_speed(E, nu, rho)


def material_xml(mat_type: int, name: str, rho: float = 1., E: float = 0., nu: float = 0., yield_: float = 0.,
                 Ep: float = 0., G: float = 0., K: float = 0., uj: int = 0) -> str:
    """<Material> block of type 1 (IsotropicMat), 9 (IsoPlasticity with linear
    hardening), 28 (Neohookean, G and K input, U(J) option uj) or 35 (rigid
    contact material, RigidMaterial in multimaterial mode: no properties)."""
    if mat_type == 35:
        return f'  <Material Type="35" Name="{name}">\n  </Material>\n'
    body = f"    <rho>{_fmt(rho)}</rho>\n"
    if mat_type == 28:
        body += f"    <G>{_fmt(G)}</G>\n    <K>{_fmt(K)}</K>\n    <UJOption>{int(uj)}</UJOption>\n"
    else:
        body += f"    <E>{_fmt(E)}</E>\n    <nu>{_fmt(nu)}</nu>\n"
    body += "    <alpha>0</alpha>\n"
    if mat_type == 9:
        body += f"    <yield>{_fmt(yield_)}</yield>\n    <Ep>{_fmt(Ep)}</Ep>\n"
    return f'  <Material Type="{mat_type}" Name="{name}">\n{body}  </Material>\n'


def cfl_timestep(cell_mm: float, wave_speed: float, cfl: float) -> float:
    """Time step of NairnMPM::CFLTimeStep (NairnMPM.cpp:1207-1240), seconds."""
    return cfl * (cell_mm / wave_speed)


def _fmt(v: float) -> str:
    return repr(float(v))


def _header(analysis: int, method: int, gimp: str, maxtime_s: float, cfl: float,
            archive_root: str, ppe: int, order: str, inc_terms: int = 0) -> str:
    # <DefGradTerms> sets MaterialBase::incrementalDefGradTerms (MPMReadHandler.cpp:492-495)
    terms = f"    <DefGradTerms>{int(inc_terms)}</DefGradTerms>\n" if inc_terms > 0 else ""
    return f"""<?xml version='1.0'?>
<!DOCTYPE JANFEAInput SYSTEM "NairnMPM.dtd">
<JANFEAInput version='3'>
  <Header>
    <Description>synthetic workload</Description>
    <Analysis>{analysis}</Analysis>
  </Header>
  <MPMHeader>
    <MPMMethod>{method}</MPMMethod>
    <GIMP type="{gimp}"/>
    <MatlPtsPerElement>{ppe}</MatlPtsPerElement>
    <Timing CFL="{_fmt(cfl)}"/>
    <MaxTime units="ms">{_fmt(maxtime_s * 1.e3)}</MaxTime>
    <ArchiveTime units="ms">{_fmt(maxtime_s * 1.e3 * 10.)}</ArchiveTime>
    <ArchiveRoot>{archive_root}</ArchiveRoot>
    <MPMArchiveOrder>{order}</MPMArchiveOrder>
{terms}  </MPMHeader>
"""


def xpic_xml(xpic) -> str:
    """The PeriodicXPIC custom task (Custom_Tasks/PeriodicXPIC.cpp:55-145) for
    xpic = (order, fmpm, period): XPICOrder (or FMPMOrder when fmpm) on every
    period-th step; empty for None."""
    if not xpic:
        return ""
    order, fmpm, period = xpic
    key = "FMPMOrder" if fmpm else "XPICOrder"
    return f"""  <CustomTasks>
    <Schedule name='PeriodicXPIC'>
      <Parameter name='{key}'>{int(order)}</Parameter>
      <Parameter name='periodicSteps'>{int(period)}</Parameter>
    </Schedule>
  </CustomTasks>
"""


# archive items: velocity, stress, strain, plastic strain, work energy,
# plastic energy, history 1 (ArchiveData.hpp:22-32)
ARCHIVE_ORDER = "iYYYYYNYNYNNNYNNNN"


def cantilever_2d(nx: int = 100, ny: int = 20, cell: float = 1.0, ppc_side: int = 2,
                  E: float = 1000., nu: float = 0.33, rho: float = 1.0, v0: float = 1000.,
                  steps: int = 1000, cfl: float = 0.4, gimp: str = "uGIMP", method: int = 2,
                  margin_cells: int = 4, archive_root: str = "Results/cant.", mat_type: int = 1,
                  G: float = 0., K: float = 0., uj: int = 0, inc_terms: int = 0, xpic=None) -> tuple[str, dict]:
    """2D plane-strain cantilever of nx*ny cells, left edge fixed, initial
    v_y = v0*sin(pi*x/(2L)) (mm/s); elastic (mat_type 1, E and nu) or
    Neo-Hookean (mat_type 28, G and K).  Returns (xml, info)."""
    L = nx * cell
    H = ny * cell
    c = wave_speed(mat_type, rho, E=E, nu=nu, G=G, K=K)
    dt = cfl_timestep(cell, c, cfl)
    maxtime = (steps - 0.5) * dt
    m = margin_cells * cell
    xml = _header(10, method, gimp, maxtime, cfl, archive_root, ppc_side * ppc_side, ARCHIVE_ORDER, inc_terms)
    xml += f"""  <Mesh output="file">
    <Grid xmin="{_fmt(-m)}" xmax="{_fmt(L + m)}" ymin="{_fmt(-m)}" ymax="{_fmt(H + m)}" thickness="1">
      <Horiz cellsize="{_fmt(cell)}"/>
      <Vert cellsize="{_fmt(cell)}"/>
    </Grid>
  </Mesh>
  <MaterialPoints>
    <Body mat="1" angle="0" thick="1" vx="0" vy="0">
      <!-- velocity expressions apply to the shapes that follow them -->
      <vel0Y>{_fmt(v0)}*sin(pi*x/(2*{_fmt(L)}))</vel0Y>
      <Rect xmin="0" xmax="{_fmt(L)}" ymin="0" ymax="{_fmt(H)}"/>
    </Body>
  </MaterialPoints>
{material_xml(mat_type, "beam", rho, E=E, nu=nu, G=G, K=K, uj=uj)}  <GridBCs>
    <BCLine x1="0" y1="{_fmt(-0.5 * cell)}" x2="0" y2="{_fmt(H + 0.5 * cell)}" tolerance="{_fmt(0.01)}">
      <DisBC dir="1" disp="0"/>
      <DisBC dir="2" disp="0"/>
    </BCLine>
  </GridBCs>
{xpic_xml(xpic)}</JANFEAInput>
"""
    return xml, {"dt": dt, "steps": steps, "maxtime": maxtime, "dim": 2}


def taylor_3d(radius: float = 5.0, length: float = 25.0, cell: float = 0.25, ppc_side: int = 2,
              v0: float = -200000., E: float = 200000., nu: float = 0.3, yield_: float = 300.,
              Ep: float = 2000., rho: float = 7.8, steps: int = 2000, cfl: float = 0.5,
              gimp: str = "uGIMP", method: int = 2, lateral_margin: float | None = None,
              archive_root: str = "Results/taylor.", mat_type: int = 9, G: float = 0., K: float = 0.,
              uj: int = 0, inc_terms: int = 0, xpic=None) -> tuple[str, dict]:
    """3D Taylor impact: cylinder along z from z=0 to z=length moving at v0
    (mm/s) onto a rigid wall at z=0 (zero z-velocity on the z=0 node plane);
    von Mises (mat_type 9), elastic (1) or Neo-Hookean (28)."""
    c = wave_speed(mat_type, rho, E=E, nu=nu, G=G, K=K)
    dt = cfl_timestep(cell, c, cfl)
    maxtime = (steps - 0.5) * dt
    lm = lateral_margin if lateral_margin is not None else max(4 * cell, 0.8 * radius)
    xr = radius + lm
    xml = _header(12, method, gimp, maxtime, cfl, archive_root, ppc_side ** 3, ARCHIVE_ORDER, inc_terms)
    xml += f"""  <Mesh output="file">
    <Grid xmin="{_fmt(-xr)}" xmax="{_fmt(xr)}" ymin="{_fmt(-xr)}" ymax="{_fmt(xr)}" zmin="{_fmt(-4 * cell)}" zmax="{_fmt(length + 4 * cell)}">
      <Horiz cellsize="{_fmt(cell)}"/>
      <Vert cellsize="{_fmt(cell)}"/>
      <Depth cellsize="{_fmt(cell)}"/>
    </Grid>
  </Mesh>
  <MaterialPoints>
    <Body mat="1" angle="0" vx="0" vy="0" vz="{_fmt(v0)}">
      <Cylinder xmin="{_fmt(-radius)}" xmax="{_fmt(radius)}" ymin="{_fmt(-radius)}" ymax="{_fmt(radius)}" zmin="0" zmax="{_fmt(length)}" axis="z"/>
    </Body>
  </MaterialPoints>
{material_xml(mat_type, "bar", rho, E=E, nu=nu, yield_=yield_, Ep=Ep, G=G, K=K, uj=uj)}  <GridBCs>
    <BCBox xmin="{_fmt(-xr - cell)}" xmax="{_fmt(xr + cell)}" ymin="{_fmt(-xr - cell)}" ymax="{_fmt(xr + cell)}" zmin="{_fmt(-0.01 * cell)}" zmax="{_fmt(0.01 * cell)}">
      <DisBC dir="3" disp="0"/>
    </BCBox>
  </GridBCs>
{xpic_xml(xpic)}</JANFEAInput>
"""
    return xml, {"dt": dt, "steps": steps, "maxtime": maxtime, "dim": 3}


def _mm_mode(normals: int, friction: float) -> str:
    """<MultiMaterialMode> with the normal method and a Coulomb friction law
    (<Friction>: < 0 stick, 0 frictionless; ContactLaw::ConvertOldStyleToContactLaw)."""
    return (f'    <MultiMaterialMode Normals="{int(normals)}">\n'
            f'      <Friction>{_fmt(friction)}</Friction>\n'
            f'    </MultiMaterialMode>\n')


def contact_2d(plate=(20, 4), block=(6, 4), block_x0=5.0, gap=0.0, cell=1.0, ppc_side=2, v=(2000., -2000.),
               plate_mat=None, block_mat=None, friction=0.3, normals=2, steps=200, cfl=0.4, gimp="uGIMP",
               method=2, margin_cells=4, archive_root: str = "Results/contact.", inc_terms: int = 0,
               xpic=None) -> tuple[str, dict]:
    """2D plane-strain multimaterial contact: a block (plate=(nx, ny) and
    block=(nx, ny) in cells) moving at v onto an elastic plate whose base is
    held; materials (type, properties) as dicts for material_xml; optionally
    a PeriodicXPIC task (xpic_xml)."""
    pm = dict(mat_type=1, rho=2.7, E=70000., nu=0.33) if plate_mat is None else dict(plate_mat)
    bm = dict(mat_type=28, rho=1.1, G=10., K=50.) if block_mat is None else dict(block_mat)
    Lp, Hp = plate[0] * cell, plate[1] * cell
    Lb, Hb = block[0] * cell, block[1] * cell
    y0 = Hp + gap
    c = max(wave_speed(pm["mat_type"], pm["rho"], E=pm.get("E", 0.), nu=pm.get("nu", 0.), G=pm.get("G", 0.),
                       K=pm.get("K", 0.)),
            wave_speed(bm["mat_type"], bm["rho"], E=bm.get("E", 0.), nu=bm.get("nu", 0.), G=bm.get("G", 0.),
                       K=bm.get("K", 0.)))
    dt = cfl_timestep(cell, c, cfl)
    maxtime = (steps - 0.5) * dt
    m = margin_cells * cell
    xml = _header(10, method, gimp, maxtime, cfl, archive_root, ppc_side * ppc_side, ARCHIVE_ORDER, inc_terms)
    xml = xml.replace("  </MPMHeader>\n", _mm_mode(normals, friction) + "  </MPMHeader>\n")
    xml += f"""  <Mesh output="file">
    <Grid xmin="{_fmt(-m)}" xmax="{_fmt(Lp + m)}" ymin="{_fmt(-m)}" ymax="{_fmt(y0 + Hb + m)}" thickness="1">
      <Horiz cellsize="{_fmt(cell)}"/>
      <Vert cellsize="{_fmt(cell)}"/>
    </Grid>
  </Mesh>
  <MaterialPoints>
    <Body mat="1" angle="0" thick="1" vx="0" vy="0">
      <Rect xmin="0" xmax="{_fmt(Lp)}" ymin="0" ymax="{_fmt(Hp)}"/>
    </Body>
    <Body mat="2" angle="0" thick="1" vx="{_fmt(v[0])}" vy="{_fmt(v[1])}">
      <Rect xmin="{_fmt(block_x0)}" xmax="{_fmt(block_x0 + Lb)}" ymin="{_fmt(y0)}" ymax="{_fmt(y0 + Hb)}"/>
    </Body>
  </MaterialPoints>
{material_xml(pm.pop("mat_type"), "plate", **pm)}{material_xml(bm.pop("mat_type"), "block", **bm)}  <GridBCs>
    <BCLine x1="{_fmt(-0.5 * cell)}" y1="0" x2="{_fmt(Lp + 0.5 * cell)}" y2="0" tolerance="{_fmt(0.01)}">
      <DisBC dir="1" disp="0"/>
      <DisBC dir="2" disp="0"/>
    </BCLine>
  </GridBCs>
{xpic_xml(xpic)}</JANFEAInput>
"""
    return xml, {"dt": dt, "steps": steps, "maxtime": maxtime, "dim": 2}


def contact_3d(plate=(12, 12, 3), block=(4, 4, 3), block_x0=4.0, block_y0=4.0, gap=0.0, cell=0.5, ppc_side=2,
               v=(4000., 0., -4000.), plate_mat=None, block_mat=None, friction=0.3, normals=2, steps=100, cfl=0.5,
               gimp="lCPDI", method=2, margin_cells=4, archive_root: str = "Results/contact3.",
               inc_terms: int = 0, xpic=None) -> tuple[str, dict]:
    """3D multimaterial contact (the config-3 form): a Neo-Hookean block
    pressed and sliding on an elastic plate whose base plane is held;
    optionally a PeriodicXPIC task (xpic_xml)."""
    pm = dict(mat_type=1, rho=2.7, E=70000., nu=0.33) if plate_mat is None else dict(plate_mat)
    bm = dict(mat_type=28, rho=1.1, G=10., K=50.) if block_mat is None else dict(block_mat)
    Lx, Ly, Hp = plate[0] * cell, plate[1] * cell, plate[2] * cell
    bx, by, bz = block[0] * cell, block[1] * cell, block[2] * cell
    z0 = Hp + gap
    c = max(wave_speed(pm["mat_type"], pm["rho"], E=pm.get("E", 0.), nu=pm.get("nu", 0.), G=pm.get("G", 0.),
                       K=pm.get("K", 0.)),
            wave_speed(bm["mat_type"], bm["rho"], E=bm.get("E", 0.), nu=bm.get("nu", 0.), G=bm.get("G", 0.),
                       K=bm.get("K", 0.)))
    dt = cfl_timestep(cell, c, cfl)
    maxtime = (steps - 0.5) * dt
    m = margin_cells * cell
    xml = _header(12, method, gimp, maxtime, cfl, archive_root, ppc_side ** 3, ARCHIVE_ORDER, inc_terms)
    xml = xml.replace("  </MPMHeader>\n", _mm_mode(normals, friction) + "  </MPMHeader>\n")
    xml += f"""  <Mesh output="file">
    <Grid xmin="{_fmt(-m)}" xmax="{_fmt(Lx + m)}" ymin="{_fmt(-m)}" ymax="{_fmt(Ly + m)}" zmin="{_fmt(-m)}" zmax="{_fmt(z0 + bz + m)}">
      <Horiz cellsize="{_fmt(cell)}"/>
      <Vert cellsize="{_fmt(cell)}"/>
      <Depth cellsize="{_fmt(cell)}"/>
    </Grid>
  </Mesh>
  <MaterialPoints>
    <Body mat="1" angle="0" vx="0" vy="0" vz="0">
      <Box xmin="0" xmax="{_fmt(Lx)}" ymin="0" ymax="{_fmt(Ly)}" zmin="0" zmax="{_fmt(Hp)}"/>
    </Body>
    <Body mat="2" angle="0" vx="{_fmt(v[0])}" vy="{_fmt(v[1])}" vz="{_fmt(v[2])}">
      <Box xmin="{_fmt(block_x0)}" xmax="{_fmt(block_x0 + bx)}" ymin="{_fmt(block_y0)}" ymax="{_fmt(block_y0 + by)}" zmin="{_fmt(z0)}" zmax="{_fmt(z0 + bz)}"/>
    </Body>
  </MaterialPoints>
{material_xml(pm.pop("mat_type"), "plate", **pm)}{material_xml(bm.pop("mat_type"), "block", **bm)}  <GridBCs>
    <BCBox xmin="{_fmt(-m - cell)}" xmax="{_fmt(Lx + m + cell)}" ymin="{_fmt(-m - cell)}" ymax="{_fmt(Ly + m + cell)}" zmin="{_fmt(-0.01 * cell)}" zmax="{_fmt(0.01 * cell)}">
      <DisBC dir="1" disp="0"/>
      <DisBC dir="2" disp="0"/>
      <DisBC dir="3" disp="0"/>
    </BCBox>
  </GridBCs>
{xpic_xml(xpic)}</JANFEAInput>
"""
    return xml, {"dt": dt, "steps": steps, "maxtime": maxtime, "dim": 3}


def rigid_contact_2d(plate=(20, 4), indenter=(6, 3), indenter_x0=7.0, gap=0.5, cell=1.0, ppc_side=2,
                     v=(0., -2000.), plate_mat=None, friction=0.3, normals=2, steps=150, cfl=0.4, gimp="uGIMP",
                     method=2, margin_cells=4, archive_root: str = "Results/rigid.", inc_terms: int = 0) -> tuple[str, dict]:
    """2D plane-strain contact with a rigid material: a rigid indenter
    (RigidMaterial type 35, moving at the constant velocity v) pressed into
    an elastic plate whose base is held.  The plate's body comes first, so the
    reference keeps the particles in input order (non-rigid first)."""
    pm = dict(mat_type=1, rho=2.7, E=70000., nu=0.33) if plate_mat is None else dict(plate_mat)
    Lp, Hp = plate[0] * cell, plate[1] * cell
    Li, Hi = indenter[0] * cell, indenter[1] * cell
    y0 = Hp + gap
    c = wave_speed(pm["mat_type"], pm["rho"], E=pm.get("E", 0.), nu=pm.get("nu", 0.), G=pm.get("G", 0.),
                   K=pm.get("K", 0.))
    dt = cfl_timestep(cell, c, cfl)
    maxtime = (steps - 0.5) * dt
    m = margin_cells * cell
    xml = _header(10, method, gimp, maxtime, cfl, archive_root, ppc_side * ppc_side, ARCHIVE_ORDER, inc_terms)
    xml = xml.replace("  </MPMHeader>\n", _mm_mode(normals, friction) + "  </MPMHeader>\n")
    xml += f"""  <Mesh output="file">
    <Grid xmin="{_fmt(-m)}" xmax="{_fmt(Lp + m)}" ymin="{_fmt(-m)}" ymax="{_fmt(y0 + Hi + m)}" thickness="1">
      <Horiz cellsize="{_fmt(cell)}"/>
      <Vert cellsize="{_fmt(cell)}"/>
    </Grid>
  </Mesh>
  <MaterialPoints>
    <Body mat="1" angle="0" thick="1" vx="0" vy="0">
      <Rect xmin="0" xmax="{_fmt(Lp)}" ymin="0" ymax="{_fmt(Hp)}"/>
    </Body>
    <Body mat="2" angle="0" thick="1" vx="{_fmt(v[0])}" vy="{_fmt(v[1])}">
      <Rect xmin="{_fmt(indenter_x0)}" xmax="{_fmt(indenter_x0 + Li)}" ymin="{_fmt(y0)}" ymax="{_fmt(y0 + Hi)}"/>
    </Body>
  </MaterialPoints>
{material_xml(pm.pop("mat_type"), "plate", **pm)}{material_xml(35, "indenter")}  <GridBCs>
    <BCLine x1="{_fmt(-0.5 * cell)}" y1="0" x2="{_fmt(Lp + 0.5 * cell)}" y2="0" tolerance="{_fmt(0.01)}">
      <DisBC dir="1" disp="0"/>
      <DisBC dir="2" disp="0"/>
    </BCLine>
  </GridBCs>
</JANFEAInput>
"""
    return xml, {"dt": dt, "steps": steps, "maxtime": maxtime, "dim": 2}


def rigid_taylor_3d(radius: float = 1.0, length: float = 2.0, cell: float = 0.5, ppc_side: int = 2,
                    v0: float = -200000., E: float = 200000., nu: float = 0.3, yield_: float = 300.,
                    Ep: float = 2000., rho: float = 7.8, slab_cells: int = 2, vx0: float = 0., friction: float = 0.0,
                    normals: int = 2, steps: int = 40, cfl: float = 0.5, gimp: str = "uGIMP", method: int = 2,
                    archive_root: str = "Results/rtaylor.", inc_terms: int = 0) -> tuple[str, dict]:
    """The Taylor impact with a rigid wall made of particles: the bar
    (von Mises, linear hardening) moving at v0 (mm/s; vx0 along x for an
    oblique impact) onto a stationary slab of
    rigid contact material (type 35) occupying -slab_cells*cell <= z <= 0,
    in place of the zero-velocity grid condition on the z = 0 plane;
    multimaterial contact with Coulomb friction."""
    c = wave_speed(9, rho, E=E, nu=nu)
    dt = cfl_timestep(cell, c, cfl)
    maxtime = (steps - 0.5) * dt
    lm = max(4 * cell, 0.8 * radius)
    xr = radius + lm
    zs = slab_cells * cell
    xml = _header(12, method, gimp, maxtime, cfl, archive_root, ppc_side ** 3, ARCHIVE_ORDER, inc_terms)
    xml = xml.replace("  </MPMHeader>\n", _mm_mode(normals, friction) + "  </MPMHeader>\n")
    xml += f"""  <Mesh output="file">
    <Grid xmin="{_fmt(-xr)}" xmax="{_fmt(xr)}" ymin="{_fmt(-xr)}" ymax="{_fmt(xr)}" zmin="{_fmt(-zs - 4 * cell)}" zmax="{_fmt(length + 4 * cell)}">
      <Horiz cellsize="{_fmt(cell)}"/>
      <Vert cellsize="{_fmt(cell)}"/>
      <Depth cellsize="{_fmt(cell)}"/>
    </Grid>
  </Mesh>
  <MaterialPoints>
    <Body mat="1" angle="0" vx="{_fmt(vx0)}" vy="0" vz="{_fmt(v0)}">
      <Cylinder xmin="{_fmt(-radius)}" xmax="{_fmt(radius)}" ymin="{_fmt(-radius)}" ymax="{_fmt(radius)}" zmin="0" zmax="{_fmt(length)}" axis="z"/>
    </Body>
    <Body mat="2" angle="0" vx="0" vy="0" vz="0">
      <Box xmin="{_fmt(-xr + cell)}" xmax="{_fmt(xr - cell)}" ymin="{_fmt(-xr + cell)}" ymax="{_fmt(xr - cell)}" zmin="{_fmt(-zs)}" zmax="0"/>
    </Body>
  </MaterialPoints>
{material_xml(9, "bar", rho, E=E, nu=nu, yield_=yield_, Ep=Ep)}{material_xml(35, "wall")}</JANFEAInput>
"""
    return xml, {"dt": dt, "steps": steps, "maxtime": maxtime, "dim": 3}
