"""OPTIMET-3D's own interface for the sphere path, on top of the GB300 library.

This module mirrors what a user of the reference drives: the XML case file
(``simulation_input``, Reader.cpp:55-101,581-663,781-960), the model objects
(``Geometry``, ``Scatterer``, ``ElectroMagnetic``, ``Excitation``), the solver
factory and ``AbstractSolver`` (Solver.h:62-144, Solver.cpp:30-54), ``Result``
(cross sections and fields, Result.cpp) and ``Simulation`` with its two run
modes (Simulation.cpp:34-63): the wavelength scan (outputType 11, which writes
``<case>_AbsorptionCS_FF.dat``, ``<case>_ScatteringCS_FF.dat`` and, with SH
sources, ``<case>_ScatteringCS_SH.dat`` / ``<case>_AbsorptionCS_SH.dat`` in the
reference's "lambda<TAB>value" format) and the field map (outputType 0). The
reference writes fields to HDF5 (Output.cpp, OutputGrid.cpp, out of scope);
here ``<case>_FF.npz`` / ``<case>_SH.npz`` hold the grid points and E, H.

Everything numeric runs on the GPU through the C ABI; there is no CPU path.

    python -m optimet_gb300.optimet case.xml [--precision c64]
"""
from __future__ import annotations

import argparse
import math
import os
import sys
import xml.etree.ElementTree as ET
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import (ACA, C64, C128, FF, SH, SOLVE_FGMRES_MIXED, SOLVE_GMRES, SOLVE_LU, Context,
               Problem, medium, options, plane_wave, spheres_array)
from . import materials

FRNM_TO_M = 1e-9  # consFrnmTom (constants.cpp)


# ---------------------------------------------------------------------------
# Model objects
# ---------------------------------------------------------------------------
@dataclass
class ElectroMagnetic:
    """Relative material parameters of a sphere or the background
    (ElectroMagnetic::init_r, ElectroMagnetic.cpp:34-56); the dispersive
    models (GoldModel with its a, b, d parameters, SiliconModel) are
    re-evaluated by update(wavelength) (ElectroMagnetic::update,
    ElectroMagnetic.cpp:226-241)."""
    epsilon_r: complex = 1.0
    mu_r: complex = 1.0
    epsilon_r_SH: complex = 1.0
    ksippp: complex = 0.0
    ksiparppar: complex = 0.0
    gamma: complex = 0.0
    model: str = "relative"
    a_SH: complex = 0.0
    b_SH: complex = 0.0
    d_SH: complex = 0.0

    def update(self, wavelength: float):
        if self.model == "GoldModel":
            vals = materials.gold(wavelength, self.a_SH, self.b_SH, self.d_SH)
        elif self.model == "SiliconModel":
            vals = materials.silicon(wavelength)
        else:
            return
        (self.epsilon_r, self.epsilon_r_SH, self.ksippp, self.ksiparppar,
         self.gamma) = (complex(v) for v in vals)


@dataclass
class Scatterer:
    """A sphere: centre (metres, Cartesian), radius, material, nMax."""
    vR: np.ndarray
    radius: float
    elmag: ElectroMagnetic
    nMax: int
    scatterer_type: str = "sphere"


@dataclass
class Geometry:
    objects: List[Scatterer] = field(default_factory=list)
    bground: ElectroMagnetic = field(default_factory=ElectroMagnetic)
    ACA_cond: bool = False

    def nMax(self) -> int:
        return self.objects[0].nMax if self.objects else 0

    def nMaxS(self) -> int:
        return self.nMax()

    def pushObject(self, s: Scatterer):
        """Geometry::pushObject (Geometry.cpp:37-55): overlapping spheres are rejected."""
        for o in self.objects:
            if np.linalg.norm(o.vR - s.vR) <= o.radius + s.radius:
                raise RuntimeError("Objects overlap")
        self.objects.append(s)


@dataclass
class Excitation:
    """Plane wave (Excitation.cpp:31-137): wavelength (m), propagation
    angles (radians), polarisation (E_theta, E_phi), SH flag."""
    wavelength: float
    theta: float
    phi: float
    e_theta: complex
    e_phi: complex
    SH_cond: bool = False

    def updateWavelength(self, lam: float):
        self.wavelength = lam

    def omega(self) -> float:
        return 2.0 * math.pi * 299792458.0 / self.wavelength


@dataclass
class Run:
    geometry: Geometry
    excitation: Excitation
    outputType: int = -1
    params: List[float] = field(default_factory=lambda: [0.0] * 9)
    projection: bool = False
    solver: str = "scalapack"
    tolerance: float = 1e-10
    num_blocks: int = 1000
    max_iterations: int = 4000
    nMax: int = 0


# ---------------------------------------------------------------------------
# XML reader (simulation_input)
# ---------------------------------------------------------------------------
def _c(node, prefix="value") -> complex:
    if node is None:
        return 0j
    return complex(float(node.get(prefix + ".real", 0.0)), float(node.get(prefix + ".imag", 0.0)))


def _read_scatterer(node, nmax: int) -> Scatterer:
    """read_scatterer (Reader.cpp:581-663), sphere objects."""
    if node.get("type") != "sphere":
        raise NotImplementedError("only sphere objects are on this path (arbitrary.shape is srcAr/)")
    if node.find("cartesian") is not None:
        c = node.find("cartesian")
        vR = np.array([float(c.get(k, 0.0)) for k in "xyz"]) * FRNM_TO_M
    elif node.find("spherical") is not None:
        c = node.find("spherical")
        r, t, p = float(c.get("rrr", 0.0)) * FRNM_TO_M, float(c.get("the", 0.0)), float(c.get("phi", 0.0))
        vR = np.array([r * math.sin(t) * math.cos(p), r * math.sin(t) * math.sin(p), r * math.cos(t)])
    else:
        vR = np.zeros(3)
    props = node.find("properties")
    radius = float(props.get("radius")) * FRNM_TO_M if props is not None and props.get("radius") else 0.0
    em = ElectroMagnetic()
    eps, mu = node.find("epsilon"), node.find("mu")
    if eps is not None or mu is not None:
        if mu is None or mu.get("type") != "relative":
            raise RuntimeError('The type for mu must be "relative"')
        em.mu_r = _c(mu)
        kind = eps.get("type") if eps is not None else None
        if kind == "relative":
            em.epsilon_r = _c(eps)
            em.epsilon_r_SH = _c(node.find("epsilon_SH"))
            em.ksippp = _c(node.find("ksippp"))
            em.ksiparppar = _c(node.find("ksiparppar"))
            em.gamma = _c(node.find("gamma"))
        elif kind == "GoldModel":
            prm = eps.find("parameters")
            em.model = kind
            em.a_SH, em.b_SH, em.d_SH = (_c(prm, x) for x in ("a", "b", "d"))
        elif kind == "SiliconModel":
            em.model = kind
        else:
            raise RuntimeError("Unknown type for epsilon")
    return Scatterer(vR=vR, radius=radius, elmag=em, nMax=nmax)


# The zincblende (GaAs) cell of the structure generators, in units of the
# cell size: 14 large sites, then 4 small ones (Reader.cpp:205-209, 341-345).
_ZB = ((1, 0, 0), (1, .5, .5), (.5, .5, 0), (.5, 0, .5), (0, .5, .5), (0, 1, 0), (.5, 1, .5), (1, 1, 1),
       (.5, .5, 1), (0, 0, 1), (0, 0, 0), (1, 0, 1), (1, 1, 0), (0, 1, 1), (.75, .25, .25), (.25, .75, .25),
       (.75, .75, .75), (.25, .25, .75))


def _structure(st, nmax: int):
    """The structure generators of read_structure (Reader.cpp:120-573): "cube"
    (points^3 copies on a cubic lattice, a corner at the origin), "surface"
    (points^2 in the xy plane), "GaAssurf" (No_cells^2 zincblende cells in the
    xy plane; the 4 small sites have radius R / 2) and "GaAscube" (No_cells^3
    cells; small radius R / 1.7). Sites shared with an earlier cell are not
    repeated (the reference's X1 > 0 / Y1 > 0 / Z1 > 0 tests). The objects come
    out in the reference's order: it writes each generated site (the origin
    skipped in the zincblende ones) into the last object pushed and then pushes
    a fresh copy of the prototype, so object k holds site k + 1 (k + 1-th
    non-origin site) and the prototype with its own position and radius comes
    last."""
    kind = st.get("type")
    props = st.find("properties")
    proto = _read_scatterer(st.find("object"), nmax)
    sites, radii = [], []
    if kind in ("cube", "surface"):
        no, d = int(props.get("points")), float(props.get("distance")) * FRNM_TO_M
        layers = range(no) if kind == "cube" else [0]
        for k in layers:
            for j in range(no):
                for i in range(no):
                    sites.append((d * i, d * j, d * k))
                    radii.append(proto.radius)
        sites, radii = sites[1:], radii[1:]  # site 0 is the prototype's own slot
    elif kind in ("GaAssurf", "GaAscube"):
        no = int(props.get("No_cells"))
        a = float(props.get("cell_size")) * FRNM_TO_M
        R = proto.radius
        small = R / 2.0 if kind == "GaAssurf" else R / 1.7
        cell = [(a * x, a * y, a * z) for x, y, z in _ZB]
        for t in (range(no) if kind == "GaAscube" else [0]):
            for i in range(no):
                for j in range(no):
                    for k, (x, y, z) in enumerate(cell):
                        if (i > 0 and x <= 0.0) or (j > 0 and y <= 0.0) or (t > 0 and z <= 0.0):
                            continue
                        p = (x + a * i if i else x, y + a * j if j else y, z + a * t if t else z)
                        if p == (0.0, 0.0, 0.0):
                            continue
                        sites.append(p)
                        radii.append(R if k < 14 else small)
    else:
        raise NotImplementedError(f"structure type {kind!r}")
    out = [Scatterer(vR=np.array(p, dtype=float), radius=r, elmag=proto.elmag, nMax=nmax)
           for p, r in zip(sites, radii)]
    out.append(proto)
    return out


def simulation_input(source) -> Run:
    """Parse an Optimet3D case (path or XML text). The case file holds several
    top-level elements, so it is wrapped in one root before parsing."""
    text = source
    if not source.lstrip().startswith("<"):
        with open(source) as f:
            text = f.read()
    if text.lstrip().startswith("<?xml"):
        text = text[text.index("?>") + 2:]
    root = ET.fromstring("<case>" + text + "</case>")
    sim = root.find("simulation")
    if sim is None:
        raise RuntimeError("Simulation parameters not defined!")
    nmax = int(sim.find("harmonics").get("nmax"))
    aca = sim.find("ACA") is not None and sim.find("ACA").get("compression") == "yes"
    geo = root.find("geometry")
    if geo is None:
        raise RuntimeError("Geometry not defined!")
    g = Geometry(ACA_cond=aca)
    st = geo.find("structure")
    if st is not None:
        for o in _structure(st, nmax):
            g.pushObject(o)
    for node in geo.findall("object"):
        g.pushObject(_read_scatterer(node, nmax))
    bg = geo.find("background")
    # the reference reads the background only when its type is NOT "relative"
    # (Reader.cpp:84-99); a "relative" background stays vacuum
    if bg is not None and bg.get("type") != "relative":
        g.bground = ElectroMagnetic(epsilon_r=_c(bg.find("epsilon")), mu_r=_c(bg.find("mu")))
    if not g.objects:
        raise RuntimeError("No scatterers defined in input")
    src = root.find("source")
    if src is None:
        raise RuntimeError("Source not defined!")
    lam = float(src.find("wavelength").get("value")) * 1e-9
    prop = src.find("propagation")
    th = float(prop.get("theta", 0.0)) * math.pi / 180.0
    ph = float(prop.get("phi", 0.0)) * math.pi / 180.0
    pol = src.find("polarization")
    ex = Excitation(lam, th, ph, _c(pol, "Etheta"), _c(pol, "Ephi"),
                    src.find("SHsources") is not None and src.find("SHsources").get("condition") == "yes")
    run = Run(geometry=g, excitation=ex, nMax=nmax)
    out = root.find("output")
    if out is None:
        raise RuntimeError("Output not defined!")
    kind = out.get("type")
    if kind == "coefficients":
        run.outputType = 2
    elif kind == "field":
        run.outputType = 0
        grid = out.find("grid")
        for i, ax in enumerate("xyz"):
            a = grid.find(ax)
            run.params[3 * i] = float(a.get("min")) * 1e-9
            run.params[3 * i + 1] = float(a.get("max")) * 1e-9
            run.params[3 * i + 2] = float(a.get("steps"))
        pj = out.find("projection")
        run.projection = pj is not None and pj.get("spherical") == "true"
    elif kind == "response":
        scan = out.find("scan")
        wl = scan.find("wavelength") if scan is not None else None
        if wl is not None:
            lo, hi = float(wl.get("initial")), float(wl.get("final"))
            step = int(float(wl.get("stepsize")))
            run.params[0], run.params[1] = lo * 1e-9, hi * 1e-9
            run.params[2] = int(hi - lo) // step + 1  # Reader.cpp:876-878
            run.outputType = 11
        if scan is not None and scan.find("radius") is not None:
            run.outputType = 112 if wl is not None else 12
    # solver choice (read_parameter_list, Reader.cpp:909-921; LinearSystemSolver.hpp:149-160)
    plist = root.find("ParameterList")
    if plist is not None:
        for p in plist.iter("Parameter"):
            name, val = p.get("name"), p.get("value")
            if name == "Solver":
                run.solver = val
            elif name == "Convergence Tolerance":
                run.tolerance = float(val)
            elif name == "Num Blocks":
                run.num_blocks = int(val)
            elif name == "Maximum Iterations":
                run.max_iterations = int(val)
    return run


# ---------------------------------------------------------------------------
# Solver and Result
# ---------------------------------------------------------------------------
class GpuSolver:
    """solver::AbstractSolver on the GPU. Dense direct LU for the reference's
    direct solvers ("eigen" / "scalapack" / serial), GMRES otherwise; the
    precision form (complex64 matrix, FGMRES with FP32 inner iterations) on
    request."""

    def __init__(self, run: Run, precision: int = C128, ctx: Optional[Context] = None):
        self.run = run
        self.precision = precision
        self.ctx = ctx or Context(0)
        self.pr = None  # built by the first update() (the scan sets its wavelength first)

    def _form(self):
        # <ACA compression="yes">: compressed operator under Gmres_Zcomp
        if self.precision == C128 and self.run.geometry.ACA_cond:
            return ACA
        return self.precision

    def _options(self):
        if self._form() == ACA:  # PreconditionedMatrixSolver.h:48-51
            return options(SOLVE_GMRES, tol=1e-6, max_iter=240, restarts=2)
        if self.precision == C64:
            return options(SOLVE_FGMRES_MIXED, tol=min(self.run.tolerance, 1e-8), max_iter=30,
                           restarts=8, inner_iter=80, inner_tol=1e-4)
        if self.run.solver in ("scalapack", "eigen") and not self.run.geometry.ACA_cond:
            return options(SOLVE_LU)
        m = max(1, min(self.run.num_blocks, 400))
        return options(SOLVE_GMRES, tol=self.run.tolerance, max_iter=m,
                       restarts=max(1, self.run.max_iterations // m))

    def update(self, run: Optional[Run] = None):
        """AbstractSolver::update: rebuild for the current excitation."""
        if run is not None:
            self.run = run
        g, ex = self.run.geometry, self.run.excitation
        for o in g.objects:  # Geometry::update(excitation): dispersive models
            o.elmag.update(ex.wavelength)
        em = [o.elmag for o in g.objects]
        sp = spheres_array(np.array([o.vR for o in g.objects]), np.array([o.radius for o in g.objects]),
                           np.array([e.epsilon_r for e in em]), g.nMax(),
                           mu=np.array([e.mu_r for e in em]), eps_sh=np.array([e.epsilon_r_SH for e in em]),
                           ksippp=np.array([e.ksippp for e in em]),
                           ksiparppar=np.array([e.ksiparppar for e in em]),
                           gamma=np.array([e.gamma for e in em]))
        wave = plane_wave(ex.wavelength, ex.theta, ex.phi, ex.e_theta, ex.e_phi, sh=ex.SH_cond)
        if self.pr is None:
            self.pr = Problem(self.ctx, sp, medium(g.bground.epsilon_r, g.bground.mu_r), wave)
        else:
            self.pr.set_wave(wave)
        self.pr.source_vector(copy=False)

    def solve(self):
        """AbstractSolver::solve: (X_sca, X_int, X_sca_SH, X_int_SH)."""
        if self.pr is None:
            self.update()
        opts = self._options()
        form = self._form()
        self.pr.assemble(FF, form)
        self.pr.solve(opts, allow_unconverged=False)
        X_sca, X_int = self.pr.coefficients()
        X_sca_SH = X_int_SH = None
        if self.run.excitation.SH_cond:
            self.pr.assemble(SH, form)
            self.pr.solve_sh(opts)
            _, _, X_sca_SH, X_int_SH = self.pr.sh_vectors()
        return X_sca, X_int, X_sca_SH, X_int_SH


def factory(run: Run, precision: int = C128, ctx: Optional[Context] = None) -> GpuSolver:
    """solver::factory (Solver.cpp:30-54) for this path: the GPU solver."""
    return GpuSolver(run, precision, ctx)


class Result:
    """Result (Result.cpp) over a solved GpuSolver."""

    def __init__(self, solver: GpuSolver):
        self.solver = solver
        self._x = solver.pr.cross_sections()
        self._sh = solver.pr.sh_cross_sections() if solver.run.excitation.SH_cond else None

    def getExtinctionCrossSection(self) -> float:
        return float(self._x[0])

    def getScatteringCrossSection(self) -> float:
        return float(self._x[1])

    def getAbsorptionCrossSection(self) -> float:
        return float(self._x[3])

    def getScatteringCrossSection_SH(self) -> float:
        return float(self._sh[0])

    def getAbsorptionCrossSection_SH(self) -> float:
        return float(self._sh[1])

    def setFields(self, points):
        """Result::setFields (Result.cpp:889-933): E, H (and SH) at the points."""
        E, H = self.solver.pr.near_field(points)
        Esh = Hsh = None
        if self.solver.run.excitation.SH_cond:
            Esh, Hsh = self.solver.pr.near_field_sh(points)
        return E, H, Esh, Hsh


def grid_points(params) -> np.ndarray:
    """OutputGrid's regular Cartesian grid (OutputGrid.cpp:41-158): x fastest,
    x_i = min + i (max - min) / (steps - 1) + 1e-12."""
    n = [int(params[2]), int(params[5]), int(params[8])]
    ax = [abs(params[3 * i + 1] - params[3 * i]) / (n[i] - 1) for i in range(3)]
    idx = np.arange(n[0] * n[1] * n[2])
    cx, cy, cz = idx % n[0], (idx // n[0]) % n[1], idx // (n[0] * n[1])
    return np.stack([params[0] + cx * ax[0] + 1e-12, params[3] + cy * ax[1] + 1e-12,
                     params[6] + cz * ax[2] + 1e-12], axis=1)


def _fmt(v: float) -> str:
    """std::ostream's default formatting of a double (6 significant digits)."""
    return f"{v:g}"


class Simulation:
    """Simulation (Simulation.cpp:34-63): runs a case file."""

    def __init__(self, caseFile: str, precision: int = C128):
        self.caseFile = caseFile[:-4] if caseFile.endswith(".xml") else caseFile
        self.precision = precision

    def run(self) -> int:
        run = simulation_input(self.caseFile + ".xml")
        solver = factory(run, self.precision)
        if run.outputType == 0:
            self.field_simulation(run, solver)
        elif run.outputType == 11:
            self.scan_wavelengths(run, solver)
        else:
            sys.stderr.write("Nothing to do?\n")
            return 1
        return 0

    def scan_wavelengths(self, run: Run, solver: GpuSolver):
        """Simulation::scan_wavelengths (Simulation.cpp:604-685)."""
        lami, lamf, steps = run.params[0], run.params[1], int(run.params[2])
        lams = (lamf - lami) / (steps - 1) if steps > 1 else 0.0
        sh = run.excitation.SH_cond
        files = {"a": open(self.caseFile + "_AbsorptionCS_FF.dat", "w"),
                 "s": open(self.caseFile + "_ScatteringCS_FF.dat", "w")}
        if sh:
            files["ssh"] = open(self.caseFile + "_ScatteringCS_SH.dat", "w")
            files["ash"] = open(self.caseFile + "_AbsorptionCS_SH.dat", "w")
        try:
            for i in range(steps):
                lam = lami + i * lams
                run.excitation.updateWavelength(lam)
                solver.update(run)
                solver.solve()
                r = Result(solver)
                files["a"].write(f"{_fmt(lam)}\t{_fmt(r.getExtinctionCrossSection() - r.getScatteringCrossSection())}\n")
                files["s"].write(f"{_fmt(lam)}\t{_fmt(r.getScatteringCrossSection())}\n")
                if sh:
                    files["ssh"].write(f"{_fmt(lam)}\t{_fmt(r.getScatteringCrossSection_SH())}\n")
                    files["ash"].write(f"{_fmt(lam)}\t{_fmt(r.getAbsorptionCrossSection_SH())}\n")
        finally:
            for f in files.values():
                f.close()

    def field_simulation(self, run: Run, solver: GpuSolver):
        """Simulation::field_simulation (Simulation.cpp:319-370); fields in npz."""
        solver.solve()
        r = Result(solver)
        pts = grid_points(run.params)
        E, H, Esh, Hsh = r.setFields(pts)
        np.savez(self.caseFile + "_FF.npz", points=pts, E=E, H=H)
        if run.excitation.SH_cond:
            np.savez(self.caseFile + "_SH.npz", points=pts, E=Esh, H=Hsh)


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description="Run an Optimet3D case file on the GPU")
    ap.add_argument("case")
    ap.add_argument("--precision", choices=["c128", "c64"], default="c128")
    a = ap.parse_args(argv)
    return Simulation(a.case, C64 if a.precision == "c64" else C128).run()


if __name__ == "__main__":
    sys.exit(main())
