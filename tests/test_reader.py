"""The Optimet3D XML case reader and the reference-facing objects
(optimet_gb300.optimet): parsing rules of Reader.cpp on CPU, and (GPU) the
scan and field runs of Simulation against the oracle."""
import math
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = os.path.join(HERE, "cases")


def test_reader_units_angles_background_and_scan():
    from optimet_gb300 import optimet as O
    run = O.simulation_input(os.path.join(CASES, "pair_scan.xml"))
    g, ex = run.geometry, run.excitation
    assert run.nMax == 4 and g.nMax() == 4 and len(g.objects) == 2
    assert np.allclose(g.objects[0].vR, [-60e-9, 10e-9, 0.0])
    r, t, p = 150e-9, 1.2, 0.3
    assert np.allclose(g.objects[1].vR, [r * math.sin(t) * math.cos(p), r * math.sin(t) * math.sin(p),
                                         r * math.cos(t)])
    assert g.objects[0].radius == pytest.approx(55e-9)
    assert g.objects[1].elmag.epsilon_r == 9.0 + 0.12j
    assert g.objects[0].elmag.ksiparppar == 0.25
    # a background whose type is not "relative" is read (Reader.cpp:84-99)
    assert g.bground.epsilon_r == 1.7689
    assert ex.wavelength == pytest.approx(700e-9)
    assert ex.theta == pytest.approx(math.radians(30)) and ex.phi == pytest.approx(math.radians(45))
    assert ex.e_theta == 0.8 and ex.e_phi == 0.6j and ex.SH_cond
    # steps = int(final - initial) / stepsize + 1
    assert run.outputType == 11 and run.params[2] == 3
    assert run.params[0] == pytest.approx(600e-9) and run.params[1] == pytest.approx(640e-9)


def test_reader_relative_background_stays_vacuum_and_field_grid():
    from optimet_gb300 import optimet as O
    run = O.simulation_input(os.path.join(CASES, "field_map.xml"))
    # the reference ignores a background of type "relative"
    assert run.geometry.bground.epsilon_r == 1.0
    assert run.outputType == 0 and run.params[2] == 9 and run.params[5] == 7 and run.params[8] == 2
    pts = O.grid_points(run.params)
    assert pts.shape == (9 * 7 * 2, 3)
    assert pts[1, 0] - pts[0, 0] == pytest.approx(50e-9) and pts[0, 0] == pytest.approx(-200e-9 + 1e-12)
    assert pts[9, 1] - pts[0, 1] == pytest.approx(400e-9 / 6)


def test_reader_rejections():
    from optimet_gb300 import optimet as O
    base = open(os.path.join(CASES, "field_map.xml")).read()
    with pytest.raises(RuntimeError, match="overlap"):
        O.simulation_input(base.replace('z="90.0"', 'z="50.0"'))
    with pytest.raises(NotImplementedError):
        O.simulation_input(base.replace('<object type="sphere">', '<structure type="hexagonal"><object type="sphere">', 1)
                           .replace('</object>', '</object></structure>', 1))
    with pytest.raises(RuntimeError, match="Unknown type"):
        O.simulation_input(base.replace('type="relative" value.real="-17.0"', 'type="Drude" value.real="-17.0"', 1))
    with pytest.raises(RuntimeError, match="mu"):
        O.simulation_input(base.replace('<mu type="relative"', '<mu type="absolute"', 1))


def _oracle_cluster(oracle, run):
    g, ex = run.geometry, run.excitation
    em = [o.elmag for o in g.objects]
    return oracle.Cluster(xyz=np.array([o.vR for o in g.objects]), radius=np.array([o.radius for o in g.objects]),
                          eps=np.array([e.epsilon_r for e in em]), eps_sh=np.array([e.epsilon_r_SH for e in em]),
                          nmax=run.nMax, wavelength=ex.wavelength, bg_eps=g.bground.epsilon_r,
                          bg_mu=g.bground.mu_r, theta=ex.theta, phi=ex.phi, e_theta=ex.e_theta,
                          e_phi=ex.e_phi, ksippp=np.array([e.ksippp for e in em]),
                          ksiparppar=np.array([e.ksiparppar for e in em]))


@pytest.mark.gpu
def test_scan_case_matches_oracle(tmp_path, oracle):
    """Simulation.run() on the scan case writes the reference's four .dat files;
    every value equals the oracle's cross sections (to the file's 6 digits,
    and to 1e-10 before formatting)."""
    import shutil
    from optimet_gb300 import optimet as O
    case = tmp_path / "pair_scan.xml"
    shutil.copy(os.path.join(CASES, "pair_scan.xml"), case)
    assert O.Simulation(str(case)).run() == 0
    run = O.simulation_input(str(case))
    tab = oracle.clg_tables(run.nMax)
    cols = {k: np.loadtxt(str(tmp_path / f"pair_scan_{k}.dat"))
            for k in ("AbsorptionCS_FF", "ScatteringCS_FF", "ScatteringCS_SH", "AbsorptionCS_SH")}
    solver = O.factory(run)
    for i, lam in enumerate(600e-9 + 20e-9 * np.arange(3)):
        run.excitation.updateWavelength(lam)
        cl = _oracle_cluster(oracle, run)
        pr = oracle.Problem(cl)
        X = oracle.lu_solve(pr.scattering_matrix(), pr.source_vector())
        Xi = pr.internal(X)
        xs = pr.cross_sections(X)
        K, K1, Xs, Xis = pr.sh_solve(tab, Xi)
        xsh = pr.sh_cross_sections(tab, Xi, Xs, Xis)
        solver.update(run)
        solver.solve()
        r = O.Result(solver)
        assert abs(r.getExtinctionCrossSection() - xs[0]) < 1e-10 * abs(xs[0])
        assert abs(r.getScatteringCrossSection() - xs[1]) < 1e-10 * abs(xs[1])
        assert abs(r.getScatteringCrossSection_SH() - xsh[0]) < 1e-10 * abs(xsh[0])
        assert abs(r.getAbsorptionCrossSection_SH() - xsh[1]) < 1e-10 * abs(xsh[1])
        assert cols["AbsorptionCS_FF"][i, 0] == pytest.approx(lam, rel=1e-5)
        assert cols["AbsorptionCS_FF"][i, 1] == pytest.approx(xs[0] - xs[1], rel=1e-5)
        assert cols["ScatteringCS_FF"][i, 1] == pytest.approx(xs[1], rel=1e-5)
        assert cols["ScatteringCS_SH"][i, 1] == pytest.approx(xsh[0], rel=1e-5)
        assert cols["AbsorptionCS_SH"][i, 1] == pytest.approx(xsh[1], rel=1e-5)


@pytest.mark.gpu
def test_field_case_matches_oracle(tmp_path, oracle):
    import shutil
    from optimet_gb300 import optimet as O
    case = tmp_path / "field_map.xml"
    shutil.copy(os.path.join(CASES, "field_map.xml"), case)
    assert O.Simulation(str(case)).run() == 0
    out = np.load(str(tmp_path / "field_map_FF.npz"))
    run = O.simulation_input(str(case))
    pr = oracle.Problem(_oracle_cluster(oracle, run))
    X = oracle.lu_solve(pr.scattering_matrix(), pr.source_vector())
    E, H = pr.near_field(X, pr.internal(X), oracle.grid_points(run.params))
    assert np.max(np.abs(out["E"] - E)) < 1e-10 * np.max(np.abs(E))
    assert np.max(np.abs(out["H"] - H)) < 1e-10 * np.max(np.abs(H))


def test_material_models_and_cube_structure():
    """SiliconModel interpolates n, k linearly on its 10 nm grid (n^2 - k^2 +
    2ink at the fundamental, the same at lambda/2 for SH); GoldModel's chi(2)
    terms scale with (eps_r - 1) as in ElectroMagnetic.cpp:134-143; the cube
    generator puts points^3 copies on a lattice with a corner at the origin."""
    from optimet_gb300 import materials as M
    from optimet_gb300 import optimet as O
    i = 55
    lam = (0.25 + i * 0.01 + 0.004) * 1e-6
    eps, eps_sh, kp, kpp, g = M.silicon(lam)
    n = M.N_SI[i] + (M.N_SI[i + 1] - M.N_SI[i]) * 0.4
    k = M.K_SI[i] + (M.K_SI[i + 1] - M.K_SI[i]) * 0.4
    assert eps == pytest.approx(complex(n * n - k * k, 2 * n * k), rel=1e-12)
    assert (kp, kpp, g) == M.SI_CHI
    with pytest.raises(ValueError):
        M.silicon(1.47e-6)
    with pytest.raises(ValueError):
        M.silicon(0.45e-6)  # SH wavelength below the table
    e, esh, a, b, d = M.gold(800e-9, 1.0, 2.0, 4.0)
    assert e.real < -10 and e.imag > 0 and esh.imag > 0
    omega = 2 * math.pi * M.C_LIGHT / 800e-9
    scale = (e - 1) * M.Q_ELECTRON / (M.M_ELECTRON * omega ** 2)
    assert a == pytest.approx(-scale / 4) and b == pytest.approx(-scale) and d == pytest.approx(-scale / 2)
    case = open(os.path.join(CASES, "field_map.xml")).read()
    cube = case.replace('<object type="sphere">\n    <cartesian x="0.0" y="0.0" z="-90.0" />',
                        '<structure type="cube"><properties points="3" distance="200.0" />'
                        '<object type="sphere">', 1).replace('</object>', '</object></structure>', 1)
    cube = cube.replace('<object type="sphere">\n    <cartesian x="0.0" y="0.0" z="90.0" />',
                        '<object type="sphere">\n    <cartesian x="-300.0" y="0.0" z="0.0" />')
    run = O.simulation_input(cube)
    assert len(run.geometry.objects) == 28
    # the reference's order: object k holds lattice site k + 1, the prototype
    # (its own position, the origin here) comes last, then the other objects
    assert np.allclose(run.geometry.objects[0].vR, [200e-9, 0.0, 0.0])
    assert np.allclose(run.geometry.objects[25].vR, [400e-9, 400e-9, 400e-9])
    assert np.allclose(run.geometry.objects[26].vR, [0.0, 0.0, 0.0])
    assert np.allclose(run.geometry.objects[27].vR, [-300e-9, 0.0, 0.0])


def _structure_case(kind, props, radius=20.0):
    head = open(os.path.join(CASES, "field_map.xml")).read()
    i, j = head.index("<geometry>"), head.index("</geometry>")
    geo = ('<geometry>\n<structure type="%s"><properties %s />\n<object type="sphere">\n'
           '<properties radius="%g" />\n<epsilon type="relative" value.real="12.0" value.imag="0.1" />\n'
           '<mu type="relative" value.real="1.0" value.imag="0.0" />\n</object></structure>\n'
           % (kind, props, radius))
    return head[:i] + geo + head[j:]


@pytest.mark.parametrize("kind,no,count", [("GaAssurf", 1, 18), ("GaAssurf", 2, 54), ("GaAssurf", 3, 110),
                                           ("GaAscube", 1, 18), ("GaAscube", 2, 95), ("surface", 3, 9)])
def test_structure_generators(kind, no, count):
    """read_structure's generators (Reader.cpp:120-573). Zincblende cells of
    size a: 14 large sites (radius R) and 4 small ones (R / 2 on a surface,
    R / 1.7 in a cube); sites on a face shared with an earlier cell are not
    repeated, so No x No cells hold 18 + 26 (No - 1) + 10 (No - 1)^2 sites and
    No^3 cells 18 + 39 (No - 1) + 30 (No - 1)^2 + 8 (No - 1)^3 (the origin is
    the prototype's own slot). Object k holds the (k + 1)-th non-origin site;
    the prototype comes last at its own position (the origin)."""
    from optimet_gb300 import optimet as O
    a = 200.0
    props = ('No_cells="%d" cell_size="%g"' % (no, a)) if kind.startswith("GaAs") else \
        ('points="%d" distance="%g"' % (no, a))
    run = O.simulation_input(_structure_case(kind, props))
    obj = run.geometry.objects
    m = no - 1
    want = {"GaAssurf": 18 + 26 * m + 10 * m * m, "GaAscube": 18 + 39 * m + 30 * m * m + 8 * m ** 3,
            "surface": no * no}[kind]
    assert len(obj) == want == count
    xyz = np.array([o.vR for o in obj]) / 1e-9
    assert np.allclose(xyz[-1], 0.0)
    assert len({tuple(np.round(p, 6)) for p in xyz}) == len(obj)  # no site twice
    r = np.array([o.radius for o in obj]) / 1e-9
    if kind == "surface":
        assert np.allclose(xyz[0], [a, 0, 0]) and np.allclose(xyz[:, 2], 0.0) and np.allclose(r, 20.0)
        return
    assert np.allclose(xyz[0], [a, 0, 0]) and r[0] == pytest.approx(20.0)
    small = 20.0 / (2.0 if kind == "GaAssurf" else 1.7)
    assert set(np.round(r, 9)) == {20.0, round(small, 9)}
    # the small sites sit at the quarter positions of each cell
    frac = np.mod(xyz[r < 20.0] / a, 1.0)
    assert np.all(np.isin(np.round(frac, 9), [0.25, 0.75]))
    assert xyz.min() >= 0.0 and xyz.max() <= a * no + 1e-9
    if kind == "GaAssurf":
        assert xyz[:, 2].max() <= a + 1e-9

