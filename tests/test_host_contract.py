"""Host-side contracts that need no GPU: the solver roles that the
reference-facing GpuSolver picks from a case (the choice of
solver::factory, Solver.cpp:30-54, and the parameters of
LinearSystemSolver.hpp:149-160 and PreconditionedMatrixSolver.h:48-51), and
the JSON line of bench.py's reference arm (the oracle port timed on the host
cores; rank 0 alone prints under a multi-rank launch)."""
import json
import os
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CASES = os.path.join(HERE, "cases")


def _run_for(xml_text, tmp_path):
    from optimet_gb300 import optimet as O
    p = tmp_path / "case.xml"
    p.write_text(xml_text)
    return O.simulation_input(str(p))


def _with_parameters(base, params):
    # a top-level ParameterList after <simulation>, as in the reference's
    # examples (read_parameter_list, Reader.cpp:916-927)
    plist = '<ParameterList name="Belos">' + "".join(
        '<Parameter name="%s" type="%s" value="%s"/>' % (n, t, v) for n, t, v in params) + "</ParameterList>"
    return base.replace("</simulation>", "</simulation>\n" + plist)


def _solver(run, precision):
    from optimet_gb300 import optimet as O
    # the context is only used once the solver runs; the role is chosen before
    return O.GpuSolver(run, precision, ctx=object())


def test_solver_roles_follow_the_reference_factory(tmp_path):
    import optimet_gb300 as G
    base = open(os.path.join(CASES, "pair_scan.xml")).read()
    assert "</simulation>" in base
    # no ParameterList: "scalapack" (Reader.cpp:925-926), the direct solve
    run = _run_for(base, tmp_path)
    assert run.solver == "scalapack"
    o = _solver(run, G.C128)._options()
    assert o.method == G.SOLVE_LU
    # "eigen" is the serial direct solve too
    run = _run_for(_with_parameters(base, [("Solver", "string", "eigen")]), tmp_path)
    assert _solver(run, G.C128)._options().method == G.SOLVE_LU
    # anything else is Belos GMRES with the case's tolerance, blocks and iterations
    run = _run_for(_with_parameters(base, [("Solver", "string", "GMRES"),
                                           ("Convergence Tolerance", "double", "1e-8"),
                                           ("Num Blocks", "int", "50"),
                                           ("Maximum Iterations", "int", "500")]), tmp_path)
    o = _solver(run, G.C128)._options()
    assert o.method == G.SOLVE_GMRES and o.tol == pytest.approx(1e-8)
    assert o.max_iter == 50 and o.restarts == 10
    # the precision form: FP64 FGMRES around FP32 GMRES, never looser than 1e-8
    o = _solver(run, G.C64)._options()
    assert o.method == G.SOLVE_FGMRES_MIXED and o.tol == pytest.approx(1e-8)


def test_aca_case_takes_the_compressed_gmres_role(tmp_path):
    import optimet_gb300 as G
    base = open(os.path.join(CASES, "pair_scan.xml")).read()
    # <ACA> inside <simulation> (Reader.cpp:61-65)
    text = base.replace("</simulation>", '<ACA compression="yes" /></simulation>')
    run = _run_for(text, tmp_path)
    assert run.geometry.ACA_cond
    s = _solver(run, G.C128)
    assert s._form() == G.ACA
    o = s._options()
    # Gmres_Zcomp's parameters (PreconditionedMatrixSolver.h:48-51)
    assert o.method == G.SOLVE_GMRES and o.tol == pytest.approx(1e-6)
    assert o.max_iter == 240 and o.restarts == 2


def _bench(args, env_extra=None):
    env = dict(os.environ)
    env.update(env_extra or {})
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, cwd=ROOT, env=env,
                          capture_output=True, text=True, timeout=600)


def test_reference_arm_prints_one_json_line():
    r = _bench(["--impl", "reference", "--workload", "small", "--steps", "1", "--warmup", "3"])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["higher_is_better"] is True
    assert d["unit"] == "wavelength-solves/s" and d["value"] > 0
    assert d["steps"] == 1 and d["warmup"] == 3 and d["n_gpus"] == 1
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["config"]["workload"].startswith("small")


def test_reference_arm_other_ranks_exit_quietly():
    r = _bench(["--impl", "reference", "--workload", "small", "--steps", "1", "--warmup", "3"],
               {"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
