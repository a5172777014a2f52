"""The explicit time loop against dune-fem's own TimeProvider and
ExplicitRungeKuttaSolver.

tests/golden/ref_timeloop.json was made by oracle/make_ref_golden.sh, which
compiles the reference's solver/timeprovider.hh, solver/rungekutta/explicit.hh
and butchertable.cc unmodified and runs five SSP-RK3 steps (tvd3ButcherTable)
of u' = -M^{-1} A u, A the reference's DGEllipticOperator (Q2, periodic 3x2x2
cells, kappa field, mass term), M = |K| I.  The operator reports a time-step
estimate that depends on how often it was applied, so the step sizes record
which stage evaluations the TimeProvider took the minimum over (one at
initialize, then one per stage: three per step).
"""
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import relmax

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
with open(os.path.join(ROOT, "tests", "golden", "ref_timeloop.json")) as _f:
    GOLD = json.load(_f)


def estimate(k):
    """The golden operator's estimate after its k-th application."""
    return 1e-3 * (3 + (7 * k + 2) % 13) / 8.0


def initial_state():
    p = GOLD["order"]
    nl = (p + 1) ** 3
    ncell = int(np.prod(GOLD["cells"]))
    i = np.arange(ncell * nl, dtype=np.int64)
    u = ((i * 7919 + 13) % 2003 - 1001) / 1000.0
    c = np.arange(ncell, dtype=np.int64)
    idx = c[:, None] * nl + np.arange(nl, dtype=np.int64)[None, :]
    kappa = ((idx * 37 + 5) % 9 - 4) / 1000.0
    kappa[:, 0] = 1.0 + ((c * 31 + 7) % 11) / 10.0
    return u, kappa.reshape(-1)


def problem_kw():
    return dict(quad_points=GOLD["quad_points"], diffusion=GOLD["diffusion"], penalty=GOLD["penalty"],
                mass=GOLD["mass"], periodic=(1, 1, 1), weak_dirichlet=False)


def run_loop(gb, step):
    """The reference's loop: initialize applies the operator once and
    provides its estimate; tp.init(); per step solve (three applications,
    each providing the estimate) and tp.next().  Returns step sizes, start
    times and the final time."""
    tp = gb.TimeProvider(start_time=0.0, cfl=GOLD["cfl"])
    applications = 0

    def applied():
        nonlocal applications
        applications += 1
        tp.provideTimeStepEstimate(estimate(applications))

    applied()
    tp.init()
    dts, times = [], []
    while tp.timeStep() < GOLD["steps"]:
        times.append(tp.time())
        dts.append(tp.deltaT())
        step(tp.deltaT())
        for _ in range(3):
            applied()
        tp.next()
    assert applications == GOLD["applications"]
    return dts, times, tp.time()


def test_tvd3_table_is_the_one_the_gpu_step_uses():
    """The SSP-RK3 coefficients of csrc/rk.cu are the reference's compiled
    tvd3ButcherTable."""
    t = GOLD["tvd3"]
    assert t["A"] == [[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.25, 0.25, 0.0]]
    assert t["b"] == [1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0] and t["c"] == [0.0, 1.0, 0.5] and t["order"] == 3
    with open(os.path.join(ROOT, "dune-fem_gb300", "csrc", "rk.cu")) as f:
        src = f.read()
    assert "A[3][3] = {{0.0, 0.0, 0.0}, {1.0, 0.0, 0.0}, {0.25, 0.25, 0.0}}" in src
    assert "b[3] = {1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0}" in src


def test_python_time_provider_and_oracle_rk3_equal_reference(gb, orc):
    u, kappa = initial_state()
    prob = orc.DGProblem(tuple(GOLD["cells"]), GOLD["order"], **problem_kw())
    state = {"u": u}

    def step(dt):
        state["u"] = prob.rk3_step(state["u"], dt, kappa=kappa)

    dts, times, final = run_loop(gb, step)
    assert dts == GOLD["dt"] and times == GOLD["time"] and final == GOLD["final_time"]
    assert relmax(state["u"], GOLD["u"]) < 1e-13


def test_cpp_time_provider_equals_reference(gb, tmp_path):
    """include/gbfem.hpp's TimeProvider driven the same way gives the same
    step sizes and times, bit for bit."""
    src = tmp_path / "tp.cpp"
    src.write_text(r"""
#include <cstdio>
#include <cstdlib>
#include "gbfem.hpp"
static double estimate(long k) { return 1e-3 * (3 + (7 * k + 2) % 13) / 8.0; }
int main(int argc, char** argv) {
  const double cfl = std::atof(argv[1]);
  const int steps = std::atoi(argv[2]);
  gbfem_cpp::TimeProvider tp(0.0, cfl);
  long applications = 0;
  tp.provideTimeStepEstimate(estimate(++applications));
  tp.init();
  for (; tp.timeStep() < steps; tp.next()) {
    std::printf("%.17g %.17g\n", tp.time(), tp.deltaT());
    for (int s = 0; s < 3; ++s) tp.provideTimeStepEstimate(estimate(++applications));
  }
  std::printf("%.17g %ld\n", tp.time(), applications);
  return 0;
}
""")
    exe = str(tmp_path / "tp")
    lib = os.path.join(ROOT, "dune-fem_gb300", "lib")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src), "-o", exe,
                        "-L", lib, "-lgbfem", "-Wl,-rpath," + lib], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe, repr(GOLD["cfl"]), str(GOLD["steps"])], capture_output=True, text=True, check=True)
    rows = [line.split() for line in out.stdout.strip().splitlines()]
    assert [float(t) for t, _ in rows[:-1]] == GOLD["time"]
    assert [float(d) for _, d in rows[:-1]] == GOLD["dt"]
    assert float(rows[-1][0]) == GOLD["final_time"] and int(rows[-1][1]) == GOLD["applications"]


@pytest.mark.gpu
def test_gpu_rk3_time_loop_equals_reference(gb):
    u, kappa = initial_state()
    op = gb.DGOperator(tuple(GOLD["cells"]), GOLD["order"], kappa=gb.DeviceArray.from_numpy(kappa), **problem_kw())
    ud = gb.DeviceArray.from_numpy(u)
    rk = gb.RK3(op)
    dts, times, final = run_loop(gb, lambda dt: rk.step(ud, dt))
    assert dts == GOLD["dt"] and final == GOLD["final_time"]
    assert relmax(ud.numpy(), GOLD["u"]) < 1e-12
