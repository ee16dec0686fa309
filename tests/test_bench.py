"""The measurement contract of bench.py on the CPU: the c3 workload's unit
counts and the algorithmic bytes its roofline divides by (11,022,336
depth-steps per gradient; 36.8 GB per Born-adjoint launch).
"""
import importlib.util
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="module")
def c3(bench):
    from wemgpu import synthetic as S
    cfg = bench.workload()
    return cfg, S.params_of(cfg)


def test_depth_steps_per_gradient(bench, c3):
    cfg, p = c3
    assert (p.ns, p.nx, p.nz) == (32, 768, 300)
    # 2 WEM passes + 10 Born-adjoint passes, 32 shots x 96 frequencies, 299 steps
    assert bench.row_steps(p, 96) == 12 * 32 * 96 * 299 == 11022336


def test_born_adjoint_algorithmic_bytes(bench, c3):
    cfg, p = c3
    b = bench.algorithmic_bytes("k_born_adj", p, 96, 8)
    assert b == 36805017600
    # three stored fields written and read once per row-depth, two image rows
    # per group (of 8 shots) and depth, four passes over the phase and
    # split-step tables
    rows, groups, nxg = 32 * 96, 4 * 96, 768
    tables = 96 * p.nz * (768 + 768) * 8
    assert b == 3 * 16 * nxg * p.nz * rows + groups * p.nz * 16 * nxg + 4 * tables


def test_measured_per_row_constants(bench, c3):
    cfg, p = c3
    # ncu traffic of the Born adjoint scaled to the full launch agrees with the
    # algorithmic bytes (each stored row written and read once)
    traffic = bench.TRAFFIC_PER_ROW_DEPTH["k_born_adj"] * p.ns * 96 * p.nz
    assert abs(traffic / bench.algorithmic_bytes("k_born_adj", p, 96, 8) - 1) < 0.05
    for k in ("k_born_adj", "k_wem"):
        assert bench.INST_PER_ROW_DEPTH[k] > 1000


def test_gpus_flag_must_match_the_ranks():
    """--gpus N under a launcher with another world size is refused, not
    silently run as one rank."""
    import subprocess
    import sys
    env = dict(os.environ, WORLD_SIZE="2", RANK="0")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--gpus", "1"], env=env,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode != 0 and "WORLD_SIZE=2" in r.stderr
