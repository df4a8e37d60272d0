import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def vrc_lib():
    from voreen_gb300 import build
    build.build()
    import voreen_gb300
    return voreen_gb300.lib()


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def ctx(vrc_lib):
    import voreen_gb300 as v
    c = v.Context(0)
    yield c
    c.close()


def pytest_terminal_summary(terminalreporter, exitstatus, config):
    """Prints the FP64 parity reports the tests recorded: per case the max |d|
    against the FP32 and FP64 oracles, and the decision-divergent rays (count
    and their max |d|) that the 1/255 bound leaves out."""
    try:
        from helpers import REPORTS
    except ImportError:
        return
    if not REPORTS:
        return
    tr = terminalreporter
    tr.section("parity vs FP64 oracle (|d| in 1/255 units)")
    for label, r in REPORTS:
        tr.write_line(f"{label}: max vs FP32 {r['max_abs_vs_fp32'] * 255:.4f}, vs FP64 {r['max_abs_vs_fp64'] * 255:.4f} "
                      f"on agreeing rays ({r['max_abs_vs_fp64_all_rays'] * 255:.4f} on all); divergent rays "
                      f"{r['divergent_rays']} of {r['hit_rays']} hit, their max {r['divergent_max_abs_vs_fp64'] * 255:.4f}, "
                      f"above 1/255: {r['waived_rays']}; channels > 0.5/255: {r['channels_over_half_lsb_vs_fp64']}")
