import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
TESTS = os.path.dirname(os.path.abspath(__file__))
if TESTS not in sys.path:
    sys.path.insert(0, TESTS)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA decode path")
    config.addinivalue_line("markers", "slow: full-size workloads")


def pytest_terminal_summary(terminalreporter, exitstatus, config):
    """Counts reported by the parity tests: what was compared, how much of it."""
    try:
        from helpers import REPORTS
    except ImportError:
        return
    if not REPORTS:
        return
    terminalreporter.write_line("parity counts:")
    for name, counts in REPORTS:
        terminalreporter.write_line(f"  {name}: " + ", ".join(f"{k}={v}" for k, v in counts.items()))
