"""The reference's own Python tests, run unchanged against this package.

libcasm-monte's Python tests import ``libcasm.monte``; the plugin
``casmcode_monte_gb300.libcasm_alias`` maps those imports to this package.  The tests that need
neither a GPU nor libcasm.xtal (ValueMap, the random number generator, samplers, sampling
functions, completion checks and the selected-event function parameters) must all pass.  The
test files are read where the reference tree is mounted (they are not copied into this
repository); the test is skipped where it is not.
"""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REFERENCE_TESTS = os.environ.get("LIBCASM_MONTE_PYTHON_TESTS", "/root/reference/python/tests")
FILES = ["test_ValueMap.py", "test_RandomNumberGeneratory.py", "sampling/test_Sampler.py",
         "sampling/test_SamplingFunction.py", "sampling/test_CompletionCheck.py",
         "sampling/test_SelectedEventFunctionParams.py"]


def test_reference_python_tests_pass(tmp_path):
    paths = [os.path.join(REFERENCE_TESTS, f) for f in FILES]
    if not all(os.path.exists(p) for p in paths):
        pytest.skip("the reference's Python tests are not mounted here")
    env = dict(os.environ, PYTHONPATH=ROOT + os.pathsep + os.environ.get("PYTHONPATH", ""))
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-p", "casmcode_monte_gb300.libcasm_alias",
                        "-p", "no:cacheprovider", "--rootdir", str(tmp_path), *paths],
                       capture_output=True, text=True, cwd=str(tmp_path), env=env, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
    assert "21 passed" in r.stdout, r.stdout[-1000:]
