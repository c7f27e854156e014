"""The oracle's entry points run clean under AddressSanitizer and UndefinedBehaviorSanitizer
(host-only race/memory checking; compute-sanitizer is not available for the GPU side)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_oracle_selftest_under_asan_ubsan():
    if shutil.which("g++") is None or shutil.which("make") is None:
        pytest.skip("no host compiler")
    r = subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "sanitize"], capture_output=True, text=True)
    if r.returncode != 0 and "sanitize" in r.stderr and "unrecognized" in r.stderr:
        pytest.skip("compiler without sanitizers")
    assert r.returncode == 0, r.stderr[-2000:]
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0", UBSAN_OPTIONS="print_stacktrace=1")
    p = subprocess.run([os.path.join(ROOT, "oracle", "_build", "selftest_asan")], capture_output=True, text=True,
                       env=env, timeout=300)
    assert p.returncode == 0, p.stdout[-2000:] + p.stderr[-4000:]
    assert "selftest ok" in p.stdout
    assert "runtime error" not in p.stderr
