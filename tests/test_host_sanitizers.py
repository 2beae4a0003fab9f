"""Host code under AddressSanitizer and UndefinedBehaviorSanitizer (no GPU).

compute-sanitizer is closed on the GPU pool, so the host side gets the
sanitizers instead: the library's C++ sources (parser, generator, text writer,
planner, checkpoint reader, API layer) are rebuilt with -fsanitize=address,
undefined and driven by tests/host_sanitize_driver.cpp through well-formed and
malformed inputs; any out-of-bounds access, use after free or undefined
behaviour aborts the driver.
"""

import os
import shutil
import subprocess

import pytest

from oracle_util import ROOT


@pytest.mark.timeout(600)
def test_host_code_under_asan_ubsan(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("no host compiler")
    from gputucker_gb300 import build
    lib = build.build_host_sanitized(str(tmp_path / "lib"))
    drv = str(tmp_path / "drv")
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-g", *build.SANITIZE, "-I" + build.INCLUDE,
                        os.path.join(ROOT, "tests", "host_sanitize_driver.cpp"), lib,
                        "-Wl,-rpath," + os.path.dirname(lib), "-o", drv], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0:abort_on_error=1", UBSAN_OPTIONS="print_stacktrace=1")
    r = subprocess.run([drv, str(tmp_path)], capture_output=True, text=True, env=env, timeout=300)
    print(r.stdout, r.stderr[-3000:])
    assert r.returncode == 0, r.stderr[-3000:]
    assert "AddressSanitizer" not in r.stderr and "runtime error" not in r.stderr
    assert "host sanitizer driver: ok" in r.stdout
