"""The library's host C11 code (the frame set-up, clamps, parameter scenes and synthetic maps) run over
ordinary and edge inputs under AddressSanitizer and UndefinedBehaviorSanitizer: no report, exit 0."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "artful_gb300", "csrc")


def test_host_code_under_sanitizers(tmp_path):
    exe = str(tmp_path / "host_sanitized")
    cmd = [os.environ.get("CC", "gcc"), "-std=c11", "-O1", "-g", "-fno-omit-frame-pointer",
           "-fsanitize=address,undefined,float-cast-overflow", "-fno-sanitize-recover=all", "-ffp-contract=off",
           "-I" + os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "host_sanitized.c"),
           os.path.join(CSRC, "holeHost.c"), os.path.join(CSRC, "synthScene.c"), "-lm", "-o", exe]
    build = subprocess.run(cmd, capture_output=True, text=True)
    if build.returncode != 0 and "sanitize" in build.stderr:
        pytest.skip("this compiler has no sanitizer runtime")
    assert build.returncode == 0, build.stderr
    run = subprocess.run([exe], capture_output=True, text=True, timeout=300,
                         env=dict(os.environ, ASAN_OPTIONS="detect_leaks=1", UBSAN_OPTIONS="print_stacktrace=1"))
    assert run.returncode == 0, run.stdout + run.stderr
    assert "runtime error" not in run.stderr and "AddressSanitizer" not in run.stderr, run.stderr
    assert run.stdout.startswith("checksum ")
