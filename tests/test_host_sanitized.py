"""The library's host C11 code run under AddressSanitizer and UndefinedBehaviorSanitizer: the frame set-up,
clamps, parameter scenes and synthetic maps over ordinary and edge inputs, and the renderer backend's host
logic through its table over a fake device.  No report, exit 0."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "artful_gb300", "csrc")


def _build_and_run(tmp_path, driver, units):
    exe = str(tmp_path / driver.replace(".c", ""))
    cmd = [os.environ.get("CC", "gcc"), "-std=c11", "-O1", "-g", "-fno-omit-frame-pointer",
           "-fsanitize=address,undefined,float-cast-overflow", "-fno-sanitize-recover=all", "-ffp-contract=off",
           "-I" + os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", driver)] + \
          [os.path.join(CSRC, u) for u in units] + ["-lm", "-o", exe]
    build = subprocess.run(cmd, capture_output=True, text=True)
    if build.returncode != 0 and "sanitize" in build.stderr:
        pytest.skip("this compiler has no sanitizer runtime")
    assert build.returncode == 0, build.stderr
    run = subprocess.run([exe], capture_output=True, text=True, timeout=300,
                         env=dict(os.environ, ASAN_OPTIONS="detect_leaks=1", UBSAN_OPTIONS="print_stacktrace=1"))
    assert run.returncode == 0, run.stdout + run.stderr
    assert "runtime error" not in run.stderr and "AddressSanitizer" not in run.stderr, run.stderr
    return run.stdout


def test_host_code_under_sanitizers(tmp_path):
    assert _build_and_run(tmp_path, "host_sanitized.c", ["holeHost.c", "synthScene.c"]).startswith("checksum ")


def test_renderer_host_logic_under_sanitizers(tmp_path):
    out = _build_and_run(tmp_path, "renderer_sanitized.c", ["renderer.c", "holeHost.c", "synthScene.c"])
    assert "renderer checks failed: 0" in out
