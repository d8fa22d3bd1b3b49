"""The CPU restatement (oracle/gbns_oracle.c) under AddressSanitizer and
UndefinedBehaviorSanitizer: tests/cpp/oracle_sanitize.c runs every entry
point over the scheme families, coordinate maps and boundary kinds on small
ragged grids; any out-of-bounds access or undefined operation aborts it."""
import os
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_oracle_clean_under_asan_ubsan():
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "oracle_sanitize")
        cmd = ["gcc", "-std=c11", "-O1", "-g", "-fno-omit-frame-pointer", "-ffp-contract=off",
               "-fsanitize=address,undefined", "-fno-sanitize-recover=all",
               "-I" + os.path.join(ROOT, "include"),
               os.path.join(ROOT, "oracle", "gbns_oracle.c"), os.path.join(ROOT, "tests", "cpp", "oracle_sanitize.c"),
               "-o", exe, "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0 and "sanitize" in r.stderr and "unrecognized" in r.stderr:
            pytest.skip("compiler without sanitizers")
        assert r.returncode == 0, r.stderr[-3000:]
        env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=1", UBSAN_OPTIONS="print_stacktrace=1")
        out = subprocess.run([exe], capture_output=True, text=True, timeout=300, env=env)
    assert out.returncode == 0, (out.stdout + out.stderr)[-4000:]
    assert "sanitized oracle runs ok" in out.stdout
