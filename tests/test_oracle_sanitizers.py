"""The oracle (the checker of every parity test) under AddressSanitizer and
UndefinedBehaviorSanitizer: oracle/sanity_main.c drives its entry points on
seeded inputs -- every field kind, 1-cell to 33^3 grids, both topologies and
all placements, the sweeps, the draw layout, the LOD generator, the batch
driver and the FP64 fitting path -- and any out-of-bounds access, leak or
undefined operation aborts it.  CPU only."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_oracle_under_asan_ubsan():
    if shutil.which("gcc") is None or shutil.which("make") is None:
        pytest.skip("no gcc / make")
    b = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "sanitize"], capture_output=True, text=True)
    if b.returncode != 0:
        if "asan" in b.stderr.lower() or "sanitize" in b.stderr.lower():
            pytest.skip("no sanitizer runtime: " + b.stderr[-300:])
        raise AssertionError(b.stderr[-3000:])
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0", UBSAN_OPTIONS="print_stacktrace=1",
               OMP_NUM_THREADS="2")
    r = subprocess.run([os.path.join(ROOT, "oracle", "_build", "oracle_sanity")], capture_output=True, text=True,
                       env=env, timeout=600)
    assert r.returncode == 0 and "oracle sanity ok" in r.stdout, (r.stdout[-1000:], r.stderr[-4000:])
