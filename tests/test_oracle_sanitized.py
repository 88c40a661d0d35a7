"""The oracle under AddressSanitizer and UndefinedBehaviorSanitizer (CPU).

oracle/ns_oracle.c built with -fsanitize=address,undefined (abort on the
first report) runs the known-answer tests and the comparison with the
PyTorch twin in a child process that preloads the ASan runtime: any
out-of-bounds access, use after free, signed overflow or other undefined
behaviour in the restatement fails the run."""
import os
import shutil
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_oracle_kats_under_asan_ubsan(oracle_mod):
    if not shutil.which("gcc"):
        pytest.skip("gcc is needed for the sanitized build")
    libasan = subprocess.run(["gcc", "-print-file-name=libasan.so"], capture_output=True,
                             text=True).stdout.strip()
    if not libasan or not Path(libasan).exists():
        pytest.skip("no ASan runtime for this compiler")
    oracle_mod.build(sanitize=True)
    env = dict(os.environ, NS_ORACLE_SANITIZE="1", LD_PRELOAD=libasan,
               ASAN_OPTIONS="detect_leaks=0:abort_on_error=1",
               UBSAN_OPTIONS="print_stacktrace=1:halt_on_error=1", OMP_NUM_THREADS="2")
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-p", "no:cacheprovider",
                        "-m", "not gpu", "-k", "not library_tables",
                        "tests/test_oracle_kat.py", "tests/test_torch_ref.py"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=1200)
    tail = r.stdout[-3000:] + r.stderr[-3000:]
    assert r.returncode == 0, tail
    assert "ERROR: AddressSanitizer" not in r.stderr and "runtime error" not in r.stderr, tail
    assert " passed" in r.stdout
