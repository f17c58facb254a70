"""Host code under AddressSanitizer and UndefinedBehaviorSanitizer (CPU only).

The CPU oracle (oracle/pq2_port.c) and the generated HGP class code compiled
for the host (tests/host_eri_check.cpp over csrc/_gen) are built with
-fsanitize=address,undefined, and the oracle and host-codegen test modules are
run against those builds in a child Python process with the ASan runtime
preloaded.  Any out-of-bounds access, use after free, signed overflow, invalid
shift or misaligned load in that code ends the child with an error report, so
this test fails.

The generated programs are the same straight-line VRR/HRR code the CUDA class
kernels include, so an index the generator got wrong (an operand beyond the
scratch it sizes, say) shows up here as well, before any GPU run.
"""
import os
import shutil
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SAN = ["-fsanitize=address,undefined", "-fno-sanitize-recover=undefined"]


def _runtime(name):
    """Path of a gcc sanitizer runtime, or None."""
    gcc = shutil.which("gcc")
    if gcc is None:
        return None
    p = subprocess.run([gcc, "-print-file-name=" + name], capture_output=True, text=True).stdout.strip()
    return p if os.path.isabs(p) and os.path.exists(p) else None


def test_oracle_and_generated_code_clean_under_asan_ubsan(tmp_path):
    asan = _runtime("libasan.so")
    if asan is None or _runtime("libubsan.so") is None:
        pytest.skip("gcc sanitizer runtimes not installed")
    port = tmp_path / "libpq2_port_san.so"
    subprocess.run(["gcc", "-O1", "-g", "-fno-omit-frame-pointer", *SAN, "-fPIC", "-fopenmp", "-shared", "-o",
                    str(port), os.path.join(ROOT, "oracle", "pq2_port.c"), "-lm"], check=True)
    env = dict(os.environ)
    env.update({
        "LD_PRELOAD": asan,
        # CPython keeps objects alive at exit by design; leaks are not what this checks
        "ASAN_OPTIONS": "detect_leaks=0:halt_on_error=1:abort_on_error=0",
        "UBSAN_OPTIONS": "halt_on_error=1:print_stacktrace=1",
        "RCHEM_SANITIZE_PORT": str(port),
        # -O0: the generated (dd|dd) code takes minutes to compile instrumented at -O1
        "RCHEM_SANITIZE_FLAGS": " ".join(["-O0", *SAN]),
    })
    # -s: a sanitizer report goes to the real stderr (it ends the process before pytest could print it)
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-s", "-x", "-m", "not gpu", "-p", "no:cacheprovider",
                        os.path.join(ROOT, "tests", "test_oracle.py"),
                        os.path.join(ROOT, "tests", "test_codegen_host.py")],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=900)
    out = r.stdout + r.stderr
    assert r.returncode == 0, out[-6000:]
    assert "runtime error:" not in out, out[-6000:]
    assert "AddressSanitizer" not in out, out[-6000:]
    assert " passed" in out, out[-2000:]
