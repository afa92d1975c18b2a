"""The C++ drop-in header (include/si_gpu/interval_map.hpp): a C++ program written like the
reference's own unit tests (test/tests.cpp) is compiled against the header, linked to
libsi_gpu.so and run on the GPU."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build(out_dir):
    from superintervals_gb300 import build_ext
    build_ext.build()
    exe = os.path.join(out_dir, "test_dropin")
    cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "test_dropin.cpp"), "-L", build_ext.OUT_DIR, "-lsi_gpu",
           "-Wl,-rpath," + build_ext.OUT_DIR, "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_dropin_header_compiles(tmp_path):
    """Compiles and links on any machine (no GPU needed to build)."""
    assert os.path.isfile(_build(str(tmp_path)))


@pytest.mark.gpu
def test_dropin_known_answers_on_gpu(tmp_path):
    exe = _build(str(tmp_path))
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "drop-in ok" in r.stdout
