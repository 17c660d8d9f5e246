"""The C++ header (include/newman_gb300.hpp) compiles against the library and
drives the host-side calls of a reference-style caller (no GPU needed)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <cstdio>
#include "newman_gb300.hpp"
using newman_gb300::Mandelbrot;
int main() {
  Mandelbrot mandel(480, 640);                 // FractalViewer::reset, viewer.cpp:76
  if (mandel.N() != 256 || mandel.rows() != 480) return 1;
  mandel.setView({"-0.75", "0"}, {"0.0046875", "0.0046875"}, 1024);
  if (!mandel.useHardware()) return 2;
  mandel.zoomAt(2.0f, 100, 200);                // zoom drag, viewer.cpp:420
  mandel.translate(3, -4);                      // pan drag, viewer.cpp:424
  Mandelbrot saved = mandel;                    // beautyRender, viewer.cpp:193
  mandel.scaleUp(3);
  if (mandel.rows() != 1440 || saved.rows() != 480) return 3;
  mandel = saved;                               // viewer.cpp:251
  auto p = mandel.pointAt(0, 0);
  std::printf("%s %s\n", p.re.c_str(), p.im.c_str());
  try {
    mandel.setN(0);
    return 4;
  } catch (const newman_gb300::Error& e) {
    if (e.code != NM_ERR_ARG) return 5;
  }
  return 0;
}
"""


def test_cxx_wrapper_compiles_and_runs(tmp_path):
    import newman_gb300
    lib = newman_gb300.LIB_PATH
    if not os.path.exists(lib):
        pytest.skip("library not built")
    src = tmp_path / "t.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "t"
    subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                    str(exe), lib, "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, (out.returncode, out.stdout, out.stderr)
    assert out.stdout.split()[0].startswith("-0.")
