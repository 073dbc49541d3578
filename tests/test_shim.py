"""The C++ builder shim (include/gbjk_fock.hpp) compiles against the C ABI,
links libgbjk.so, and turns a failing call into std::runtime_error."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r'''
#include <cstdio>
#include "gbjk_fock.hpp"
int main() {
  int bs[2] = {3, 2}, K[2] = {5, 5}, cm[10] = {0, 1, 2, 3, 4, 0, 1, 2, 3, 4};
  gbjk_desc d{6, 10, 2, bs, K, cm, 0.0, 0};  // block sizes sum to 5 != nbf 6
  try {
    auto e = std::make_shared<gbjk_fock::engine>(d, nullptr, nullptr, nullptr);
    std::printf("no-throw\n");
    return 1;
  } catch (const std::runtime_error& ex) {
    std::printf("threw: %s\n", ex.what());
  }
  try {
    gbjk_fock::create_k(nullptr, "dfqq");
  } catch (const std::runtime_error& ex) {
    std::printf("threw: %s\n", ex.what());
  }
  return 0;
}
'''


@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_shim_compiles_links_and_throws(tmp_path):
    src = tmp_path / "shim.cpp"
    src.write_text(SRC)
    exe = tmp_path / "shim"
    lib = os.path.join(ROOT, "chem_gb300", "lib")
    subprocess.check_call(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src),
                           "-L", lib, "-lgbjk", "-Wl,-rpath," + lib, "-o", str(exe)])
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.count("threw:") == 2
    assert "Invalid kmethod" in out.stdout
