"""The C++ builder classes of include/gbjk_fock.hpp drive the GPU engine the
way megalochem's SCF drives fock::J / fock::K (src/hf/hfscf.cpp:201-259):
create_j("dfao") / create_k("dfmo") / create_k("dfmem"), the setters,
init(), compute_J() / compute_K(), get_J() / get_K_A().  A small C++ program
reads the water problem from files, runs the builders on the GPU in FP64
and writes J and K; they must equal the oracle bit for bit (DF-MEM K is the
DF-AO exchange, so it is checked against the oracle's DF-AO K)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r'''
#include <cstdio>
#include <fstream>
#include <vector>
#include "gbjk_fock.hpp"

template <class T> std::vector<T> rd(const std::string& f) {
  std::ifstream in(f, std::ios::binary | std::ios::ate);
  const size_t n = (size_t)in.tellg() / sizeof(T);
  std::vector<T> v(n);
  in.seekg(0);
  in.read(reinterpret_cast<char*>(v.data()), n * sizeof(T));
  return v;
}
template <class T> void wr(const std::string& f, const std::vector<T>& v) {
  std::ofstream out(f, std::ios::binary);
  out.write(reinterpret_cast<const char*>(v.data()), v.size() * sizeof(T));
}

int main(int argc, char** argv) {
  const std::string d = argv[1];
  auto dims = rd<int>(d + "/dims");  // nbf naux nblk nocc
  auto bs = rd<int>(d + "/bsizes"), pk = rd<int>(d + "/panelK"), cm = rd<int>(d + "/colmap");
  auto B = rd<double>(d + "/B"), Li = rd<double>(d + "/Linv"), Vi = rd<double>(d + "/Vinv");
  const int nbf = dims[0], nocc = dims[3];
  gbjk_desc desc{nbf, dims[1], dims[2], bs.data(), pk.data(), cm.data(), 1e-10, 0};
  try {
    auto eng = std::make_shared<gbjk_fock::engine>(desc, B.data(), Li.data(), Vi.data());
    auto P = std::make_shared<std::vector<double>>(rd<double>(d + "/P"));
    auto C = std::make_shared<std::vector<double>>(rd<double>(d + "/C"));
    auto j = gbjk_fock::create_j(eng, "dfao");
    j->set_density_alpha(P);
    j->init();
    j->compute_J();
    wr(d + "/J", *j->get_J());
    auto k = gbjk_fock::create_k(eng, "dfmo");
    k->set_coeff_alpha(C, nocc);
    k->init();
    k->compute_K();
    wr(d + "/K", *k->get_K_A());
    auto km = gbjk_fock::create_k(eng, "dfmem");
    km->set_density_alpha(P);
    km->init();
    km->compute_K();
    wr(d + "/Kmem", *km->get_K_A());
    try {
      gbjk_fock::create_k(eng, "dfrobust");
    } catch (const std::runtime_error& ex) {
      std::printf("dfrobust: %s\n", ex.what());
    }
  } catch (const std::exception& ex) {
    std::printf("error: %s\n", ex.what());
    return 1;
  }
  return 0;
}
'''


@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_cpp_builders_on_gpu_match_oracle(water, tmp_path):
    from chem_gb300.fock import tune_plan
    from oracle.oracle import Oracle
    ds = water
    lay = ds.layout
    rng = np.random.default_rng(11)
    C = np.ascontiguousarray(np.linalg.qr(rng.standard_normal((ds.nbf, ds.nbf)))[0][:, :ds.nocc])
    P = C @ C.T
    d = tmp_path
    np.array([lay.nbf, lay.naux, lay.nblk, ds.nocc], np.int32).tofile(d / "dims")
    np.asarray(lay.bsizes, np.int32).tofile(d / "bsizes")
    np.asarray(lay.panel_K, np.int32).tofile(d / "panelK")
    np.concatenate(lay.column_map()).astype(np.int32).tofile(d / "colmap")
    np.ascontiguousarray(ds.B).tofile(d / "B")
    np.ascontiguousarray(np.tril(ds.Linv)).tofile(d / "Linv")
    np.ascontiguousarray(ds.Vinv).tofile(d / "Vinv")
    P.tofile(d / "P")
    C.tofile(d / "C")
    src = d / "drive.cpp"
    src.write_text(SRC)
    exe = d / "drive"
    lib = os.path.join(ROOT, "chem_gb300", "lib")
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                           str(src), "-L", lib, "-lgbjk", "-Wl,-rpath," + lib, "-o", str(exe)])
    out = subprocess.run([str(exe), str(d)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "dfrobust: Cannot use robust k for method other than PARI" in out.stdout
    n = ds.nbf
    J = np.fromfile(d / "J").reshape(n, n)
    K = np.fromfile(d / "K").reshape(n, n)
    Km = np.fromfile(d / "Kmem").reshape(n, n)
    orc = Oracle(lay, ds.B)
    assert np.array_equal(J, orc.df_j(ds.Vinv, 2 * P, 1e-10))
    kc = tune_plan(n, ds.naux, ds.nocc)[0]["fp64_kchunk"]
    assert np.array_equal(K, orc.dfmo_k(np.tril(ds.Linv), C, 1e-10, kchunk=kc))
    kca = tune_plan(n, ds.naux, n)[0]["fp64_kchunk"]
    assert np.array_equal(Km, orc.dfao_k(ds.Vinv, P, 1e-10, kchunk=kca))
    assert np.abs(Km - K).max() <= 1e-10  # DF-AO/DF-MEM K = DF-MO K for P = C C^T
