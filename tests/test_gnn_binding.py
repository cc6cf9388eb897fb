"""The geogram-side binding (geogram_gb300/bindings/geogram_gnn.cpp) compiles
against the reference's own headers, links with geogram (the reference
build, oracle/_ref) and libgbv.so, and registers through
geo_register_NearestNeighborSearch_creator (points/nn_search.h:288): the
factory's create(3, "GNN") returns the GPU search, not its BNN fallback.
Without a GPU its first set_points reports the missing device; with one, its
lists equal BNN's, also when eight threads query it at once (the pattern of
delaunay_nn.cpp:57-70).  Needs the reference checkout (GEOGRAM_SRC, else the
usual mount) and its build; skipped otherwise."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

MAIN = r"""
#include <geogram/points/nn_search.h>
#include <cstdio>
#include <cstring>
#include <random>
#include <stdexcept>
#include <thread>
#include <vector>

namespace GEO { void register_gpu_nearest_neighbor_search(); }
extern "C" int ref_init(void);

int main() {
    ref_init();
    GEO::register_gpu_nearest_neighbor_search();
    GEO::NearestNeighborSearch_var gnn = GEO::NearestNeighborSearch::create(3, "GNN");
    GEO::NearestNeighborSearch_var bnn = GEO::NearestNeighborSearch::create(3, "BNN");
    if (gnn.is_null() || typeid(*gnn) == typeid(*bnn)) { std::printf("not registered\n"); return 1; }
    const unsigned n = 5000, k = 21;
    std::vector<double> pts(3 * n);
    std::mt19937_64 rng(7);
    std::uniform_real_distribution<double> u(0.0, 1.0);
    for (double& v : pts) v = u(rng);
    try {
        gnn->set_points(n, pts.data());
    } catch (const std::runtime_error& e) {
        if (std::strstr(e.what(), "GNN:")) { std::printf("registered, no gpu: %s\n", e.what()); return 0; }
        throw;
    }
    bnn->set_points(n, pts.data());
    std::vector<int> bad(8, 0);
    std::vector<std::thread> pool;
    for (int t = 0; t < 8; ++t) pool.emplace_back([&, t]() {
        std::vector<GEO::index_t> a(k + 8), b(k + 8);
        std::vector<double> da(k + 8), db(k + 8);
        for (unsigned i = t; i < n; i += 8) {
            const GEO::index_t kk = k + (i % 8);  // lists of growing length
            gnn->get_nearest_neighbors(kk, GEO::index_t(i), a.data(), da.data());
            bnn->get_nearest_neighbors(kk, GEO::index_t(i), b.data(), db.data());
            for (GEO::index_t r = 0; r < kk; ++r) if (da[r] != db[r]) ++bad[t];
        }
    });
    for (auto& th : pool) th.join();
    int total = 0;
    for (int v : bad) total += v;
    std::printf("registered, gpu, %d distance mismatches\n", total);
    return total == 0 ? 0 : 1;
}
"""


def test_binding_compiles_links_and_registers(tmp_path):
    from oracle import oracle
    ref = oracle.REF_SRC
    geo = os.path.join(ref, "src", "lib")
    lib_ref = os.path.join(ROOT, "oracle", "_ref", "libgbv_ref.so")
    lib_gbv = os.path.join(ROOT, "geogram_gb300", "libgbv.so")
    if not os.path.isdir(os.path.join(geo, "geogram")):
        pytest.skip("no reference checkout")
    if oracle.build_ref() is None or not os.path.exists(lib_ref):
        pytest.skip("reference build unavailable")
    if not os.path.exists(lib_gbv) or shutil.which("g++") is None:
        pytest.skip("libgbv.so or g++ missing")
    main = tmp_path / "main.cpp"
    main.write_text(MAIN)
    exe = tmp_path / "gnn_test"
    cmd = ["g++", "-std=c++17", "-O1", "-w", "-DGEOGRAM_VERSION=\"1.10.1\"",
           "-I", os.path.join(ROOT, "oracle", "ref", "shim"),
           "-I", os.path.join(ROOT, "oracle", "_ref", "gen"), "-I", geo,
           "-I", os.path.join(geo, "geogram", "third_party"), "-I", os.path.join(ROOT, "include"),
           str(main), os.path.join(ROOT, "geogram_gb300", "bindings", "geogram_gnn.cpp"),
           lib_ref, lib_gbv, f"-Wl,-rpath,{os.path.dirname(lib_ref)}",
           f"-Wl,-rpath,{os.path.dirname(lib_gbv)}", "-lpthread", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr[-2000:]
    assert r.stdout.startswith("registered")
