"""The L-BFGS driver of gbv_cvt_newton (geogram_gb300/csrc/gbv_lbfgs.h),
host code compiled here with g++ and run without a GPU: the extended
Rosenbrock function and a quadratic converge (as scipy's L-BFGS does on
the same functions), every
accepted step satisfies the sufficient-decrease condition, and a stop after
nb_iter iterations with epsg = 0 (the reference's CVT::Newton_iterations
settings, voronoi/CVT.cpp:295-302) does exactly nb_iter iterations."""
import os
import subprocess
import textwrap

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

HARNESS = textwrap.dedent(r"""
    #include <cstdio>
    #include <cmath>
    #include "gbv_lbfgs.h"
    using namespace gbv;
    int main() {
      // extended Rosenbrock, n = 100, start (-1.2, 1, -1.2, 1, ...)
      {
        const size_t n = 100;
        std::vector<double> x(n);
        for (size_t i = 0; i < n; i += 2) { x[i] = -1.2; x[i + 1] = 1.0; }
        LbfgsParams p; p.m = 7; p.max_iter = 500; p.epsg = 1e-10;
        double fprev = 1e300; int bad = 0;
        auto fg = [&](const std::vector<double>& v, std::vector<double>& g) {
          double f = 0;
          for (size_t i = 0; i < n; i += 2) {
            const double t1 = 1 - v[i], t2 = 10 * (v[i + 1] - v[i] * v[i]);
            f += t1 * t1 + t2 * t2;
            g[i] = -2 * t1 - 40 * v[i] * t2;
            g[i + 1] = 20 * t2;
          }
          return f;
        };
        auto cb = [&](int, const std::vector<double>&, double f, const std::vector<double>&) {
          if (!(f < fprev)) ++bad;
          fprev = f;
        };
        LbfgsResult r = lbfgs_minimize(x, p, fg, cb);
        double err = 0; for (double v : x) err = std::fmax(err, std::fabs(v - 1.0));
        std::printf("rosen %d %d %.3e %.3e %d %d\n", r.iterations, r.evaluations, r.f, err, bad,
                    r.line_search_info);
      }
      // quadratic with condition number 1e2, n = 50: fixed iteration count
      {
        const size_t n = 50;
        std::vector<double> x(n, 1.0), a(n);
        for (size_t i = 0; i < n; ++i) a[i] = std::pow(1e2, double(i) / (n - 1));
        auto fg = [&](const std::vector<double>& v, std::vector<double>& g) {
          double f = 0;
          for (size_t i = 0; i < n; ++i) { f += 0.5 * a[i] * v[i] * v[i]; g[i] = a[i] * v[i]; }
          return f;
        };
        LbfgsParams p; p.m = 7; p.max_iter = 30;
        int calls = 0;
        LbfgsResult r = lbfgs_minimize(x, p, fg,
            [&](int, const std::vector<double>&, double, const std::vector<double>&) { ++calls; });
        std::printf("quad30 %d %d %.3e\n", r.iterations, calls, r.f);
        p.max_iter = 400; p.epsg = 1e-9;
        std::vector<double> y(n, 1.0);
        r = lbfgs_minimize(y, p, fg, nullptr);
        std::printf("quad %d %.3e\n", r.iterations, r.f);
      }
      return 0;
    }
""")


def test_lbfgs_converges_and_counts_iterations(tmp_path):
    src = tmp_path / "h.cpp"
    src.write_text(HARNESS)
    exe = tmp_path / "h"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "geogram_gb300", "csrc"),
                    str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    ros = out[0].split()
    assert ros[0] == "rosen"
    assert float(ros[3]) < 1e-16 and float(ros[4]) < 1e-7  # f and max |x - 1| at the minimum
    assert int(ros[5]) == 0                                # every accepted step decreased f
    q30 = out[1].split()
    assert int(q30[1]) == 30 and int(q30[2]) == 30         # nb_iter iterations, one callback each
    q = out[2].split()
    assert float(q[2]) < 1e-15


CVT_HARNESS = textwrap.dedent(r"""
    #include <cstdio>
    #include <cstdlib>
    #include <vector>
    #include "gbv_lbfgs.h"
    extern "C" int ref_init();
    extern "C" int ref_rvd_volume(const double*, unsigned, const unsigned*, unsigned,
                                  const double*, unsigned, double*, double*, double*, double*);
    int main(int argc, char** argv) {
      // argv: mesh file, tets file, seeds file (raw binary), iterations, output file
      auto slurp = [](const char* p, size_t& bytes) {
        FILE* f = std::fopen(p, "rb"); std::fseek(f, 0, SEEK_END); bytes = std::ftell(f);
        std::fseek(f, 0, SEEK_SET); std::vector<char> b(bytes);
        if (std::fread(b.data(), 1, bytes, f) != bytes) std::exit(2); std::fclose(f); return b;
      };
      size_t bv, bt, bx;
      auto V = slurp(argv[1], bv); auto T = slurp(argv[2], bt); auto X = slurp(argv[3], bx);
      const unsigned nv = bv / 24, nt = bt / 16, n = bx / 24;
      const double* v = (const double*)V.data(); const unsigned* t = (const unsigned*)T.data();
      std::vector<double> x((const double*)X.data(), (const double*)X.data() + 3 * n);
      ref_init();
      gbv::LbfgsParams p; p.m = 7; p.max_iter = std::atoi(argv[4]);
      std::vector<double> m(n), mg(3 * n);
      auto fg = [&](const std::vector<double>& y, std::vector<double>& g) {
        double f = 0; ref_rvd_volume(v, nv, t, nt, y.data(), n, mg.data(), m.data(), &f, g.data());
        return f;
      };
      gbv::LbfgsResult r = gbv::lbfgs_minimize(x, p, fg, nullptr);
      FILE* o = std::fopen(argv[5], "wb"); std::fwrite(x.data(), 8, x.size(), o); std::fclose(o);
      std::printf("%d %.17g\n", r.iterations, r.f);
      return 0;
    }
""")


def test_lbfgs_restatement_follows_the_reference_hlbfgs(tmp_path):
    """Our L-BFGS driven by the reference's own CVT energy and gradient
    (oracle/_ref) against the reference's CVT::Newton_iterations (HLBFGS):
    Newton_iterations(1) and (10) take 2 and 11 steps (HLBFGS stops once its
    count exceeds max_iter), and after as many steps the seeds agree to
    rounding (fixtures from tests/golden/make_golden.py)."""
    import numpy as np
    from oracle import oracle
    if not oracle.ref_available():
        pytest.skip("oracle/_ref is not built (reference checkout absent)")
    from conftest import load_golden
    src = tmp_path / "c.cpp"
    src.write_text(CVT_HARNESS)
    exe = tmp_path / "c"
    lib = os.path.dirname(oracle.REF_LIB)
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "geogram_gb300", "csrc"),
                    str(src), "-o", str(exe), "-L", lib, "-lgbv_ref", f"-Wl,-rpath,{lib}"],
                   check=True)
    for name in ("cube_300", "lshape_500"):
        d = load_golden(f"cvt_newton_{name}.npz")
        files = []
        for key, dt in (("mesh_xyz", np.float64), ("tets", np.uint32), ("x", np.float64)):
            p = tmp_path / f"{name}_{key}.bin"
            np.ascontiguousarray(d[key], dtype=dt).tofile(p)
            files.append(str(p))
        for it in (1, 10):
            out = tmp_path / f"{name}_{it}.bin"
            r = subprocess.run([str(exe), *files, str(it + 1), str(out)], capture_output=True,
                               text=True, check=True)
            its, f = r.stdout.split()
            x = np.fromfile(out).reshape(-1, 3)
            assert int(its) == it + 1
            assert np.max(np.abs(x - d[f"x{it}"])) < 1e-12
            assert abs(float(f) - float(d[f"f{it}"])) <= 1e-12 * float(d[f"f{it}"])
