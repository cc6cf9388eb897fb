// Limited-memory BFGS with the More-Thuente line search, host code.
//
// This is the method of the reference's default optimizer (HLBFGS with
// update strategy 0, third_party/HLBFGS/HLBFGS.cpp, driven by
// numerics/lbfgs_optimizers.cpp:159-196 and voronoi/CVT.cpp:272-307): the
// two-loop recursion over the last m pairs (s, y) with the initial inverse
// Hessian (s'y / y'y) I, a first step of 1 / |g| along -g and of 1 after
// that, and a line search for the sufficient decrease and curvature
// conditions (ftol 1e-4, gtol 0.9, xtol 1e-16, steps in [1e-20, 1e20], at
// most 20 evaluations; INIT_HLBFGS, HLBFGS.cpp:30-54).  The line search is
// the published algorithm of J. J. More and D. J. Thuente ("Line search
// algorithms with guaranteed sufficient decrease", ACM TOMS 20(3), 1994),
// written here from the paper, with HLBFGS's one departure from it (a
// bracketing step keeps at least 1/1000 of the interval, LineSearch.cpp's
// SAFE_SEARCH).  Everything is plain C++ on std::vector so
// that it builds and is tested without a GPU; the objective is a callback.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <functional>
#include <vector>

namespace gbv {

struct LbfgsParams {
  int m = 7;                // pairs kept
  int max_iter = 100;
  double ftol = 1e-4;       // sufficient decrease
  double gtol = 0.9;        // curvature
  double xtol = 1e-16;      // relative width of the bracket
  double stpmin = 1e-20, stpmax = 1e20;
  int maxfev = 20;          // evaluations per line search
  double epsg = 0.0;        // stop once |g| <= epsg (0: never)
};

struct LbfgsResult {
  int iterations = 0;
  int evaluations = 0;
  int line_search_info = 0;  // 1: conditions met; other values: why it stopped
  double f = 0.0;
};

namespace lbfgs_detail {

inline double dot(const std::vector<double>& a, const std::vector<double>& b) {
  double s = 0.0;
  for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
  return s;
}

// One safeguarded step of the More-Thuente search: the interval
// [stx, sty] with the values and derivatives at its ends, the trial stp
// with fp, dp; returns the next trial in stp and updates the interval.
inline void step(double& stx, double& fx, double& dx, double& sty, double& fy, double& dy,
                 double& stp, double fp, double dp, bool& brackt, double stpmin, double stpmax,
                 int& info) {
  info = 0;
  if ((brackt && (stp <= std::min(stx, sty) || stp >= std::max(stx, sty))) || dx * (stp - stx) >= 0.0 ||
      stpmax < stpmin)
    return;
  const double sgnd = dp * (dx / std::fabs(dx));
  double stpf, stpc, stpq;
  bool bound;
  if (fp > fx) {
    // 1: a higher value; the minimum is bracketed
    info = 1;
    bound = true;
    const double theta = (fx - fp) * 3.0 / (stp - stx) + dx + dp;
    const double s = std::max({std::fabs(theta), std::fabs(dx), std::fabs(dp)});
    double gamma = s * std::sqrt((theta / s) * (theta / s) - (dx / s) * (dp / s));
    if (stp < stx) gamma = -gamma;
    const double p = (gamma - dx) + theta, q = ((gamma - dx) + gamma) + dp;
    stpc = stx + (p / q) * (stp - stx);
    stpq = stx + ((dx / ((fx - fp) / (stp - stx) + dx)) / 2.0) * (stp - stx);
    stpf = std::fabs(stpc - stx) < std::fabs(stpq - stx) ? stpc : stpc + (stpq - stpc) / 2.0;
    // HLBFGS's safeguard (from TNPACK): at least 1/1000 of the way from stx
    stpf = stp > stx ? std::max(stx + 0.001 * (stp - stx), stpf)
                     : std::min(stx + 0.001 * (stp - stx), stpf);
    brackt = true;
  } else if (sgnd < 0.0) {
    // 2: a lower value and derivatives of opposite signs
    info = 2;
    bound = false;
    const double theta = (fx - fp) * 3.0 / (stp - stx) + dx + dp;
    const double s = std::max({std::fabs(theta), std::fabs(dx), std::fabs(dp)});
    double gamma = s * std::sqrt((theta / s) * (theta / s) - (dx / s) * (dp / s));
    if (stp > stx) gamma = -gamma;
    const double p = (gamma - dp) + theta, q = ((gamma - dp) + gamma) + dx;
    stpc = stp + (p / q) * (stx - stp);
    stpq = stp + (dp / (dp - dx)) * (stx - stp);
    stpf = std::fabs(stpc - stp) > std::fabs(stpq - stp) ? stpc : stpq;
    brackt = true;
  } else if (std::fabs(dp) < std::fabs(dx)) {
    // 3: a lower value, same signs, the derivative decreases in magnitude
    info = 3;
    bound = true;
    const double theta = (fx - fp) * 3.0 / (stp - stx) + dx + dp;
    const double s = std::max({std::fabs(theta), std::fabs(dx), std::fabs(dp)});
    double gamma = s * std::sqrt(std::max(0.0, (theta / s) * (theta / s) - (dx / s) * (dp / s)));
    if (stp > stx) gamma = -gamma;
    const double p = (gamma - dp) + theta, q = (gamma + (dx - dp)) + gamma;
    const double r = p / q;
    if (r < 0.0 && gamma != 0.0) stpc = stp + r * (stx - stp);
    else stpc = stp > stx ? stpmax : stpmin;
    stpq = stp + (dp / (dp - dx)) * (stx - stp);
    if (brackt) stpf = std::fabs(stp - stpc) < std::fabs(stp - stpq) ? stpc : stpq;
    else stpf = std::fabs(stp - stpc) > std::fabs(stp - stpq) ? stpc : stpq;
  } else {
    // 4: a lower value, same signs, the derivative does not decrease
    info = 4;
    bound = false;
    if (brackt) {
      const double theta = (fp - fy) * 3.0 / (sty - stp) + dy + dp;
      const double s = std::max({std::fabs(theta), std::fabs(dy), std::fabs(dp)});
      double gamma = s * std::sqrt((theta / s) * (theta / s) - (dy / s) * (dp / s));
      if (stp > sty) gamma = -gamma;
      const double p = (gamma - dp) + theta, q = ((gamma - dp) + gamma) + dy;
      stpf = stp + (p / q) * (sty - stp);
    } else {
      stpf = stp > stx ? stpmax : stpmin;
    }
  }
  // the new interval
  if (fp > fx) {
    sty = stp;
    fy = fp;
    dy = dp;
  } else {
    if (sgnd < 0.0) {
      sty = stx;
      fy = fx;
      dy = dx;
    }
    stx = stp;
    fx = fp;
    dx = dp;
  }
  stpf = std::max(stpmin, std::min(stpmax, stpf));
  stp = stpf;
  if (brackt && bound) {
    const double mid = stx + 0.66 * (sty - stx);
    stp = sty > stx ? std::min(mid, stp) : std::max(mid, stp);
  }
}

}  // namespace lbfgs_detail

// f(x, g) returns the objective at x and writes its gradient to g.
// newiter(iteration, x, f, g) is called after every accepted step.
// x holds the start and receives the last accepted point.
inline LbfgsResult lbfgs_minimize(
    std::vector<double>& x, const LbfgsParams& prm,
    const std::function<double(const std::vector<double>&, std::vector<double>&)>& fg,
    const std::function<void(int, const std::vector<double>&, double,
                             const std::vector<double>&)>& newiter) {
  using lbfgs_detail::dot;
  const size_t n = x.size();
  LbfgsResult res;
  std::vector<double> g(n), d(n), x0(n), g0(n), q(n);
  std::vector<std::vector<double>> S, Y;
  std::vector<double> rho;
  double f = fg(x, g);
  ++res.evaluations;
  res.f = f;
  for (int it = 0; it < prm.max_iter; ++it) {
    const double gnorm = std::sqrt(dot(g, g));
    if (gnorm <= prm.epsg || gnorm == 0.0) break;
    // ---- direction: two-loop recursion
    double stp = 1.0;
    if (S.empty()) {
      for (size_t i = 0; i < n; ++i) d[i] = -g[i];
      stp = 1.0 / gnorm;
    } else {
      q = g;
      const int k = (int)S.size();
      std::vector<double> alpha(k);
      for (int j = k - 1; j >= 0; --j) {
        alpha[j] = rho[j] * dot(S[j], q);
        for (size_t i = 0; i < n; ++i) q[i] -= alpha[j] * Y[j][i];
      }
      const double gamma = dot(S[k - 1], Y[k - 1]) / dot(Y[k - 1], Y[k - 1]);
      for (size_t i = 0; i < n; ++i) q[i] *= gamma;
      for (int j = 0; j < k; ++j) {
        const double beta = rho[j] * dot(Y[j], q);
        for (size_t i = 0; i < n; ++i) q[i] += S[j][i] * (alpha[j] - beta);
      }
      for (size_t i = 0; i < n; ++i) d[i] = -q[i];
    }
    // ---- More-Thuente line search from x0 along d
    x0 = x;
    g0 = g;
    const double finit = f, dginit = dot(g, d);
    if (!(dginit < 0.0)) {
      res.line_search_info = 0;  // not a descent direction
      break;
    }
    const double dgtest = prm.ftol * dginit;
    double width = prm.stpmax - prm.stpmin, width1 = 2.0 * width;
    double stx = 0.0, fx = finit, dgx = dginit, sty = 0.0, fy = finit, dgy = dginit;
    bool brackt = false, stage1 = true;
    int infoc = 1, info = 0, nfev = 0;
    double stmin = 0.0, stmax = 0.0;
    for (;;) {
      if (brackt) {
        stmin = std::min(stx, sty);
        stmax = std::max(stx, sty);
      } else {
        stmin = stx;
        stmax = stp + 4.0 * (stp - stx);
      }
      stp = std::max(prm.stpmin, std::min(prm.stpmax, stp));
      if ((brackt && (stp <= stmin || stp >= stmax)) || nfev >= prm.maxfev - 1 || infoc == 0 ||
          (brackt && stmax - stmin <= prm.xtol * stmax))
        stp = stx;
      for (size_t i = 0; i < n; ++i) x[i] = x0[i] + stp * d[i];
      f = fg(x, g);
      ++nfev;
      ++res.evaluations;
      const double dg = dot(g, d);
      const double ftest1 = finit + stp * dgtest;
      if ((brackt && (stp <= stmin || stp >= stmax)) || infoc == 0) info = 6;
      if (stp == prm.stpmax && f <= ftest1 && dg <= dgtest) info = 5;
      if (stp == prm.stpmin && (f > ftest1 || dg >= dgtest)) info = 4;
      if (nfev >= prm.maxfev) info = 3;
      if (brackt && stmax - stmin <= prm.xtol * stmax) info = 2;
      if (f <= ftest1 && std::fabs(dg) <= prm.gtol * (-dginit)) info = 1;
      if (info != 0) break;
      if (stage1 && f <= ftest1 && dg >= std::min(prm.ftol, prm.gtol) * dginit) stage1 = false;
      if (stage1 && f <= fx && f > ftest1) {
        // the modified function psi(stp) = f(stp) - f(0) - ftol stp f'(0)
        double fm = f - stp * dgtest, fxm = fx - stx * dgtest, fym = fy - sty * dgtest;
        double dgm = dg - dgtest, dgxm = dgx - dgtest, dgym = dgy - dgtest;
        lbfgs_detail::step(stx, fxm, dgxm, sty, fym, dgym, stp, fm, dgm, brackt, stmin, stmax,
                           infoc);
        fx = fxm + stx * dgtest;
        fy = fym + sty * dgtest;
        dgx = dgxm + dgtest;
        dgy = dgym + dgtest;
      } else {
        lbfgs_detail::step(stx, fx, dgx, sty, fy, dgy, stp, f, dg, brackt, stmin, stmax, infoc);
      }
      if (brackt) {
        if (std::fabs(sty - stx) >= 0.66 * width1) stp = stx + 0.5 * (sty - stx);
        width1 = width;
        width = std::fabs(sty - stx);
      }
    }
    res.line_search_info = info;
    if (info != 1) {
      // the search failed: keep the best point it has seen
      if (!(f < finit)) {
        x = x0;
        g = g0;
        f = finit;
      }
      res.f = f;
      break;
    }
    // ---- the new pair
    std::vector<double> s(n), y(n);
    for (size_t i = 0; i < n; ++i) {
      s[i] = x[i] - x0[i];
      y[i] = g[i] - g0[i];
    }
    const double ys = dot(y, s);
    if (ys > 0.0) {
      if ((int)S.size() == prm.m) {
        S.erase(S.begin());
        Y.erase(Y.begin());
        rho.erase(rho.begin());
      }
      S.push_back(std::move(s));
      Y.push_back(std::move(y));
      rho.push_back(1.0 / ys);
    }
    res.iterations = it + 1;
    res.f = f;
    if (newiter) newiter(it + 1, x, f, g);
  }
  return res;
}

}  // namespace gbv
