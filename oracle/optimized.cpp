// optimized.cpp -- an optimised CPU port of the plain two-electron VMC + SR
// path, timed beside the faithful one for an honest CPU/GPU ratio.
//
// TEST/BENCH INFRASTRUCTURE ONLY (the CPU baseline legs of bench.py). It
// runs the algorithm of the GPU walker kernel on the CPU instead of the
// reference's call pattern: one walker's state in a struct (no allocation),
// orbital values/gradients/Laplacians and the pair terms cached at the
// current configuration and replaced only on accepted moves, the
// single-electron Metropolis ratio sigma(r') / sigma(r) x exp(2 du), the
// local energy assembled from the caches every sweep, and the SR sums
// (sum O, sum E O, sum O O^T over the exponent and the Pade b). Chains run on
// std::thread workers, each owning a contiguous range of walkers. The
// system is psi = sigma(r1) sigma(r2) exp(u(r12)), sigma = sum_I exp(-a r_I),
// u = r / (2 (1 + b r)) (He: one centre at the origin, Z = 2; H2: centres at
// z = +-0.7, Z = 1), Gaussian moves of width `step`.
#include <chrono>
#include <cmath>
#include <cstdint>
#include <thread>
#include <vector>

namespace {

struct Sys {
  int M;
  double R[2][3];
  double Z;
  double vnn;
  double a, b;
};

struct Orb {  // sigma at one electron: value, gradient, Laplacian, d/da, e-n potential
  double v, g[3], l, da, ven;
};

inline void orbital(const Sys& s, const double* r, Orb& o) {
  o.v = o.l = o.da = o.ven = 0.0;
  o.g[0] = o.g[1] = o.g[2] = 0.0;
  for (int I = 0; I < s.M; ++I) {
    const double d0 = r[0] - s.R[I][0], d1 = r[1] - s.R[I][1], d2 = r[2] - s.R[I][2];
    const double n = std::sqrt(d0 * d0 + d1 * d1 + d2 * d2), inv = 1.0 / n;
    const double e = std::exp(-s.a * n), f = -s.a * e * inv;
    o.v += e;
    o.g[0] += f * d0;
    o.g[1] += f * d1;
    o.g[2] += f * d2;
    o.l += e * (s.a * s.a - 2.0 * s.a * inv);
    o.da += -n * e;
    o.ven -= s.Z * inv;
  }
}

struct Pair {  // u, u'/r, u'' + 2u'/r, 1/r, du/db
  double u, f, l, inv, db;
};

inline void pair(const Sys& s, const double* d, Pair& p) {
  const double r = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  const double q = 1.0 / (1.0 + s.b * r);
  p.inv = 1.0 / r;
  p.u = 0.5 * r * q;
  const double up = 0.5 * q * q, upp = -s.b * q * q * q;
  p.f = up * p.inv;
  p.l = upp + 2.0 * p.f;
  p.db = -0.5 * r * r * q * q;
}

struct Rng {  // splitmix64 -> two uniforms -> Box-Muller
  uint64_t x;
  inline uint64_t next() {
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  inline double u01() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
  inline void normal3(double* z) {
    const double r1 = std::sqrt(-2.0 * std::log(u01())), t1 = 6.283185307179586 * u01();
    const double r2 = std::sqrt(-2.0 * std::log(u01())), t2 = 6.283185307179586 * u01();
    z[0] = r1 * std::cos(t1);
    z[1] = r1 * std::sin(t1);
    z[2] = r2 * std::cos(t2);
  }
};

struct Sums {
  double n = 0, e = 0, e2 = 0, o[2] = {0, 0}, eo[2] = {0, 0}, oo[3] = {0, 0, 0}, acc = 0;
};

void chains(const Sys& s, int w0, int w1, int n_eq, int n_steps, double step, uint64_t seed, Sums* out) {
  Sums S;
  for (int w = w0; w < w1; ++w) {
    Rng rng{seed * 0x100000001B3ull + (uint64_t)w};
    double x[2][3];
    for (int i = 0; i < 2; ++i) rng.normal3(x[i]);
    Orb o[2];
    orbital(s, x[0], o[0]);
    orbital(s, x[1], o[1]);
    Pair p;
    double d[3] = {x[0][0] - x[1][0], x[0][1] - x[1][1], x[0][2] - x[1][2]};
    pair(s, d, p);
    for (int it = 0; it < n_eq + n_steps; ++it) {
      for (int i = 0; i < 2; ++i) {
        double z[3], xn[3];
        rng.normal3(z);
        for (int c = 0; c < 3; ++c) xn[c] = x[i][c] + step * z[c];
        Orb on;
        orbital(s, xn, on);
        const double* xo = x[1 - i];
        double dn[3] = {xn[0] - xo[0], xn[1] - xo[1], xn[2] - xo[2]};
        Pair pn;
        pair(s, dn, pn);
        const double ratio = on.v / o[i].v;
        if (ratio * ratio * std::exp(2.0 * (pn.u - p.u)) > rng.u01()) {
          for (int c = 0; c < 3; ++c) x[i][c] = xn[c];
          o[i] = on;
          p = pn;
          S.acc += 1.0;
        }
      }
      if (it < n_eq) continue;
      // E_L from the caches
      const double d0 = x[0][0] - x[1][0], d1 = x[0][1] - x[1][1], d2 = x[0][2] - x[1][2];
      double lap = 0.0;
      for (int i = 0; i < 2; ++i) {
        const double sg = i == 0 ? 1.0 : -1.0;
        const double gj[3] = {sg * p.f * d0, sg * p.f * d1, sg * p.f * d2};
        const double iv = 1.0 / o[i].v;
        const double gd[3] = {o[i].g[0] * iv, o[i].g[1] * iv, o[i].g[2] * iv};
        lap += o[i].l * iv + p.l + 2.0 * (gd[0] * gj[0] + gd[1] * gj[1] + gd[2] * gj[2]) +
               gj[0] * gj[0] + gj[1] * gj[1] + gj[2] * gj[2];
      }
      const double E = -0.5 * lap + o[0].ven + o[1].ven + p.inv + s.vnn;
      const double O[2] = {o[0].da / o[0].v + o[1].da / o[1].v, p.db};
      S.n += 1.0;
      S.e += E;
      S.e2 += E * E;
      for (int k = 0; k < 2; ++k) {
        S.o[k] += O[k];
        S.eo[k] += E * O[k];
      }
      S.oo[0] += O[0] * O[0];
      S.oo[1] += O[0] * O[1];
      S.oo[2] += O[1] * O[1];
    }
  }
  *out = S;
}

}  // namespace

extern "C" {

// Returns wall seconds; writes the mean energy and the acceptance ratio.
// system 0: He (Z = 2 at the origin), 1: H2 (nuclei at z = +-0.7).
double optimized_vmc(int system, int n_walkers, int n_eq, int n_steps, double step, double a, double b,
                     int n_threads, uint64_t seed, double* energy_mean, double* acceptance) {
  Sys s;
  if (system == 0) {
    s.M = 1;
    s.R[0][0] = s.R[0][1] = s.R[0][2] = 0.0;
    s.Z = 2.0;
    s.vnn = 0.0;
  } else {
    s.M = 2;
    s.R[0][0] = s.R[0][1] = 0.0;
    s.R[0][2] = -0.7;
    s.R[1][0] = s.R[1][1] = 0.0;
    s.R[1][2] = 0.7;
    s.Z = 1.0;
    s.vnn = 1.0 / 1.4;
  }
  s.a = a;
  s.b = b;
  if (n_threads < 1) n_threads = 1;
  std::vector<Sums> part(n_threads);
  std::vector<std::thread> th;
  const auto t0 = std::chrono::steady_clock::now();
  for (int k = 0; k < n_threads; ++k) {
    const int w0 = (int)((int64_t)n_walkers * k / n_threads), w1 = (int)((int64_t)n_walkers * (k + 1) / n_threads);
    th.emplace_back(chains, std::cref(s), w0, w1, n_eq, n_steps, step, seed, &part[k]);
  }
  for (auto& t : th) t.join();
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  Sums tot;
  for (const Sums& p : part) {
    tot.n += p.n;
    tot.e += p.e;
    tot.acc += p.acc;
  }
  if (energy_mean) *energy_mean = tot.n > 0 ? tot.e / tot.n : 0.0;
  if (acceptance) *acceptance = tot.acc / (2.0 * (double)n_walkers * (n_eq + n_steps));
  return secs;
}

}  // extern "C"
