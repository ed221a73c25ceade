// faithful.cpp -- the reference's CPU VMC path restated in C++ for timing.
//
// TEST/BENCH INFRASTRUCTURE ONLY (the CPU baseline leg of bench.py and the
// `--impl reference` arm). It keeps the reference's call pattern, which is
// what a user of Jvanrhijn/mole runs today:
//   * every proposal clones the configuration on the heap
//     (src/metropolis/src/metrop.rs:60-71 box, 150-163 diffuse);
//   * acceptance recomputes psi(x') and psi(x) from scratch
//     (metrop.rs:73-82), or psi and grad psi three times for the diffuse
//     move (metrop.rs:165-198);
//   * samples are Operator::act_on(psi, cfg) / psi(cfg) for every observable
//     (src/montecarlo/src/samplers.rs:81-104), with the electronic
//     Hamiltonian composed as T psi + V_ion psi + V_ee psi
//     (src/operator/src/operator.rs:177-184), so psi is evaluated three more
//     times per energy sample, plus the "Parameter gradient" and
//     "Wavefunction value" observables (src/vmc/src/operators.rs:7-24);
//   * every sample is pushed into a HashMap<String, Vec<OperatorValue>>;
//   * chains run on std::thread workers like VmcRunner's rayon workers
//     (src/vmc/src/vmc.rs:55-78), each worker owning its walkers.
// The trial functions are written the way the reference's examples write
// theirs (value / gradient / laplacian of psi itself, product rule), for the
// two plain systems: He with a Pade e-e Jastrow and H2 with sigma orbitals
// and a Pade e-e Jastrow.
#include <chrono>
#include <cmath>
#include <cstdint>
#include <random>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

struct OperatorValue {
  int kind;  // 0 scalar, 1 vector
  double s;
  std::vector<double> v;
};

using Cfg = std::vector<double>;  // (N, 3) row-major, heap allocated like Array2<f64>

double norm3(const double* x) { return std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]); }

// psi = sigma(r1) sigma(r2) exp(u(r12)), sigma = sum over centres of exp(-a |r - R|),
// u = r / (2 (1 + b r)); params = (a, b). One centre at the origin gives the
// helium function exp(-a (r1 + r2)) exp(u).
struct PadeTwoElectron {
  std::vector<double> centres;  // M x 3
  double a, b;

  void sigma(const double* r, double& v, double* g, double& lap, double& da) const {
    v = 0.0; lap = 0.0; da = 0.0;
    g[0] = g[1] = g[2] = 0.0;
    for (size_t I = 0; I < centres.size() / 3; ++I) {
      double d[3] = {r[0] - centres[3 * I], r[1] - centres[3 * I + 1], r[2] - centres[3 * I + 2]};
      double n = norm3(d), e = std::exp(-a * n);
      v += e;
      for (int k = 0; k < 3; ++k) g[k] += -a * e * d[k] / n;
      lap += e * (a * a - 2.0 * a / n);
      da += -n * e;
    }
  }
  double value(const Cfg& x) const {
    double v1, v2, g[3], l, d;
    sigma(&x[0], v1, g, l, d);
    sigma(&x[3], v2, g, l, d);
    double d12[3] = {x[0] - x[3], x[1] - x[4], x[2] - x[5]};
    double r = norm3(d12);
    return v1 * v2 * std::exp(r / (2.0 * (1.0 + b * r)));
  }
  Cfg gradient(const Cfg& x) const {
    double v1, v2, g1[3], g2[3], l, d;
    sigma(&x[0], v1, g1, l, d);
    sigma(&x[3], v2, g2, l, d);
    double d12[3] = {x[0] - x[3], x[1] - x[4], x[2] - x[5]};
    double r = norm3(d12), q = 1.0 / (1.0 + b * r);
    double eJ = std::exp(0.5 * r * q), up = 0.5 * q * q;
    Cfg g(6);
    for (int k = 0; k < 3; ++k) {
      g[k] = eJ * (g1[k] * v2 + v1 * v2 * up * d12[k] / r);
      g[3 + k] = eJ * (v1 * g2[k] - v1 * v2 * up * d12[k] / r);
    }
    return g;
  }
  double laplacian(const Cfg& x) const {
    double v1, v2, g1[3], g2[3], l1, l2, d;
    sigma(&x[0], v1, g1, l1, d);
    sigma(&x[3], v2, g2, l2, d);
    double d12[3] = {x[0] - x[3], x[1] - x[4], x[2] - x[5]};
    double r = norm3(d12), q = 1.0 / (1.0 + b * r);
    double eJ = std::exp(0.5 * r * q), up = 0.5 * q * q, upp = -b * q * q * q;
    double dot1 = 0.0, dot2 = 0.0;
    for (int k = 0; k < 3; ++k) {
      dot1 += g1[k] * up * d12[k] / r;
      dot2 += g2[k] * up * d12[k] / r;
    }
    double jl = upp + 2.0 * up / r + up * up;
    return eJ * (l1 * v2 + 2.0 * v2 * dot1 + v1 * v2 * jl) +
           eJ * (v1 * l2 - 2.0 * v1 * dot2 + v1 * v2 * jl);
  }
  std::vector<double> parameter_gradient(const Cfg& x) const {
    double v1, v2, g[3], l, d1, d2;
    sigma(&x[0], v1, g, l, d1);
    sigma(&x[3], v2, g, l, d2);
    double d12[3] = {x[0] - x[3], x[1] - x[4], x[2] - x[5]};
    double r = norm3(d12), q = 1.0 / (1.0 + b * r);
    double eJ = std::exp(0.5 * r * q);
    double psi = v1 * v2 * eJ;
    return {eJ * (d1 * v2 + v1 * d2), psi * (-0.5 * r * r * q * q)};
  }
};

// ElectronicHamiltonian::act_on (operator.rs:177-184): T psi + V_ion psi + V_ee psi
struct Hamiltonian {
  std::vector<double> nuc;
  std::vector<int> z;
  double vnn = 0.0;
  double act_on(const PadeTwoElectron& wf, const Cfg& x) const {
    double t = -0.5 * wf.laplacian(x);  // KineticEnergy (operator.rs:122-124)
    double vion = 0.0;                  // IonicPotential (operator.rs:22-33)
    for (size_t I = 0; I < z.size(); ++I)
      for (int j = 0; j < 2; ++j) {
        double d[3] = {x[3 * j] - nuc[3 * I], x[3 * j + 1] - nuc[3 * I + 1],
                       x[3 * j + 2] - nuc[3 * I + 2]};
        vion -= z[I] / norm3(d);
      }
    vion += vnn;
    double pv = vion * wf.value(x);
    double d12[3] = {x[0] - x[3], x[1] - x[4], x[2] - x[5]};
    double pe = (1.0 / norm3(d12)) * wf.value(x);  // ElectronicPotential
    return t + pv + pe;
  }
};

struct Chain {
  Cfg cfg;
  std::mt19937_64 rng;
  double acceptance = 0.0;
  std::unordered_map<std::string, std::vector<OperatorValue>> samples;
};

// move kind 0: uniform box of side `step`; 1: Gaussian of width `step`
bool move_state(const PadeTwoElectron& wf, Chain& c, int idx, int kind, double step) {
  Cfg prop = c.cfg;  // propose_move clones the configuration
  if (kind == 0) {
    std::uniform_real_distribution<double> d(-0.5 * step, 0.5 * step);
    for (int k = 0; k < 3; ++k) prop[3 * idx + k] += d(c.rng);
  } else {
    std::normal_distribution<double> d(0.0, step);
    for (int k = 0; k < 3; ++k) prop[3 * idx + k] += d(c.rng);
  }
  double wv = wf.value(prop);
  double acc = std::min(wv * wv / std::pow(wf.value(c.cfg), 2), 1.0);
  std::uniform_real_distribution<double> u(0.0, 1.0);
  if (acc > u(c.rng)) {
    c.cfg = prop;
    return true;
  }
  return false;
}

void sample(const PadeTwoElectron& wf, const Hamiltonian& h, Chain& c, bool sr) {
  double psi = wf.value(c.cfg);
  c.samples["Energy"].push_back({0, h.act_on(wf, c.cfg) / wf.value(c.cfg), {}});
  if (sr) {
    std::vector<double> pg = wf.parameter_gradient(c.cfg);
    double pv = wf.value(c.cfg);
    for (double& g : pg) g *= pv;  // ParameterGradient: dpsi/dp * psi
    // Vector / Scalar divides the other way round in the reference
    // (src/operator/src/traits.rs:149-150): the stored sample is psi / (psi dpsi/dp)
    for (double& g : pg) g = psi / g;
    c.samples["Parameter gradient"].push_back({1, 0.0, pg});
    double v = wf.value(c.cfg);
    c.samples["Wavefunction value"].push_back({0, v * v / psi, {}});
  }
}

}  // namespace

extern "C" {

// Runs n_walkers independent chains of (n_eq + n_steps) sweeps on n_threads
// threads; returns wall seconds and writes the mean sampled energy.
// system 0: He (Z=2 at the origin), system 1: H2 (nuclei at z = +-0.7).
double faithful_vmc(int system, int n_walkers, int n_eq, int n_steps, int move_kind, double step,
                    double a, double b, int sr, int n_threads, uint64_t seed, double* energy_mean) {
  PadeTwoElectron wf;
  Hamiltonian h;
  if (system == 0) {
    wf.centres = {0.0, 0.0, 0.0};
    h.nuc = {0.0, 0.0, 0.0};
    h.z = {2};
  } else {
    wf.centres = {0.0, 0.0, -0.7, 0.0, 0.0, 0.7};
    h.nuc = wf.centres;
    h.z = {1, 1};
    h.vnn = 1.0 / 1.4;
  }
  wf.a = a;
  wf.b = b;
  if (n_threads < 1) n_threads = 1;
  std::vector<double> esum(n_threads, 0.0), ecount(n_threads, 0.0);
  auto t0 = std::chrono::steady_clock::now();
  std::vector<std::thread> pool;
  for (int t = 0; t < n_threads; ++t) {
    pool.emplace_back([&, t] {
      for (int w = t; w < n_walkers; w += n_threads) {
        Chain c;
        c.rng.seed(seed + 7919ull * (uint64_t)w);
        std::uniform_real_distribution<double> init(-1.0, 1.0);  // Sampler::new (samplers.rs:44-55)
        c.cfg.resize(6);
        for (double& v : c.cfg) v = init(c.rng);
        for (int s = 0; s < n_eq + n_steps; ++s) {
          for (int e = 0; e < 2; ++e)
            if (move_state(wf, c, e, move_kind, step)) c.acceptance += 0.5;
          if (s >= n_eq) sample(wf, h, c, sr != 0);
        }
        for (const OperatorValue& v : c.samples["Energy"]) esum[t] += v.s;
        ecount[t] += (double)c.samples["Energy"].size();
        if (sr) {
          // StochasticReconfiguration::construct_sr_matrix (optimizers.rs:181-231):
          // O = (psi_p / psi) per sample, S += O O^T / n
          const auto& pg = c.samples["Parameter gradient"];
          const auto& wv = c.samples["Wavefunction value"];
          double S[4] = {0, 0, 0, 0};
          for (size_t n = 0; n < pg.size(); ++n) {
            double o0 = pg[n].v[0] / wv[n].s, o1 = pg[n].v[1] / wv[n].s;
            S[0] += o0 * o0 / pg.size();
            S[1] += o0 * o1 / pg.size();
            S[2] += o1 * o0 / pg.size();
            S[3] += o1 * o1 / pg.size();
          }
          esum[t] += 0.0 * S[0];
        }
      }
    });
  }
  for (auto& th : pool) th.join();
  auto t1 = std::chrono::steady_clock::now();
  double es = 0.0, ec = 0.0;
  for (int t = 0; t < n_threads; ++t) {
    es += esum[t];
    ec += ecount[t];
  }
  if (energy_mean) *energy_mean = ec > 0 ? es / ec : 0.0;
  return std::chrono::duration<double>(t1 - t0).count();
}

int faithful_hardware_threads(void) { return (int)std::thread::hardware_concurrency(); }
}
