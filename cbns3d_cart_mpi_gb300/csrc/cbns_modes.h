// cbns_modes.h — the project-defined random solenoidal velocity perturbation of
// the Taylor-Green initial state (no counterpart in the reference), shared by
// the host library and the GPU library so both draw identical modes.
//
// nmodes modes, each an integer wavevector k with 1 <= |k| <= kmax, a unit
// direction a perpendicular to k (so the mode is divergence-free), a phase and a
// weight, drawn from splitmix64(seed); weights are normalised so their sum is amp.
//   du(x) = sum_m a_m * (amp * w_m / sum w) * cos(k_m . x + phase_m)
#pragma once

#include <cmath>
#include <cstdint>
#include <vector>

namespace cbns {

struct PerturbMode {
  double k[3];
  double a[3];  // unit direction times amp * weight / sum(weights)
  double phase;
};

inline uint64_t splitmix64(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
inline double uniform01(uint64_t& s) { return (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }

inline std::vector<PerturbMode> draw_modes(uint64_t seed, double amp, int nmodes, int kmax) {
  const double PI = 3.14159265358979323846;
  uint64_t s = seed;
  std::vector<PerturbMode> modes;
  std::vector<double> weight;
  double wsum = 0.0;
  while ((int)modes.size() < nmodes) {
    PerturbMode m;
    for (int d = 0; d < 3; ++d) m.k[d] = std::floor(uniform01(s) * (2 * kmax + 1)) - kmax;
    double k2 = m.k[0] * m.k[0] + m.k[1] * m.k[1] + m.k[2] * m.k[2];
    if (k2 < 1.0 || k2 > (double)kmax * kmax) continue;
    double r[3], a2 = 0.0;
    for (int d = 0; d < 3; ++d) r[d] = uniform01(s) * 2.0 - 1.0;
    m.a[0] = m.k[1] * r[2] - m.k[2] * r[1];
    m.a[1] = m.k[2] * r[0] - m.k[0] * r[2];
    m.a[2] = m.k[0] * r[1] - m.k[1] * r[0];
    for (int d = 0; d < 3; ++d) a2 += m.a[d] * m.a[d];
    if (a2 < 1e-12) continue;
    for (int d = 0; d < 3; ++d) m.a[d] /= std::sqrt(a2);
    m.phase = uniform01(s) * 2.0 * PI;
    double w = 0.5 + uniform01(s);
    wsum += w;
    weight.push_back(w);
    modes.push_back(m);
  }
  for (size_t i = 0; i < modes.size(); ++i) {
    double amp_m = amp * weight[i] / wsum;
    for (int d = 0; d < 3; ++d) modes[i].a[d] *= amp_m;
  }
  return modes;
}

}  // namespace cbns
