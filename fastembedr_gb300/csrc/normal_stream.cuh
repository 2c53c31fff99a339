// Normal draws from std::mt19937 in the stream order of std::normal_distribution<double>, with
// the logarithms and roots spread over host threads.
#pragma once

#include <cstddef>
#include <random>

namespace fe {

// Draws of N(mean, sd) from an engine in the order std::normal_distribution<double> gives them:
// Marsaglia's polar method (two uniforms per attempt, accepted when 0 < x^2 + y^2 <= 1; the pair
// yields y * m first and keeps x * m for the next call, m = sqrt(-2 log(r2) / r2)) on uniforms
// made as generate_canonical<double, 53> makes them from a 32-bit engine (two words, the first
// the low one, scaled by 2^-64). fill() runs the engine and the acceptance tests on the calling
// thread and the logarithms and roots on host threads. At first use the polar path is compared
// bit for bit with std::normal_distribution (draws and engine state); where the standard library
// differs, every draw goes through std::normal_distribution instead.
class NormalStream {
 public:
  NormalStream(double mean, double sd) : mean_(mean), sd_(sd), std_(mean, sd) {}
  double next(std::mt19937& g);
  // out[i] = next(g) * scale for i < count
  void fill(std::mt19937& g, double* out, std::size_t count, double scale);
  // whether the polar path reproduces std::normal_distribution here (and is used)
  static bool polar_path();

 private:
  double next_polar(std::mt19937& g);
  void fill_polar(std::mt19937& g, double* out, std::size_t count, double scale, std::size_t parallel_min);
  static bool self_check();

  double mean_, sd_;
  std::normal_distribution<double> std_;
  bool has_saved_ = false;
  double saved_ = 0.0;
};

}  // namespace fe
