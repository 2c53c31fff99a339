// Host-side normal draws for the UMAP spectral start (see normal_stream.cuh).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "../../include/fastembedr_cuda.h"
#include "normal_stream.cuh"

namespace fe {
namespace {

constexpr std::size_t kParallelPairs = 32768;  // below this many pairs fill() stays on one thread

// A uniform draw in [0, 1) as generate_canonical<double, 53> makes it from a 32-bit engine.
double canonical(std::mt19937& g) {
  const double lo = (double)g();
  const double hi = (double)g();
  const double r = (lo + hi * 4294967296.0) / 18446744073709551616.0;
  return r >= 1.0 ? std::nextafter(1.0, 0.0) : r;
}

struct PolarPoint {
  double x, y, r2;
};

PolarPoint polar_point(std::mt19937& g) {
  for (;;) {
    const double x = 2.0 * canonical(g) - 1.0;
    const double y = 2.0 * canonical(g) - 1.0;
    const double r2 = x * x + y * y;
    if (r2 <= 1.0 && r2 != 0.0) return {x, y, r2};
  }
}

double polar_mult(double r2) { return std::sqrt(-2 * std::log(r2) / r2); }

bool same_bits(const double* a, const double* b, std::size_t count) {
  return std::memcmp(a, b, sizeof(double) * count) == 0;
}

}  // namespace

double NormalStream::next_polar(std::mt19937& g) {
  double z;
  if (has_saved_) {
    has_saved_ = false;
    z = saved_;
  } else {
    const PolarPoint p = polar_point(g);
    const double m = polar_mult(p.r2);
    saved_ = p.x * m;
    has_saved_ = true;
    z = p.y * m;
  }
  return z * sd_ + mean_;
}

void NormalStream::fill_polar(std::mt19937& g, double* out, std::size_t count, double scale,
                              std::size_t parallel_min) {
  std::size_t first = 0;
  if (count > 0 && has_saved_) out[first++] = next_polar(g) * scale;
  const std::size_t pairs = (count - first + 1) / 2;
  if (pairs < parallel_min) {
    for (std::size_t i = first; i < count; ++i) out[i] = next_polar(g) * scale;
    return;
  }
  // the engine and the acceptance tests in stream order, then the pairs' values in parallel
  std::vector<PolarPoint> pts(pairs);
  for (PolarPoint& p : pts) p = polar_point(g);
  auto work = [&](std::size_t a, std::size_t b) {
    for (std::size_t k = a; k < b; ++k) {
      const double m = polar_mult(pts[k].r2);
      const double zy = pts[k].y * m, zx = pts[k].x * m;
      const std::size_t o = first + 2 * k;
      out[o] = (zy * sd_ + mean_) * scale;
      if (o + 1 < count) out[o + 1] = (zx * sd_ + mean_) * scale;
    }
  };
  const std::size_t hw = std::max(1u, std::thread::hardware_concurrency());
  const std::size_t nt = std::min<std::size_t>({hw, 16, pairs / 4096 + 1});
  std::vector<std::thread> pool;
  const std::size_t chunk = (pairs + nt - 1) / nt;
  for (std::size_t t = 1; t < nt; ++t) {
    const std::size_t a = t * chunk, b = std::min(pairs, a + chunk);
    if (a < b) pool.emplace_back(work, a, b);
  }
  work(0, std::min(pairs, chunk));
  for (std::thread& th : pool) th.join();
  if ((count - first) % 2 == 1) {
    // the last pair's x value is left over for the next draw
    saved_ = pts.back().x * polar_mult(pts.back().r2);
    has_saved_ = true;
  }
}

bool NormalStream::self_check() {
  const std::uint32_t seeds[] = {1u, 42u, 2026u};
  for (std::uint32_t seed : seeds) {
    // single draws, an odd-length parallel fill (the leftover value carried into the next
    // draws), then an even-length fill starting from a leftover value
    std::mt19937 ga(seed), gb(seed);
    NormalStream mine(0.0, 1e-4);
    std::normal_distribution<double> ref(0.0, 1e-4);
    const std::size_t lens[] = {1001, 2 * 4096 + 1, 3, 2 * 4096};
    for (int part = 0; part < 4; ++part) {
      const std::size_t len = lens[part];
      std::vector<double> a(len), b(len);
      const double scale = part == 1 ? 10000.0 : 1.0;
      if (part == 0 || part == 2) {
        for (std::size_t i = 0; i < len; ++i) a[i] = mine.next_polar(ga) * scale;
      } else {
        mine.fill_polar(ga, a.data(), len, scale, 1);
      }
      for (std::size_t i = 0; i < len; ++i) b[i] = ref(gb) * scale;
      if (!same_bits(a.data(), b.data(), len)) return false;
    }
    if (!(ga == gb)) return false;
  }
  return true;
}

bool NormalStream::polar_path() {
  static const bool ok = self_check();
  return ok;
}

double NormalStream::next(std::mt19937& g) { return polar_path() ? next_polar(g) : std_(g); }

void NormalStream::fill(std::mt19937& g, double* out, std::size_t count, double scale) {
  if (polar_path()) {
    fill_polar(g, out, count, scale, kParallelPairs);
    return;
  }
  for (std::size_t i = 0; i < count; ++i) out[i] = std_(g) * scale;
}

}  // namespace fe

extern "C" int fastembedr_host_normal_stream_check(void) { return fe::NormalStream::polar_path() ? 1 : 0; }
