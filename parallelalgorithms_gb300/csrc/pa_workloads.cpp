// Seeded synthetic inputs for the radix hot path, generated on the host so
// that the GPU path and the CPU checkers see identical bytes.
//
// The uniform 32-bit recipe is the reference's own: std::mt19937_64 seeded
// with 1234, key = low 32 bits of each draw (ParallelAlgorithms.cpp:91,
// 112-115).  The other distributions have no reference recipe; they are
// project-defined and documented beside each function.
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <random>
#include <vector>

namespace {

// 53 random bits -> [0, 1)
inline double unit(std::mt19937_64& g) { return (double)(g() >> 11) * (1.0 / 9007199254740992.0); }

inline uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

}  // namespace

extern "C" {

// out[i] = (uint32_t)g() with g = std::mt19937_64(seed).
void pa_gen_uniform_u32(uint64_t seed, size_t n, uint32_t* out) {
  std::mt19937_64 g(seed);
  for (size_t i = 0; i < n; ++i) out[i] = (uint32_t)g();
}

// out[i] = g() with g = std::mt19937_64(seed).
void pa_gen_uniform_u64(uint64_t seed, size_t n, uint64_t* out) {
  std::mt19937_64 g(seed);
  for (size_t i = 0; i < n; ++i) out[i] = g();
}

// Zipf(s) over `ranks` ranks: rank r (1-based) has probability proportional
// to r^-s; ranks are drawn by inverse CDF (binary search of the cumulative
// table with a uniform draw of std::mt19937_64(seed)) and mapped to the key
// splitmix64(r), so every byte of the key varies.
void pa_gen_zipf_u64(uint64_t seed, size_t n, double s, uint32_t ranks, uint64_t* out) {
  if (ranks == 0) return;
  std::vector<double> cdf(ranks);
  double acc = 0.0;
  for (uint32_t r = 0; r < ranks; ++r) {
    acc += std::pow((double)(r + 1), -s);
    cdf[r] = acc;
  }
  for (uint32_t r = 0; r < ranks; ++r) cdf[r] /= acc;
  std::mt19937_64 g(seed);
  for (size_t i = 0; i < n; ++i) {
    const double u = unit(g);
    size_t lo = 0, hi = ranks - 1;
    while (lo < hi) {
      const size_t mid = (lo + hi) / 2;
      if (cdf[mid] > u)
        hi = mid;
      else
        lo = mid + 1;
    }
    out[i] = splitmix64((uint64_t)lo + 1);
  }
}

// float32 N(0,1) by Box-Muller (one value per pair of uniform draws) from
// std::mt19937_64(seed), with special values planted at seeded positions:
// each key is, with probability `frac` each, +0.0, -0.0, +inf, -inf, or a
// denormal (random non-zero 23-bit mantissa, random sign).
void pa_gen_normal_specials_f32(uint64_t seed, size_t n, double frac, float* out) {
  std::mt19937_64 g(seed);
  const double two_pi = 6.283185307179586476925286766559;
  for (size_t i = 0; i < n; ++i) {
    const double c = unit(g);
    uint32_t bits;
    if (c < frac) {
      bits = 0x00000000u;
    } else if (c < 2 * frac) {
      bits = 0x80000000u;
    } else if (c < 3 * frac) {
      bits = 0x7F800000u;
    } else if (c < 4 * frac) {
      bits = 0xFF800000u;
    } else if (c < 5 * frac) {
      const uint64_t r = g();
      uint32_t mant = (uint32_t)(r & 0x7FFFFFu);
      if (mant == 0) mant = 1;
      bits = ((uint32_t)(r >> 32) & 0x80000000u) | mant;
    } else {
      const double u1 = ((double)(g() >> 11) + 1.0) * (1.0 / 9007199254740992.0);
      const double u2 = unit(g);
      const float z = (float)(std::sqrt(-2.0 * std::log(u1)) * std::cos(two_pi * u2));
      std::memcpy(&bits, &z, 4);
    }
    std::memcpy(&out[i], &bits, 4);
  }
}

// count sizes round(exp(U(ln lo, ln hi))) from std::mt19937_64(seed).
void pa_gen_log_uniform_sizes(uint64_t seed, size_t count, double lo, double hi, uint64_t* out) {
  std::mt19937_64 g(seed);
  const double a = std::log(lo), b = std::log(hi);
  for (size_t i = 0; i < count; ++i) out[i] = (uint64_t)std::llround(std::exp(a + (b - a) * unit(g)));
}

}  // extern "C"
