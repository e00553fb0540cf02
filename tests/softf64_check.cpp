// Host check of the integer-pipe binary64 routines (py-orbit_gb300/csrc/
// softf64.cuh) against the host's IEEE arithmetic: sf::mul, sf::add,
// sf::fma and sf::scale2 must return the same bits as a * b, a + b,
// fma(a, b, c) and a * 2^k, and sf::to_float / sf::from_float the same as
// the casts, on random normal operands over wide and narrow
// exponent spreads, near-cancellations, exact ties, zeros and random bit
// patterns (subnormals, infinities, NaN).  Prints the mismatch count.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "softf64.cuh"

using namespace orbit;

static std::mt19937_64 g(12345);

static double normal(int spread) {
  double x = std::ldexp(1.0 + (double)(g() >> 12) * 0x1p-52, (int)(g() % (2 * spread + 1)) - spread);
  return (g() & 1) ? -x : x;
}

static bool same(double a, double b) { return sf::bits(a) == sf::bits(b) || (std::isnan(a) && std::isnan(b)); }

int main(int argc, char** argv) {
  const long n = argc > 1 ? std::atol(argv[1]) : 2000000;
  long bad = 0;
  for (long i = 0; i < n; ++i) {
    const int spread = (i % 4 == 0) ? 1000 : (i % 4 == 1 ? 60 : (i % 4 == 2 ? 5 : 0));
    double a = normal(spread), b = normal(spread), c = normal(spread);
    switch (i % 10) {
      case 1: c = -(a * b); break;                                          // total cancellation
      case 2: c = sf::from_bits(sf::bits(-(a * b)) ^ (g() & 0xFF)); break;  // near cancellation
      case 3: b = sf::from_bits(sf::bits(-a) ^ (g() & 0xFFF)); break;       // add cancellation
      case 4: c = std::ldexp(c, -(int)(g() % 200)); break;
      case 5: c = std::ldexp(c, (int)(g() % 200)); break;
      case 6: b = std::ldexp(b, (int)(g() % 130) - 65); break;
      case 7: c = std::ldexp(a * b, -53) * ((g() & 1) ? 1.5 : 0.5); break;  // ties of a * b + tiny
      case 8: a = sf::from_bits(g()); b = sf::from_bits(g()); c = sf::from_bits(g()); break;
      case 9: a = (g() & 1) ? 0.0 : -0.0; break;
      default: break;
    }
    if (!same(a * b, sf::mul(a, b))) ++bad;
    if (!same(a + b, sf::add(a, b))) ++bad;
    if (!same(std::fma(a, b, c), sf::fma(a, b, c))) ++bad;
    if (!same(a * 0.5, sf::scale2(a, -1)) || !same(a * 2.0, sf::scale2(a, 1))) ++bad;
    // conversions: doubles near float ties and over the float range, and
    // random float bit patterns
    double t = (i % 3 == 0) ? a : std::ldexp(a, (int)(g() % 300) - 150);
    if (i % 5 == 0) t = sf::from_bits((sf::bits(t) & ~((1ull << 29) - 1)) | (1ull << 28));  // exact tie
    const float tf = (float)t, sf32 = sf::to_float(t);
    if (!(sf::fbits(tf) == sf::fbits(sf32) || (std::isnan(tf) && std::isnan(sf32)))) ++bad;
    const float r = sf::from_fbits((uint32_t)g());
    const double rd = (double)r, sd = sf::from_float(r);
    if (!same(rd, sd)) ++bad;
  }
  std::printf("%ld\n", bad);
  return bad != 0;
}
