// Checks ek_ffbits.h against the hardware conversions on random doubles
// over many binades.  Prints the mismatch counts; exit 0
// when all are zero.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "ek_ffbits.h"

int main(int argc, char **argv) {
  const long n = argc > 1 ? std::atol(argv[1]) : 2000000;
  std::mt19937_64 rng(12345);
  std::uniform_real_distribution<double> mant(1.0, 2.0);
  std::uniform_int_distribution<int> expo(-70, 70);
  long bad_d2f = 0, bad_f2d = 0;
  for (long t = 0; t < n; ++t) {
    double x = std::ldexp(mant(rng), expo(rng));
    if (rng() & 1) x = -x;
    if (t % 97 == 0) x = std::ldexp(1.0, expo(rng));             // powers of two
    if (t % 89 == 0) x = (double)(float)x;                      // exact floats
    if (t % 83 == 0) x = std::nextafter((double)(float)x, 3.0);  // just off a float
    const float h_ref = (float)x;
    if (ek::fbits(ek::d2f_bits(x)) != ek::fbits(h_ref)) ++bad_d2f;
    if (ek::dbits(ek::f2d_bits(h_ref)) != ek::dbits((double)h_ref)) ++bad_f2d;
  }
  // infinities both ways; NaN stays NaN with its sign
  for (double x : {INFINITY, -INFINITY}) {
    if (ek::fbits(ek::d2f_bits(x)) != ek::fbits((float)x)) ++bad_d2f;
    if (ek::dbits(ek::f2d_bits((float)x)) != ek::dbits(x)) ++bad_f2d;
  }
  for (double x : {NAN, -NAN}) {
    const float f = ek::d2f_bits(x);
    if (!std::isnan(f) || std::signbit(f) != std::signbit(x)) ++bad_d2f;
    const double y = ek::f2d_bits((float)x);
    if (!std::isnan(y) || std::signbit(y) != std::signbit(x)) ++bad_f2d;
  }
  std::printf("n=%ld d2f=%ld f2d=%ld\n", n, bad_d2f, bad_f2d);
  return (bad_d2f | bad_f2d) ? 1 : 0;
}
