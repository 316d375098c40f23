// Host check of the exact phi step (gpu_inscy_gb300/csrc/phi_exact.cuh): the
// integer form against the reference's double expression on pseudo-random
// and edge inputs.  Prints "<cases> <mismatches> <cases with sum >= 2^10>".
#include <cstdio>
#include <cstdlib>

#include "../gpu_inscy_gb300/csrc/phi_exact.cuh"

using namespace inscy;

static uint64_t mix(uint64_t x) {
  x ^= x >> 31;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  x ^= x >> 29;
  return x;
}

int main(int argc, char** argv) {
  const long long n = argc > 1 ? atoll(argv[1]) : 10000000;
  long long bad = 0, large = 0, cases = 0;
  auto check = [&](float sum, float sq) {
    ++cases;
    if (sum >= 1024.f) ++large;
    if (f2u(phi_step_exact(sum, sq)) != f2u(phi_step_double(sum, sq))) {
      if (++bad <= 5) std::printf("mismatch sum=%a sq=%a\n", sum, sq);
    }
  };
  // edges: sums around powers of two and the 2^10 switch, sq at 0, 1 and tiny values
  const float sums[] = {0.f, 5.9604645e-8f, 1.f, 1.0000001f, 2.f, 1023.99994f, 1024.f, 1e6f, 3.f, 16777215.f, 16777216.f, 3.4028235e38f};
  const float sqs[] = {0.f, 1.f, 0.99999994f, 0.5f, 1e-10f, 9.3132257e-10f, 8.6736174e-19f, 5.421011e-20f, 2e-30f};
  for (float s : sums)
    for (float q : sqs) check(s, q);
  for (long long i = 0; i < n; ++i) {
    const uint64_t x = mix((uint64_t)i * 0x9e3779b97f4a7c15ull + 1), y = mix(x + 0x632be59bd9b4e019ull);
    float sum;
    switch (x & 7) {
      case 0:  // an integer-valued count
        sum = (float)((x >> 8) % 3000);
        break;
      case 1:
      case 2:  // the range phi sums take
        sum = u2f((uint32_t)(((x >> 8) % 34 + 127 - 24) << 23) | (uint32_t)((x >> 20) & 0x7fffffu));
        break;
      case 3:
      case 4:
      case 5:  // [1, 2^13): most steps of the density kernel
        sum = u2f((uint32_t)(((x >> 8) % 13 + 127) << 23) | (uint32_t)((x >> 20) & 0x7fffffu));
        break;
      default:  // wide exponents
        sum = u2f((uint32_t)(((x >> 8) % 90 + 127 - 30) << 23) | (uint32_t)((x >> 20) & 0x7fffffu));
    }
    float sq;
    if (y & 1) {
      sq = u2f((uint32_t)((y >> 8) % 0x3f800001u));
    } else {
      const float dd = (float)((double)(y >> 11) * 0x1p-53);
      sq = dd * dd;
    }
    check(sum, sq);
  }
  std::printf("%lld %lld %lld\n", cases, bad, large);
  return 0;
}
