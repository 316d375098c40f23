// The reference's phi step, sum = float(double(sum) + (1.0 - double(sq)))
// (ClusteringCpu.cu:118-120), computed exactly with 64-bit integer arithmetic.
//
// GB300's FP64 rate is a small fraction of its FP32/INT32 rate, and this step
// runs once per (neighbour, subspace, point).  In units of 2^-53:
//   * k = sq * 2^53, rounded to an integer as the double subtraction 1 - sq
//     rounds (exact for sq >= 2^-30; ties to even below);
//   * T = 2^53 - k is then exactly the double 1 - sq;
//   * sum is 0 or >= 2^-24 (it only grows by terms that are 0 or >= 2^-24),
//     so for sum < 2^10 it is an integer ms << (es + 30) below 2^63 and
//     U = sum + T fits 64 bits exactly.  For larger sums the work moves to
//     units of 2^(es - 62): the bits of T dropped by that shift become a
//     sticky bit, which is exact for both roundings since they happen at
//     least ten bits higher.
// Rounding U to 53 significant bits (the double addition) and then to 24 (the
// conversion to float), both to nearest even, reproduces the reference's two
// roundings.  Inputs outside the domain (negative or subnormal sum, sq
// outside [0, 1]) take the double expression.
#pragma once
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define PHI_HD __host__ __device__ __forceinline__
#else
#define PHI_HD inline
#endif

namespace inscy {

PHI_HD int msb64(uint64_t v) {  // index of the highest set bit, v > 0
#ifdef __CUDA_ARCH__
  return 63 - __clzll((long long)v);
#else
  return 63 - __builtin_clzll(v);
#endif
}

PHI_HD uint32_t f2u(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
#endif
}
PHI_HD float u2f(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  std::memcpy(&f, &u, 4);
  return f;
#endif
}

// v rounded to a multiple of 2^r (r >= 1), ties to even; returns v >> r rounded
PHI_HD uint64_t round_shift(uint64_t v, int r) {
  const uint64_t q = v >> r, rem = v & ((1ull << r) - 1), half = 1ull << (r - 1);
  return q + ((rem > half || (rem == half && (q & 1))) ? 1 : 0);
}

PHI_HD float phi_step_double(float sum, float sq) {
  return (float)((double)sum + (1.0 - (double)sq));
}

PHI_HD float phi_step_exact(float sum, float sq) {
  const uint32_t sb = f2u(sum), qb = f2u(sq);
  const uint32_t bs = sb >> 23, bq = qb >> 23;
  if ((sb != 0 && (bs < 127 - 24 || bs > 254)) || qb > 0x3f800000u) return phi_step_double(sum, sq);
  // k = sq in units of 2^-53, rounded as the double subtraction 1 - sq rounds
  // (a subnormal sq leaves 1 - sq = 1: k = 0)
  uint64_t k = 0;
  if (bq != 0) {
    const uint64_t mq = (qb & 0x7fffffu) | 0x800000u;
    const int sh = (int)bq - 127 + 30;  // sq = mq * 2^sh units
    if (sh >= 0)
      k = mq << sh;
    else if (sh >= -24)
      k = round_shift(mq, -sh);  // below that, mq * 2^sh < 1/2 rounds to 0
  }
  const uint64_t T = (1ull << 53) - k;
  uint64_t U;
  int g = 0;  // U is in units of 2^(g - 53)
  if (sb == 0) {
    U = T;
  } else {
    const uint64_t ms = (sb & 0x7fffffu) | 0x800000u;
    const int es = (int)bs - 127;
    if (es <= 9) {
      U = (ms << (es + 30)) + T;
    } else {
      g = es - 9;
      const uint64_t Tg = g >= 64 ? (uint64_t)(T != 0) : ((T >> g) | (uint64_t)((T & ((1ull << g) - 1)) != 0));
      U = (ms << 39) + Tg;
    }
  }
  if (U == 0) return 0.f;
  // U >= 2^29 here (sum >= 2^-24 or 1 - sq >= 2^-24): both rounding shifts are >= 6
  int p = msb64(U);
  if (p > 52) {  // the double addition: 53 significant bits
    U = round_shift(U, p - 52) << (p - 52);
    p = msb64(U);
  }
  uint64_t q = round_shift(U, p - 23);  // the conversion to float: 24 significant bits
  int e = p - 53 + g;                   // value = (q / 2^23) * 2^e
  if (q >> 24) {                        // rounded up to 2^24
    q >>= 1;
    ++e;
  }
  return u2f(((uint32_t)(e + 127) << 23) | ((uint32_t)q & 0x7fffffu));
}

}  // namespace inscy
