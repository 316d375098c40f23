// The reference's phi step, sum = float(double(sum) + (1.0 - double(sq)))
// (ClusteringCpu.cu:118-120), computed exactly with integer arithmetic.
//
// GB300's FP64 rate is a small fraction of its FP32/INT32 rate, and this step
// runs once per (neighbour, subspace, point).  Both operands live on a common
// fixed-point grid: sum is 0 or >= 2^-24 (it only ever grows by terms that
// are 0 or >= 2^-24), so its bits sit at or above 2^-47; the term 1 - sq is
// kept exactly on the 2^-53 grid (when sq < 2^-30 it is first rounded to that
// grid exactly as the double subtraction rounds it).  The exact sum in units
// of 2^-53 fits in 128 bits; rounding it to 53 significant bits (the double
// addition) and then to 24 bits (the conversion to float), both to nearest
// even, reproduces the reference's two roundings.  Sums of 2^60 and above
// (never reached: a sum of at most n terms <= 1) take the double path.
#pragma once
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define PHI_HD __host__ __device__ __forceinline__
#else
#define PHI_HD inline
#endif

namespace inscy {

typedef unsigned __int128 u128;

PHI_HD int msb128(u128 v) {  // index of the highest set bit, v > 0
  uint64_t hi = (uint64_t)(v >> 64), lo = (uint64_t)v;
#ifdef __CUDA_ARCH__
  return hi ? 127 - __clzll((long long)hi) : 63 - __clzll((long long)lo);
#else
  return hi ? 127 - __builtin_clzll(hi) : 63 - __builtin_clzll(lo);
#endif
}

// round v to a multiple of 2^r (r >= 1), ties to even
PHI_HD u128 round_even(u128 v, int r) {
  u128 q = v >> r;
  u128 rem = v - (q << r);
  u128 half = (u128)1 << (r - 1);
  if (rem > half || (rem == half && (q & 1))) ++q;
  return q << r;
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

// double-precision reference of the step (used outside the exact range)
PHI_HD float phi_step_double(float sum, float sq) {
  return (float)((double)sum + (1.0 - (double)sq));
}

// sum >= 0 (0 or >= 2^-24), sq in [0, 1]
PHI_HD float phi_step_exact(float sum, float sq) {
  const uint32_t sb = f2u(sum), qb = f2u(sq);
  const int es = (int)(sb >> 23) - 127;
  if (sb != 0 && (es < -24 || es > 60)) return phi_step_double(sum, sq);
  // T = (1 - sq) in units of 2^-53, rounded as the double subtraction does
  uint64_t k;  // sq in units of 2^-53
  if (qb == 0) {
    k = 0;
  } else {
    const int eq = (int)(qb >> 23) - 127;  // sq <= 1: eq <= 0
    const uint64_t mq = (qb & 0x7fffffu) | (((qb >> 23) != 0) ? 0x800000u : 0u);
    const int sh = eq + 30;  // sq = mq * 2^(eq - 23) = mq * 2^(sh) * 2^-53
    if ((qb >> 23) == 0) {
      k = 0;  // subnormal sq < 2^-126: 1 - sq rounds to 1
    } else if (sh >= 0) {
      k = mq << sh;
    } else if (sh < -40) {
      k = 0;  // below half a unit of 2^-53
    } else {
      // round mq * 2^sh to an integer, ties to even (the result 2^53 - k then
      // has an even last bit, as the double subtraction's tie rule requires)
      const int r = -sh;
      uint64_t q = mq >> r, rem = mq & ((1ull << r) - 1), half = 1ull << (r - 1);
      if (rem > half || (rem == half && (q & 1))) ++q;
      k = q;
    }
  }
  const uint64_t T = (1ull << 53) - k;
  u128 V = (u128)T;
  if (sb != 0) {
    const uint64_t ms = (sb & 0x7fffffu) | 0x800000u;
    V += (u128)ms << (es + 30);  // sum = ms * 2^(es - 23) = ms << (es + 30) units
  }
  if (V == 0) return 0.f;
  // the double addition: 53 significant bits
  int p = msb128(V);
  if (p > 52) V = round_even(V, p - 52);
  // the conversion to float: 24 significant bits
  p = msb128(V);
  if (p > 23) V = round_even(V, p - 23);
  p = msb128(V);
  // value = V * 2^-53 with V = m * 2^(p - 23), m in [2^23, 2^24)
  const uint32_t m = (uint32_t)(V >> (p - 23));
  const int e = p - 53;
  return u2f(((uint32_t)(e + 127) << 23) | (m & 0x7fffffu));
}

}  // namespace inscy
