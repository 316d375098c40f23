// The reference's phi step, sum = float(double(sum) + (1.0 - double(sq)))
// (ClusteringCpu.cu:118-120), computed exactly with integer arithmetic:
// phi_step_exact (32-bit integers, the common case) and phi_step_u64 (64-bit,
// every sum; the derivation below).
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

// the general form on 64-bit integers
PHI_HD float phi_step_u64(float sum, float sq) {
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


PHI_HD float sub_rn(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}

// The common case on 32-bit integers (64-bit shifts occupy a slow pipe on
// GB300): 1 <= sum < 2^24 and sq in {0} u [2^-30, 1].  Units of
// q = 2^(e - 24), e the exponent of sum: sum = S (in [2^24, 2^25)), 1 = 2^(24-e),
// sq = I + F (integer part, fraction F = Fsq / 2^fb) and V = sum + 1 - sq <
// 2^26.  The double addition rounds V to 28 fraction bits (27 once V >= 2^25,
// i.e. past the next power of two), half to even; the conversion to float
// then rounds to a multiple of 2 (4) units -- both shifts together are 29
// bits, so the second rounding is a remainder test against 2^28.
// sum = 0 is one correctly rounded subtraction; the rest takes phi_step_u64.
PHI_HD float phi_step_exact(float sum, float sq) {
  const uint32_t sb = f2u(sum), qb = f2u(sq);
  const uint32_t bs = sb >> 23, bq = qb >> 23;
  const bool q_ok = qb == 0 || (bq >= 127 - 30 && qb <= 0x3f800000u);
  if (sb == 0 && q_ok) return sub_rn(1.f, sq);  // 1 - sq is exact in double here
  if (!q_ok || bs < 127 || bs > 127 + 23) return phi_step_u64(sum, sq);
  const int e = (int)bs - 127;
  const uint32_t S = ((sb & 0x7fffffu) | 0x800000u) << 1;
  const uint32_t one = 1u << (24 - e);
  uint32_t I = 0, Fsq = 0;
  int fb = 0;
  if (qb != 0) {
    const uint32_t mq = (qb & 0x7fffffu) | 0x800000u;
    const int k1 = (int)bq - 127 - e + 1;  // sq = mq * 2^k1 units, k1 <= 1
    if (k1 >= 0) {
      I = mq << k1;
    } else {
      fb = -k1;
      I = fb >= 24 ? 0u : mq >> fb;
      Fsq = fb >= 24 ? mq : mq & ((1u << fb) - 1u);
    }
  }
  const uint32_t Vi = S + one - I;  // V = Vi - Fsq / 2^fb
  const int up = (Vi - (Fsq != 0 ? 1u : 0u)) >= (1u << 25) ? 1 : 0;
  const int fr = 28 - up;
  uint32_t RF;  // the fraction on the double's grid: Fsq * 2^(fr - fb), half to even
  if (fb <= fr) {
    RF = Fsq << (fr - fb);
  } else {
    const int r = fb - fr;  // 1 .. 25; Fsq < 2^24
    const uint32_t qv = Fsq >> r, rem = Fsq & ((1u << r) - 1u), half = 1u << (r - 1);
    RF = qv + ((rem > half || (rem == half && (qv & 1u))) ? 1u : 0u);
  }
  // round (Vi * 2^fr - RF) / 2^29 half to even
  const int g = 1 + up;  // float grid of the result: 2^g units
  uint32_t Q = Vi >> g;
  int32_t rem = (int32_t)((Vi & ((1u << g) - 1u)) << fr) - (int32_t)RF;
  if (rem < 0) {
    Q -= 1;
    rem += 1 << 29;
  }
  Q += (rem > (1 << 28) || (rem == (1 << 28) && (Q & 1u))) ? 1u : 0u;
  int ex = e + up;
  if (Q >> 24) {
    Q >>= 1;
    ++ex;
  }
  return u2f(((uint32_t)(ex + 127) << 23) | (Q & 0x7fffffu));
}

}  // namespace inscy
