// Shared device code: determinant bit operations, integral accessors and the
// Slater-Condon rules, written for sm_103a.
//
// Determinant layout (same bit convention as Dice, SHCI/Determinants.h:247-602):
// two 64-bit words per determinant, spin-orbital p at bit p%64 of word p/64,
// alpha orbital k = spin-orbital 2k, beta orbital k = spin-orbital 2k+1.
// Alpha/beta strings are single 64-bit words with orbital k at bit k.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace shci {

constexpr int kMaxOrb = 64;      // spatial orbitals
constexpr int kMaxSpin = 128;    // spin orbitals
constexpr unsigned kFull = 0xffffffffu;

struct Det2 {
  uint64_t w0, w1;
};

__host__ __device__ inline bool det_getocc(const Det2& d, int p) {
  return p < 64 ? ((d.w0 >> p) & 1ull) : ((d.w1 >> (p - 64)) & 1ull);
}
__host__ __device__ inline void det_flip(Det2& d, int p) {
  if (p < 64)
    d.w0 ^= (1ull << p);
  else
    d.w1 ^= (1ull << (p - 64));
}

// Determinant::operator< (SHCI/Determinants.h:490-498): signed words, top down.
__host__ __device__ inline bool det_less(const Det2& a, const Det2& b) {
  if ((int64_t)a.w1 != (int64_t)b.w1) return (int64_t)a.w1 < (int64_t)b.w1;
  return (int64_t)a.w0 < (int64_t)b.w0;
}
__host__ __device__ inline bool det_eq(const Det2& a, const Det2& b) { return a.w0 == b.w0 && a.w1 == b.w1; }

// Even-bit extraction: bits 0,2,4,... of x packed into the low 32 bits.
__host__ __device__ inline uint32_t compact_even(uint64_t x) {
  x &= 0x5555555555555555ull;
  x = (x | (x >> 1)) & 0x3333333333333333ull;
  x = (x | (x >> 2)) & 0x0f0f0f0f0f0f0f0full;
  x = (x | (x >> 4)) & 0x00ff00ff00ff00ffull;
  x = (x | (x >> 8)) & 0x0000ffff0000ffffull;
  x = (x | (x >> 16)) & 0x00000000ffffffffull;
  return (uint32_t)x;
}
__host__ __device__ inline uint64_t spread_even(uint32_t v) {
  uint64_t x = v;
  x = (x | (x << 16)) & 0x0000ffff0000ffffull;
  x = (x | (x << 8)) & 0x00ff00ff00ff00ffull;
  x = (x | (x << 4)) & 0x0f0f0f0f0f0f0f0full;
  x = (x | (x << 2)) & 0x3333333333333333ull;
  x = (x | (x << 1)) & 0x5555555555555555ull;
  return x;
}
// getAlpha / getBeta (SHCI/Determinants.h:471-487)
__host__ __device__ inline uint64_t det_alpha(const Det2& d) {
  return (uint64_t)compact_even(d.w0) | ((uint64_t)compact_even(d.w1) << 32);
}
__host__ __device__ inline uint64_t det_beta(const Det2& d) {
  return (uint64_t)compact_even(d.w0 >> 1) | ((uint64_t)compact_even(d.w1 >> 1) << 32);
}
__host__ __device__ inline Det2 det_from_strings(uint64_t a, uint64_t b) {
  Det2 d;
  d.w0 = spread_even((uint32_t)a) | (spread_even((uint32_t)b) << 1);
  d.w1 = spread_even((uint32_t)(a >> 32)) | (spread_even((uint32_t)(b >> 32)) << 1);
  return d;
}

// The alpha <-> beta flip of a determinant (Determinant::flipAlphaBeta,
// SHCI/Determinants.h:278-282) and whether it is the standard member of its
// pair (Determinant::isStandard, :241-258: not smaller than its flip, words
// compared as unsigned integers from the top word down; a closed shell is its
// own flip and standard).
__host__ __device__ inline Det2 det_flip_pair(const Det2& d) {
  const uint64_t ev = 0x5555555555555555ull, od = 0xAAAAAAAAAAAAAAAAull;
  Det2 f;
  f.w0 = ((d.w0 & ev) << 1) | ((d.w0 & od) >> 1);
  f.w1 = ((d.w1 & ev) << 1) | ((d.w1 & od) >> 1);
  return f;
}
__host__ __device__ inline bool det_is_standard(const Det2& d) {
  const Det2 f = det_flip_pair(d);
  if (d.w1 != f.w1) return d.w1 > f.w1;
  return d.w0 >= f.w0;
}

// Number of occupied spin orbitals strictly between lo and hi (lo < hi).
__device__ inline int occ_between(const Det2& d, int lo, int hi) {
  // bits (lo, hi): mask of bits < hi minus bits <= lo
  auto below = [](uint64_t w, int k) -> uint64_t {  // bits of w below position k (0..64)
    return k >= 64 ? w : (k <= 0 ? 0ull : (w & ((1ull << k) - 1ull)));
  };
  int c = __popcll(below(d.w0, hi)) + __popcll(below(d.w1, hi - 64));
  c -= __popcll(below(d.w0, lo + 1)) + __popcll(below(d.w1, lo + 1 - 64));
  return c;
}

// Device view of the integrals (SHCI/integral.h:47-101).
struct IntsView {
  const double* I1;        // (2n)x(2n) spin-orbital matrix
  const double* I2;        // 8-fold packed spatial (ij|kl)
  const double* Direct;    // n x n, (ii|jj)
  const double* Exchange;  // n x n, (ij|ji)
  int norb;
  const float* I1f;  // FP32 copies for the FP32 matrix-free sigma
  const float* I2f;
  // Terms of Hij_1Excite per spin-orbital pair (a, i) of one spin s and
  // occupied spin orbital j, at [((s n + a/2) n + i/2) 2n + j]:
  // (ai|jj) - (aj|ji) for j of spin s, (ai|jj) otherwise, each the FP64
  // difference the sum adds (V1) and its FP32 counterpart (V1f). Optional.
  const double* V1;
  const float* V1f;
};

__device__ __forceinline__ int pair_index(int i, int j) {
  int a = i > j ? i : j, b = i > j ? j : i;
  return a * (a + 1) / 2 + b;
}
// twoInt::operator() on spatial indices
__device__ __forceinline__ double i2_spatial(const double* __restrict__ I2, int i, int j, int k, int l) {
  int ij = pair_index(i, j), kl = pair_index(k, l);
  size_t A = ij > kl ? ij : kl, B = ij > kl ? kl : ij;
  return __ldg(I2 + A * (A + 1) / 2 + B);
}
// twoInt::operator() on spin orbitals: zero unless both pairs are same-spin
__device__ __forceinline__ double i2_spin(const double* __restrict__ I2, int i, int j, int k, int l) {
  if (((i ^ j) & 1) || ((k ^ l) & 1)) return 0.0;
  return i2_spatial(I2, i >> 1, j >> 1, k >> 1, l >> 1);
}

// Hij_1Excite (SHCI/Determinants.cpp:437-505): `a` created, `i` destroyed,
// the sum running over the ket's occupied spin orbitals in ascending order.
// Adds are kept un-fused and in the reference's order so the FP64 result is
// bit-identical to it.
__device__ inline double hij_single(const IntsView& I, const Det2& ket, int a, int i) {
  const int n2 = 2 * I.norb;
  double energy = __ldg(I.I1 + (size_t)a * n2 + i);
  if (I.V1) {  // the same terms, read from the table, summed in the same order
    const double* v = I.V1 + ((size_t)((a & 1) * I.norb + (a >> 1)) * I.norb + (i >> 1)) * n2;
#pragma unroll 1
    for (int w = 0; w < 2; ++w) {
      uint64_t bits = w ? ket.w1 : ket.w0;
      while (bits) {
        const int j = __ffsll((long long)bits) - 1 + 64 * w;
        bits &= bits - 1;
        energy = __dadd_rn(energy, __ldg(v + j));
      }
    }
    const int lo = a < i ? a : i, hi = a < i ? i : a;
    return (occ_between(ket, lo, hi) & 1) ? -energy : energy;
  }
  const int sa = a & 1;
  const int ai = pair_index(a >> 1, i >> 1);
#pragma unroll 1
  for (int w = 0; w < 2; ++w) {
    uint64_t bits = w ? ket.w1 : ket.w0;
    while (bits) {
      int j = __ffsll((long long)bits) - 1 + 64 * w;
      bits &= bits - 1;
      // (ai|jj) - (aj|ji); the exchange term vanishes for opposite spins
      int jj = pair_index(j >> 1, j >> 1);
      size_t A = ai > jj ? ai : jj, B = ai > jj ? jj : ai;
      double d = __ldg(I.I2 + A * (A + 1) / 2 + B);
      double x = 0.0;
      if ((j & 1) == sa) x = i2_spatial(I.I2, a >> 1, j >> 1, j >> 1, i >> 1);
      energy = __dadd_rn(energy, __dsub_rn(d, x));
    }
  }
  int lo = a < i ? a : i, hi = a < i ? i : a;
  return (occ_between(ket, lo, hi) & 1) ? -energy : energy;
}

// Hij_2Excite (SHCI/Determinants.cpp:406-434): i<j destroyed, a<b created.
__device__ inline double hij_double(const IntsView& I, const Det2& ket, int i, int j, int a, int b) {
  int c = occ_between(ket, i < a ? i : a, i < a ? a : i) + occ_between(ket, j < b ? j : b, j < b ? b : j);
  double sgn = (c & 1) ? -1.0 : 1.0;
  if (a > j || b < i) sgn = -sgn;
  double v = __dsub_rn(i2_spin(I.I2, a, i, b, j), i2_spin(I.I2, a, j, b, i));
  return sgn * v;
}

// Hij(bra, ket) for determinants at excitation distance 1 or 2
// (SHCI/Determinants.cpp:564-631).
__device__ inline double hij_any(const IntsView& I, const Det2& bra, const Det2& ket) {
  uint64_t u0 = bra.w0 ^ ket.w0, u1 = bra.w1 ^ ket.w1;
  uint64_t c0 = u0 & bra.w0, c1 = u1 & bra.w1;  // created
  uint64_t d0 = u0 & ket.w0, d1 = u1 & ket.w1;  // destroyed
  int ncre = __popcll(c0) + __popcll(c1);
  int cre[2], des[2];
  int k = 0;
  while (c0 && k < 2) { cre[k++] = __ffsll((long long)c0) - 1; c0 &= c0 - 1; }
  while (c1 && k < 2) { cre[k++] = __ffsll((long long)c1) - 1 + 64; c1 &= c1 - 1; }
  k = 0;
  while (d0 && k < 2) { des[k++] = __ffsll((long long)d0) - 1; d0 &= d0 - 1; }
  while (d1 && k < 2) { des[k++] = __ffsll((long long)d1) - 1 + 64; d1 &= d1 - 1; }
  if (ncre == 1) return hij_single(I, ket, cre[0], des[0]);
  if (ncre == 2) return hij_double(I, ket, des[0], des[1], cre[0], cre[1]);
  return 0.0;
}

// FP32 counterparts of hij_single / hij_double / hij_any on the FP32 integral
// copies, for the FP32 matrix-free sigma: same excitation and sign logic,
// FP32 arithmetic (about 1e-7 relative error per element: the rounding of
// the integrals to FP32 plus the FP32 sum of a single excitation's terms).
__device__ __forceinline__ float i2f_spatial(const float* __restrict__ I2f, int i, int j, int k, int l) {
  int ij = pair_index(i, j), kl = pair_index(k, l);
  size_t A = ij > kl ? ij : kl, B = ij > kl ? kl : ij;
  return __ldg(I2f + A * (A + 1) / 2 + B);
}
__device__ inline float hij_single_f32(const IntsView& I, const Det2& ket, int a, int i) {
  const int n2 = 2 * I.norb;
  float energy = __ldg(I.I1f + (size_t)a * n2 + i);
  if (I.V1f) {
    const float* v = I.V1f + ((size_t)((a & 1) * I.norb + (a >> 1)) * I.norb + (i >> 1)) * n2;
#pragma unroll 1
    for (int w = 0; w < 2; ++w) {
      uint64_t bits = w ? ket.w1 : ket.w0;
      while (bits) {
        const int j = __ffsll((long long)bits) - 1 + 64 * w;
        bits &= bits - 1;
        energy += __ldg(v + j);
      }
    }
    const int lo = a < i ? a : i, hi = a < i ? i : a;
    return (occ_between(ket, lo, hi) & 1) ? -energy : energy;
  }
  const int sa = a & 1;
  const int ai = pair_index(a >> 1, i >> 1);
#pragma unroll 1
  for (int w = 0; w < 2; ++w) {
    uint64_t bits = w ? ket.w1 : ket.w0;
    while (bits) {
      const int j = __ffsll((long long)bits) - 1 + 64 * w;
      bits &= bits - 1;
      const int jj = pair_index(j >> 1, j >> 1);
      const size_t A = ai > jj ? ai : jj, B = ai > jj ? jj : ai;
      float t = __ldg(I.I2f + A * (A + 1) / 2 + B);
      if ((j & 1) == sa) t -= i2f_spatial(I.I2f, a >> 1, j >> 1, j >> 1, i >> 1);
      energy += t;
    }
  }
  const int lo = a < i ? a : i, hi = a < i ? i : a;
  return (occ_between(ket, lo, hi) & 1) ? -energy : energy;
}
__device__ inline float hij_double_f32(const IntsView& I, const Det2& ket, int i, int j, int a, int b) {
  int c = occ_between(ket, i < a ? i : a, i < a ? a : i) + occ_between(ket, j < b ? j : b, j < b ? b : j);
  bool neg = (c & 1) != 0;
  if (a > j || b < i) neg = !neg;
  float v = 0.f;
  if (!(((a ^ i) & 1) || ((b ^ j) & 1))) v = i2f_spatial(I.I2f, a >> 1, i >> 1, b >> 1, j >> 1);
  if (!(((a ^ j) & 1) || ((b ^ i) & 1))) v -= i2f_spatial(I.I2f, a >> 1, j >> 1, b >> 1, i >> 1);
  return neg ? -v : v;
}
__device__ inline float hij_any_f32(const IntsView& I, const Det2& bra, const Det2& ket) {
  uint64_t u0 = bra.w0 ^ ket.w0, u1 = bra.w1 ^ ket.w1;
  uint64_t c0 = u0 & bra.w0, c1 = u1 & bra.w1;
  uint64_t d0 = u0 & ket.w0, d1 = u1 & ket.w1;
  int ncre = __popcll(c0) + __popcll(c1);
  int cre[2], des[2];
  int k = 0;
  while (c0 && k < 2) { cre[k++] = __ffsll((long long)c0) - 1; c0 &= c0 - 1; }
  while (c1 && k < 2) { cre[k++] = __ffsll((long long)c1) - 1 + 64; c1 &= c1 - 1; }
  k = 0;
  while (d0 && k < 2) { des[k++] = __ffsll((long long)d0) - 1; d0 &= d0 - 1; }
  while (d1 && k < 2) { des[k++] = __ffsll((long long)d1) - 1 + 64; d1 &= d1 - 1; }
  if (ncre == 1) return hij_single_f32(I, ket, cre[0], des[0]);
  if (ncre == 2) return hij_double_f32(I, ket, des[0], des[1], cre[0], cre[1]);
  return 0.f;
}

// Compensated FP32 accumulator (s + c): TwoSum of every addition and the FMA
// residual of every product are collected in c.
struct Acc {
  float s, c;
};
__device__ __forceinline__ void acc_add(Acc& a, float h, float x) {
  const float p = __fmul_rn(h, x);
  const float pe = __fmaf_rn(h, x, -p);  // exact product residual
  const float t = __fadd_rn(a.s, p);
  const float bp = __fsub_rn(t, a.s);
  const float e = __fadd_rn(__fsub_rn(a.s, __fsub_rn(t, bp)), __fsub_rn(p, bp));
  a.s = t;
  a.c = __fadd_rn(a.c, __fadd_rn(e, pe));
}
// The same without the product's rounding residual: the rounded product h*x
// does not depend on the order of the sum (so a row and its alpha <-> beta
// flipped row still sum the same products, compensated for order), and its
// rounding, 2^-24 of the product, is the size of the FP32 rounding of h and x
// themselves. Used where several vectors share each loaded element.
__device__ __forceinline__ void acc_add_rounded(Acc& a, float h, float x) {
  const float p = __fmul_rn(h, x);
  const float t = __fadd_rn(a.s, p);
  const float bp = __fsub_rn(t, a.s);
  const float e = __fadd_rn(__fsub_rn(a.s, __fsub_rn(t, bp)), __fsub_rn(p, bp));
  a.s = t;
  a.c = __fadd_rn(a.c, e);
}
__device__ __forceinline__ void acc_merge(Acc& a, const Acc& b) {
  const float t = __fadd_rn(a.s, b.s);
  const float bp = __fsub_rn(t, a.s);
  const float e = __fadd_rn(__fsub_rn(a.s, __fsub_rn(t, bp)), __fsub_rn(b.s, bp));
  a.s = t;
  a.c = __fadd_rn(a.c, __fadd_rn(e, b.c));
}

// Determinant::Energy without the core energy (SHCI/Determinants.cpp:252-300).
__device__ inline double det_energy(const IntsView& I, const Det2& d, const double* sDirect,
                                    const double* sExchange) {
  const int n = I.norb, n2 = 2 * n;
  int closed[kMaxSpin];
  int nc = 0;
  uint64_t b0 = d.w0, b1 = d.w1;
  while (b0) { closed[nc++] = __ffsll((long long)b0) - 1; b0 &= b0 - 1; }
  while (b1) { closed[nc++] = __ffsll((long long)b1) - 1 + 64; b1 &= b1 - 1; }
  double energy = 0.0;
  for (int i = 0; i < nc; i++) {
    int P = closed[i];
    energy = __dadd_rn(energy, __ldg(I.I1 + (size_t)P * n2 + P));
    for (int j = i + 1; j < nc; j++) {
      int Q = closed[j];
      energy = __dadd_rn(energy, sDirect[(P >> 1) * n + (Q >> 1)]);
      if (((P ^ Q) & 1) == 0) energy = __dsub_rn(energy, sExchange[(P >> 1) * n + (Q >> 1)]);
    }
  }
  return energy;
}

// 64-bit mixing hash for determinant keys (splitmix64 finaliser).
__host__ __device__ inline uint64_t mix64(uint64_t x) {
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  x ^= x >> 31;
  return x;
}
__host__ __device__ inline uint64_t det_hash(const Det2& d) { return mix64(d.w0 ^ mix64(d.w1 + 0x9e3779b97f4a7c15ull)); }

}  // namespace shci
