// ORACLE — test infrastructure only. Nothing in the product links or calls this file.
//
// dSFMT-19937 (double-precision SIMD-oriented Fast Mersenne Twister, Saito & Matsumoto,
// "A PRNG specialized in double precision floating point numbers using an affine
// transition", MCQMC 2008), restated in portable scalar C++ from the published algorithm.
// The reference vendors the original library in mt/dSFMT.c and seeds it through
// Random::init (Random.hpp:12-14); the parameter set is the one the reference builds with
// (-DDSFMT_MEXP=19937, include.mk:9; constants as published in mt/dSFMT-params19937.h:6-15).
//
// Pinned: tests/golden/dsfmt_*.json hold outputs of the reference's own mt/dSFMT.c and
// Random.hpp, compiled from the reference sources by oracle/ref_build.sh.
#pragma once
#include <cstdint>
#include <cstring>

namespace ora {

class Dsfmt19937 {
 public:
  static constexpr int kN = (19937 - 128) / 104 + 1;  // 191 128-bit words
  static constexpr int kN64 = kN * 2;

  void seed(uint32_t s) {
    // 32-bit linear-congruential fill of the whole state (including the lung word),
    // little-endian 32-bit view of the 64-bit words.
    uint32_t w[(kN + 1) * 4];
    w[0] = s;
    for (int i = 1; i < (kN + 1) * 4; ++i)
      w[i] = 1812433253u * (w[i - 1] ^ (w[i - 1] >> 30)) + static_cast<uint32_t>(i);
    for (int k = 0; k < (kN + 1) * 2; ++k)
      st_[k] = static_cast<uint64_t>(w[2 * k]) | (static_cast<uint64_t>(w[2 * k + 1]) << 32);
    // force every word into [1,2) IEEE-754 form
    for (int k = 0; k < kN * 2; ++k) st_[k] = (st_[k] & kLowMask) | kHighConst;
    certify_period();
    idx_ = kN64;
  }

  // [1, 2)
  double close1_open2() {
    if (idx_ >= kN64) {
      refill();
      idx_ = 0;
    }
    return as_double(st_[idx_++]);
  }
  // [0, 1)
  double close_open() { return close1_open2() - 1.0; }
  // (0, 1]
  double open_close() { return 2.0 - close1_open2(); }
  // (0, 1)
  double open_open() {
    if (idx_ >= kN64) {
      refill();
      idx_ = 0;
    }
    return as_double(st_[idx_++] | 1u) - 1.0;
  }

 private:
  static constexpr int kPos1 = 117;
  static constexpr int kSl1 = 19;
  static constexpr int kSr = 12;
  static constexpr uint64_t kMsk1 = 0x000ffafffffffb3fULL;
  static constexpr uint64_t kMsk2 = 0x000ffdfffc90fffdULL;
  static constexpr uint64_t kFix1 = 0x90014964b32f4329ULL;
  static constexpr uint64_t kFix2 = 0x3b8d12ac548a7c7aULL;
  static constexpr uint64_t kPcv1 = 0x3d84e1ac0dc82880ULL;
  static constexpr uint64_t kPcv2 = 0x0000000000000001ULL;
  static constexpr uint64_t kLowMask = 0x000FFFFFFFFFFFFFULL;
  static constexpr uint64_t kHighConst = 0x3FF0000000000000ULL;

  static double as_double(uint64_t u) {
    double d;
    std::memcpy(&d, &u, sizeof d);
    return d;
  }

  // one step of the 128-bit recursion; word w is (st_[2w], st_[2w+1]); lung is (l0, l1)
  void recurse(int r, int a, int b, uint64_t &l0, uint64_t &l1) {
    const uint64_t t0 = st_[2 * a], t1 = st_[2 * a + 1];
    const uint64_t o0 = l0, o1 = l1;
    l0 = (t0 << kSl1) ^ (o1 >> 32) ^ (o1 << 32) ^ st_[2 * b];
    l1 = (t1 << kSl1) ^ (o0 >> 32) ^ (o0 << 32) ^ st_[2 * b + 1];
    st_[2 * r] = (l0 >> kSr) ^ (l0 & kMsk1) ^ t0;
    st_[2 * r + 1] = (l1 >> kSr) ^ (l1 & kMsk2) ^ t1;
  }

  void refill() {
    uint64_t l0 = st_[2 * kN], l1 = st_[2 * kN + 1];
    int i = 0;
    for (; i < kN - kPos1; ++i) recurse(i, i, i + kPos1, l0, l1);
    for (; i < kN; ++i) recurse(i, i, i + kPos1 - kN, l0, l1);
    st_[2 * kN] = l0;
    st_[2 * kN + 1] = l1;
  }

  void certify_period() {
    uint64_t inner = ((st_[2 * kN] ^ kFix1) & kPcv1) ^ ((st_[2 * kN + 1] ^ kFix2) & kPcv2);
    for (int s = 32; s > 0; s >>= 1) inner ^= inner >> s;
    if (inner & 1u) return;
    st_[2 * kN + 1] ^= 1u;  // the lowest set bit of PCV2 is bit 0
  }

  uint64_t st_[(kN + 1) * 2];
  int idx_ = kN64;
};

}  // namespace ora
