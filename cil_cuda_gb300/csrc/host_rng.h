// Host random stream of oracle mode (CIL_RNG_DSFMT).
//
// dSFMT-19937 (Saito & Matsumoto, MCQMC 2008) in portable scalar C++, seeded like the
// reference's Random::init (Random.hpp:12-14, vendored mt/dSFMT.c built with
// -DDSFMT_MEXP=19937, include.mk:9), plus the reference's draw functions on top of it:
// uniform / uniform0x / Leva's normal / onDSphere (Random.hpp:16-118). With the same seed
// this stream reproduces the reference's Random:: sequence bit for bit, so the library
// draws noise, division axes, cycle lengths and apoptosis tests in the reference's order.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

namespace cil {

class HostRng {
 public:
  void seed(uint32_t s) {
    uint32_t w[(kN + 1) * 4];
    w[0] = s;
    for (int i = 1; i < (kN + 1) * 4; ++i)
      w[i] = 1812433253u * (w[i - 1] ^ (w[i - 1] >> 30)) + static_cast<uint32_t>(i);
    for (int k = 0; k < (kN + 1) * 2; ++k)
      st_[k] = static_cast<uint64_t>(w[2 * k]) | (static_cast<uint64_t>(w[2 * k + 1]) << 32);
    for (int k = 0; k < kN * 2; ++k)
      st_[k] = (st_[k] & 0x000FFFFFFFFFFFFFULL) | 0x3FF0000000000000ULL;
    uint64_t inner = ((st_[2 * kN] ^ 0x90014964b32f4329ULL) & 0x3d84e1ac0dc82880ULL) ^
                     ((st_[2 * kN + 1] ^ 0x3b8d12ac548a7c7aULL) & 0x0000000000000001ULL);
    for (int sh = 32; sh > 0; sh >>= 1) inner ^= inner >> sh;
    if (!(inner & 1u)) st_[2 * kN + 1] ^= 1u;
    idx_ = 2 * kN;
  }

  double close_open() { return bits(next()) - 1.0; }
  double open_open() { return bits(next() | 1u) - 1.0; }

  double uniform() { return (open_open() - 0.5) * 2.0; }
  double uniform0x(double x) { return close_open() * x; }
  double normal() {
    const double s = 0.449871, t = -0.386595, a = 0.19600, b = 0.25472;
    const double r1 = 0.27597, r2 = 0.27846;
    double u, v, x, y, q;
    do {
      u = 1.0 - close_open();
      v = 1.7156 * (close_open() - 0.5);
      x = u - s;
      y = std::fabs(v) - t;
      q = x * x + y * (a * y - b * x);
    } while (q >= r1 && (q > r2 || v * v > -4.0 * u * u * std::log(u)));
    return v / u;
  }
  double normal(double mu, double sigma) { return mu + sigma * normal(); }
  void on_dsphere(int dim, double *ni) {
    double r2;
    for (;;) {
      r2 = 0.0;
      for (int d = 0; d < dim; ++d) {
        ni[d] = uniform();
        r2 += ni[d] * ni[d];
      }
      if (r2 <= 1.0) break;
    }
    const double norm = 1.0 / std::sqrt(r2);
    for (int d = 0; d < dim; ++d) ni[d] *= norm;
  }

 private:
  static constexpr int kN = (19937 - 128) / 104 + 1;

  static double bits(uint64_t u) {
    double d;
    std::memcpy(&d, &u, sizeof d);
    return d;
  }
  uint64_t next() {
    if (idx_ >= 2 * kN) {
      refill();
      idx_ = 0;
    }
    return st_[idx_++];
  }
  void refill() {
    const int pos1 = 117, sl1 = 19, sr = 12;
    const uint64_t m1 = 0x000ffafffffffb3fULL, m2 = 0x000ffdfffc90fffdULL;
    uint64_t l0 = st_[2 * kN], l1 = st_[2 * kN + 1];
    for (int i = 0; i < kN; ++i) {
      const int b = i + pos1 < kN ? i + pos1 : i + pos1 - kN;
      const uint64_t t0 = st_[2 * i], t1 = st_[2 * i + 1];
      const uint64_t o0 = l0, o1 = l1;
      l0 = (t0 << sl1) ^ (o1 >> 32) ^ (o1 << 32) ^ st_[2 * b];
      l1 = (t1 << sl1) ^ (o0 >> 32) ^ (o0 << 32) ^ st_[2 * b + 1];
      st_[2 * i] = (l0 >> sr) ^ (l0 & m1) ^ t0;
      st_[2 * i + 1] = (l1 >> sr) ^ (l1 & m2) ^ t1;
    }
    st_[2 * kN] = l0;
    st_[2 * kN + 1] = l1;
  }

  uint64_t st_[(kN + 1) * 2];
  int idx_ = 2 * kN;
};

}  // namespace cil
