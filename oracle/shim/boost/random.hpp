// Minimal stand-in for the three Boost.Random 1.80 types that SpAc's
// Feynman-Kac solver uses (boost::mt19937, normal_distribution<double>,
// exponential_distribution<double>).  Written for this project; it exists only
// so that the reference sources compile unmodified as a test oracle.
//
// Differences from Boost, all documented and all confined to the random
// stream (the reference's parity contract is statistical):
//  * normal_distribution is Box-Muller from two 32-bit words per draw (no
//    cached second value), not Boost's ziggurat.  The oracle restatement's
//    "sequential stream" mode uses the identical transform, so that the
//    oracle and the compiled reference consume the same numbers.
//  * mt19937::discard(z) for z >= 2^24 re-seeds from z instead of skipping z
//    words one by one (the reference discards 1e10 words per OpenMP thread).
#ifndef SPAC_ORACLE_SHIM_BOOST_RANDOM
#define SPAC_ORACLE_SHIM_BOOST_RANDOM
#include <cmath>
#include <cstdint>
#include <random>

namespace boost {

class mt19937 {
 public:
  typedef std::uint32_t result_type;
  mt19937() : e_(5489u) {}
  explicit mt19937(std::uint32_t s) : e_(s) {}
  result_type operator()() { return static_cast<result_type>(e_()); }
  void seed(std::uint32_t s) { e_.seed(s); }
  void discard(unsigned long long z) {
    if (z < (1ull << 24)) {
      e_.discard(z);
    } else {
      std::seed_seq sq{static_cast<std::uint32_t>(z), static_cast<std::uint32_t>(z >> 32), 0x5eedu};
      e_.seed(sq);
    }
  }

 private:
  std::mt19937 e_;
};

namespace random {
using ::boost::mt19937;
}

template <typename RealType = double>
class normal_distribution {
 public:
  explicit normal_distribution(RealType mean = 0, RealType sigma = 1) : mean_(mean), sigma_(sigma) {}
  template <typename Engine>
  RealType operator()(Engine& e) {
    const double inv32 = 2.3283064365386962890625e-10;  // 2^-32
    std::uint32_t a = static_cast<std::uint32_t>(e());
    std::uint32_t b = static_cast<std::uint32_t>(e());
    double u1 = (static_cast<double>(a) + 0.5) * inv32;
    double u2 = (static_cast<double>(b) + 0.5) * inv32;
    double z = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    return mean_ + sigma_ * z;
  }

 private:
  RealType mean_, sigma_;
};

template <typename RealType = double>
class exponential_distribution {
 public:
  explicit exponential_distribution(RealType lambda = 1) : lambda_(lambda) {}
  template <typename Engine>
  RealType operator()(Engine& e) {
    const double inv32 = 2.3283064365386962890625e-10;
    std::uint32_t a = static_cast<std::uint32_t>(e());
    double u = (static_cast<double>(a) + 0.5) * inv32;
    return -std::log(u) / lambda_;
  }

 private:
  RealType lambda_;
};

}  // namespace boost
#endif
