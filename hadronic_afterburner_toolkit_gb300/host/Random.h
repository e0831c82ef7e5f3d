// Shared random-number source of an analysis.
//
// Same engine and distributions as the reference's RandomUtil::Random
// (src/Random.{h,cpp}): std::mt19937 seeded with `seed` (-1: from
// std::random_device), rand_uniform() from uniform_real_distribution<double>
// over [min, max), rand_int_uniform() from uniform_int_distribution<int> over
// [0, INT_MAX].  Mixed-event partners and rotation angles are drawn from it in
// the reference's order, so a given seed selects the same partners.
#pragma once

#include <memory>
#include <random>

namespace RandomUtil {

class Random {
  public:
    explicit Random(int seed_in, double min = 0.0, double max = 1.0);
    double rand_uniform() { return uniform_(*gen_); }
    int rand_int_uniform() { return int_uniform_(*gen_); }
    int get_seed() const { return seed_; }

  private:
    int seed_;
    std::unique_ptr<std::mt19937> gen_;
    std::uniform_real_distribution<double> uniform_;
    std::uniform_int_distribution<int> int_uniform_;
};

}  // namespace RandomUtil
