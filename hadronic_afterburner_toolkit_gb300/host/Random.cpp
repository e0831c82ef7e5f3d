#include "Random.h"

namespace RandomUtil {

Random::Random(int seed_in, double min, double max) : seed_(seed_in), uniform_(min, max) {
    if (seed_ == -1) {
        std::random_device dev;
        seed_ = static_cast<int>(dev());
    }
    gen_.reset(new std::mt19937(static_cast<std::mt19937::result_type>(seed_)));
}

}  // namespace RandomUtil
