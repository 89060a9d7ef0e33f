// Kokkos_Random.hpp -- shim of Random_XorShift64_Pool (test infrastructure).
//
// The reference draws one frand(0,1) per random measurement per shot
// (MeasurementFunctors.hpp:245-251).  Kokkos' own stream is backend and
// thread dependent, so parity runs replace it with forced draws: when a bit
// table is installed, frand returns 0.25 for a 1 bit and 0.75 for a 0 bit of
// the current shot (the RangePolicy index), so `frand < bias` yields the bit
// at the default bias 0.5.  Without a table a plain xorshift64 is used
// (outcomes then are not meant to be compared bit-wise).
#pragma once
#include "Kokkos_Core.hpp"

namespace Kokkos {
namespace shim {
inline const std::uint8_t *&forced_bits() {
    static const std::uint8_t *p = nullptr;
    return p;
}
} // namespace shim

class Random_XorShift64 {
  public:
    explicit Random_XorShift64(std::uint64_t s) : state_(s ? s : 0x9E3779B97F4A7C15ull) {}
    float frand(float lo, float hi) {
        const std::uint8_t *bits = shim::forced_bits();
        float u;
        if (bits) {
            std::int64_t b = shim::current_index;
            u = ((bits[b >> 3] >> (b & 7)) & 1) ? 0.25f : 0.75f;
        } else {
            state_ ^= state_ << 13;
            state_ ^= state_ >> 7;
            state_ ^= state_ << 17;
            u = static_cast<float>(state_ >> 40) * (1.0f / 16777216.0f);
        }
        return lo + (hi - lo) * u;
    }

  private:
    std::uint64_t state_;
};

template <class ExecSpace = DefaultExecutionSpace> class Random_XorShift64_Pool {
  public:
    Random_XorShift64_Pool() = default;
    explicit Random_XorShift64_Pool(std::uint64_t seed) : seed_(seed) {}
    Random_XorShift64 get_state() const {
        return Random_XorShift64(seed_ ^ (0x9E3779B97F4A7C15ull * static_cast<std::uint64_t>(shim::current_index + 1)));
    }
    void free_state(const Random_XorShift64 &) const {}

  private:
    std::uint64_t seed_ = 0;
};
} // namespace Kokkos
