// MT19937 generator (M. Matsumoto and T. Nishimura, ACM TOMACS 8(1), 1998)
// with the 53-bit real draw the reference uses for its barostat and its input
// generators: MTRand(seed) followed by rand53()
// (include/algorithms/MersenneTwister.h:167-200, 337-341).  The host driver
// draws the Monte-Carlo box-move trials from it, as MD.cpp:149,595,690 do.
#pragma once
#include <cstdint>

namespace smd {

class Mt19937 {
 public:
  explicit Mt19937(uint32_t seed) {
    s_[0] = seed;
    for (int i = 1; i < 624; ++i) s_[i] = 1812433253u * (s_[i - 1] ^ (s_[i - 1] >> 30)) + (uint32_t)i;
    regen();
  }
  uint32_t next_u32() {
    if (pos_ == 624) regen();
    uint32_t y = s_[pos_++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    return y ^ (y >> 18);
  }
  double rand53() {
    const uint32_t hi = next_u32() >> 5, lo = next_u32() >> 6;
    return (hi * 67108864.0 + lo) * (1.0 / 9007199254740992.0);
  }

 private:
  void regen() {
    for (int i = 0; i < 624; ++i) {
      const uint32_t y = (s_[i] & 0x80000000u) | (s_[(i + 1) % 624] & 0x7fffffffu);
      s_[i] = s_[(i + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    pos_ = 0;
  }
  uint32_t s_[624];
  int pos_ = 624;
};

}  // namespace smd
