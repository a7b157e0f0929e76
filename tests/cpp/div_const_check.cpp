// Checks u8_over_255 and u16_over_65535 (gbr_math.h: the reciprocal product
// with one residual correction) against the correctly rounded IEEE division
// fdiv(t, 255.0f) / fdiv(t, 65535.0f), bit for bit, for every integer t of
// their ranges.  Usage: div_const_check.  Exit code 0 when all match.
#include <cstdio>
#include <cstring>

#include "../../openclrenderer_gb300/csrc/gbr_math.h"

static uint32_t bits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
}

int main() {
  long bad255 = 0, bad65535 = 0;
  for (uint32_t t = 0; t <= 255; t++)
    if (bits(gbr::u8_over_255(t)) != bits(gbr::fdiv((float)t, 255.0f))) {
      if (bad255 < 5) std::printf("t=%u: %a vs %a\n", t, gbr::u8_over_255(t), gbr::fdiv((float)t, 255.0f));
      bad255++;
    }
  for (uint32_t t = 0; t <= 65535; t++)
    if (bits(gbr::u16_over_65535(t)) != bits(gbr::fdiv((float)t, 65535.0f))) {
      if (bad65535 < 5)
        std::printf("t=%u: %a vs %a\n", t, gbr::u16_over_65535(t), gbr::fdiv((float)t, 65535.0f));
      bad65535++;
    }
  std::printf("mismatches_255=%ld mismatches_65535=%ld\n", bad255, bad65535);
  return bad255 || bad65535 ? 1 : 0;
}
