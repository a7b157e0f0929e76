// Checks walk_visits (gbr_math.h, the rule the tile rasteriser applies) against
// the literal fragment walk of the oracle (the reference state machine,
// cl2.cl:5046-5126) on whole bounding boxes: for each (w, h, miny, chunk) the
// set of pixels visited by all ceil(w*h/chunk) fragments must equal the set
// walk_visits accepts.  Usage: walk_rule_check <seed> <random cases>
// Exit code 0 when every case matches.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "../../oracle/gbr_oracle.cpp"

static long check(int w, int h, int miny, int chunk, int screen_w, int screen_h) {
  // a triangle whose rounded bbox is [0, w) x [miny, miny + h) after the -1 / clamp
  f3 tp[3] = {mk3(1.0f, (float)miny + 1.0f, 100.f), mk3((float)w, (float)miny + 1.0f, 100.f),
              mk3(1.0f, (float)(miny + h), 100.f)};
  float mm[4];
  bbox4(tp[0], tp[1], tp[2], (float)screen_w, (float)screen_h, mm);
  if ((int)mm[0] != 0 || (int)(mm[1] - mm[0]) != w || (int)mm[2] != miny || (int)(mm[3] - mm[2]) != h) {
    printf("bad construction w=%d h=%d miny=%d\n", w, h, miny);
    return 1;
  }
  std::vector<unsigned char> lit((size_t)w * h, 0);
  int nfrag = (int)ceilf((float)(w * h) / (float)chunk);
  for (int a = 0; a < nfrag; a++)
    walk(tp, (float)screen_w, (float)screen_h, chunk, (uint32_t)a, false, [&](float x, float y) {
      lit[(size_t)((int)y - miny) * w + (int)x] = 1;
    });
  long bad = 0;
  for (int r = 0; r < h; r++)
    for (int j = 0; j < w; j++) {
      bool rule = walk_visits(j, r, w, h, (float)miny, chunk);
      if (rule != (lit[(size_t)r * w + j] != 0)) {
        if (bad < 5) printf("mismatch w=%d h=%d miny=%d chunk=%d at (%d,%d): literal %d rule %d\n", w, h, miny, chunk, j, r, lit[(size_t)r * w + j], (int)rule);
        bad++;
      }
    }
  return bad;
}

int main(int argc, char** argv) {
  unsigned seed = argc > 1 ? (unsigned)atoi(argv[1]) : 1;
  int ncases = argc > 2 ? atoi(argv[2]) : 2000;
  long bad = 0, cases = 0, holes = 0;
  // exhaustive small boxes
  for (int w = 1; w <= 48; w++)
    for (int h = 1; h <= 24; h++)
      for (int miny : {0, 1, 7, 100, 513, 1000, 1079})
        for (int chunk : {500, 300}) {
          bad += check(w, h, miny, chunk, 3840, 2160);
          cases++;
        }
  // random boxes up to 3840 x 2160
  std::mt19937 rng(seed);
  for (int i = 0; i < ncases; i++) {
    int w = 1 + (int)(rng() % 3000);
    int miny = (int)(rng() % 2000);
    int hmax = std::min(2160 - 1 - miny, 1 + (int)(400000 / w));
    if (hmax < 1) continue;
    int h = 1 + (int)(rng() % hmax);
    int chunk = (rng() & 1) ? 500 : 300;
    bad += check(w, h, miny, chunk, 3840, 2160);
    for (int r = 1; r < h; r++) holes += walk_row_late(w, (float)miny, r);
    cases++;
  }
  printf("cases=%ld mismatching_pixels=%ld late_rows_seen=%ld\n", cases, bad, holes);
  return bad == 0 ? 0 : 1;
}
