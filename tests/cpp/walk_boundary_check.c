/* Exhaustive check of the row-change points of the reference fragment walk
 * (cl2.cl:5046-5081: y = floor(mad(k, 1.f/w, miny))).
 *
 * For every bbox width w <= W, top row miny < H and row boundary k = r*w
 * (1 <= r <= H - miny) it evaluates the row index the walk computes at k-1, k
 * and k+1 and counts boundaries where the row changes early (at k-1), one step
 * late (at k+1) or two steps late (after k+1).  Prints the counts; the
 * rasteriser's walk rule (gbr_math.h walk_visits) assumes early == 0 and
 * late2 == 0.  Build: cc -O2 -fopenmp -ffp-contract=off walk_boundary_check.c -lm
 * Usage: walk_boundary_check W H
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  int W = atoi(argv[1]), H = atoi(argv[2]);
  long early = 0, late1 = 0, late2 = 0;
#pragma omp parallel for schedule(dynamic, 8) reduction(+ : early, late1, late2)
  for (int w = 1; w <= W; w++) {
    float iw = 1.f / (float)w;
    for (int miny = 0; miny < H; miny++) {
      float fm = (float)miny;
      for (int r = 1; r <= H - miny; r++) {
        long k0 = (long)r * w;
        float ya = floorf(fmaf((float)(k0 - 1), iw, fm)) - fm;
        float yb = floorf(fmaf((float)k0, iw, fm)) - fm;
        float yc = floorf(fmaf((float)(k0 + 1), iw, fm)) - fm;
        if (ya != (float)(r - 1)) early++;
        if (yb != (float)r) late1++;
        if (w > 1 && yc != (float)r) late2++;
      }
    }
  }
  printf("W=%d H=%d early=%ld late1=%ld late2=%ld\n", W, H, early, late1, late2);
  return (early == 0 && late2 == 0) ? 0 : 1;
}
