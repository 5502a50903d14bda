// k-chunking of the stage kernel's work items (fw::stage_chunk, kernels.h), checked on the
// host for every grid depth up to 60 planes, every chunk length up to 20 and every pair of
// band edges: the chunks tile [k1, k2] in order, none is longer than kc, and none straddles
// a band edge; and the default chunk length's bounds.  Built and run by
// tests/test_stage_chunks.py.
#include <cstdio>
#include "kernels.h"
int main() {
  int bad = 0, cases = 0;
  for (int nk = 1; nk <= 60; ++nk)
    for (int kc = 1; kc <= 20; ++kc)
      for (int lo_off = 0; lo_off <= nk; ++lo_off)
        for (int hi_off = lo_off; hi_off <= nk; ++hi_off) {
          fw::Geom g{}; g.k1 = 3; g.k2 = 3 + nk - 1; g.nk = nk;
          const int lo = g.k1 + lo_off, hi = g.k1 + hi_off;
          const int n = fw::stage_chunk_count(g, kc, lo, hi);
          int next = g.k1;
          ++cases;
          for (int bz = 0; bz < n; ++bz) {
            int kb, ke;
            fw::stage_chunk(g, kc, lo, hi, bz, &kb, &ke);
            if (kb != next || ke < kb || ke - kb + 1 > kc || (kb < lo && ke >= lo) || (kb < hi && ke >= hi)) { ++bad; break; }
            next = ke + 1;
          }
          if (next != g.k2 + 1) ++bad;
        }
  // the default planes per CTA (fw::stage_planes_per_cta): within [3, 24] unless the grid
  // is deeper than 2047 x 24 planes, never more than 2047 plain chunks, and the banded
  // chunk count always fits the 12 bits an item gives it
  for (int ty : {8, 16})
    for (int ni = 8; ni <= 32768; ni = ni < 64 ? ni + 7 : ni * 2)
      for (int nj = 8; nj <= 8192; nj = nj < 64 ? nj + 5 : nj * 2)
        for (int nk = 8; nk <= 8188; nk = nk < 64 ? nk + 1 : nk + 97) {
          fw::Geom g{}; g.ni = ni; g.nj = nj; g.nk = nk; g.k1 = 3; g.k2 = 3 + nk - 1;
          const int kc = fw::stage_planes_per_cta(g, 152, ty);
          ++cases;
          const int lo = g.k1 + (nk > 12 ? 12 : 0), hi = g.k2 - 3;
          if (kc < 3 || kc > 24 || (nk + kc - 1) / kc > 2047 || fw::stage_chunk_count(g, kc, lo, hi) > 4095) ++bad;
        }
  printf("cases %d bad %d\n", cases, bad);
  return bad != 0;
}
