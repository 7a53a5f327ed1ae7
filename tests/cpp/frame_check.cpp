// The lateral-frame numbering of vibe_internal.cuh (frame_count /
// frame_column) against the direct definition: every column of an nx x ny
// cell grid with min(i, nx-1-i, j, ny-1-j) < f appears exactly once, and
// nothing else. Prints "bad <n>"; exit status 0 when n = 0.
#include <cstdio>
#include <set>
#include <utility>

#include "vibe_internal.cuh"

int main() {
  using namespace vgb;
  int bad = 0;
  for (int nx = 1; nx <= 40; ++nx)
    for (int ny = 1; ny <= 40; ++ny)
      for (int f = 1; f <= 22; ++f) {
        std::set<std::pair<int, int>> want, got;
        for (int j = 0; j < ny; ++j)
          for (int i = 0; i < nx; ++i)
            if (imin(imin(i, nx - 1 - i), imin(j, ny - 1 - j)) < f) want.insert({i, j});
        const int n = frame_count(nx, ny, f);
        for (int e = 0; e < n; ++e) {
          int i = -1, j = -1;
          frame_column(e, nx, ny, f, i, j);
          if (i < 0 || i >= nx || j < 0 || j >= ny || !got.insert({i, j}).second) ++bad;
        }
        if (got != want) ++bad;
      }
  std::printf("bad %d\n", bad);
  return bad != 0;
}
