// Host check of exshalos_gb300/csrc/taus_index.h (run by
// tests/test_fixedpoint.py): the draw index of every drawn mode and the total
// against a replay of the reference's mode loop (density_grid.c:94-186),
// which walks i, j, k over the half-complex grid, skips the Hermitian copies
// of the k = 0 and k = nz/2 planes (the four copy rules of :109-150) and
// draws one deviate for the self-conjugate modes, two for the others
// (`fixed`: nothing / one phase).
#include <cstdio>
#include "taus_index.h"

int main() {
  long bad = 0, checked = 0;
  const int sizes[][3] = {{4, 4, 4}, {6, 6, 6}, {8, 8, 8}, {4, 6, 8}, {8, 4, 6}, {12, 10, 4}, {16, 16, 16},
                          {32, 32, 32}, {10, 14, 18}, {64, 48, 32}, {48, 64, 16}, {34, 36, 38}};
  for (const auto& sz : sizes) {
    const int n0 = sz[0], n1 = sz[1], n2 = sz[2], nz2 = n2 / 2 + 1;
    for (int fixed = 0; fixed < 2; fixed++) {
      long long d = 0;
      for (int i = 0; i < n0; i++)
        for (int j = 0; j < n1; j++)
          for (int k = 0; k < nz2; k++) {
            if ((k == 0 || k == n2 / 2) && (i > n0 / 2 || j > n1 / 2)) {
              if ((i > n0 / 2 && j > n1 / 2) || i == 0 || i == n0 / 2 || j == 0 || j == n1 / 2 ||
                  (i > n0 / 2 && j < n1 / 2))
                continue;                       // a copy: no draw
            }
            const long long got = exh::taus_draw_index(i, j, k, n0, n1, n2, fixed);
            checked++;
            if (got != d) {
              if (bad < 5) printf("%d %d %d (%d,%d,%d) fixed %d: %lld vs %lld\n", n0, n1, n2, i, j, k, fixed, got, d);
              bad++;
            }
            const bool selfc = (i == 0 || i == n0 / 2) && (j == 0 || j == n1 / 2) && (k == 0 || k == n2 / 2);
            d += fixed ? (selfc ? 0 : 1) : (selfc ? 1 : 2);
          }
      if (exh::taus_draw_total(n0, n1, n2, fixed) != d) {
        printf("total %d %d %d fixed %d: %lld vs %lld\n", n0, n1, n2, fixed,
               exh::taus_draw_total(n0, n1, n2, fixed), d);
        bad++;
      }
    }
  }
  printf("checked %ld bad %ld\n", checked, bad);
  return bad != 0;
}
