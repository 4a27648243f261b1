// Position of a Fourier mode in the reference's random stream: the number of
// draws the mode loop of Compute_Den (src/exshalos/density_grid.c:94-186)
// makes before it.  Plain C++ (host and device), checked on the CPU against a
// replay of that loop.
#pragma once

#if defined(__CUDACC__)
#define EXH_HD __host__ __device__ __forceinline__
#else
#define EXH_HD inline
#endif

namespace exh {

// Draws the reference's mode loop (density_grid.c:94-186) makes before mode
// (i, j, k), which must be a drawn mode (not a Hermitian copy): rows are
// visited in (i, j) order with k = 0 .. n2/2 inside; a mode draws two
// deviates (`fixed`: one phase), the eight self-conjugate modes one deviate
// (`fixed`: none), the copies on the k = 0 and k = n2/2 planes nothing.
// A row (i, j) holds copies when i > n0/2, or i in {0, n0/2} and j > n1/2;
// self-conjugate modes when i in {0, n0/2} and j in {0, n1/2}.
EXH_HD long long taus_draw_index(int i, int j, int k, int n0, int n1, int n2,
                                                              int fixed) {
  const int h0 = n0 / 2, h1 = n1 / 2;
  const long long nc = n2 / 2 + 1;
  const bool edge_i = (i == 0 || i == h0);
  const long long rows = (long long)i * n1 + j;
  long long copy_rows = (i > 0 ? n1 - 1 - h1 : 0) + (i > h0 ? n1 - 1 - h1 : 0) +
                        (i > h0 + 1 ? (long long)(i - h0 - 1) * n1 : 0);
  copy_rows += (i > h0) ? j : (edge_i ? (j > h1 + 1 ? j - h1 - 1 : 0) : 0);
  const long long self_rows = (i > 0 ? 2 : 0) + (i > h0 ? 2 : 0) + (edge_i ? (j > 0) + (j > h1) : 0);
  const bool copy_row = (i > h0) || (edge_i && j > h1);
  const bool self_row = edge_i && (j == 0 || j == h1);
  if (fixed) {
    const long long first = copy_row || self_row ? 0 : 1;
    return nc * rows - 2 * copy_rows - 2 * self_rows + (k > 0 ? first + (k - 1) : 0);
  }
  const long long first = copy_row ? 0 : (self_row ? 1 : 2);
  return 2 * nc * rows - 4 * copy_rows - 2 * self_rows + (k > 0 ? first + 2 * (long long)(k - 1) : 0);
}

// every draw of the field: the index the loop reaches after its last row
EXH_HD long long taus_draw_total(int n0, int n1, int n2, int fixed) {
  return taus_draw_index(n0, 0, 0, n0, n1, n2, fixed);
}

}  // namespace exh
