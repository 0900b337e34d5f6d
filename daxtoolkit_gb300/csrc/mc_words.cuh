// Row-word helpers of the marching-cubes count passes: the eight corner
// windows of a word's cells, their case indices and the packed per-word
// counts (triangles << 16 | crossing edges).
#pragma once
#include <cstdint>

#include "common.cuh"
#include "mc_case.cuh"

namespace daxgb {

struct CornerWords {
  uint32_t a, a1, b, b1, c, c1, d, d1;
};

// Case index of cell q of the word; vertex order v0..v7 =
// (i,j,k) (i+1,j,k) (i+1,j+1,k) (i,j+1,k) and the same at k+1
// (dax/exec/internal/TopologyUniform.h:150-157); bit n = value[n] > iso.
__device__ __forceinline__ int case_of(const CornerWords& w, int q) {
  return (int)(((w.a >> q) & 1u) | (((w.a1 >> q) & 1u) << 1) | (((w.b1 >> q) & 1u) << 2) |
               (((w.b >> q) & 1u) << 3) | (((w.c >> q) & 1u) << 4) | (((w.c1 >> q) & 1u) << 5) |
               (((w.d1 >> q) & 1u) << 6) | (((w.d >> q) & 1u) << 7));
}

// Cells of the word that are neither all-inside nor all-outside.
__device__ __forceinline__ uint32_t active_cells(const CornerWords& w, uint32_t cell_mask) {
  const uint32_t all1 = w.a & w.a1 & w.b & w.b1 & w.c & w.c1 & w.d & w.d1;
  const uint32_t any1 = w.a | w.a1 | w.b | w.b1 | w.c | w.c1 | w.d | w.d1;
  return any1 & ~all1 & cell_mask;
}

// The eight corner words of word m of row r (a, a+x of rows (j..j+1,
// k..k+1)) and the masks that decide which of them are meaningful.
struct WordBits {
  CornerWords w;
  uint32_t pmask, xmask;
  bool hy, hz;
};

template <bool CG = false>
__device__ __forceinline__ WordBits load_word_bits(const Grid& g, const uint32_t* bits, unsigned r,
                                                   int m) {
  WordBits wb;
  int j, k;
  split_row(g, r, j, k);
  wb.hy = j < g.ny - 1;
  wb.hz = k < g.nz - 1;
  const long long dy = g.nx, dz = (long long)g.nx * g.ny;
  const long long pos = (long long)r * g.nx + 32ll * m;
  wb.pmask = low_mask(g.nx - 32 * m);
  wb.xmask = low_mask(g.nx - 1 - 32 * m);
  wb.w = CornerWords{};
  bits_at2<CG>(bits, pos, wb.w.a, wb.w.a1);
  if (wb.hy) bits_at2<CG>(bits, pos + dy, wb.w.b, wb.w.b1);
  if (wb.hz) bits_at2<CG>(bits, pos + dz, wb.w.c, wb.w.c1);
  if (wb.hy && wb.hz) bits_at2<CG>(bits, pos + dy + dz, wb.w.d, wb.w.d1);
  return wb;
}

// Counts of one word from its eight corner words.
__device__ __forceinline__ uint32_t packed_counts(const CornerWords& w, bool hy, bool hz,
                                                  uint32_t pmask, uint32_t xmask,
                                                  const unsigned char* nf) {
  int v = __popc((w.a ^ w.a1) & xmask);
  if (hy) v += __popc((w.a ^ w.b) & pmask);
  if (hz) v += __popc((w.a ^ w.c) & pmask);
  int t = 0;
  if (hy && hz)
    for (uint32_t u = active_cells(w, xmask); u; u &= u - 1) t += nf[case_of(w, __ffs(u) - 1)];
  return ((uint32_t)t << 16) | (uint32_t)v;
}

}  // namespace daxgb
