// Cell threshold on the in-range bit stream (bit = lo <= f <= hi), on the
// row-word pipeline marching cubes uses.
//
// K2a (k_thr_count): per row word w = (point row r = (j, k), word m)
//     kept[w] = cells 32m .. 32m+31 of cell row r whose 8 corners are all in
//               range (ThresholdFunction, dax/worklet/Threshold.h:30-66)
//     used[w] = points 32m .. 32m+31 of point row r that are a corner of a
//               kept cell (FillPointMask,
//               dax/cont/DispatcherGenerateTopology.h:206-227)
//     wc[w]   = popc(kept) << 16 | popc(used)
// K2b (k_mc_scan, shared with marching cubes): per-word exclusive offsets
//     wt (kept cells) and wv (used points), the compacted list act of the
//     words with either, and the totals.
// K3 (k_thr_emit): a warp loads 32 active words at once (lane = word), then
//     walks them with lane = bit: the word's used points (coordinates and
//     field: StreamCompact with the point mask, :237-239 and :98-113) and
//     its kept cells, whose 8 corner ids are each corner's rank among the
//     used points.  That equals the reference's Copy/Sort/Unique/LowerBounds
//     of the connectivity (:229-258), because the used ids sorted ascending
//     are exactly the used points in point order.
#include "common.cuh"
#include "kernels.cuh"

namespace daxgb {

namespace {

// Cells of point row (j+dj, k+dk) whose two x-corners are in range: bit b
// is cell 32m+b; *carry = the same for cell 32m-1 (m > 0).
__device__ __forceinline__ uint32_t x_pairs(const Grid& g, const uint32_t* __restrict__ bits,
                                            long long pos, int m, uint32_t* carry) {
  uint32_t a, a1;
  bits_at2(bits, pos, a, a1);
  if (m > 0) {
    const long long q = pos - 1;
    *carry = ((__ldg(bits + (q >> 5)) >> (unsigned)(q & 31)) & a) & 1u;
  } else {
    *carry = 0u;
  }
  return a & a1;
}

}  // namespace

__global__ void __launch_bounds__(256) k_thr_count(Grid g, const uint32_t* __restrict__ bits,
                                                   uint32_t* __restrict__ kept,
                                                   uint32_t* __restrict__ used,
                                                   uint32_t* __restrict__ wc) {
  const long long W = g.R * g.wr;  // < 2^27 for grids below 2^31 points
  const long long dy = g.nx, dz = (long long)g.nx * g.ny;
  for (long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x; w < W;
       w += (long long)gridDim.x * blockDim.x) {
    const unsigned r = (unsigned)w / (unsigned)g.wr;
    const int m = (int)((unsigned)w - r * (unsigned)g.wr);
    const int j = (int)(r % (unsigned)g.ny), k = (int)(r / (unsigned)g.ny);
    const long long pos = (long long)r * g.nx + 32ll * m;
    // x-pairs of the 3 x 3 point rows around (j, k): px[dk + 1][dj + 1]
    uint32_t px[3][3], pc[3][3];
#pragma unroll
    for (int dk = -1; dk <= 1; ++dk) {
#pragma unroll
      for (int dj = -1; dj <= 1; ++dj) {
        const int jj = j + dj, kk = k + dk;
        if (jj < 0 || jj >= g.ny || kk < 0 || kk >= g.nz) {
          px[dk + 1][dj + 1] = 0u;
          pc[dk + 1][dj + 1] = 0u;
        } else {
          px[dk + 1][dj + 1] = x_pairs(g, bits, pos + dj * dy + dk * dz, m, &pc[dk + 1][dj + 1]);
        }
      }
    }
    // kept cells of the 4 cell rows (j + cj, k + ck), cj, ck in {-1, 0}
    const uint32_t cmask = low_mask(g.nx - 1 - 32 * m);
    uint32_t own = 0u, u = 0u;
#pragma unroll
    for (int ck = -1; ck <= 0; ++ck) {
#pragma unroll
      for (int cj = -1; cj <= 0; ++cj) {
        const int jc = j + cj, kc = k + ck;
        if (jc < 0 || jc >= g.ny - 1 || kc < 0 || kc >= g.nz - 1) continue;
        const uint32_t K = px[ck + 1][cj + 1] & px[ck + 1][cj + 2] & px[ck + 2][cj + 1] &
                           px[ck + 2][cj + 2] & cmask;
        const uint32_t Kc = pc[ck + 1][cj + 1] & pc[ck + 1][cj + 2] & pc[ck + 2][cj + 1] &
                            pc[ck + 2][cj + 2];
        u |= K | (K << 1) | Kc;
        if (cj == 0 && ck == 0) own = K;
      }
    }
    u &= low_mask(g.nx - 32 * m);
    kept[w] = own;
    used[w] = u;
    wc[w] = ((uint32_t)__popc(own) << 16) | (uint32_t)__popc(u);
  }
}

void launch_thr_count(const Grid& g, const uint32_t* bits, uint32_t* kept, uint32_t* used,
                      uint32_t* wc, int num_sms, cudaStream_t s) {
  const long long want = (g.R * g.wr + 255) / 256;
  const int blocks = resident_blocks(k_thr_count, 256, 0, num_sms, want);
  k_thr_count<<<blocks, 256, 0, s>>>(g, bits, kept, used, wc);
}

// Per active word, what the emit loop needs: its masks and offsets, and for
// kept cells the used masks / offsets of the 7 other corner words: rows
// q = dj + 2 dk (q = 1..3) at word m, and rows q = 0..3 at word m + 1.
struct ThrWord {
  uint32_t w, u, kw, v0, t0;
  uint32_t cu[7], cv[7];
};

__global__ void __launch_bounds__(256) k_thr_emit(Grid g, const float* __restrict__ f,
                                                  const uint32_t* __restrict__ kept,
                                                  const uint32_t* __restrict__ used,
                                                  const uint32_t* __restrict__ wt,
                                                  const uint32_t* __restrict__ wv,
                                                  const uint32_t* __restrict__ act,
                                                  Info* __restrict__ info,
                                                  int32_t* __restrict__ conn, long long kcap,
                                                  float* __restrict__ coords,
                                                  float* __restrict__ fout, long long ucap) {
  const long long K = info->total_a, U = info->total_b, A = info->total_c;
  if (K > kcap || U > ucap || (info->error & (kErrOverflow | kErrTimeout))) {
    if (blockIdx.x == 0 && threadIdx.x == 0 && (K > kcap || U > ucap))
      atomicOr(&info->error, kErrCapacity);
    return;
  }
  const int lane = threadIdx.x & 31;
  const uint32_t below = (1u << lane) - 1u;
  const bool conn16 = (reinterpret_cast<uintptr_t>(conn) & 15) == 0;
  const long long warp0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  const unsigned wr = (unsigned)g.wr;
  for (long long a0 = warp0 * 32; a0 < A; a0 += nwarps * 32) {
    // lane L gathers active word a0 + L
    ThrWord d{};
    const int cnt = (int)min(32ll, A - a0);
    if (lane < cnt) {
      d.w = __ldg(act + a0 + lane);
      d.u = __ldg(used + d.w);
      d.kw = __ldg(kept + d.w);
      d.v0 = __ldg(wv + d.w);
      d.t0 = __ldg(wt + d.w);
      if (d.kw) {  // a kept cell implies rows j + 1 and k + 1 exist
        const unsigned r = d.w / wr, m = d.w - r * wr;
        const uint32_t rows[4] = {d.w, d.w + wr, d.w + (unsigned)g.ny * wr,
                                  d.w + (unsigned)(g.ny + 1) * wr};
#pragma unroll
        for (int q = 1; q < 4; ++q) {
          d.cu[q - 1] = __ldg(used + rows[q]);
          d.cv[q - 1] = __ldg(wv + rows[q]);
        }
        if (m + 1 < wr) {
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            d.cu[3 + q] = __ldg(used + rows[q] + 1);
            d.cv[3 + q] = __ldg(wv + rows[q] + 1);
          }
        }
      }
    }
    for (int s = 0; s < cnt; ++s) {
      const uint32_t w = __shfl_sync(kFull, d.w, s);
      const uint32_t u = __shfl_sync(kFull, d.u, s);
      const uint32_t kw = __shfl_sync(kFull, d.kw, s);
      const uint32_t r = w / wr, m = w - r * wr;
      const int j = (int)(r % (unsigned)g.ny), k = (int)(r / (unsigned)g.ny);
      const int i = 32 * (int)m + lane;
      const long long p = (long long)r * g.nx + i;
      const uint32_t v0 = __shfl_sync(kFull, d.v0, s);
      if ((u >> lane) & 1u) {
        const long long id = (long long)v0 + __popc(u & below);
        float* c = coords + 3 * id;
        c[0] = coord(g.ox, g.sx, i, g.mx);
        c[1] = coord(g.oy, g.sy, j, g.my);
        c[2] = coord(g.oz, g.sz, k, g.mz);
        if (fout) fout[id] = __ldg(f + p);
      }
      if (kw == 0u) continue;  // uniform across the warp
      const uint32_t t0 = __shfl_sync(kFull, d.t0, s);
      uint32_t cu[8], cv[8];  // corner rows q at word m (0..3) and m + 1 (4..7)
      cu[0] = u;
      cv[0] = v0;
#pragma unroll
      for (int e = 0; e < 7; ++e) {
        cu[e + 1] = __shfl_sync(kFull, d.cu[e], s);
        cv[e + 1] = __shfl_sync(kFull, d.cv[e], s);
      }
      if ((kw >> lane) & 1u) {
        const long long cid = (long long)t0 + __popc(kw & below);
        int32_t ids[8];
#pragma unroll
        for (int v = 0; v < 8; ++v) {
          // v0..v7: (i,j,k) (i+1,j,k) (i+1,j+1,k) (i,j+1,k), then the same at k+1
          const int di = ((v & 3) == 1 || (v & 3) == 2) ? 1 : 0;
          const int dj = ((v & 3) >= 2) ? 1 : 0;
          const int q = dj + 2 * (v >> 2);
          uint32_t uq = cu[q], vq = cv[q], lm = below;
          if (di) {
            if (lane == 31) {  // corner i + 1 is bit 0 of word m + 1
              uq = cu[4 + q];
              vq = cv[4 + q];
              lm = 0u;
            } else {
              lm = (2u << lane) - 1u;
            }
          }
          ids[v] = (int32_t)(vq + (uint32_t)__popc(uq & lm));
        }
        if (conn16) {
          int4* dst = reinterpret_cast<int4*>(conn + 8 * cid);
          dst[0] = make_int4(ids[0], ids[1], ids[2], ids[3]);
          dst[1] = make_int4(ids[4], ids[5], ids[6], ids[7]);
        } else {
#pragma unroll
          for (int v = 0; v < 8; ++v) conn[8 * cid + v] = ids[v];
        }
      }
    }
  }
}

void launch_thr_emit(const Grid& g, const float* f, const WordOffsets& o, const uint32_t* kept,
                     const uint32_t* used, Info* info, int32_t* conn, long long kcap,
                     float* coords, float* fout, long long ucap, int num_sms, cudaStream_t s) {
  // the active count lives on the device: one resident wave, grid-stride
  const long long want = (g.R * g.wr + 255) / 256;
  const int blocks = resident_blocks(k_thr_emit, 256, 0, num_sms, want);
  k_thr_emit<<<blocks, 256, 0, s>>>(g, f, kept, used, o.wt, o.wv, o.act, info, conn, kcap, coords,
                                    fout, ucap);
}

}  // namespace daxgb
