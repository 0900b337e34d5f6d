// Cell threshold on the in-range bit stream (bit = lo <= f <= hi).
//
// K2 (k_thr_rows): per point row r = (j, k)
//     K[r] = kept cells of cell row r (all 8 corner bits set,
//            ThresholdFunction, dax/worklet/Threshold.h:30-66)
//     U[r] = used points of point row r (a corner of some kept cell,
//            FillPointMask, dax/cont/DispatcherGenerateTopology.h:206-227)
//   writes the used-point mask (row-padded, one word per 32 points) and scans
//   (K, U) with the decoupled look-back.
// K3 (k_thr_emit): kept cells' connectivity = rank of each corner among the
//   used points (equal to the reference's Copy/Sort/Unique/LowerBounds of the
//   connectivity, :229-258, since used ids sorted ascending are exactly the
//   used points in point order), plus the compacted coordinates and field
//   (StreamCompact with the point mask, :237-239 and :98-113).
#include "common.cuh"
#include "kernels.cuh"

namespace daxgb {

// bits_at that also accepts pos == -1 (the cell left of the first point).
__device__ __forceinline__ uint32_t bits_at_signed(const uint32_t* bits, long long pos) {
  return pos >= 0 ? bits_at(bits, pos) : (bits_at(bits, 0) << 1);
}

// Kept mask of cells s..s+31 of cell row (j, k) (s may be -1); requires
// 0 <= j < ny-1 and 0 <= k < nz-1.
__device__ __forceinline__ uint32_t kept_word(const Grid& g, const uint32_t* bits, int j, int k,
                                              int s) {
  const long long dy = g.nx, dz = (long long)g.nx * g.ny;
  const long long pos = ((long long)k * g.ny + j) * g.nx + s;
  uint32_t w = bits_at_signed(bits, pos) & bits_at(bits, pos + 1) &
               bits_at_signed(bits, pos + dy) & bits_at(bits, pos + dy + 1) &
               bits_at_signed(bits, pos + dz) & bits_at(bits, pos + dz + 1) &
               bits_at_signed(bits, pos + dy + dz) & bits_at(bits, pos + dy + dz + 1);
  uint32_t valid = low_mask(g.nx - 1 - s);
  if (s < 0) valid &= ~1u;
  return w & valid;
}

// Used-point mask of point row (j, k), word m.
__device__ __forceinline__ uint32_t used_word(const Grid& g, const uint32_t* bits, int j, int k,
                                              int m) {
  uint32_t u = 0;
  const int s = 32 * m;
#pragma unroll
  for (int dk = -1; dk <= 0; ++dk) {
    const int kc = k + dk;
    if (kc < 0 || kc >= g.nz - 1) continue;
#pragma unroll
    for (int dj = -1; dj <= 0; ++dj) {
      const int jc = j + dj;
      if (jc < 0 || jc >= g.ny - 1) continue;
      u |= kept_word(g, bits, jc, kc, s) | kept_word(g, bits, jc, kc, s - 1);
    }
  }
  return u & low_mask(g.nx - s);
}

template <int G>
__global__ void __launch_bounds__(256) k_thr_rows(Grid g, const uint32_t* __restrict__ bits,
                                                  uint32_t* __restrict__ used,
                                                  long long* __restrict__ row_k,
                                                  long long* __restrict__ row_u,
                                                  unsigned long long* __restrict__ status,
                                                  Info* __restrict__ info, int tiles) {
  constexpr int RT = kRowsPerTile;
  constexpr int GPB = 256 / G;
  __shared__ int s_tile;
  __shared__ int s_k[RT], s_u[RT];
  __shared__ long long s_wk[8], s_wu[8];
  __shared__ long long s_ex[2];
  if (threadIdx.x == 0) s_tile = (int)atomicAdd(&info->ticket, 1u);
  __syncthreads();
  const int tile = s_tile;
  const long long r0 = (long long)tile * RT;
  const int gl = threadIdx.x & (G - 1);
  const int grp = threadIdx.x / G;
  for (int lr = grp; lr < RT; lr += GPB) {
    const long long r = r0 + lr;
    int kc = 0, uc = 0;
    if (r < g.R) {
      const int j = (int)(r % g.ny), k = (int)(r / g.ny);
      const bool cells = (j < g.ny - 1) && (k < g.nz - 1);
      for (int m = gl; m < g.wr; m += G) {
        if (cells) kc += __popc(kept_word(g, bits, j, k, 32 * m));
        const uint32_t u = used_word(g, bits, j, k, m);
        used[r * g.wr + m] = u;
        uc += __popc(u);
      }
    }
    kc = group_sum(kc, G);
    uc = group_sum(uc, G);
    if (gl == 0) {
      s_k[lr] = kc;
      s_u[lr] = uc;
    }
  }
  __syncthreads();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long long k0 = s_k[tid], u0 = s_u[tid];
  long long ki = k0, ui = u0;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long a = __shfl_up_sync(kFull, ki, o), b = __shfl_up_sync(kFull, ui, o);
    if (lane >= o) { ki += a; ui += b; }
  }
  if (lane == 31) { s_wk[warp] = ki; s_wu[warp] = ui; }
  __syncthreads();
  long long wk = 0, wu = 0, aggk = 0, aggu = 0;
#pragma unroll
  for (int w = 0; w < 8; ++w) {
    if (w < warp) { wk += s_wk[w]; wu += s_wu[w]; }
    aggk += s_wk[w];
    aggu += s_wu[w];
  }
  if (warp == 0) s_ex[0] = warp_lookback(status, tile, aggk, &info->error);
  if (warp == 1) s_ex[1] = warp_lookback(status + tiles, tile, aggu, &info->error);
  __syncthreads();
  const long long r = r0 + tid;
  if (r < g.R) {
    row_k[r] = s_ex[0] + wk + ki - k0;
    row_u[r] = s_ex[1] + wu + ui - u0;
  }
  if (tile == tiles - 1 && tid == 0) {
    row_k[g.R] = s_ex[0] + aggk;
    row_u[g.R] = s_ex[1] + aggu;
    info->total_a = s_ex[0] + aggk;
    info->total_b = s_ex[1] + aggu;
  }
}

void launch_thr_rows(const Grid& g, const uint32_t* bits, uint32_t* used, long long* row_k,
                     long long* row_u, unsigned long long* status, Info* info, int tiles,
                     cudaStream_t s) {
#define DAXGB_THR(G) k_thr_rows<G><<<tiles, 256, 0, s>>>(g, bits, used, row_k, row_u, status, info, tiles)
  switch (lanes_per_row(g.wr)) {
    case 1: DAXGB_THR(1); break;
    case 2: DAXGB_THR(2); break;
    case 4: DAXGB_THR(4); break;
    case 8: DAXGB_THR(8); break;
    case 16: DAXGB_THR(16); break;
    default: DAXGB_THR(32); break;
  }
#undef DAXGB_THR
}

template <int G>
__global__ void __launch_bounds__(256) k_thr_emit(Grid g, const float* __restrict__ f,
                                                  const uint32_t* __restrict__ bits,
                                                  const uint32_t* __restrict__ used,
                                                  const long long* __restrict__ row_k,
                                                  const long long* __restrict__ row_u,
                                                  Info* __restrict__ info,
                                                  int32_t* __restrict__ conn, long long kcap,
                                                  float* __restrict__ coords,
                                                  float* __restrict__ fout, long long ucap) {
  constexpr int GPB = 256 / G;
  extern __shared__ uint32_t s_rows[];  // [GPB][4 rows][mask, prefix][wr]
  if (info->total_a > kcap || info->total_b > ucap) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&info->error, kErrCapacity);
    return;
  }
  const int gl = threadIdx.x & (G - 1);
  const int grp = threadIdx.x / G;
  const int wr = g.wr;
  const unsigned gm = group_mask(G);
  const bool conn_al16 = (reinterpret_cast<uintptr_t>(conn) & 15) == 0;
  uint32_t* sm = s_rows + (size_t)grp * 8 * wr;
  const long long ngroups = (long long)gridDim.x * GPB;
  for (long long r = (long long)blockIdx.x * GPB + grp; r < g.R; r += ngroups) {
    const long long kb = row_k[r], ke = row_k[r + 1];
    const long long ub = row_u[r], ue = row_u[r + 1];
    if (kb == ke && ub == ue) continue;
    const int j = (int)(r % g.ny), k = (int)(r / g.ny);
    const int nq = ke > kb ? 4 : 1;
    long long qbase[4] = {ub, 0, 0, 0};
    for (int qi = 0; qi < nq; ++qi) {
      const long long rq = (long long)(k + (qi >> 1)) * g.ny + (j + (qi & 1));
      if (qi) qbase[qi] = row_u[rq];
      int carry = 0;
      for (int m0 = 0; m0 < wr; m0 += G) {
        const int m = m0 + gl;
        const uint32_t u = m < wr ? used[rq * wr + m] : 0u;
        const int cnt = __popc(u);
        const int incl = group_inclusive_scan(cnt, G);
        if (m < wr) {
          sm[qi * 2 * wr + m] = u;
          sm[qi * 2 * wr + wr + m] = (uint32_t)(carry + incl - cnt);
        }
        carry += group_last(incl, G);
      }
    }
    __syncwarp(gm);
    // compacted coordinates and field of the used points of row r
    if (ue > ub) {
      const float y = coord(g.oy, g.sy, j, g.my), z = coord(g.oz, g.sz, k, g.mz);
      for (int m = gl; m < wr; m += G) {
        long long id = ub + sm[wr + m];
        for (uint32_t u = sm[m]; u; u &= u - 1) {
          const int i = 32 * m + __ffs(u) - 1;
          coords[3 * id + 0] = coord(g.ox, g.sx, i, g.mx);
          coords[3 * id + 1] = y;
          coords[3 * id + 2] = z;
          if (fout) fout[id] = __ldg(f + r * g.nx + i);
          ++id;
        }
      }
    }
    // kept cells of cell row r, 8 compacted point ids each (hex order)
    if (ke > kb) {
      long long carry = 0;
      for (int m0 = 0; m0 < wr; m0 += G) {
        const int m = m0 + gl;
        const uint32_t km = m < wr ? kept_word(g, bits, j, k, 32 * m) : 0u;
        const int cnt = __popc(km);
        const int incl = group_inclusive_scan(cnt, G);
        long long cid = kb + carry + incl - cnt;
        for (uint32_t u = km; u; u &= u - 1, ++cid) {
          const int i = 32 * m + __ffs(u) - 1;
          int32_t ids[8];
#pragma unroll
          for (int v = 0; v < 8; ++v) {
            // v0..v7: (i,j,k) (i+1,j,k) (i+1,j+1,k) (i,j+1,k), then k+1
            const int di = ((v & 3) == 1 || (v & 3) == 2) ? 1 : 0;
            const int dj = ((v & 3) >= 2) ? 1 : 0;
            const int dk = v >> 2;
            const int qi = dj + 2 * dk;
            const int ii = i + di;
            const uint32_t* qs = sm + qi * 2 * wr;
            const int wq = ii >> 5, bq = ii & 31;
            ids[v] = (int32_t)(qbase[qi] + qs[wr + wq] + __popc(qs[wq] & ((1u << bq) - 1u)));
          }
          if (conn_al16) {
            int4* dst = reinterpret_cast<int4*>(conn + 8 * cid);
            dst[0] = make_int4(ids[0], ids[1], ids[2], ids[3]);
            dst[1] = make_int4(ids[4], ids[5], ids[6], ids[7]);
          } else {
#pragma unroll
            for (int v = 0; v < 8; ++v) conn[8 * cid + v] = ids[v];
          }
        }
        carry += group_last(incl, G);
      }
    }
    __syncwarp(gm);
  }
}

template <int G>
static void launch_thr_emit_g(const Grid& g, const float* f, const uint32_t* bits,
                              const uint32_t* used, const long long* row_k,
                              const long long* row_u, Info* info, int32_t* conn, long long kcap,
                              float* coords, float* fout, long long ucap, int num_sms,
                              cudaStream_t s) {
  constexpr int GPB = 256 / G;
  const size_t smem = (size_t)GPB * 8 * g.wr * sizeof(uint32_t);
  const long long want = (g.R + GPB - 1) / GPB;
  const long long cap = (long long)num_sms * 8;
  const int blocks = (int)(want < 1 ? 1 : (want < cap ? want : cap));
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(k_thr_emit<G>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_thr_emit<G><<<blocks, 256, smem, s>>>(g, f, bits, used, row_k, row_u, info, conn, kcap, coords,
                                          fout, ucap);
}

void launch_thr_emit(const Grid& g, const float* f, const uint32_t* bits, const uint32_t* used,
                     const long long* row_k, const long long* row_u, Info* info, int32_t* conn,
                     long long kcap, float* coords, float* fout, long long ucap, int num_sms,
                     cudaStream_t s) {
#define DAXGB_THR(G) \
  launch_thr_emit_g<G>(g, f, bits, used, row_k, row_u, info, conn, kcap, coords, fout, ucap, num_sms, s)
  switch (lanes_per_row(g.wr)) {
    case 1: DAXGB_THR(1); break;
    case 2: DAXGB_THR(2); break;
    case 4: DAXGB_THR(4); break;
    case 8: DAXGB_THR(8); break;
    case 16: DAXGB_THR(16); break;
    default: DAXGB_THR(32); break;
  }
#undef DAXGB_THR
}

}  // namespace daxgb
