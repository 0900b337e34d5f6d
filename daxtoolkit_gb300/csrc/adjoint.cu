// Adjoints of the isosurface vertices and of CellGradient with respect to the
// point field, as one deterministic gather per point (no atomics).
//
// Isosurface (merged): vertex v on edge (A, B) along `axis` is
//     x_v = c_A + w (c_B - c_A),   w = (iso - f_A) / (f_B - f_A)
// (dax/worklet/MarchingCubes.h:160-161, dax/math/VectorAnalysis.h:35-50).
// Only the axis component of c_B - c_A is non-zero (h = its float value), so
//     dL/df_A += g (iso - f_B) / d^2,   dL/df_B -= g (iso - f_A) / d^2,
// with g = dL/dx_v[axis] * h and d = f_B - f_A.  Point p gathers its <= 6
// incident crossing edges in a fixed order: forward x, y, z (p = A), then
// backward x, y, z (p = B); each edge's vertex id is its owner word's offset
// plus its rank in that word, exactly as the forward pass numbered it.
//
// CellGradient: g_c[a] = sum_v f_v dW_v[a] / width_c[a] with dW = +-0.25
// (dax/exec/Derivative.h:37-58), so
//     dL/df_p += sum over the <= 8 cells c containing p, a in {x,y,z}:
//                s_a * 0.25 * dL/dg_c[a] / width_c[a]
// where s_a = +1 when p is on the cell's upper face along a, else -1; the
// cells are visited in a fixed (k, j, i) order.
//
// Both contributions are summed into one write of dL/df per point (4 B/point
// of HBM write, the dominant traffic; the bit stream and the per-row offsets
// are L2-resident).
#include "common.cuh"
#include "kernels.cuh"

namespace daxgb {

namespace {

__device__ __forceinline__ void row_masks(const Grid& g, const uint32_t* bits, int j, int k, int m,
                                          uint32_t& X, uint32_t& Y, uint32_t& Z) {
  const long long pos = ((long long)k * g.ny + j) * g.nx + 32ll * m;
  const int i0 = 32 * m;
  const uint32_t a = bits_at(bits, pos);
  X = (a ^ bits_at(bits, pos + 1)) & low_mask(g.nx - 1 - i0);
  Y = (j < g.ny - 1) ? ((a ^ bits_at(bits, pos + g.nx)) & low_mask(g.nx - i0)) : 0u;
  Z = (k < g.nz - 1) ? ((a ^ bits_at(bits, pos + (long long)g.nx * g.ny)) & low_mask(g.nx - i0))
                     : 0u;
}

// vertex id of edge (i, axis) of an owner row staged as [X, Y, Z, word offset][wr]
__device__ __forceinline__ long long edge_rank(const uint32_t* qs, int wr, int i, int axis) {
  const int w = i >> 5, b = i & 31;
  const uint32_t lm = (1u << b) - 1u;
  const uint32_t X = qs[w], Y = qs[wr + w], Z = qs[2 * wr + w];
  long long r = (long long)qs[3 * wr + w] + __popc(X & lm) + __popc(Y & lm) + __popc(Z & lm);
  if (axis >= 1) r += (X >> b) & 1u;
  if (axis >= 2) r += (Y >> b) & 1u;
  return r;
}

__device__ __forceinline__ float axis_step(const Grid& g, int axis, int idx) {
  if (axis == 0) return coord(g.ox, g.sx, idx + 1, g.mx) - coord(g.ox, g.sx, idx, g.mx);
  if (axis == 1) return coord(g.oy, g.sy, idx + 1, g.my) - coord(g.oy, g.sy, idx, g.my);
  return coord(g.oz, g.sz, idx + 1, g.mz) - coord(g.oz, g.sz, idx, g.mz);
}

// contribution of edge (pa -> pb) with vertex vid to dL/df at one end point
__device__ __forceinline__ float edge_term(const Grid& g, const float* f, float iso,
                                           const float* dverts, long long vid, int axis,
                                           long long pa, long long pb, int idx_a, bool at_a) {
  const float fa = __ldg(f + pa), fb = __ldg(f + pb);
  const float d = fb - fa;
  const float gv = __ldg(dverts + 3 * vid + axis) * axis_step(g, axis, idx_a);
  const float num = at_a ? (iso - fb) : -(iso - fa);
  return gv * num / (d * d);
}

}  // namespace

template <int G>
__global__ void __launch_bounds__(256) k_field_adjoint(Grid g, const float* __restrict__ f,
                                                       float iso,
                                                       const uint32_t* __restrict__ bits,
                                                       const uint32_t* __restrict__ wv,
                                                       const float* __restrict__ dverts,
                                                       const float* __restrict__ dgrad,
                                                       float* __restrict__ out) {
  constexpr int GPB = 256 / G;
  extern __shared__ uint32_t s_rows[];  // [GPB][3 rows][X, Y, Z, word vertex offset][wr]
  const int gl = threadIdx.x & (G - 1);
  const int grp = threadIdx.x / G;
  const int wr = g.wr;
  uint32_t* sm = s_rows + (size_t)grp * 12 * wr;
  const long long dy = g.nx, dz = (long long)g.nx * g.ny;
  const int cx = g.nx - 1, cy = g.ny - 1;
  const long long ngroups = (long long)gridDim.x * GPB;
  for (long long r = (long long)blockIdx.x * GPB + grp; r < g.R; r += ngroups) {
    const int j = (int)(r % g.ny), k = (int)(r / g.ny);
    const long long qbase[3] = {0, 0, 0};
    if (dverts) {
      // owner rows: 0 = (j, k), 1 = (j-1, k), 2 = (j, k-1); per word the
      // crossing masks and the word's global vertex offset
      for (int qi = 0; qi < 3; ++qi) {
        const int jq = j - (qi == 1), kq = k - (qi == 2);
        if (jq < 0 || kq < 0) continue;  // uniform within the group
        const long long rq = (long long)kq * g.ny + jq;
        for (int m = gl; m < wr; m += G) {
          uint32_t X, Y, Z;
          row_masks(g, bits, jq, kq, m, X, Y, Z);
          uint32_t* q = sm + qi * 4 * wr;
          q[m] = X;
          q[wr + m] = Y;
          q[2 * wr + m] = Z;
          q[3 * wr + m] = __ldg(wv + rq * wr + m);
        }
      }
      __syncwarp(group_mask(G));
    }
    const long long prow = r * g.nx;
    for (int i = gl; i < g.nx; i += G) {
      const long long p = prow + i;
      float acc = 0.0f;
      if (dverts) {
        const uint32_t* q0 = sm;
        const int w = i >> 5, b = i & 31;
        const uint32_t X = q0[w], Y = q0[wr + w], Z = q0[2 * wr + w];
        if ((X >> b) & 1u)
          acc += edge_term(g, f, iso, dverts, qbase[0] + edge_rank(q0, wr, i, 0), 0, p, p + 1, i, true);
        if ((Y >> b) & 1u)
          acc += edge_term(g, f, iso, dverts, qbase[0] + edge_rank(q0, wr, i, 1), 1, p, p + dy, j, true);
        if ((Z >> b) & 1u)
          acc += edge_term(g, f, iso, dverts, qbase[0] + edge_rank(q0, wr, i, 2), 2, p, p + dz, k, true);
        if (i > 0 && ((q0[(i - 1) >> 5] >> ((i - 1) & 31)) & 1u))
          acc += edge_term(g, f, iso, dverts, qbase[0] + edge_rank(q0, wr, i - 1, 0), 0, p - 1, p,
                           i - 1, false);
        if (j > 0) {
          const uint32_t* q1 = sm + 4 * wr;
          if ((q1[wr + w] >> b) & 1u)
            acc += edge_term(g, f, iso, dverts, qbase[1] + edge_rank(q1, wr, i, 1), 1, p - dy, p,
                             j - 1, false);
        }
        if (k > 0) {
          const uint32_t* q2 = sm + 8 * wr;
          if ((q2[2 * wr + w] >> b) & 1u)
            acc += edge_term(g, f, iso, dverts, qbase[2] + edge_rank(q2, wr, i, 2), 2, p - dz, p,
                             k - 1, false);
        }
      }
      if (dgrad) {
#pragma unroll
        for (int dk = 1; dk >= 0; --dk) {
          const int kc = k - dk;
          if (kc < 0 || kc >= g.nz - 1) continue;
          const float wz = axis_step(g, 2, kc);
#pragma unroll
          for (int dj = 1; dj >= 0; --dj) {
            const int jc = j - dj;
            if (jc < 0 || jc >= g.ny - 1) continue;
            const float wy = axis_step(g, 1, jc);
#pragma unroll
            for (int di = 1; di >= 0; --di) {
              const int ic = i - di;
              if (ic < 0 || ic >= g.nx - 1) continue;
              const float wx = axis_step(g, 0, ic);
              const long long c = ic + (long long)cx * (jc + (long long)cy * kc);
              const float gx = __ldg(dgrad + 3 * c), gy = __ldg(dgrad + 3 * c + 1),
                          gz = __ldg(dgrad + 3 * c + 2);
              acc += (di ? 0.25f : -0.25f) * gx / wx + (dj ? 0.25f : -0.25f) * gy / wy +
                     (dk ? 0.25f : -0.25f) * gz / wz;
            }
          }
        }
      }
      out[p] = acc;
    }
    __syncwarp(group_mask(G));
  }
}

template <int G>
static void launch_adj_g(const Grid& g, const float* f, float iso, const uint32_t* bits,
                         const WordOffsets* o, const float* dverts, const float* dgrad,
                         float* out, int num_sms, cudaStream_t s) {
  constexpr int GPB = 256 / G;
  const size_t smem = dverts ? (size_t)GPB * 12 * g.wr * sizeof(uint32_t) : 0;
  const long long want = (g.R + GPB - 1) / GPB;
  const long long cap = (long long)num_sms * 8;
  const int blocks = (int)(want < 1 ? 1 : (want < cap ? want : cap));
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(k_field_adjoint<G>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_field_adjoint<G><<<blocks, 256, smem, s>>>(g, f, iso, bits, o ? o->wv : nullptr, dverts,
                                                dgrad, out);
}

void launch_field_adjoint(const Grid& g, const float* f, float iso, const uint32_t* bits,
                          const WordOffsets* o, const float* dverts, const float* dgrad,
                          float* out, int num_sms, cudaStream_t s) {
#define DAXGB_ADJ(G) launch_adj_g<G>(g, f, iso, bits, o, dverts, dgrad, out, num_sms, s)
  switch (lanes_per_row(g.wr)) {
    case 1: DAXGB_ADJ(1); break;
    case 2: DAXGB_ADJ(2); break;
    case 4: DAXGB_ADJ(4); break;
    case 8: DAXGB_ADJ(8); break;
    case 16: DAXGB_ADJ(16); break;
    default: DAXGB_ADJ(32); break;
  }
#undef DAXGB_ADJ
}

}  // namespace daxgb
