// Slice on a uniform grid (dax/worklet/Slice.h:28-168).
//
// SliceCount / SliceGenerate classify and interpolate every cell with
//     s = dot(normal, coords[v] - origin)    per cell vertex,
// against the isovalue dot(normal, origin), with the voxel edges listed lower
// point first (Slice.h:144-148) and marching cubes' TriTable, weight and
// merge.  s depends only on the point, so a slice is the marching-cubes
// pipeline on the implicit point field s(p) at that isovalue.  Nothing of s
// is stored: the classification bits come straight from the coordinates
// (P/8 bytes of traffic instead of the 4P-byte field read), the count and
// scan passes only read bits, and the emit pass evaluates s at the two end
// points of each crossing edge (slot_value).  k_slice_field writes s itself
// for callers that want the field.  dax::dot accumulates in
// component order, a0*b0 + a1*b1 + a2*b2 (dax/Types.h:611-621); every
// rounding is spelled out so the values equal the reference's float
// arithmetic bit for bit.
#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "kernels.cuh"

namespace daxgb {

// Per-point classification, for planes and grids whose values may overflow
// or be NaN.  Each warp walks a contiguous run of steps, one 32-bit word of
// the flat bit stream (bit p of word p / 32) per step; lane l holds point
// p = 32 * step + l with its (i, row) and the y and z terms of its row, and
// moves 32 points per step (the division happens once per warp, split_row
// once per row).  The x terms of the row, nx floats, sit in shared memory:
// consecutive lanes read consecutive entries.  Points p >= P classify as 0;
// each lane keeps one word of every 32 steps so the warp stores whole
// 128-byte lines.
__global__ void __launch_bounds__(256) k_slice_points(Grid g, float3 o, float3 n, float iso,
                                                      long long steps, long long per,
                                                      unsigned long long mnx,
                                                      uint32_t* __restrict__ bits) {
  extern __shared__ float s_tx[];  // [nx]: n.x * (x(i) - o.x)
  for (int i = threadIdx.x; i < g.nx; i += blockDim.x)
    s_tx[i] = __fmul_rn(n.x, __fsub_rn(coord(g.ox, g.sx, i, g.mx), o.x));
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long s0 = warp * per;
  if (s0 >= steps) return;
  const long long s1 = s0 + per < steps ? s0 + per : steps;
  unsigned p = (unsigned)(s0 * 32 + lane);
  unsigned row = div_by(p, mnx);
  int i = (int)(p - row * (unsigned)g.nx);
  int j, k;
  split_row(g, row, j, k);
  float ty = __fmul_rn(n.y, __fsub_rn(coord(g.oy, g.sy, j, g.my), o.y));
  float tz = __fmul_rn(n.z, __fsub_rn(coord(g.oz, g.sz, k, g.mz), o.z));
  uint32_t mine = 0;
  for (long long st = s0; st < s1; ++st) {
    const float v = __fadd_rn(__fadd_rn(s_tx[i], ty), tz);
    const uint32_t word = __ballot_sync(kFull, (long long)p < g.P && v > iso);
    const int q = (int)((st - s0) & 31);
    if (q == lane) mine = word;
    if (q == 31 || st + 1 == s1) {
      if (lane <= q) bits[st - q + lane] = mine;
    }
    p += 32;
    i += 32;
    if (i >= g.nx) {
      do {
        i -= g.nx;
        ++row;
      } while (i >= g.nx);
      split_row(g, row, j, k);
      ty = __fmul_rn(n.y, __fsub_rn(coord(g.oy, g.sy, j, g.my), o.y));
      tz = __fmul_rn(n.z, __fsub_rn(coord(g.oz, g.sz, k, g.mz), o.z));
    }
  }
}

// The field itself: warps take whole point rows (contiguous in memory), the
// lanes write consecutive points, four per lane in flight.
__global__ void __launch_bounds__(256) k_slice_field(Grid g, float3 o, float3 n,
                                                     float* __restrict__ out) {
  extern __shared__ float s_tx[];  // [nx]: n.x * (x(i) - o.x)
  for (int i = threadIdx.x; i < g.nx; i += blockDim.x)
    s_tx[i] = __fmul_rn(n.x, __fsub_rn(coord(g.ox, g.sx, i, g.mx), o.x));
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < g.R;
       r += nwarps) {
    int j, k;
    split_row(g, (unsigned)r, j, k);
    const float ty = __fmul_rn(n.y, __fsub_rn(coord(g.oy, g.sy, j, g.my), o.y));
    const float tz = __fmul_rn(n.z, __fsub_rn(coord(g.oz, g.sz, k, g.mz), o.z));
    float* __restrict__ row = out + r * g.nx;
    int i = lane;
    for (; i + 96 < g.nx; i += 128) {
      const float v0 = __fadd_rn(__fadd_rn(s_tx[i], ty), tz);
      const float v1 = __fadd_rn(__fadd_rn(s_tx[i + 32], ty), tz);
      const float v2 = __fadd_rn(__fadd_rn(s_tx[i + 64], ty), tz);
      const float v3 = __fadd_rn(__fadd_rn(s_tx[i + 96], ty), tz);
      __stcs(row + i, v0);
      __stcs(row + i + 32, v1);
      __stcs(row + i + 64, v2);
      __stcs(row + i + 96, v3);
    }
    for (; i < g.nx; i += 32) __stcs(row + i, __fadd_rn(__fadd_rn(s_tx[i], ty), tz));
  }
}

// ---- row-split classification -------------------------------------------
// Along a point row (j, k fixed) only the x term varies:
//   s(i) = (tx(i) + ty) + tz,  tx(i) = n.x * (x(i) - o.x),
//   x(i) = o_grid.x + spacing.x * float(i + min.x).
// Every step is a correctly rounded float operation, each monotone in its
// varying argument, so while no value is NaN or infinite s(i) is monotone in
// i (non-decreasing when n.x * spacing.x > 0, non-increasing when < 0,
// constant when 0), and the points with s > iso form a suffix, a prefix, or
// all or none of the row.  k_slice_rows finds, per row, the first i whose
// test differs from i = 0's by binary search (about log2(nx) evaluations of
// the very expression the per-point kernels evaluate); k_slice_words then
// writes each 32-bit word of the flat bit stream from the splits of the one
// or more rows it covers.  The host takes this path only when every
// intermediate value is provably finite (see slice_rows_exact); otherwise
// k_slice_points tests every point.

__device__ __forceinline__ bool slice_inside(const Grid& g, float3 o, float3 n, float iso, int i,
                                             float ty, float tz) {
  const float tx = __fmul_rn(n.x, __fsub_rn(coord(g.ox, g.sx, i, g.mx), o.x));
  return __fadd_rn(__fadd_rn(tx, ty), tz) > iso;
}

// split[r] = number of leading points of row r whose test equals point 0's;
// bit 31 holds point 0's test.
__global__ void __launch_bounds__(256) k_slice_rows(Grid g, float3 o, float3 n, float iso,
                                                    uint32_t* __restrict__ split) {
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < g.R;
       r += (long long)gridDim.x * blockDim.x) {
    int j, k;
    split_row(g, (unsigned)r, j, k);
    const float ty = __fmul_rn(n.y, __fsub_rn(coord(g.oy, g.sy, j, g.my), o.y));
    const float tz = __fmul_rn(n.z, __fsub_rn(coord(g.oz, g.sz, k, g.mz), o.z));
    const bool first = slice_inside(g, o, n, iso, 0, ty, tz);
    int lo = 1, hi = g.nx;  // the answer lies in [lo, hi]
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (slice_inside(g, o, n, iso, mid, ty, tz) != first) hi = mid; else lo = mid + 1;
    }
    split[r] = (uint32_t)lo | (first ? 0x80000000u : 0u);
  }
}

// Word w of the bit stream: points 32w .. 32w+31, across as many rows as
// they touch; points past P are 0.
__global__ void __launch_bounds__(256) k_slice_words(Grid g, unsigned long long mnx,
                                                     const uint32_t* __restrict__ split,
                                                     uint32_t* __restrict__ bits,
                                                     long long nwords) {
  for (long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x; w < nwords;
       w += (long long)gridDim.x * blockDim.x) {
    const long long p0 = w << 5;
    uint32_t word = 0;
    if (p0 < g.P) {
      unsigned row = div_by((unsigned)p0, mnx);
      int i = (int)((unsigned)p0 - row * (unsigned)g.nx);
      int pos = 0;
      while (pos < 32 && (long long)row < g.R) {
        const int len = min(g.nx - i, 32 - pos);  // points of this row in the word
        const uint32_t sp = __ldg(split + row);
        const int cut = (int)(sp & 0x7fffffffu);
        // inside range of the row: [0, cut) if point 0 is inside, else [cut, nx)
        const int a = (sp >> 31) ? 0 : cut, b = (sp >> 31) ? cut : g.nx;
        const int lo = max(a, i), hi = min(b, i + len);
        if (lo < hi) {
          const uint32_t m = (hi - lo == 32) ? 0xffffffffu : ((1u << (hi - lo)) - 1u);
          word |= m << (pos + lo - i);
        }
        pos += len;
        i = 0;
        ++row;
      }
    }
    bits[w] = word;
  }
}

namespace {

// Dynamic shared memory of the x-term table, opted in above 48 KB.
template <typename K>
size_t tx_smem(K kernel, const Grid& g) {
  const size_t smem = sizeof(float) * (size_t)g.nx;
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  return smem;
}

}  // namespace

float slice_isovalue(const float origin[3], const float normal[3]) {
  // each step through a volatile float, so no compiler fuses it into an FMA
  volatile float r = normal[0] * origin[0];
  volatile float t1 = normal[1] * origin[1];
  r = r + t1;
  volatile float t2 = normal[2] * origin[2];
  r = r + t2;
  return r;
}

// True when no value of the slice expression can be NaN or infinite on this
// grid, so each row's test is monotone in i (bounds taken in double, with a
// wide margin over float rounding).
bool slice_rows_exact(const Grid& g, float3 o, float3 n) {
  const double og[3] = {g.ox, g.oy, g.oz}, sp[3] = {g.sx, g.sy, g.sz};
  const double mn[3] = {(double)g.mx, (double)g.my, (double)g.mz};
  const double dim[3] = {(double)g.nx, (double)g.ny, (double)g.nz};
  const double po[3] = {o.x, o.y, o.z}, pn[3] = {n.x, n.y, n.z};
  double sum = 0.0;
  for (int a = 0; a < 3; ++a) {
    if (!std::isfinite(og[a]) || !std::isfinite(sp[a]) || !std::isfinite(po[a]) ||
        !std::isfinite(pn[a]))
      return false;
    const double idx = std::max(std::fabs(mn[a]), std::fabs(mn[a] + dim[a]));
    const double x = std::fabs(og[a]) + std::fabs(sp[a]) * idx;  // |coordinate| bound
    sum += std::fabs(pn[a]) * (x + std::fabs(po[a]));
  }
  return sum < 1e36;  // FLT_MAX is 3.4e38
}

void launch_slice_bits(const Grid& g, float3 o, float3 n, float iso, uint32_t* bits,
                       long long nwords, uint32_t* row_scratch, int num_sms, cudaStream_t s) {
  if (row_scratch && std::isfinite(iso) && slice_rows_exact(g, o, n)) {
    const int rb = resident_blocks(k_slice_rows, 256, 0, num_sms, (g.R + 255) / 256);
    k_slice_rows<<<rb, 256, 0, s>>>(g, o, n, iso, row_scratch);
    const int wb = resident_blocks(k_slice_words, 256, 0, num_sms, (nwords + 255) / 256);
    k_slice_words<<<wb, 256, 0, s>>>(g, div_multiplier((unsigned)g.nx), row_scratch, bits, nwords);
    return;
  }
  const size_t smem = tx_smem(k_slice_points, g);
  // at least 32 steps per warp (one whole line of bit words), 8 warps a block
  const int blocks =
      resident_blocks(k_slice_points, 256, smem, num_sms, (nwords + 8 * 32 - 1) / (8 * 32));
  const long long warps = (long long)blocks * 8;
  long long per = (nwords + warps - 1) / warps;
  per = (per + 31) / 32 * 32;
  k_slice_points<<<blocks, 256, smem, s>>>(g, o, n, iso, nwords, per,
                                           div_multiplier((unsigned)g.nx), bits);
}

void launch_slice_field(const Grid& g, float3 o, float3 n, float* out, int num_sms,
                        cudaStream_t s) {
  const size_t smem = tx_smem(k_slice_field, g);
  const int blocks = resident_blocks(k_slice_field, 256, smem, num_sms, (g.R + 7) / 8);
  k_slice_field<<<blocks, 256, smem, s>>>(g, o, n, out);
}

}  // namespace daxgb
