// Shared device-side building blocks for the uniform-grid kernels.
//
// Data layout in HBM (one grid of nx*ny*nz points, x fastest):
//   field  : float32[P]                 caller-owned, read once by K1
//   bits   : uint32[bit_words(P)]       1 bit per point, flat point order
//   row words: W = R * wr (R = ny*nz point rows, wr = ceil(nx/32)); word
//            (r, m) covers points 32m..32m+31 of point row r and the cells
//            with those first points; per-word counts, exclusive offsets and
//            masks are uint32[W] arrays in that order
// "Row" always means a row of POINTS (fixed j, k); the cells whose first point
// lies in point row r form cell row r (valid when j < ny-1 and k < nz-1).
// Cell id order (dax/Extent.h:128-137) equals row-word order restricted to
// the valid rows, so per-word offsets give the reference's output order.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace daxgb {

constexpr unsigned kFull = 0xffffffffu;

// Host-prepared, device-consumed description of one uniform grid.
struct Grid {
  int nx, ny, nz;         // point dimensions
  int wr;                 // 32-bit words per point row: ceil(nx / 32)
  float ox, oy, oz;       // origin
  float sx, sy, sz;       // spacing
  int mx, my, mz;         // extent minimum (added to ijk for coordinates)
  long long P;            // points
  long long R;            // point rows = ny * nz
  unsigned long long mwr, mny;  // division multipliers for wr and ny (div_by)
};

// n / d for 32-bit n and a divisor fixed per grid, from the multiplier
// M = floor((2^64 - 1) / d) + 1 (0 for d = 1): q = high 64 bits of n * M.
// Exact for every 32-bit n and 2 <= d < 2^32: n/d <= n*M/2^64 < n/d + 2^-32
// and 2^-32 <= 1/d (T. Granlund, P. Montgomery, "Division by Invariant
// Integers using Multiplication", PLDI 1994).
__host__ __device__ inline unsigned long long div_multiplier(unsigned d) {
  return d >= 2 ? ~0ull / d + 1ull : 0ull;
}
__device__ __forceinline__ unsigned div_by(unsigned n, unsigned long long M) {
  return M ? (unsigned)__umul64hi((unsigned long long)n, M) : n;
}
// Row r and word m of a grid's row word lw (lw < R * wr < 2^32).
__device__ __forceinline__ unsigned split_word(const Grid& g, unsigned lw, int& m) {
  const unsigned r = div_by(lw, g.mwr);
  m = (int)(lw - r * (unsigned)g.wr);
  return r;
}
// (j, k) of point row r.
__device__ __forceinline__ void split_row(const Grid& g, unsigned r, int& j, int& k) {
  const unsigned kk = div_by(r, g.mny);
  k = (int)kk;
  j = (int)(r - kk * (unsigned)g.ny);
}

// One grid of a batch (device-resident table entry, or passed by value).
struct GridSlot {
  Grid g;
  const float* field;     // the grid's point field
  float iso;              // its isovalue (MC) / lower bound (threshold)
  float iso_hi;           // upper bound (threshold)
  long long chunk0;       // first global 128-point chunk (classification pass)
  long long word0;        // first bit word of the grid's bits (= 4 * chunk0)
  long long row0;         // first global point row
  long long rw0;          // first global row word (row-padded word arrays)
  float3 plane_o;         // field == NULL: the implicit slice field
  float3 plane_n;         //   dot(plane_n, coord - plane_o)
  long long cell0;        // first cell / point of the grid in per-cell and
  long long point0;       //   per-point arrays concatenated over a grid set
};

// A set of grids processed by one launch per pass.  count == 1: the grid is
// `one` (no table lookups); count > 1: `slots` is a device table sorted by
// chunk0 / row0 and rows / chunks are resolved by binary search.
struct GridSet {
  const GridSlot* slots;
  int count;
  long long rows;         // total point rows
  long long chunks;       // total 128-point chunks
  long long rowwords;     // total row words: sum of R * wr
  GridSlot one;
};

__device__ __forceinline__ int slot_of_row(const GridSet& S, long long grow) {
  int lo = 0, hi = S.count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(&S.slots[mid].row0) <= grow) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ int slot_of_chunk(const GridSet& S, long long chunk) {
  int lo = 0, hi = S.count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(&S.slots[mid].chunk0) <= chunk) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ int slot_of_rowword(const GridSet& S, long long rw) {
  int lo = 0, hi = S.count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(&S.slots[mid].rw0) <= rw) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Slot search keys (each slot's first chunk or first row word) staged in a
// block's shared memory: a grid-set kernel looks up a slot per chunk or per
// word, and a search through the slot table in global memory is a chain of
// dependent loads that the field stream evicts from L1.
constexpr int kStagedSlots = 512;

// Stages key(slot) for every slot when the set has at most kStagedSlots
// (call from every thread of the block; ends with a block barrier).
// Returns whether the keys were staged.
template <typename Key>
__device__ __forceinline__ bool stage_slot_keys(const GridSet& S, long long* keys, Key key) {
  const bool staged = S.count > 1 && S.count <= kStagedSlots;
  if (staged)
    for (int i = threadIdx.x; i < S.count; i += blockDim.x) keys[i] = key(S.slots[i]);
  __syncthreads();
  return staged;
}

// The last slot whose key is <= x.
__device__ __forceinline__ int slot_search(const long long* keys, int count, long long x) {
  int lo = 0, hi = count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (keys[mid] <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// The slot of x for x at or after slot `from`'s start: steps forward over
// the slots that start at or before x (keys staged by stage_slot_keys, or
// null: the slots' first row words, rw0, from global memory).  A warp whose
// items lie in few slots searches once and steps.
__device__ __forceinline__ int slot_after(const GridSet& S, const long long* keys, int from,
                                          long long x) {
  int si = from;
  while (si + 1 < S.count && (keys ? keys[si + 1] : __ldg(&S.slots[si + 1].rw0)) <= x) ++si;
  return si;
}

// The slot whose first block (block0[slot], ascending) is the last at or
// before block b: the grid a block of a grid-set launch works for.
__device__ __forceinline__ int block_slot(const long long* block0, int count, long long b) {
  int lo = 0, hi = count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(block0 + mid) <= b) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ GridSlot load_slot(const GridSet& S, int i) {
  return S.count == 1 ? S.one : S.slots[i];
}

// Device info block at the head of every scratch buffer.
struct Info {
  long long total_a;      // triangles (MC) / kept cells (threshold)
  long long total_b;      // merged vertices (MC) / used points (threshold)
  long long total_c;      // active row words
  int error;              // kErr* bits raised on the device
  unsigned ticket;        // next batch of active words for the MC emit warps
  unsigned done;          // MC emit blocks finished (the last resets both)
  int aborted;            // a count kernel's bounded wait ran out (the scan
                          //   reports it as kErrTimeout); cleared with error
  int pad[6];
};

constexpr int kErrCapacity = 2;    // output buffer too small
constexpr int kErrOverflow = 4;    // more than 2^31 - 1 triangles or vertices
constexpr int kErrBadIndex = 8;    // a cell lists a point id outside [0, P)
constexpr int kErrState = 16;      // a merge scratch that no merge pass of this count wrote
constexpr int kErrBadCount = 32;   // a count array asks a cell for a triangle its case lacks
constexpr int kErrTimeout = 64;    // a bounded device-side wait ran out (the fused count pass)

// Coordinate of grid index i along one axis: origin + spacing * (i + min),
// computed in float with no fused multiply-add, as the reference's implicit
// coordinate portal does (dax/cont/UniformGrid.h:82-89).
__device__ __forceinline__ float coord(float o, float s, int i, int m) {
  return __fadd_rn(o, __fmul_rn(s, (float)(i + m)));
}

// Division by a divisor d used many times, from its correctly rounded
// reciprocal r = recip_or_zero(d): q = RN(x r), e = x - q d (exact with one
// fused multiply-add), result RN(q + e r).  With r within half an ulp of 1/d
// and q within one ulp of x/d this is the correctly rounded x / d (P.
// Markstein, "Computation of elementary functions on the IBM RISC System/6000
// processor", IBM J. Res. Develop. 34(1), 1990; J.-M. Muller et al.,
// Handbook of Floating-Point Arithmetic, 2010, Markstein's theorem), provided
// no intermediate leaves the normal range: outside 2^-90 < |x|, |q| < 2^90
// (and for r = 0, a divisor outside that band) it falls back to __fdiv_rn;
// x = 0 gives the signed zero x r directly.
__device__ __forceinline__ float recip_or_zero(float d) {
  const float a = fabsf(d);
  return (a > 0x1p-90f && a < 0x1p90f) ? __frcp_rn(d) : 0.0f;
}
__device__ __forceinline__ float div_by_recip(float x, float d, float r) {
  const float q = __fmul_rn(x, r);
  const float ax = fabsf(x), aq = fabsf(q);
  if (ax > 0x1p-90f && ax < 0x1p90f && aq > 0x1p-90f && aq < 0x1p90f)
    return __fmaf_rn(__fmaf_rn(-q, d, x), r, q);
  if (x == 0.0f && r != 0.0f) return q;
  return __fdiv_rn(x, d);
}

__device__ __forceinline__ unsigned mag_bits(float v) { return __float_as_uint(v) & 0x7fffffffu; }

// Divisor band of div_fast: 2^-30 <= |w| < 2^30 (magnitude bit patterns).
constexpr unsigned kFastWidthLo = 0x30800000u;
constexpr unsigned kFastWidthHi = 0x4e800000u;
__device__ __forceinline__ bool width_in_band(float w) {
  return mag_bits(w) - kFastWidthLo < kFastWidthHi - kFastWidthLo;
}

// x / w for x = 0 or 2^-85 <= |x| < 2^87 and 2^-30 <= |w| < 2^30 with
// r = RN(1/w): div_by_recip's correction step without its range checks
// (every intermediate is normal on that domain).  The sign comes from
// q = RN(x r), which is the correctly signed zero when x is +-0 (where the
// correction step alone would give +0 for x = -0).
__device__ __forceinline__ float div_fast(float x, float w, float r) {
  const float q = __fmul_rn(x, r);
  const float y = __fmaf_rn(__fmaf_rn(-q, w, x), r, q);
  return __uint_as_float(mag_bits(y) | (__float_as_uint(q) & 0x80000000u));
}

// dax::math::Lerp(a, b, w) = a + w * (b - a), dax/math/VectorAnalysis.h:35-50.
__device__ __forceinline__ float lerp_rn(float a, float b, float w) {
  return __fadd_rn(a, __fmul_rn(w, __fsub_rn(b, a)));
}

// The slice field at point (i, j, k): dot(N, coord - O) with dax::dot's
// component order, a0*b0 + a1*b1 + a2*b2, every step rounded on its own
// (dax/worklet/Slice.h:64-73, :131-138; dax/Types.h:611-621).
__device__ __forceinline__ float plane_value(const Grid& g, const float3& o, const float3& n, int i,
                                             int j, int k) {
  const float dx = __fsub_rn(coord(g.ox, g.sx, i, g.mx), o.x);
  const float dy = __fsub_rn(coord(g.oy, g.sy, j, g.my), o.y);
  const float dz = __fsub_rn(coord(g.oz, g.sz, k, g.mz), o.z);
  return __fadd_rn(__fadd_rn(__fmul_rn(n.x, dx), __fmul_rn(n.y, dy)), __fmul_rn(n.z, dz));
}

// Point value of slot sl at flat point p = (i, j, k): the stored field, or
// the implicit slice field when the slot has none.
__device__ __forceinline__ float slot_value(const GridSlot& sl, long long p, int i, int j, int k) {
  return sl.field ? __ldg(sl.field + p) : plane_value(sl.g, sl.plane_o, sl.plane_n, i, j, k);
}

// Bit-stream loads.  CG = false: the read-only path (the stream was written
// by an earlier launch); CG = true: L2 only, for a stream that other blocks
// of the same launch wrote (the fused classify + count kernel), which the
// non-coherent path and L1 could serve stale.
template <bool CG>
__device__ __forceinline__ uint32_t ld_bits(const uint32_t* p) {
  return CG ? __ldcg(p) : __ldg(p);
}

// 32 consecutive bits of the flat bit stream starting at bit `pos` (any
// alignment).  The stream is padded so pos+63 is always readable.
template <bool CG = false>
__device__ __forceinline__ uint32_t bits_at(const uint32_t* __restrict__ bits, long long pos) {
  const long long w = pos >> 5;
  const uint32_t lo = ld_bits<CG>(bits + w);
  const uint32_t hi = ld_bits<CG>(bits + w + 1);
  return __funnelshift_r(lo, hi, (unsigned)(pos & 31));
}

// bits_at(pos) and bits_at(pos + 1) (the +x neighbours) from the same two
// words: the second is the first shifted down one bit with bit pos+32 on top.
template <bool CG = false>
__device__ __forceinline__ void bits_at2(const uint32_t* __restrict__ bits, long long pos,
                                         uint32_t& a, uint32_t& a1) {
  const long long w = pos >> 5;
  const unsigned sh = (unsigned)(pos & 31);
  const uint32_t w0 = ld_bits<CG>(bits + w), w1 = ld_bits<CG>(bits + w + 1);
  a = __funnelshift_r(w0, w1, sh);
  a1 = __funnelshift_rc(w0, w1, sh + 1u);  // sh = 31: w1 whole
}

// Four consecutive 32-bit windows of a row (x = 32m .. 32m+127) and their +x
// neighbours, from five word fetches.
template <bool CG = false>
__device__ __forceinline__ void row_windows4(const uint32_t* __restrict__ bits, long long pos,
                                             uint32_t (&a)[4], uint32_t (&a1)[4]) {
  const long long w = pos >> 5;
  const unsigned sh = (unsigned)(pos & 31);
  uint32_t x[5];
#pragma unroll
  for (int e = 0; e < 5; ++e) x[e] = ld_bits<CG>(bits + w + e);
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    a[e] = __funnelshift_r(x[e], x[e + 1], sh);
    a1[e] = __funnelshift_rc(x[e], x[e + 1], sh + 1u);  // sh = 31: the next word whole
  }
}

// Mask of the low n bits (n in [0, 32]).
// Programmatic dependent launch: a kernel launched with programmatic stream
// serialization (launch_pdl) may start while the kernel before it on the
// stream drains.  pdl_wait() blocks until that kernel has completed and its
// writes are visible (a no-op after an ordinary launch); pdl_trigger() lets
// the next kernel launch once every block of this one has issued it or
// exited.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

__device__ __forceinline__ uint32_t low_mask(int n) {
  return n >= 32 ? kFull : (n <= 0 ? 0u : ((1u << n) - 1u));
}

// Block-wide sums of three per-thread values (256 threads); all threads get
// the totals.  s holds 3 x 8 scratch words.
__device__ __forceinline__ void block_sum3(uint32_t& a, uint32_t& b, uint32_t& c, uint32_t* s) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(kFull, a, o);
    b += __shfl_xor_sync(kFull, b, o);
    c += __shfl_xor_sync(kFull, c, o);
  }
  if (lane == 0) {
    s[warp] = a;
    s[8 + warp] = b;
    s[16 + warp] = c;
  }
  __syncthreads();
  a = b = c = 0;
#pragma unroll
  for (int w = 0; w < 8; ++w) {
    a += s[w];
    b += s[8 + w];
    c += s[16 + w];
  }
  __syncthreads();
}

}  // namespace daxgb
