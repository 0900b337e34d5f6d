// Shared device-side building blocks for the uniform-grid kernels.
//
// Data layout in HBM (one grid of nx*ny*nz points, x fastest):
//   field  : float32[P]                       caller-owned, read once by K1
//   bits   : uint32[bit_words(P)]             1 bit per point, flat point order
//   row_a  : int64[R+1], row_b : int64[R+1]   exclusive per-row offsets (R = ny*nz)
//   status : uint64[2][tiles]                 decoupled look-back state
// "Row" always means a row of POINTS (fixed j, k); the cells whose first point
// lies in point row r form cell row r (valid when j < ny-1 and k < nz-1).
// Cell id order (dax/Extent.h:128-137) equals point-row order restricted to
// the valid rows, so per-row offsets give the reference's output order.
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
};

// One grid of a batch (device-resident table entry, or passed by value).
struct GridSlot {
  Grid g;
  const float* field;     // the grid's point field
  float iso;              // its isovalue (MC) / lower bound (threshold)
  float iso_hi;           // upper bound (threshold)
  long long chunk0;       // first global 128-point chunk (classification pass)
  long long word0;        // first bit word of the grid's bits (= 4 * chunk0)
  long long row0;         // first global point row
  long long blk0;         // first global row block (emit pass)
  long long rw0;          // first global row word (row-padded word arrays)
};

// A set of grids processed by one launch per pass.  count == 1: the grid is
// `one` (no table lookups); count > 1: `slots` is a device table sorted by
// chunk0 / row0 and rows / chunks are resolved by binary search.
struct GridSet {
  const GridSlot* slots;
  int count;
  long long rows;         // total point rows
  long long chunks;       // total 128-point chunks
  long long blocks;       // total row blocks (emit pass)
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

__device__ __forceinline__ int slot_of_block(const GridSet& S, long long blk) {
  int lo = 0, hi = S.count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(&S.slots[mid].blk0) <= blk) lo = mid; else hi = mid - 1;
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

__device__ __forceinline__ GridSlot load_slot(const GridSet& S, int i) {
  return S.count == 1 ? S.one : S.slots[i];
}

// Device info block at the head of every scratch buffer.
struct Info {
  long long total_a;      // triangles (MC) / kept cells (threshold)
  long long total_b;      // merged vertices (MC) / used points (threshold)
  long long total_c;      // active row words (MC)
  int error;              // kErr* bits raised on the device
  unsigned ticket;        // dynamic tile counter of the look-back scan
  int pad[8];
};

constexpr int kErrTimeout = 1;     // a look-back wait gave up
constexpr int kErrCapacity = 2;    // output buffer too small
constexpr int kErrOverflow = 4;    // more than 2^31 - 1 triangles or vertices

// Coordinate of grid index i along one axis: origin + spacing * (i + min),
// computed in float with no fused multiply-add, as the reference's implicit
// coordinate portal does (dax/cont/UniformGrid.h:82-89).
__device__ __forceinline__ float coord(float o, float s, int i, int m) {
  return __fadd_rn(o, __fmul_rn(s, (float)(i + m)));
}

// dax::math::Lerp(a, b, w) = a + w * (b - a), dax/math/VectorAnalysis.h:35-50.
__device__ __forceinline__ float lerp_rn(float a, float b, float w) {
  return __fadd_rn(a, __fmul_rn(w, __fsub_rn(b, a)));
}

// 32 consecutive bits of the flat bit stream starting at bit `pos` (any
// alignment).  The stream is padded so pos+63 is always readable.
__device__ __forceinline__ uint32_t bits_at(const uint32_t* __restrict__ bits, long long pos) {
  const long long w = pos >> 5;
  const uint32_t lo = __ldg(bits + w);
  const uint32_t hi = __ldg(bits + w + 1);
  return __funnelshift_r(lo, hi, (unsigned)(pos & 31));
}

// bits_at(pos) and bits_at(pos + 1) (the +x neighbours) from the same two
// words: the second is the first shifted down one bit with bit pos+32 on top.
__device__ __forceinline__ void bits_at2(const uint32_t* __restrict__ bits, long long pos,
                                         uint32_t& a, uint32_t& a1) {
  const long long w = pos >> 5;
  const unsigned sh = (unsigned)(pos & 31);
  const uint32_t w0 = __ldg(bits + w), w1 = __ldg(bits + w + 1);
  a = __funnelshift_r(w0, w1, sh);
  a1 = (a >> 1) | (((w1 >> sh) & 1u) << 31);
}

// Mask of the low n bits (n in [0, 32]).
__device__ __forceinline__ uint32_t low_mask(int n) {
  return n >= 32 ? kFull : (n <= 0 ? 0u : ((1u << n) - 1u));
}

// ---- decoupled look-back ------------------------------------------------
// Status word: bits 63..62 = flag (0 none, 1 aggregate, 2 inclusive prefix),
// bits 61..0 = value.
constexpr unsigned long long kFlagAgg = 1ull << 62;
constexpr unsigned long long kFlagInc = 2ull << 62;
constexpr unsigned long long kValMask = (1ull << 62) - 1;
constexpr int kSpinLimit = 1 << 22;   // ~0.3 s of 64 ns sleeps, then give up

__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Called by ONE full warp for tile `tile`: publishes the tile aggregate, walks
// back over predecessors (32 per step) until an inclusive prefix is found and
// returns the exclusive prefix.  Waits are bounded: on timeout the error bit
// is raised, the missing predecessors count as 0 and the tile still publishes
// so that no successor waits forever.
__device__ __forceinline__ long long warp_lookback(unsigned long long* status, int tile,
                                                  long long agg, int* err) {
  const int lane = threadIdx.x & 31;
  if (tile == 0) {
    if (lane == 0) st_release(status, kFlagInc | (unsigned long long)agg);
    return 0;
  }
  if (lane == 0) st_release(status + tile, kFlagAgg | (unsigned long long)agg);
  long long excl = 0;
  int p = tile - 1;
  int spins = 0;
  while (true) {
    const int idx = p - lane;
    const unsigned long long w = idx >= 0 ? ld_acquire(status + idx) : kFlagInc;
    const unsigned flag = (unsigned)(w >> 62);
    const unsigned inc = __ballot_sync(kFull, flag == 2u);
    const unsigned none = __ballot_sync(kFull, flag == 0u);
    const int first_inc = inc ? __ffs(inc) - 1 : 32;
    const unsigned need = first_inc >= 31 ? kFull : ((2u << first_inc) - 1u);
    if (none & need) {
      if (++spins > kSpinLimit) {
        if (lane == 0) atomicOr(err, kErrTimeout);
        break;
      }
      __nanosleep(64);
      continue;
    }
    long long v = (lane <= first_inc && idx >= 0) ? (long long)(w & kValMask) : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    excl += v;
    if (first_inc < 32) break;
    p -= 32;
  }
  if (lane == 0) st_release(status + tile, kFlagInc | (unsigned long long)(excl + agg));
  return excl;
}

// Called by ALL threads of a 256-thread block for tile `tile`: publishes the
// N aggregates, then walks back 256 predecessors per step (one status word
// per thread and chain) until each chain meets an inclusive prefix.  Bounded
// like warp_lookback.  ex[c] receives chain c's exclusive prefix.
template <int N>
__device__ __forceinline__ void block_lookback(unsigned long long* st, long long stride, int tile,
                                               const long long (&agg)[N], int* err,
                                               long long (&ex)[N]) {
  __shared__ int s_first[N][8];
  __shared__ long long s_sum[N][8];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    const unsigned long long f = tile == 0 ? kFlagInc : kFlagAgg;
#pragma unroll
    for (int c = 0; c < N; ++c) st_release(st + c * stride + tile, f | (unsigned long long)agg[c]);
  }
#pragma unroll
  for (int c = 0; c < N; ++c) ex[c] = 0;
  if (tile == 0) return;
  bool done[N];
#pragma unroll
  for (int c = 0; c < N; ++c) done[c] = false;
  int p = tile - 1, spins = 0;
  while (true) {
    bool all = true;
#pragma unroll
    for (int c = 0; c < N; ++c) all = all && done[c];
    if (all) break;
    const int idx = p - tid;
    unsigned long long wv[N];
    bool miss = false;
    int first[N];
#pragma unroll
    for (int c = 0; c < N; ++c) {
      wv[c] = (!done[c] && idx >= 0) ? ld_acquire(st + c * stride + idx) : kFlagInc;
      const unsigned b = __ballot_sync(kFull, (wv[c] >> 62) == 2u);
      if (lane == 0) s_first[c][warp] = b ? warp * 32 + __ffs(b) - 1 : 256;
    }
    __syncthreads();
#pragma unroll
    for (int c = 0; c < N; ++c) {
      first[c] = 256;
#pragma unroll
      for (int w = 0; w < 8; ++w) first[c] = min(first[c], s_first[c][w]);
      miss = miss || ((wv[c] >> 62) == 0u && tid <= first[c]);
    }
    if (__syncthreads_or(miss)) {
      if (++spins > kSpinLimit) {
        if (tid == 0) atomicOr(err, kErrTimeout);
        break;
      }
      __nanosleep(64);
      continue;
    }
#pragma unroll
    for (int c = 0; c < N; ++c) {
      long long v = (tid <= first[c] && idx >= 0) ? (long long)(wv[c] & kValMask) : 0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
      if (lane == 0) s_sum[c][warp] = v;
    }
    __syncthreads();
#pragma unroll
    for (int c = 0; c < N; ++c) {
      long long t = 0;
#pragma unroll
      for (int w = 0; w < 8; ++w) t += s_sum[c][w];
      if (!done[c]) ex[c] += t;
      done[c] = done[c] || first[c] < 256;
    }
    p -= 256;
    __syncthreads();  // s_first / s_sum reused by the next step
  }
  if (tid == 0) {
#pragma unroll
    for (int c = 0; c < N; ++c)
      st_release(st + c * stride + tile, kFlagInc | (unsigned long long)(ex[c] + agg[c]));
  }
}

// Exclusive scan of N per-thread values over a 256-thread block; returns the
// block totals in tot.  All threads must call.
template <int N>
__device__ __forceinline__ void block_exclusive_scan(const long long (&v)[N], long long (&ex)[N],
                                                     long long (&tot)[N]) {
  __shared__ long long s_w[N][8];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  long long inc[N];
#pragma unroll
  for (int c = 0; c < N; ++c) {
    inc[c] = v[c];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long u = __shfl_up_sync(kFull, inc[c], o);
      if (lane >= o) inc[c] += u;
    }
    if (lane == 31) s_w[c][warp] = inc[c];
  }
  __syncthreads();
#pragma unroll
  for (int c = 0; c < N; ++c) {
    long long before = 0, all = 0;
#pragma unroll
    for (int w = 0; w < 8; ++w) {
      if (w < warp) before += s_w[c][w];
      all += s_w[c][w];
    }
    ex[c] = before + inc[c] - v[c];
    tot[c] = all;
  }
  __syncthreads();
}

// Lanes of the aligned group of G lanes (G a power of two <= 32) that the
// calling lane belongs to.  Groups of one warp may take different branches,
// so every group-level shuffle names only its own group.
__device__ __forceinline__ unsigned group_mask(int G) {
  if (G >= 32) return kFull;
  const int lane = threadIdx.x & 31;
  return ((1u << G) - 1u) << (lane & ~(G - 1));
}

template <typename T>
__device__ __forceinline__ T group_inclusive_scan(T v, int G) {
  const unsigned gm = group_mask(G);
  const int gl = threadIdx.x & (G - 1);
  for (int o = 1; o < G; o <<= 1) {
    T u = __shfl_up_sync(gm, v, o, G);
    if (gl >= o) v += u;
  }
  return v;
}

template <typename T>
__device__ __forceinline__ T group_sum(T v, int G) {
  const unsigned gm = group_mask(G);
  for (int o = G >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(gm, v, o, G);
  return v;
}

// Value of `v` on the last lane of the caller's group.
template <typename T>
__device__ __forceinline__ T group_last(T v, int G) {
  return __shfl_sync(group_mask(G), v, G - 1, G);
}

}  // namespace daxgb
