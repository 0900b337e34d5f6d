// The count pass of one uniform grid -- classification and per-word counts
// -- fused into one persistent launch (marching cubes: MODE 0, threshold:
// MODE 1); k_word_scan then turns the counts into offsets.
//
// Run as separate launches, the count (K2a) starts only after the whole field
// has streamed through the classification (K1), and HBM idles while it runs
// from L2.  Here the blocks of one persistent launch take classification
// units from a device ticket counter, in field order:
//
//   classify unit u: chunks [u UC, (u + 1) UC) of 128 points.  The block
//       streams them into shared memory with bulk TMA copies (cp.async.bulk,
//       a ring of kRing 16 KB stages, completion counted on mbarriers) and
//       turns each stage into bit words exactly as K1 does.
//
// and count the scan tiles whose bits are complete:
//
//   count tile i: the kScanTile row words of scan tile i read the bits of
//       their rows, the next row and the next z-plane (threshold: also the
//       previous row and plane).  Each tile keeps a dependency count in
//       global memory; a block that finishes a unit adds to it, and the
//       addition that completes it puts the tile in a device queue of ready
//       tiles.  Blocks take tiles from the queue (one per unit while units
//       are left, all that remain after) and count them from the bit stream
//       in L2 -- the packed counts wc and per-tile totals of k_mc_count, or
//       the kept / used masks, counts and totals of k_thr_kept + k_thr_used,
//       bit for bit.
//
// So the counts of plane k run while other blocks stream the planes after
// it.  (Measured at 512^3 the pass is still slower than the separate
// launches, 0.146 against 0.134 ms: a block spends about 40% of its time off
// the field stream, on its dependency additions and tile counts, which is
// why it is off by default.)  A count never waits for another tile (a
// decoupled look-back scan inside this launch was measured to chain the
// tiles' look-backs behind one another), so the only waits are for a queue
// slot whose tile a running block has reserved, or, once every unit is handed
// out, for the last tiles to become ready; both end, and both are bounded
// (kSpinIters polls and kSpinNs of %globaltimer), after which the block sets
// the abort word, the launch winds down and the scan reports kErrTimeout.
//
// Control words (fctl, cleared before the launch): [0] unit ticket counter,
// [1] abort, [2] queue pushes, [3] queue pops, [4 .. 4 + tiles) dependency
// counts, [4 + tiles .. 4 + 2 tiles) the queue (tile + 1 per slot).
#include "common.cuh"
#include "kernels.cuh"
#include "mc_case.cuh"
#include "mc_words.cuh"
#include "tma.cuh"

namespace daxgb {

namespace {

constexpr int kStageChunks = 32;                  // 128-point chunks per TMA stage
constexpr int kStagePoints = 128 * kStageChunks;  // 4096
constexpr int kStageBytes = 4 * kStagePoints;     // 16 KB
constexpr int kRing = 3;                          // stages in flight per block
constexpr int kFusedThreads = 256;
constexpr int kFusedMinBlocks = 4;
constexpr int kWalk = 128;                        // tiles a unit's walk handles at a time

int g_fused_enabled = 0;  // off by default: slower than the separate passes at 512^3
int g_unit_stages = 16;  // classify unit = 16 stages = 512 chunks = 65536 points (a power of 2)

struct FusedArgs {
  Grid g;
  const float* f;
  float a, b;            // isovalue, or the threshold range [a, b]
  uint32_t* bits;
  long long nwords;      // bit words including the zero padding
  long long nchunks;     // 128-point chunks
  int unit_chunks;       // chunks per classify unit (kStageChunks x a power of 2)
  int unit_shift;        // log2 of the points per unit
  int units, tiles;
  long long W;           // row words
  uint32_t* wc;          // packed per-word counts
  uint32_t* tile_tot;    // [3][tiles] per-tile totals
  uint32_t* kept;        // threshold: per-word kept-cell and used-point masks
  uint32_t* used;
  uint32_t* ctl;
  uint32_t* deps;        // per tile: dependency additions so far
  uint32_t* queue;       // ready tiles, tile + 1 per slot
};

__device__ __forceinline__ void raise_timeout(const FusedArgs& A) { atomicExch(A.ctl + 1, 1u); }

// Bytes of stage s of unit u that the TMA copies (16-byte multiple); the
// stage's remaining points below P are read directly.
__device__ __forceinline__ unsigned stage_bytes(const FusedArgs& A, long long first_point) {
  const long long rem = A.g.P - first_point;
  if (rem <= 0) return 0u;
  const long long pts = rem < kStagePoints ? rem : kStagePoints;
  return (unsigned)(4 * pts) & ~15u;
}

// ---- work order ------------------------------------------------------------
// Points of the window of rows a count tile reads, [lo, hi), before the
// z-plane offsets: its rows from one row before its first (threshold reads
// the previous row) to the row after its last, plus the word padding that
// row_windows4 and the x-pair reads fetch past a row.
__device__ __forceinline__ void tile_rows(const FusedArgs& A, int i, long long& lo, long long& hi) {
  const long long w0 = (long long)i * kScanTile;
  const long long we = w0 + kScanTile < A.W ? w0 + kScanTile : A.W;
  const long long r_lo = div_by((unsigned)w0, A.g.mwr), r_hi = div_by((unsigned)(we - 1), A.g.mwr);
  lo = (r_lo - 1) * (long long)A.g.nx - 64;
  hi = (r_hi + 2) * (long long)A.g.nx + 192;
}

__device__ __forceinline__ int unit_of(const FusedArgs& A, long long point) {
  const long long u = point < 0 ? 0 : point >> A.unit_shift;
  return (int)(u < A.units - 1 ? u : A.units - 1);
}

// A count tile reads the bit stream over its row window [lo, hi) shifted by
// the plane offsets of its mode: window o (0: -dz, 1: 0, 2: +dz) -- marching
// cubes reads windows 1 and 2, threshold all three.  Window o of tile i
// covers units u0 .. u1 (none when it lies wholly before the field); the
// tile's dependency count is the sum of their numbers.  A unit's completion
// adds to every tile the number of its windows covering the unit; the block
// whose addition reaches the tile's count counts the tile right away.
__device__ __forceinline__ bool window_units(const FusedArgs& A, int i, int o, int& u0, int& u1) {
  long long lo, hi;
  tile_rows(A, i, lo, hi);
  const long long off = (long long)(o - 1) * A.g.nx * A.g.ny;
  if (hi + off <= 0) return false;
  u0 = unit_of(A, lo + off);
  u1 = unit_of(A, hi + off - 1);
  return true;
}

template <int MODE>
__device__ __forceinline__ unsigned tile_deps(const FusedArgs& A, int i) {
  unsigned d = 0;
  for (int o = MODE == 1 ? 0 : 1; o < 3; ++o) {
    int u0, u1;
    if (window_units(A, i, o, u0, u1)) d += (unsigned)(u1 - u0 + 1);
  }
  return d;
}

// Tiles whose window o covers unit u: [t0, t1] (empty when t0 > t1).
// Windows move forward with the tile, so both ends are binary searches.
__device__ void tiles_of_unit(const FusedArgs& A, int u, int o, int& t0, int& t1) {
  int lo = 0, hi = A.tiles;  // first tile with a window whose last unit is >= u
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    int a, b;
    if (window_units(A, mid, o, a, b) && b >= u)
      hi = mid;
    else
      lo = mid + 1;
  }
  t0 = lo;
  lo = -1;
  hi = A.tiles - 1;  // last tile whose window's first unit is <= u
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    long long wlo, whi;
    tile_rows(A, mid, wlo, whi);
    if (unit_of(A, wlo + (long long)(o - 1) * A.g.nx * A.g.ny) <= u)
      lo = mid;
    else
      hi = mid - 1;
  }
  t1 = lo;
}

// ---- classify unit ---------------------------------------------------------
template <int MODE>
__device__ __forceinline__ uint32_t in_bit(float v, float a, float b) {
  // MODE 0: values[i] > iso (dax/worklet/MarchingCubes.h:40-47)
  // MODE 1: min <= value <= max (dax/worklet/Threshold.h:40-43)
  if (MODE == 0) return v > a ? 1u : 0u;
  return (v >= a && v <= b) ? 1u : 0u;
}

// Issues the first kRing stage copies of unit u at ring positions ring_pos..
// (the ring's earlier reads ordered before them); classify_unit consumes them.
__device__ void unit_prologue(const FusedArgs& A, int u, unsigned char* ring, uint64_t* bar,
                              unsigned long long ring_pos, unsigned long long policy) {
  fence_proxy_async();
  __syncthreads();
  if (threadIdx.x != 0) return;
  const long long c_begin = (long long)u * A.unit_chunks;
  const long long c_end =
      c_begin + A.unit_chunks < A.nchunks ? c_begin + A.unit_chunks : A.nchunks;
  const int nst = (int)((c_end - c_begin + kStageChunks - 1) / kStageChunks);
  for (int s = 0; s < nst && s < kRing; ++s) {
    const unsigned long long pos = ring_pos + s;
    const int slot = (int)(pos % kRing);
    const long long fp = (c_begin + (long long)kStageChunks * s) * 128;
    const unsigned bytes = stage_bytes(A, fp);
    if (bytes) {
      mbar_arrive_tx(bar + slot, bytes);
      bulk_load(ring + slot * kStageBytes, A.f + fp, bytes, bar + slot, policy);
    } else {
      mbar_arrive(bar + slot);
    }
  }
}

// Classifies unit u, whose first stages unit_prologue issued.  Returns false
// when a stage's copy did not complete in time (the block then stops taking
// work).
template <int MODE>
__device__ bool classify_unit(const FusedArgs& A, int u, unsigned char* ring, uint64_t* bar,
                              unsigned long long& ring_pos, unsigned long long policy) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long long c_begin = (long long)u * A.unit_chunks;
  const long long c_end =
      c_begin + A.unit_chunks < A.nchunks ? c_begin + A.unit_chunks : A.nchunks;
  const int nst = (int)((c_end - c_begin + kStageChunks - 1) / kStageChunks);
  const float nan = __int_as_float(0x7fc00000);  // classifies as 0 in both modes
  auto issue = [&](int s) {
    const unsigned long long pos = ring_pos + s;
    const int slot = (int)(pos % kRing);
    const long long fp = (c_begin + (long long)kStageChunks * s) * 128;
    const unsigned bytes = stage_bytes(A, fp);
    if (bytes) {
      mbar_arrive_tx(bar + slot, bytes);
      bulk_load(ring + slot * kStageBytes, A.f + fp, bytes, bar + slot, policy);
    } else {
      mbar_arrive(bar + slot);
    }
  };
  // the first kRing stages were issued by unit_prologue
  bool ok = true;
  int s_fail = nst;
  for (int s = 0; s < nst; ++s) {
    const unsigned long long pos = ring_pos + s;
    const int slot = (int)(pos % kRing);
    const unsigned parity = (unsigned)((pos / kRing) & 1ull);
    Spin sp;
    while (!mbar_test(bar + slot, parity)) {
      if (!sp.more()) {
        ok = false;
        break;
      }
    }
    if (__syncthreads_or(!ok)) {
      ok = false;
      s_fail = s;
      break;
    }
    const long long cs0 = c_begin + (long long)kStageChunks * s;
    const long long fp = cs0 * 128;
    const unsigned bytes = stage_bytes(A, fp);
    const float4* st4 = reinterpret_cast<const float4*>(ring + slot * kStageBytes);
    const float* st1 = reinterpret_cast<const float*>(ring + slot * kStageBytes);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int cl = warp * 4 + q;  // chunk within the stage
      const long long c = cs0 + cl;
      const int off = cl * 128 + lane * 4;  // first of the lane's 4 points, in the stage
      float4 v;
      if ((unsigned)(4 * off + 16) <= bytes) {
        v = st4[cl * 32 + lane];
      } else {
        float e[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const long long p = fp + off + t;
          e[t] = (unsigned)(4 * (off + t)) < bytes ? st1[off + t] : (p < A.g.P ? __ldcs(A.f + p) : nan);
        }
        v = make_float4(e[0], e[1], e[2], e[3]);
      }
      const uint32_t nib = in_bit<MODE>(v.x, A.a, A.b) | (in_bit<MODE>(v.y, A.a, A.b) << 1) |
                           (in_bit<MODE>(v.z, A.a, A.b) << 2) | (in_bit<MODE>(v.w, A.a, A.b) << 3);
      uint32_t w = nib << (4 * (lane & 7));
      w |= __shfl_xor_sync(kFull, w, 1);
      w |= __shfl_xor_sync(kFull, w, 2);
      w |= __shfl_xor_sync(kFull, w, 4);
      if ((lane & 7) == 0 && c < c_end) A.bits[(c << 2) + (lane >> 3)] = w;
    }
    // every thread is done with the slot before the next copy overwrites it
    fence_proxy_async();
    __syncthreads();
    if (tid == 0 && s + kRing < nst) issue(s + kRing);
  }
  if (!ok) {
    // a copy that did not arrive: wait (bounded) for the copies still in
    // flight (stages s_fail .. s_fail + kRing - 1), so that none lands in
    // shared memory after the block exits
    if (tid == 0) {
      raise_timeout(A);
      for (int s = s_fail; s < nst && s < s_fail + kRing; ++s) {
        const unsigned long long pos = ring_pos + s;
        Spin sp;
        while (!mbar_test(bar + (int)(pos % kRing), (unsigned)((pos / kRing) & 1ull)) && sp.more()) {
        }
      }
    }
    __syncthreads();
    return false;
  }
  ring_pos += nst;
  if (c_end == A.nchunks && tid < 8) {
    // zero the padding words after the last chunk (read by unaligned fetches)
    const long long w = (A.nchunks << 2) + tid;
    if (w < A.nwords) A.bits[w] = 0u;
  }
  __syncthreads();
  return true;
}

// Marching cubes: packed counts (triangles << 16 | crossing edges) of the
// four row words g0..g0+3 (0 past W), from the bit stream in L2.
__device__ __forceinline__ void mc_counts4(const FusedArgs& A, long long g0,
                                           const unsigned char* nf, uint32_t (&out)[4]) {
  const Grid& g = A.g;
  out[0] = out[1] = out[2] = out[3] = 0u;
  if (g0 >= A.W) return;
  int m;
  const unsigned r = split_word(g, (unsigned)g0, m);
  if (m + 4 <= g.wr && g0 + 4 <= A.W) {
    // the four words lie in one row
    int j, k;
    split_row(g, r, j, k);
    const bool hy = j < g.ny - 1, hz = k < g.nz - 1;
    const long long dy = g.nx, dz = (long long)g.nx * g.ny;
    const long long pos = (long long)r * g.nx + 32ll * m;
    uint32_t a[4], a1[4], b[4] = {0, 0, 0, 0}, b1[4] = {0, 0, 0, 0}, c[4] = {0, 0, 0, 0},
             c1[4] = {0, 0, 0, 0}, d[4] = {0, 0, 0, 0}, d1[4] = {0, 0, 0, 0};
    row_windows4<true>(A.bits, pos, a, a1);
    if (hy) row_windows4<true>(A.bits, pos + dy, b, b1);
    if (hz) row_windows4<true>(A.bits, pos + dz, c, c1);
    if (hy && hz) row_windows4<true>(A.bits, pos + dy + dz, d, d1);
    uint32_t diff = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      diff |= a[q] ^ a1[q];
      if (hy) diff |= (a[q] ^ b[q]) | (a[q] ^ b1[q]);
      if (hz) diff |= (a[q] ^ c[q]) | (a[q] ^ c1[q]);
      if (hy && hz) diff |= (a[q] ^ d[q]) | (a[q] ^ d1[q]);
    }
    if (diff) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const CornerWords w{a[q], a1[q], b[q], b1[q], c[q], c1[q], d[q], d1[q]};
        out[q] = packed_counts(w, hy, hz, low_mask(g.nx - 32 * (m + q)),
                               low_mask(g.nx - 1 - 32 * (m + q)), nf);
      }
    }
  } else {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const long long gw = g0 + q;
      if (gw >= A.W) break;
      int mq;
      const unsigned rq = split_word(g, (unsigned)gw, mq);
      const WordBits wb = load_word_bits<true>(g, A.bits, rq, mq);
      out[q] = packed_counts(wb.w, wb.hy, wb.hz, wb.pmask, wb.xmask, nf);
    }
  }
}

// Threshold: the pair masks of point row `pos` at words m..m+3 (bit x set
// when points x and x + 1 are both in range) and the pair (32m - 1, 32m).
__device__ __forceinline__ void row_pairs4(const uint32_t* bits, long long pos, bool pre_word,
                                           uint32_t (&pp)[4], uint32_t& pre) {
  uint32_t a[4], a1[4];
  row_windows4<true>(bits, pos, a, a1);
#pragma unroll
  for (int q = 0; q < 4; ++q) pp[q] = a[q] & a1[q];
  pre = 0u;
  if (pre_word) {
    const uint32_t x = bits_at<true>(bits, pos - 1);
    pre = x & (x >> 1) & 1u;
  }
}

// Kept-cell mask of cell row (j, k), word m (0 on rows without cells).
__device__ __forceinline__ uint32_t kept_of(const Grid& g, const uint32_t* bits, int j, int k,
                                            int m) {
  if (j < 0 || k < 0 || j + 1 >= g.ny || k + 1 >= g.nz) return 0u;
  const long long dy = g.nx, dz = (long long)g.nx * g.ny;
  const long long pos = ((long long)k * g.ny + j) * g.nx + 32ll * m;
  uint32_t a, a1, b, b1, c, c1, d, d1;
  bits_at2<true>(bits, pos, a, a1);
  bits_at2<true>(bits, pos + dy, b, b1);
  bits_at2<true>(bits, pos + dz, c, c1);
  bits_at2<true>(bits, pos + dy + dz, d, d1);
  return a & a1 & b & b1 & c & c1 & d & d1 & low_mask(g.nx - 1 - 32 * m);
}

// Threshold: kept and used masks of row words g0..g0+3 (as k_thr_kept and
// k_thr_used: kept = cells whose 8 corners are in range, used = points that
// are a corner of a kept cell of cell rows (j-1..j, k-1..k)), written to the
// kept / used arrays; packed counts popc(kept) << 16 | popc(used).
__device__ __forceinline__ void thr_counts4(const FusedArgs& A, long long g0, uint32_t (&out)[4]) {
  const Grid& g = A.g;
  out[0] = out[1] = out[2] = out[3] = 0u;
  if (g0 >= A.W) return;
  int m;
  const unsigned r = split_word(g, (unsigned)g0, m);
  uint32_t own[4] = {0u, 0u, 0u, 0u}, U[4] = {0u, 0u, 0u, 0u};
  if (m + 4 <= g.wr && g0 + 4 <= A.W) {
    int j, k;
    split_row(g, r, j, k);
    const long long dy = g.nx;
    const bool pre_word = m > 0;
    // plane by plane: y-pairs of cell rows j - 1 (0) and j (1); a cell row
    // of cell plane kk - 1 is the AND of its y-pairs on planes kk - 1 and kk
    uint32_t yp[2][4], ypp[2];
    bool have = false;
#pragma unroll
    for (int dk = -1; dk <= 1; ++dk) {
      const int kk = k + dk;
      if (kk < 0 || kk >= g.nz) {
        have = false;
        continue;
      }
      const long long base = ((long long)kk * g.ny + j) * g.nx + 32ll * m;
      uint32_t p0[4] = {0u, 0u, 0u, 0u}, p1[4], p2[4] = {0u, 0u, 0u, 0u}, e0 = 0u, e1, e2 = 0u;
      row_pairs4(A.bits, base, pre_word, p1, e1);
      if (j >= 1) row_pairs4(A.bits, base - dy, pre_word, p0, e0);
      if (j + 1 < g.ny) row_pairs4(A.bits, base + dy, pre_word, p2, e2);
      uint32_t yc[2][4], ycp[2];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        yc[0][q] = p0[q] & p1[q];
        yc[1][q] = p1[q] & p2[q];
      }
      ycp[0] = e0 & e1;
      ycp[1] = e1 & e2;
      if (have) {
#pragma unroll
        for (int cj = 0; cj < 2; ++cj) {
          // cell row (j - 1 + cj, kk - 1)
          if (j - 1 + cj < 0 || j + cj >= g.ny) continue;
          uint32_t K[4];
#pragma unroll
          for (int q = 0; q < 4; ++q)
            K[q] = yp[cj][q] & yc[cj][q] & low_mask(g.nx - 1 - 32 * (m + q));
          const uint32_t kp = ypp[cj] & ycp[cj];  // cell 32m - 1
#pragma unroll
          for (int q = 0; q < 4; ++q)
            U[q] |= K[q] | (K[q] << 1) | (q > 0 ? (K[q - 1] >> 31) : kp);
          if (dk == 1 && cj == 1) {
#pragma unroll
            for (int q = 0; q < 4; ++q) own[q] = K[q];
          }
        }
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        yp[0][q] = yc[0][q];
        yp[1][q] = yc[1][q];
      }
      ypp[0] = ycp[0];
      ypp[1] = ycp[1];
      have = true;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) U[q] &= low_mask(g.nx - 32 * (m + q));
    *reinterpret_cast<uint4*>(A.kept + g0) = make_uint4(own[0], own[1], own[2], own[3]);
    *reinterpret_cast<uint4*>(A.used + g0) = make_uint4(U[0], U[1], U[2], U[3]);
  } else {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const long long gw = g0 + q;
      if (gw >= A.W) break;
      int mq, jq, kq;
      const unsigned rq = split_word(g, (unsigned)gw, mq);
      split_row(g, rq, jq, kq);
      own[q] = kept_of(g, A.bits, jq, kq, mq);
      uint32_t u = 0u;
#pragma unroll
      for (int c = 0; c < 4; ++c) {  // cell rows (jq - (c & 1), kq - (c >> 1))
        const int cj = jq - (c & 1), ck = kq - (c >> 1);
        if (cj < 0 || ck < 0) continue;
        const uint32_t K = c == 0 ? own[q] : kept_of(g, A.bits, cj, ck, mq);
        const uint32_t Kp = mq > 0 ? kept_of(g, A.bits, cj, ck, mq - 1) : 0u;
        u |= K | (K << 1) | (Kp >> 31);
      }
      U[q] = u & low_mask(g.nx - 32 * mq);
      A.kept[gw] = own[q];
      A.used[gw] = U[q];
    }
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) out[q] = (uint32_t)__popc(own[q]) << 16 | (uint32_t)__popc(U[q]);
}

// Counts of tile i: the packed per-word counts to wc and the tile's totals
// (triangles / kept cells, vertices / used points, active words) to
// tile_tot, as the separate count passes write them.
template <int MODE>
__device__ void count_tile(const FusedArgs& A, int i, const unsigned char* nf, uint32_t* s_red) {
  const int tid = threadIdx.x;
  const long long t0 = (long long)i * kScanTile;
  uint32_t st = 0, sv = 0, sa = 0;
  // coalesced groups of 4 words: thread t takes groups t + 256 e
#pragma unroll 1
  for (int e = 0; e < kScanItems / 4; ++e) {
    const long long g0 = t0 + 4ll * (tid + 256 * e);
    if (g0 >= A.W) break;
    uint32_t out[4];
    if (MODE == 0)
      mc_counts4(A, g0, nf, out);
    else
      thr_counts4(A, g0, out);
    if (g0 + 4 <= A.W) {
      *reinterpret_cast<uint4*>(A.wc + g0) = make_uint4(out[0], out[1], out[2], out[3]);
    } else {
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (g0 + q < A.W) A.wc[g0 + q] = out[q];
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      st += out[q] >> 16;
      sv += out[q] & 0xffffu;
      sa += out[q] ? 1u : 0u;
    }
  }
  __syncthreads();  // s_red of an earlier tile is read
  block_sum3(st, sv, sa, s_red);
  if (tid == 0) {
    A.tile_tot[i] = st;
    A.tile_tot[A.tiles + i] = sv;
    A.tile_tot[2 * A.tiles + i] = sa;
  }
}

template <int MODE>
__global__ void __launch_bounds__(kFusedThreads, kFusedMinBlocks) k_fused_count(FusedArgs A) {
  extern __shared__ __align__(128) unsigned char s_ring[];  // kRing TMA stages
  __shared__ __align__(8) uint64_t s_bar[kRing];
  __shared__ unsigned char s_nf[256];  // NumFaces (marching cubes)
  __shared__ int s_t[6];
  __shared__ int s_walk[kWalk];
  __shared__ unsigned char s_inc[kWalk];
  __shared__ int s_nwalk, s_next, s_unit, s_tile;
  __shared__ uint32_t s_red[24];
  const int tid = threadIdx.x;
  if (MODE == 0) s_nf[tid] = (unsigned char)mc_num_tris(tid);
  if (tid == 0) {
    for (int s = 0; s < kRing; ++s) mbar_init(s_bar + s, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  unsigned long long policy;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(policy));
  unsigned long long ring_pos = 0;
  // units in field order; each one's first stages are issued before the
  // previous unit's dependency walk and tile count, so the copies run while
  // those do
  auto take_unit = [&]() -> int {
    if (tid == 0) {
      const int v = ld_relaxed(A.ctl + 1) == 0u ? (int)atomicAdd(A.ctl, 1u) : A.units;
      s_unit = v < A.units ? v : -1;
    }
    __syncthreads();
    const int v = s_unit;
    __syncthreads();
    if (v >= 0) unit_prologue(A, v, s_ring, s_bar, ring_pos, policy);
    return v;
  };
  int u = take_unit();
  bool ok = true;
  for (;;) {
    if (u >= 0) {
      if (!classify_unit<MODE>(A, u, s_ring, s_bar, ring_pos, policy)) break;
    }
    const int un = u >= 0 ? take_unit() : -1;
    if (u >= 0) {
      // the unit's dependency additions: per window a range of tiles (one
      // search per warp), walked as their union in increasing order, kWalk
      // tiles at a time (warp 0, a tile per lane); the tiles an addition
      // completes go to the queue
      if ((tid & 31) == 0 && tid < 96) {
        const int o = tid >> 5;
        int t0 = 0, t1 = -1;
        if (MODE == 1 || o > 0) tiles_of_unit(A, u, o, t0, t1);
        s_t[o] = t0;
        s_t[3 + o] = t1;
      }
      __syncthreads();
      int cur = A.tiles;
      for (int o = 0; o < 3; ++o)
        if (s_t[o] <= s_t[3 + o] && s_t[o] < cur) cur = s_t[o];
      while (cur < A.tiles) {
        if (tid == 0) {
          int n = 0, i = cur;
          while (i < A.tiles && n < kWalk) {
            int inc = 0, next = A.tiles;
            for (int o = 0; o < 3; ++o) {
              if (s_t[o] > s_t[3 + o]) continue;
              inc += (s_t[o] <= i && i <= s_t[3 + o]) ? 1 : 0;
              const int c = i + 1 > s_t[o] ? i + 1 : s_t[o];
              if (c <= s_t[3 + o] && c < next) next = c;
            }
            s_walk[n] = i;
            s_inc[n] = (unsigned char)inc;
            ++n;
            i = next;
          }
          s_nwalk = n;
          s_next = i;
        }
        __syncthreads();
        const int n = s_nwalk;
        cur = s_next;
        if (tid < 32) {
          __threadfence();  // the unit's bits before its additions
          for (int k0 = 0; k0 < n; k0 += 32) {
            const int k = k0 + tid;
            bool ready = false;
            if (k < n && s_inc[k]) {
              const unsigned old = atomicAdd(A.deps + s_walk[k], (unsigned)s_inc[k]);
              ready = old + s_inc[k] == tile_deps<MODE>(A, s_walk[k]);
            }
            const unsigned m = __ballot_sync(kFull, ready);
            if (m) {
              unsigned base = 0;
              if (tid == 0) base = atomicAdd(A.ctl + 2, (unsigned)__popc(m));
              base = __shfl_sync(kFull, base, 0);
              if (ready) {
                __threadfence();  // every unit of the tile before the slot
                st_release(A.queue + base + __popc(m & ((1u << tid) - 1u)),
                           (unsigned)s_walk[k] + 1u);
              }
            }
          }
        }
        __syncthreads();
      }
    }
    // ---- ready tiles: one per unit while units are left (a slot already
    // reserved by a push, taken with a compare-and-swap), every remaining one
    // after (slots in order; their pushes may still be on the way)
    bool done = false;
    for (;;) {
      if (tid == 0) {
        int tile = -1;
        if (ld_relaxed(A.ctl + 1) != 0u) {
          tile = -2;
        } else {
          int slot = -1;
          if (u >= 0) {
            const unsigned p = ld_relaxed(A.ctl + 3);
            if (p < ld_relaxed(A.ctl + 2) && atomicCAS(A.ctl + 3, p, p + 1u) == p) slot = (int)p;
          } else {
            const unsigned p = atomicAdd(A.ctl + 3, 1u);
            if (p < (unsigned)A.tiles) slot = (int)p;
            else tile = -2;
          }
          if (slot >= 0) {
            Spin sp;
            unsigned v;
            while ((v = ld_acquire(A.queue + slot)) == 0u && sp.more() &&
                   ld_relaxed(A.ctl + 1) == 0u)
              __nanosleep(64);
            if (v == 0u) {
              raise_timeout(A);
              tile = -2;
            } else {
              tile = (int)v - 1;
            }
          }
        }
        s_tile = tile;
      }
      __syncthreads();
      const int tile = s_tile;
      if (tile >= 0) count_tile<MODE>(A, tile, s_nf, s_red);
      __syncthreads();
      if (tile == -2) {
        done = true;
        break;
      }
      if (u >= 0) break;  // back to the units
    }
    if (done) {
      // the launch aborted while the next unit's copies may be in flight:
      // wait (bounded) for them before leaving
      if (un >= 0 && tid == 0)
        for (int s2 = 0; s2 < kRing; ++s2) {
          const unsigned long long pos = ring_pos + s2;
          Spin sp;
          while (!mbar_test(s_bar + (int)(pos % kRing), (unsigned)((pos / kRing) & 1ull)) &&
                 sp.more()) {
          }
        }
      break;
    }
    u = un;
  }
  (void)ok;
}

}  // namespace

void set_fused_count(int enabled, int unit_stages) {
  if (enabled >= 0) g_fused_enabled = enabled ? 1 : 0;
  if (unit_stages > 0) {
    int p = 1;  // the largest power of 2 at or below the request, at most 1024
    while (p * 2 <= unit_stages && p < 1024) p *= 2;
    g_unit_stages = p;
  }
}
int fused_count_enabled() { return g_fused_enabled; }
int fused_unit_stages() { return g_unit_stages; }

size_t fused_ctl_bytes(const Grid& g) {
  const int tiles = word_scan_tiles(g.R * g.wr);
  return 4 * (size_t)(4 + 2 * tiles);
}

namespace {
int fused_units(const Grid& g, int unit_stages) {
  const long long nchunks = (g.P + 127) / 128;
  const long long uc = (long long)kStageChunks * unit_stages;
  return (int)((nchunks + uc - 1) / uc);
}
}  // namespace

int launch_fused_count(int mode, const Grid& g, const float* f, float a, float b, uint32_t* bits,
                       long long nwords, const WordOffsets& o, Info* info, uint32_t* kept,
                       uint32_t* used, uint32_t* fctl, int num_sms, cudaStream_t s) {
  FusedArgs A{};
  A.g = g;
  A.f = f;
  A.a = a;
  A.b = b;
  A.bits = bits;
  A.nwords = nwords;
  A.nchunks = (g.P + 127) / 128;
  A.unit_chunks = kStageChunks * g_unit_stages;
  A.unit_shift = 0;
  while ((128ll << A.unit_shift) < 128ll * A.unit_chunks) ++A.unit_shift;
  A.unit_shift += 7;
  A.units = fused_units(g, g_unit_stages);
  A.W = g.R * g.wr;
  A.tiles = word_scan_tiles(A.W);
  A.wc = o.wc;
  A.tile_tot = o.tile;
  A.kept = kept;
  A.used = used;
  A.ctl = fctl;
  A.deps = fctl + 4;
  A.queue = fctl + 4 + A.tiles;
  // Info (the error words) and the control words lie together at the start
  // of the scratch
  cudaError_t e = cudaMemsetAsync(info, 0,
                                  (size_t)(reinterpret_cast<char*>(fctl) -
                                           reinterpret_cast<char*>(info)) +
                                      fused_ctl_bytes(g),
                                  s);
  if (e != cudaSuccess) return (int)e;
  const size_t smem = (size_t)kRing * kStageBytes;
  // the ring plus the static shared memory is above the 48 KB a launch gets
  // without opting in; set once per device and kernel
  static int opted[2][64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && !opted[mode ? 1 : 0][dev]) {
    const void* k = mode == 0 ? reinterpret_cast<const void*>(k_fused_count<0>)
                              : reinterpret_cast<const void*>(k_fused_count<1>);
    e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    // all of the unified L1 / shared memory as shared: four blocks per SM
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout,
                               (int)cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return (int)e;
    opted[mode ? 1 : 0][dev] = 1;
  }
  if (mode == 0) {
    const int blocks = resident_blocks(k_fused_count<0>, kFusedThreads, smem, num_sms, A.units,
                                       kPassFused);
    k_fused_count<0><<<blocks, kFusedThreads, smem, s>>>(A);
  } else {
    const int blocks = resident_blocks(k_fused_count<1>, kFusedThreads, smem, num_sms, A.units,
                                       kPassFused);
    k_fused_count<1><<<blocks, kFusedThreads, smem, s>>>(A);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return (int)e;
  // the per-word offsets, the active-word list and the totals (the abort word
  // becomes kErrTimeout)
  launch_word_scan(A.W, o.wc, o.tile, o.wt, o.wv, o.act, info, s, fctl + 1);
  return (int)cudaGetLastError();
}

}  // namespace daxgb
