// K1: point classification into a bit stream, and the per-cell count kernels
// behind DispatcherMapCell<MarchingCubesCount | ThresholdCount>.
//
// K1 is the only kernel that reads the whole field.  It is a pure stream: each
// warp step loads 32 x float4 (512 B, fully coalesced, evict-first) and emits
// four 32-bit words of classification bits, so HBM traffic is 4 B/point read +
// 1/8 B/point written.  Everything downstream (counts, scans, generation)
// works on the 16x smaller bit stream, which stays resident in L2.
#include "common.cuh"
#include "kernels.cuh"
#include "mc_case.cuh"

namespace daxgb {

template <int MODE>
__device__ __forceinline__ uint32_t classify_point(float v, float a, float b) {
  // MODE 0: marching-cubes inside test, values[i] > iso (dax/worklet/MarchingCubes.h:40-47)
  // MODE 1: threshold test, min <= value <= max (dax/worklet/Threshold.h:40-43)
  if (MODE == 0) return v > a ? 1u : 0u;
  return (v >= a && v <= b) ? 1u : 0u;
}

// Each warp-chunk covers 128 points = 4 bit words.  UNROLL chunks per warp
// step keep several 512 B loads in flight per warp.  Chunks are global over
// the grid set; each grid's chunks start on a fresh chunk, so a chunk never
// straddles two grids and each grid's bits start on a word boundary.
//
// [c_begin, c_end) restricts a one-grid launch to a range of chunks (the
// slabs of the pipelined marching cubes); `init`, when not null, is the Info
// block whose error words and emit counters this launch clears (it runs
// before every other pass of its count pass).
//
// KEEP: the field is read with the default cache policy instead of
// evict-first, so that a slab's values can still be in L2 when the emit of
// that slab gathers its crossing-edge end points (pipelined calls).
template <typename T>
__device__ __forceinline__ T ld_field(const T* p, bool keep) {
  return keep ? __ldg(p) : __ldcs(p);
}

template <int MODE, bool VEC, bool KEEP>
__global__ void __launch_bounds__(256) k_classify_bits(GridSet S, uint32_t* __restrict__ bits,
                                                       long long nwords, long long c_begin,
                                                       long long c_end, Info* init) {
  constexpr int UNROLL = 4;
  const int lane = threadIdx.x & 31;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  const long long nchunks = S.chunks;
  const float nan = __int_as_float(0x7fc00000);  // classifies as 0 in both modes
  __shared__ long long s_keys[kStagedSlots];
  const long long* keys =
      stage_slot_keys(S, s_keys, [](const GridSlot& sl) { return sl.chunk0; }) ? s_keys : nullptr;
  pdl_trigger();  // the count pass may launch into the SMs this grid frees
  if (init && blockIdx.x == 0 && threadIdx.x == 0) {
    init->error = 0;
    init->aborted = 0;
    init->ticket = 0;
    init->done = 0;
  }
  if (S.count == 1) {
    // one grid: field pointer and thresholds are loop invariants
    const float* __restrict__ f = S.one.field;
    const long long P = S.one.g.P;
    const float a = S.one.iso, b = S.one.iso_hi;
    for (long long c0 = c_begin + warp * UNROLL; c0 < c_end; c0 += nwarps * UNROLL) {
      float4 v[UNROLL];
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) {
        const long long base = ((c0 + u) << 7) + lane * 4;
        if (c0 + u >= c_end) {
          v[u] = make_float4(nan, nan, nan, nan);
        } else if (VEC && base + 3 < P) {
          v[u] = ld_field(reinterpret_cast<const float4*>(f + base), KEEP);
        } else {
          v[u].x = base + 0 < P ? ld_field(f + base + 0, KEEP) : nan;
          v[u].y = base + 1 < P ? ld_field(f + base + 1, KEEP) : nan;
          v[u].z = base + 2 < P ? ld_field(f + base + 2, KEEP) : nan;
          v[u].w = base + 3 < P ? ld_field(f + base + 3, KEEP) : nan;
        }
      }
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) {
        const uint32_t nib = classify_point<MODE>(v[u].x, a, b) |
                             (classify_point<MODE>(v[u].y, a, b) << 1) |
                             (classify_point<MODE>(v[u].z, a, b) << 2) |
                             (classify_point<MODE>(v[u].w, a, b) << 3);
        uint32_t w = nib << (4 * (lane & 7));
        w |= __shfl_xor_sync(kFull, w, 1);
        w |= __shfl_xor_sync(kFull, w, 2);
        w |= __shfl_xor_sync(kFull, w, 4);
        if ((lane & 7) == 0 && c0 + u < c_end) bits[((c0 + u) << 2) + (lane >> 3)] = w;
      }
    }
  } else {
    // one search per warp step (the step's chunks are consecutive), then a
    // step forward where a chunk starts a later grid; the next step's search
    // runs while this step's loads are in flight
    const long long stride = nwarps * UNROLL;
    int snext = warp * UNROLL < nchunks
                    ? (keys ? slot_search(keys, S.count, warp * UNROLL) : slot_of_chunk(S, warp * UNROLL))
                    : 0;
    for (long long c0 = warp * UNROLL; c0 < nchunks; c0 += stride) {
      float4 v[UNROLL];
      float a[UNROLL], b[UNROLL];
      long long wout[UNROLL];
      int si = snext;
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) {
        const long long c = c0 + u;
        v[u] = make_float4(nan, nan, nan, nan);
        a[u] = b[u] = 0.0f;
        wout[u] = -1;
        if (c < nchunks) {
          while (si + 1 < S.count && (keys ? keys[si + 1] : __ldg(&S.slots[si + 1].chunk0)) <= c) ++si;
          const GridSlot& sl = S.slots[si];
          const long long lc = c - sl.chunk0;
          const long long base = (lc << 7) + lane * 4;
          const float* f = sl.field;
          const long long P = sl.g.P;
          a[u] = sl.iso;
          b[u] = sl.iso_hi;
          wout[u] = sl.word0 + (lc << 2);
          if (VEC && base + 3 < P) {
            v[u] = __ldcs(reinterpret_cast<const float4*>(f + base));
          } else {
            if (base + 0 < P) v[u].x = __ldcs(f + base + 0);
            if (base + 1 < P) v[u].y = __ldcs(f + base + 1);
            if (base + 2 < P) v[u].z = __ldcs(f + base + 2);
            if (base + 3 < P) v[u].w = __ldcs(f + base + 3);
          }
        }
      }
      if (c0 + stride < nchunks)
        snext = keys ? slot_search(keys, S.count, c0 + stride) : slot_of_chunk(S, c0 + stride);
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) {
        const uint32_t nib = classify_point<MODE>(v[u].x, a[u], b[u]) |
                             (classify_point<MODE>(v[u].y, a[u], b[u]) << 1) |
                             (classify_point<MODE>(v[u].z, a[u], b[u]) << 2) |
                             (classify_point<MODE>(v[u].w, a[u], b[u]) << 3);
        uint32_t w = nib << (4 * (lane & 7));
        w |= __shfl_xor_sync(kFull, w, 1);
        w |= __shfl_xor_sync(kFull, w, 2);
        w |= __shfl_xor_sync(kFull, w, 4);
        if ((lane & 7) == 0 && wout[u] >= 0) bits[wout[u] + (lane >> 3)] = w;
      }
    }
  }
  // zero the padding words after the last chunk (read by unaligned fetches)
  if (blockIdx.x == 0 && threadIdx.x < 8 && c_end == nchunks) {
    const long long w = (nchunks << 2) + threadIdx.x;
    if (w < nwords) bits[w] = 0u;
  }
}

void launch_classify_bits(int mode, const GridSet& S, bool all_aligned, uint32_t* bits,
                          long long nwords, int num_sms, cudaStream_t s) {
  launch_classify_range(mode, S, all_aligned, bits, nwords, 0, S.chunks, nullptr, kPassClassify,
                        false, num_sms, s);
}

void launch_classify_range(int mode, const GridSet& S, bool all_aligned, uint32_t* bits,
                           long long nwords, long long c_begin, long long c_end, Info* init,
                           int pass, bool keep, int num_sms, cudaStream_t s) {
  // blocks of 8 warps x 4 chunks
  const long long want = (c_end - c_begin + 4 * 8 - 1) / (4 * 8);
#define DAXGB_K1(M, V, K)                                                      \
  {                                                                            \
    const int blocks = resident_blocks(k_classify_bits<M, V, K>, 256, 0, num_sms, want, pass); \
    k_classify_bits<M, V, K><<<blocks, 256, 0, s>>>(S, bits, nwords, c_begin, c_end, init); \
  }
  if (mode == 0 && keep) {
    if (all_aligned) DAXGB_K1(0, true, true) else DAXGB_K1(0, false, true)
  } else if (mode == 0) {
    if (all_aligned) DAXGB_K1(0, true, false) else DAXGB_K1(0, false, false)
  } else {
    if (all_aligned) DAXGB_K1(1, true, false) else DAXGB_K1(1, false, false)
  }
#undef DAXGB_K1
}

// ---- per-cell count arrays (the Dax count handles) ---------------------
// One thread per cell, cells in id order; the 8 corner loads of neighbouring
// threads overlap and are served by L1/L2.
template <int MODE>
__global__ void __launch_bounds__(256) k_cell_count(Grid g, const float* __restrict__ f, float a,
                                                    float b, int32_t* __restrict__ count,
                                                    uint8_t* __restrict__ cases) {
  const int cx = g.nx - 1, cy = g.ny - 1;
  const long long C = (long long)cx * cy * (g.nz - 1);
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < C;
       c += (long long)gridDim.x * blockDim.x) {
    const long long row = c / cx;
    const int i = (int)(c - row * cx);
    const int j = (int)(row % cy);
    const int k = (int)(row / cy);
    const long long p0 = i + (long long)g.nx * (j + (long long)g.ny * k);
    const long long dy = g.nx, dz = (long long)g.nx * g.ny;
    const float v[8] = {__ldg(f + p0),          __ldg(f + p0 + 1),          __ldg(f + p0 + dy + 1),
                        __ldg(f + p0 + dy),     __ldg(f + p0 + dz),         __ldg(f + p0 + dz + 1),
                        __ldg(f + p0 + dz + dy + 1), __ldg(f + p0 + dz + dy)};
    if (MODE == 0) {
      int cs = 0;
#pragma unroll
      for (int n = 0; n < 8; ++n) cs |= (v[n] > a) << n;
      count[c] = (int32_t)mc_num_tris(cs);
      if (cases) cases[c] = (uint8_t)cs;
    } else {
      int valid = 1;
#pragma unroll
      for (int n = 0; n < 8; ++n) valid &= (v[n] >= a && v[n] <= b);
      count[c] = valid;
    }
  }
}

void launch_cell_count(int mode, const Grid& g, const float* f, float a, float b, int32_t* count,
                       uint8_t* cases, int num_sms, cudaStream_t s) {
  const long long C = (long long)(g.nx - 1) * (g.ny - 1) * (g.nz - 1);
  const long long want = (C + 255) / 256;
  const long long cap = (long long)num_sms * 16;
  const int blocks = (int)(want < 1 ? 1 : (want < cap ? want : cap));
  if (mode == 0) k_cell_count<0><<<blocks, 256, 0, s>>>(g, f, a, b, count, cases);
  else k_cell_count<1><<<blocks, 256, 0, s>>>(g, f, a, b, count, cases);
}

}  // namespace daxgb
