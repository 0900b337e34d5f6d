// The marching-cubes count pass (K2a) of one grid with each tile's bits
// staged in shared memory.
//
// A scan tile (kScanTile row words) reads the bit stream of its point rows
// r_lo .. r_hi + 1 and of the same rows one z-plane up.  Read from L2 one
// window at a time (k_mc_count) each 4-word group waits for 20 dependent L2
// loads.  Here a block copies those two contiguous runs of bit words, each
// about the tile's own bits, into shared memory with bulk TMA copies
// (cp.async.bulk, completion on an mbarrier) and counts from there.  The
// outputs are k_mc_count's, bit for bit: packed counts wc and per-tile
// totals.  (The same staging of the threshold's three planes, with the kept
// and used masks in one pass, measured slower than k_thr_kept + k_thr_used
// at 512^3 -- 0.155 ms against 0.138 ms for the whole count pass -- and is
// not built.)
#include "common.cuh"
#include "kernels.cuh"
#include "mc_case.cuh"
#include "mc_words.cuh"
#include "tma.cuh"

namespace daxgb {

namespace {

// 32 bits of a staged range from bit `lpos` (relative to the range's first
// word) and the +x neighbours (bits_at2 on shared memory).
__device__ __forceinline__ void s_bits2(const uint32_t* s, long long lpos, uint32_t& a,
                                        uint32_t& a1) {
  const int w = (int)(lpos >> 5);
  const unsigned sh = (unsigned)(lpos & 31);
  const uint32_t w0 = s[w], w1 = s[w + 1];
  a = __funnelshift_r(w0, w1, sh);
  a1 = __funnelshift_rc(w0, w1, sh + 1u);
}

// row_windows4 on shared memory.
__device__ __forceinline__ void s_windows4(const uint32_t* s, long long lpos, uint32_t (&a)[4],
                                           uint32_t (&a1)[4]) {
  const int w = (int)(lpos >> 5);
  const unsigned sh = (unsigned)(lpos & 31);
  uint32_t x[5];
#pragma unroll
  for (int e = 0; e < 5; ++e) x[e] = s[w + e];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    a[e] = __funnelshift_r(x[e], x[e + 1], sh);
    a1[e] = __funnelshift_rc(x[e], x[e + 1], sh + 1u);
  }
}

// The staged ranges of tile `tile`: range p (rows one plane up per p)
// starts at bit word w0[p] (a multiple of 4) and holds n[p] words.
struct Ranges {
  long long w0[2];
  int n[2];
};

__device__ __forceinline__ Ranges tile_ranges(const Grid& g, long long nwords, int tile) {
  const long long W = g.R * g.wr;
  const long long t0 = (long long)tile * kScanTile;
  const long long te = t0 + kScanTile < W ? t0 + kScanTile : W;
  const long long r_lo = div_by((unsigned)t0, g.mwr), r_hi = div_by((unsigned)(te - 1), g.mwr);
  const long long dz = (long long)g.nx * g.ny;
  Ranges R;
  for (int p = 0; p < 2; ++p) {
    R.w0[p] = 0;
    R.n[p] = 0;
    const long long off = (long long)p * dz;
    long long lo = r_lo * (long long)g.nx + off - 64;
    const long long hi = (r_hi + 2) * (long long)g.nx + off + 64;  // bits, exclusive
    if (lo < 0) lo = 0;
    long long a = (lo >> 5) & ~3ll;
    long long b = ((hi + 31) >> 5) + 2;
    b = (b + 3) & ~3ll;
    if (b > nwords) b = nwords;
    if (a >= b) continue;
    R.w0[p] = a;
    R.n[p] = (int)(b - a);  // <= the staged range's words (staged_range_words)
  }
  return R;
}

// Copies the tile's ranges into s (range p at p * range_words) and waits for
// them (bounded); false when they did not arrive in time.
__device__ bool stage_tile(const uint32_t* bits, const Ranges& R, uint32_t* s, int range_words,
                           uint64_t* bar, unsigned& phase, unsigned long long policy) {
  fence_proxy_async();  // the previous tile's reads of s before the copies
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned bytes = 0;
    for (int p = 0; p < 2; ++p) bytes += 4u * (unsigned)R.n[p];
    if (bytes) {
      mbar_arrive_tx(bar, bytes);
      for (int p = 0; p < 2; ++p)
        if (R.n[p]) bulk_load(s + p * range_words, bits + R.w0[p], 4u * (unsigned)R.n[p], bar, policy);
    } else {
      mbar_arrive(bar);
    }
  }
  Spin sp;
  bool ok = true;
  while (!mbar_test(bar, phase))
    if (!sp.more()) {
      ok = false;
      break;
    }
  ok = __syncthreads_and(ok) != 0;
  if (!ok && threadIdx.x == 0) {
    // wait (bounded) once more for the copies, so that none lands in shared
    // memory after the block leaves
    Spin sp2;
    while (!mbar_test(bar, phase) && sp2.more()) {
    }
  }
  phase ^= 1u;
  return ok;
}

// Packed counts (triangles << 16 | crossing edges) of row words g0..g0+3
// (0 past W) from the staged ranges: sa holds rows r_lo .. r_hi + 1, its
// first word at global bit ba; sb the same rows one plane up, its first word
// at global bit bb + dz (so a row's own position minus bb indexes its
// plane-up row).
__device__ __forceinline__ void staged_counts4(const Grid& g, long long W, long long g0,
                                               const uint32_t* sa, const uint32_t* sb,
                                               long long ba, long long bb,
                                               const unsigned char* s_nf, uint32_t (&out)[4]) {
  const long long dy = g.nx;
  out[0] = out[1] = out[2] = out[3] = 0u;
  int m;
  const unsigned r = split_word(g, (unsigned)g0, m);
  if (m + 4 <= g.wr && g0 + 4 <= W) {
    int j, k;
    split_row(g, r, j, k);
    const bool hy = j < g.ny - 1, hz = k < g.nz - 1;
    const long long pos = (long long)r * g.nx + 32ll * m;
    uint32_t a[4], a1[4], b[4] = {0, 0, 0, 0}, b1[4] = {0, 0, 0, 0}, c[4] = {0, 0, 0, 0},
             c1[4] = {0, 0, 0, 0}, d[4] = {0, 0, 0, 0}, d1[4] = {0, 0, 0, 0};
    s_windows4(sa, pos - ba, a, a1);
    if (hy) s_windows4(sa, pos + dy - ba, b, b1);
    if (hz) s_windows4(sb, pos - bb, c, c1);
    if (hy && hz) s_windows4(sb, pos + dy - bb, d, d1);
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
                               low_mask(g.nx - 1 - 32 * (m + q)), s_nf);
      }
    }
  } else {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const long long gw = g0 + q;
      if (gw >= W) break;
      int mq, jq, kq;
      const unsigned rq = split_word(g, (unsigned)gw, mq);
      split_row(g, rq, jq, kq);
      const bool hy = jq < g.ny - 1, hz = kq < g.nz - 1;
      const long long pos = (long long)rq * g.nx + 32ll * mq;
      CornerWords w{};
      s_bits2(sa, pos - ba, w.a, w.a1);
      if (hy) s_bits2(sa, pos + dy - ba, w.b, w.b1);
      if (hz) s_bits2(sb, pos - bb, w.c, w.c1);
      if (hy && hz) s_bits2(sb, pos + dy - bb, w.d, w.d1);
      out[q] = packed_counts(w, hy, hz, low_mask(g.nx - 32 * mq), low_mask(g.nx - 1 - 32 * mq),
                             s_nf);
    }
  }
}

// Marching cubes, one grid: packed counts (triangles << 16 | crossing
// edges) of every row word and the per-tile totals, as k_mc_count writes
// them.  Range 0 holds rows r_lo .. r_hi + 1, range 1 the same rows one
// plane up.
__global__ void __launch_bounds__(256) k_mc_count_staged(Grid g, const uint32_t* __restrict__ bits,
                                                         long long nwords, uint32_t* __restrict__ wc,
                                                         uint32_t* __restrict__ tile_tot, int tiles,
                                                         int range_words, Info* __restrict__ info) {
  extern __shared__ __align__(128) uint32_t s_bits[];  // [2][range_words]
  __shared__ __align__(8) uint64_t s_bar;
  __shared__ unsigned char s_nf[256];  // NumFaces
  __shared__ uint32_t s_red[24];
  s_nf[threadIdx.x] = (unsigned char)mc_num_tris(threadIdx.x);
  if (threadIdx.x == 0) {
    mbar_init(&s_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  pdl_trigger();
  pdl_wait();  // the classification's bits
  unsigned long long policy;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(policy));
  unsigned phase = 0;
  const long long W = g.R * g.wr;
  const long long dy = g.nx, dz = (long long)g.nx * g.ny;
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const Ranges R = tile_ranges(g, nwords, tile);
    if (!stage_tile(bits, R, s_bits, range_words, &s_bar, phase, policy)) {
      if (threadIdx.x == 0) atomicExch(&info->aborted, 1);
      return;  // every copy of this block has arrived or been waited for
    }
    const uint32_t* sa = s_bits;
    const uint32_t* sb = s_bits + range_words;
    const long long ba = 32 * R.w0[0], bb = 32 * R.w0[1] - dz;  // global bit of local 0, minus the plane
    uint32_t st = 0, sv = 0, sact = 0;
#pragma unroll 1
    for (int e = 0; e < kScanItems / 4; ++e) {
      const long long g0 = (long long)tile * kScanTile + 4ll * (threadIdx.x + 256 * e);
      if (g0 >= W) break;
      uint32_t out[4];
      staged_counts4(g, W, g0, sa, sb, ba, bb, s_nf, out);
      if (g0 + 4 <= W) {
        *reinterpret_cast<uint4*>(wc + g0) = make_uint4(out[0], out[1], out[2], out[3]);
      } else {
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (g0 + q < W) wc[g0 + q] = out[q];
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        st += out[q] >> 16;
        sv += out[q] & 0xffffu;
        sact += out[q] ? 1u : 0u;
      }
    }
    block_sum3(st, sv, sact, s_red);
    if (threadIdx.x == 0) {
      tile_tot[tile] = st;
      tile_tot[tiles + tile] = sv;
      tile_tot[2 * tiles + tile] = sact;
    }
  }
}


// Words a staged range can need: the tile's rows (at most kScanTile / wr + 2
// of them) plus the two rows after, the margins and the alignment.
int staged_range_words(const Grid& g) {
  const long long rows = kScanTile / g.wr + 2 + 2;
  const long long w = (rows * (long long)g.nx + 128) / 32 + 8;
  return (int)((w + 3) & ~3ll);
}

constexpr size_t kStagedMaxBytes = 120 * 1024;

template <typename K>
bool opt_in(K kernel, size_t smem) {
  static int done[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return false;
  if (!done[dev]) {
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kStagedMaxBytes) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    done[dev] = 1;
  }
  return smem <= kStagedMaxBytes;
}

}  // namespace

bool launch_mc_count_staged(const Grid& g, const uint32_t* bits, long long nwords,
                            const WordOffsets& o, Info* info, int num_sms, cudaStream_t s) {
  const int rw = staged_range_words(g);
  const size_t smem = 2 * 4 * (size_t)rw;
  if (!opt_in(k_mc_count_staged, smem)) return false;
  const int tiles = word_scan_tiles(g.R * g.wr);
  const int blocks = resident_blocks(k_mc_count_staged, 256, smem, num_sms, tiles, kPassCount);
  // a failed launch is reported by the caller's launch check
  (void)launch_pdl(k_mc_count_staged, blocks, 256, smem, s, g, bits, nwords, o.wc, o.tile, tiles, rw,
                   info);
  return true;
}


}  // namespace daxgb
