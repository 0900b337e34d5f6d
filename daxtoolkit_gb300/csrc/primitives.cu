// Generic data-parallel primitives of the device adapter
// (dax::cont::DeviceAdapterAlgorithm, dax/cont/internal/DeviceAdapterAlgorithm.h:44-331;
// the reference's generic versions are dax/cont/internal/DeviceAdapterAlgorithmGeneral.h):
// ScanInclusive / ScanExclusive, Sort / SortByKey, Unique, LowerBounds /
// UpperBounds and StreamCompact, on the element types the Dax pipelines use
// (dax::Id = int32, int64, unsigned, dax::Scalar = float) with values of up
// to 16 bytes (a dax::Vector3 is 12).
//
// Tiles: the float scan and the sort work on kPTile elements (256 threads x
// 16), the integer scan and the compaction on 64 KB of elements:
//   scan     integers: one pass, each tile's prefix found by a decoupled
//            look-back over the tiles before it; floats (and the sort's
//            histograms): reduce-then-scan, tile sums, one block scanning
//            the sums, then each tile scanned with its prefix, whose fixed
//            order of additions gives the same result on every run (in place
//            allowed for both);
//   sort     LSD radix sort, 8-bit digits, stable: per pass a per-tile digit
//            histogram, a scan of the histograms in digit-major order, and a
//            scatter that ranks each element among equal digits of its tile
//            (warp match + per-warp counts) in element order;
//   compact  one pass on the integer scan's machinery: a tile's kept
//            elements are counted as it lands, its offset found by the
//            look-back, and the kept elements written at their places
//            (Unique = compact of "differs from the previous key", in place;
//            StreamCompact = compact of "stencil != 0").
#include <cstdint>
#include <cstring>
#include <string>

#include "../../include/dax_gb300.h"
#include "common.cuh"
#include "kernels.cuh"
#include "tma.cuh"

namespace daxgb {

namespace {

constexpr int kPT = 256;
constexpr int kPI = 16;
constexpr int kPTile = kPT * kPI;

int ptiles(long long n) { return (int)((n + kPTile - 1) / kPTile); }

// Integer sums wrap like the reference's dax::Id arithmetic: accumulate in
// the unsigned type of the same width.
template <typename T> struct Acc { typedef T type; };
template <> struct Acc<int32_t> { typedef uint32_t type; };
template <> struct Acc<int64_t> { typedef unsigned long long type; };

template <typename A>
__device__ __forceinline__ A block_exclusive(A v, A* s_warp, A* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  A x = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const A y = __shfl_up_sync(kFull, x, d);
    if (lane >= d) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  A base = 0, tot = 0;
#pragma unroll
  for (int w = 0; w < kPT / 32; ++w) {
    if (w < warp) base += s_warp[w];
    tot += s_warp[w];
  }
  __syncthreads();
  *total = tot;
  return base + x - v;
}

// ---- scan -----------------------------------------------------------------

template <typename T>
__global__ void __launch_bounds__(kPT) k_tile_sum(const T* __restrict__ in, long long n,
                                                  typename Acc<T>::type* __restrict__ sums,
                                                  int tiles) {
  typedef typename Acc<T>::type A;
  __shared__ A s_warp[kPT / 32];
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    A v = 0;
    const long long b = (long long)tile * kPTile;
#pragma unroll 4
    for (int e = 0; e < kPI; ++e) {
      const long long i = b + e * kPT + threadIdx.x;
      if (i < n) v += (A)in[i];
    }
    A tot;
    block_exclusive(v, s_warp, &tot);
    if (threadIdx.x == 0) sums[tile] = tot;
  }
}

// One block: exclusive scan of the tile sums in place; the grand total goes
// to sums[tiles].
template <typename A>
__global__ void __launch_bounds__(1024) k_scan_sums(A* __restrict__ sums, int tiles) {
  __shared__ A s_warp[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  A carry = 0;
  for (int c0 = 0; c0 < tiles; c0 += 1024) {
    const int i = c0 + threadIdx.x;
    const A v = i < tiles ? sums[i] : (A)0;
    A x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const A y = __shfl_up_sync(kFull, x, d);
      if (lane >= d) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    A base = 0, tot = 0;
    for (int w = 0; w < 32; ++w) {
      if (w < warp) base += s_warp[w];
      tot += s_warp[w];
    }
    if (i < tiles) sums[i] = carry + base + x - v;
    carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) sums[tiles] = carry;
}

// A tile is loaded with coalesced (striped) loads into shared memory, each
// thread then scans 16 consecutive elements, and the results leave the same
// way.  The tile's prefix comes from the scanned sums.  Every element of a
// tile is read before any is written: in place is fine.
__device__ __forceinline__ int pad(int i) { return i + (i >> 5); }

template <typename T>
__global__ void __launch_bounds__(kPT) k_tile_scan(const T* __restrict__ in, T* out, long long n,
                                                   const typename Acc<T>::type* __restrict__ pre,
                                                   int tiles, int exclusive) {
  typedef typename Acc<T>::type A;
  __shared__ A s_warp[kPT / 32];
  __shared__ A s_t[kPTile + kPTile / 32];
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const long long b = (long long)tile * kPTile;
#pragma unroll
    for (int e = 0; e < kPI; ++e) {
      const int li = e * kPT + threadIdx.x;
      s_t[pad(li)] = b + li < n ? (A)in[b + li] : (A)0;
    }
    __syncthreads();
    A v[kPI];
    A sum = 0;
#pragma unroll
    for (int e = 0; e < kPI; ++e) {
      v[e] = s_t[pad(threadIdx.x * kPI + e)];
      sum += v[e];
    }
    A tot;
    A run = pre[tile] + block_exclusive(sum, s_warp, &tot);
#pragma unroll
    for (int e = 0; e < kPI; ++e) {
      const A next = run + v[e];
      s_t[pad(threadIdx.x * kPI + e)] = exclusive ? run : next;
      run = next;
    }
    __syncthreads();
#pragma unroll
    for (int e = 0; e < kPI; ++e) {
      const int li = e * kPT + threadIdx.x;
      if (b + li < n) out[b + li] = (T)s_t[pad(li)];
    }
    __syncthreads();
  }
}

// Two-level scan of many sums: chunks of 1024 scanned in parallel (each
// chunk's total to aux), the totals scanned by one block, then added back.
template <typename A>
__global__ void __launch_bounds__(1024) k_chunk_scan(A* __restrict__ v, int count,
                                                     A* __restrict__ aux) {
  __shared__ A s_warp[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int i = blockIdx.x * 1024 + threadIdx.x;
  const A x0 = i < count ? v[i] : (A)0;
  A x = x0;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const A y = __shfl_up_sync(kFull, x, d);
    if (lane >= d) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  A base = 0, tot = 0;
  for (int w = 0; w < 32; ++w) {
    if (w < warp) base += s_warp[w];
    tot += s_warp[w];
  }
  if (i < count) v[i] = base + x - x0;
  if (threadIdx.x == 0) aux[blockIdx.x] = tot;
}

template <typename A>
__global__ void __launch_bounds__(1024) k_chunk_add(A* __restrict__ v, int count,
                                                    const A* __restrict__ aux, int chunks) {
  const int i = blockIdx.x * 1024 + threadIdx.x;
  if (i < count) v[i] += aux[blockIdx.x];
  if (blockIdx.x == 0 && threadIdx.x == 0) v[count] = aux[chunks];
}

// Exclusive scan of v[0..count) in place, total to v[count]; aux holds
// count / 1024 + 2 entries.
template <typename A>
void scan_sums(A* v, int count, A* aux, cudaStream_t s) {
  if (count <= 8192) {
    k_scan_sums<A><<<1, 1024, 0, s>>>(v, count);
    return;
  }
  const int chunks = (count + 1023) / 1024;
  k_chunk_scan<A><<<chunks, 1024, 0, s>>>(v, count, aux);
  k_scan_sums<A><<<1, 1024, 0, s>>>(aux, chunks);
  k_chunk_add<A><<<chunks, 1024, 0, s>>>(v, count, aux, chunks);
}

int sum_slots(long long n) { return ptiles(n) + 1 + ptiles(n) / 1024 + 2; }

int resident(const void* kernel, int threads, int num_sms, long long want) {
  int per = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, 0) != cudaSuccess ||
      per < 1)
    per = 1;
  const long long cap = (long long)num_sms * per;
  return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

template <typename T>
void scan_t(const T* in, T* out, long long n, bool exclusive, void* scratch, void* d_total,
            int num_sms, cudaStream_t s) {
  typedef typename Acc<T>::type A;
  const int tiles = ptiles(n);
  A* sums = static_cast<A*>(scratch);
  const int b = resident((const void*)k_tile_sum<T>, kPT, num_sms, tiles);
  k_tile_sum<T><<<b, kPT, 0, s>>>(in, n, sums, tiles);
  scan_sums<A>(sums, tiles, sums + tiles + 1, s);
  k_tile_scan<T><<<b, kPT, 0, s>>>(in, out, n, sums, tiles, exclusive ? 1 : 0);
  if (d_total) cudaMemcpyAsync(d_total, sums + tiles, sizeof(T), cudaMemcpyDeviceToDevice, s);
}

// ---- single-pass scan of integer elements ---------------------------------
//
// One read and one write of every element, by one persistent block an SM.
// The block takes tiles (64 KB) from a ticket counter and keeps kSStages of
// them in a ring of shared-memory stages, each filled by one bulk TMA copy.
// Its eight compute warps reduce a tile as soon as it lands and publish the
// tile's sum (AGG); a ninth warp then finds the tile's prefix by looking back
// over the published states of the tiles before it (32 a step, lane = tile)
// and publishes the inclusive prefix (INC), while the compute warps reduce
// the next tile; they then scan the tile in shared memory and write it back
// with one bulk copy, and the stage loads the block's next ticket.
//
// Why this shape (measured at 2^30 int32): a plain copy with the same
// tickets and bulk copies runs at 7.1 TB/s, but a block that waits in its own
// look-back holds its tile and starves the loads (one tile a block: 0.61 of
// the copy bandwidth); the look-back step is an L2 round trip and the prefix
// crosses the ~152 tiles in flight 32 tiles a step, so the look-back runs
// beside the reductions instead.  Wider steps and smaller tiles polled more
// and measured slower; a short sleep between polls helped a little.
//
// Tiles are taken in ticket order and each block's tickets increase in the
// order it processes them, so the smallest unfinished tile always has all
// its predecessors' sums published and its block working on it: no tile
// waits on a later one.  Every wait is still bounded (Spin), and a wait that
// runs out marks the scan failed (DAX_GB300_ERROR_TIMEOUT when the total is
// read).
//
// Integer sums wrap, so any split of the look-back gives the same result;
// float scans keep the deterministic reduce-then-scan above.
//
// Shared-memory layout of a tile: warp w owns elements [w, w + 1) * kWarpElems;
// its lane reads and writes 16-byte chunk c at element c * 32 * E + lane * E
// of that range (E elements a chunk), so every access of a warp covers 512
// consecutive bytes and no two lanes share a bank.  The scan goes chunk by
// chunk: a lane's E elements, a warp scan of the chunk totals, and the carry
// of the chunks before.  Arrays that are not 16-byte aligned, and the ragged
// last tile, are loaded and stored element by element instead.
//
// Scratch (zeroed before the launch, the states included): ticket, error,
// total, then per tile its state: flag << 32 | sum in one 64-bit word for
// 32-bit sums, two such words (low and high halves) for 64-bit sums.
constexpr unsigned kStAgg = 1u, kStInc = 2u;
constexpr size_t kScanHead = 64;
constexpr int kSThreads = 256;                                // compute threads
constexpr int kSChunks = 16;                                  // 16-byte chunks a thread
constexpr unsigned kSTileBytes = 16u * kSChunks * kSThreads;  // 64 KB
constexpr int kSStages = 3;

struct ScanCtl {
  unsigned ticket, error;
  unsigned long long total;
};

__device__ __forceinline__ unsigned long long ld_relaxed64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

template <typename A> struct TileStates;

template <> struct TileStates<uint32_t> {
  unsigned long long* word;
  __host__ __device__ static size_t bytes(int tiles) { return (size_t)tiles * 8; }
  __host__ __device__ static size_t clear_bytes(int tiles) { return (size_t)tiles * 8; }
  __host__ __device__ explicit TileStates(char* base, int) : word((unsigned long long*)base) {}
  __device__ void publish(int t, unsigned flag, uint32_t v) const {
    st_relaxed64(word + t, (unsigned long long)flag << 32 | v);
  }
  __device__ unsigned read(int t, uint32_t& v) const {
    const unsigned long long w = ld_relaxed64(word + t);
    v = (uint32_t)w;
    return (unsigned)(w >> 32);
  }
};

// 64-bit sums: two 64-bit words, each the flag above 32 bits of the sum,
// stored and loaded as one 16-byte access (each word is single-copy atomic,
// the pair need not be); words with different flags are a read that caught a
// publication half done, and count as not yet published.
template <> struct TileStates<unsigned long long> {
  unsigned long long* pair;
  __host__ __device__ static size_t bytes(int tiles) { return (size_t)tiles * 16; }
  __host__ __device__ static size_t clear_bytes(int tiles) { return (size_t)tiles * 16; }
  __host__ __device__ explicit TileStates(char* base, int) : pair((unsigned long long*)base) {}
  __device__ void publish(int t, unsigned flag, unsigned long long v) const {
    const unsigned long long f = (unsigned long long)flag << 32;
    asm volatile("st.relaxed.gpu.global.v2.u64 [%0], {%1, %2};" ::"l"(pair + 2 * t),
                 "l"(f | (v & 0xffffffffull)), "l"(f | (v >> 32))
                 : "memory");
  }
  __device__ unsigned read(int t, unsigned long long& v) const {
    unsigned long long lo, hi;
    asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];"
                 : "=l"(lo), "=l"(hi)
                 : "l"(pair + 2 * t)
                 : "memory");
    const unsigned f = (unsigned)(lo >> 32);
    if (f != (unsigned)(hi >> 32)) return 0u;
    v = (lo & 0xffffffffull) | (hi << 32);
    return f;
  }
};

template <typename A>
__device__ __forceinline__ A warp_inclusive(A x, int lane) {
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const A y = __shfl_up_sync(kFull, x, d);
    if (lane >= d) x += y;
  }
  return x;
}

// The exclusive prefix of `tile` from the states of the tiles before it
// (one warp; every lane returns it).  A step reads the states of tiles
// top - lane, polls those not yet published (a short sleep between polls),
// and ends at the nearest inclusive prefix.  Sets `failed` if a wait ran out.
template <typename A>
__device__ A look_back(const TileStates<A>& st, int tile, int lane, bool& failed) {
  A prefix = 0;
  for (int top = tile - 1; top >= 0; top -= 32) {
    const int t = top - lane;
    A x = 0;
    unsigned f = kStInc;  // before tile 0: an inclusive zero
    if (t >= 0) {
      Spin spin;
      while ((f = st.read(t, x)) == 0u) {
        if (!spin.more()) {
          failed = true;
          f = kStInc;
          x = 0;
          break;
        }
        __nanosleep(300);
      }
    }
    // the nearest tile with its inclusive prefix ends the look-back
    const unsigned incl = __ballot_sync(kFull, f == kStInc);
    const int last = incl ? __ffs(incl) - 1 : 31;
    A part = lane <= last ? x : (A)0;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) part += __shfl_xor_sync(kFull, part, d);
    prefix += part;
    if (incl) break;
  }
  return prefix;
}

__device__ __forceinline__ void compute_sync() {  // the compute warps only
  asm volatile("bar.sync 1, %0;" ::"r"(kSThreads) : "memory");
}

__device__ __forceinline__ bool wait_phase(uint64_t* bar, unsigned parity) {
  Spin sp;
  while (!mbar_test(bar, parity))
    if (!sp.more()) return false;
  return true;
}

// A lane's first 16-byte chunk of a staged tile: warp w owns elements
// [w, w + 1) * (tile / warps); chunk c of the lane is 32 * c chunks further.
template <typename Staged>
__device__ __forceinline__ Staged* lane_chunk0(Staged* s_data, int warp, int lane) {
  constexpr int kWarpElems = (int)(kSTileBytes / sizeof(Staged)) / (kSThreads / 32);
  return s_data + warp * kWarpElems + lane * (16 / (int)sizeof(Staged));
}

// The single-pass driver the integer scan and the compaction share (run by
// one persistent block an SM, kSThreads compute threads plus a look-back
// warp).  Op is the pass's policy:
//   Staged, Sum        the ring's element type; the tile sums
//   src                the staged array
//   on_take(t)         thread 0, when a stage's bulk copy of whole tile t is issued
//   on_land(k, b, aux) thread 0, when the tile of stage k (first element b)
//                      has landed, before it is summed; aux[k] is the pass's
//                      own per-stage word
//   thread_sum(...)    a compute thread's part of the tile's sum
//   finish(...)        the compute threads' output of the tile, given the
//                      sum of everything before the thread's first element
//   store(...)         after finish and a barrier: the stage's bytes out
//                      (the scan), or nothing
template <class Op>
__device__ __forceinline__ void single_pass(const Op& op, long long n, int tiles, ScanCtl* ctl,
                                            char* states, int bulk) {
  typedef typename Op::Staged Staged;
  typedef typename Op::Sum Sum;
  constexpr int kTileElems = (int)(kSTileBytes / sizeof(Staged));
  constexpr int kWarps = kSThreads / 32;
  const TileStates<Sum> st(states, tiles);
  extern __shared__ __align__(128) unsigned char scan_smem[];
  __shared__ __align__(8) uint64_t b_full[kSStages], b_agg[kSStages], b_pre[kSStages];
  __shared__ int s_tile[kSStages];  // the stage's occupant
  __shared__ int s_seen[kSStages];  // the occupant as handed to the look-back warp
  __shared__ Sum s_tot[kSStages], s_pre[kSStages], s_wsum[kSStages][kWarps];
  __shared__ unsigned long long s_aux[kSStages];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // a tile is copied in bulk when it is whole and the arrays are 16-byte aligned
  auto whole = [&](int t) { return bulk && (long long)(t + 1) * kTileElems <= n; };
  auto stage = [&](int k) { return reinterpret_cast<Staged*>(scan_smem + (size_t)k * kSTileBytes); };
  unsigned long long policy = 0;  // read once: evict first
  auto fill = [&](int k) {        // thread 0: the stage's next tile
    const int t = (int)atomicAdd(&ctl->ticket, 1u);
    s_tile[k] = t;
    if (t < tiles && whole(t)) {
      mbar_arrive_tx(&b_full[k], kSTileBytes);
      bulk_load(stage(k), op.src + (long long)t * kTileElems, kSTileBytes, &b_full[k], policy);
      op.on_take(t);
    }
  };
  if (threadIdx.x == 0) {
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(policy));
    for (int k = 0; k < kSStages; ++k) {
      mbar_init(&b_full[k], 1);
      mbar_init(&b_agg[k], 1);
      mbar_init(&b_pre[k], 1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    for (int k = 0; k < kSStages; ++k) fill(k);
  }
  __syncthreads();

  if (warp == kWarps) {
    // the look-back warp: the block's tiles in order
    for (int i = 0;; ++i) {
      const int k = i % kSStages;
      bool failed = !wait_phase(&b_agg[k], (i / kSStages) & 1);
      const int tile = s_seen[k];
      if (tile >= tiles) break;
      const Sum tot = s_tot[k];
      const Sum prefix = look_back(st, tile, lane, failed);
      failed = __any_sync(kFull, failed);
      if (lane == 0) {
        if (tile > 0) st.publish(tile, kStInc, prefix + tot);
        if (failed) atomicOr(&ctl->error, 1u);
        if (tile == tiles - 1) ctl->total = (unsigned long long)(prefix + tot);
        s_pre[k] = prefix;
        mbar_arrive(&b_pre[k]);
      }
      __syncwarp();
    }
    return;
  }

  // compute warps.  reduce(k): the stage's tile lands (bulk) or is loaded
  // here (elements), is summed, and its sum published and handed on; false
  // once the tiles are done (the later stages hold later tickets)
  unsigned fullp = 0;  // bit k: the parity stage k's next bulk copy completes
  auto reduce = [&](int k) -> bool {
    const int tile = s_tile[k];
    if (tile >= tiles) {
      if (threadIdx.x == 0) {
        s_seen[k] = tile;
        mbar_arrive(&b_agg[k]);
      }
      return false;
    }
    Staged* s_data = stage(k);
    const long long b = (long long)tile * kTileElems;
    bool ok = true;
    if (whole(tile)) {
      ok = wait_phase(&b_full[k], (fullp >> k) & 1u);
      fullp ^= 1u << k;
    } else {
      const long long cnt = n - b < kTileElems ? n - b : kTileElems;
      for (int i = threadIdx.x; i < kTileElems; i += kSThreads)
        s_data[i] = i < cnt ? op.src[b + i] : (Staged)0;
      compute_sync();
    }
    if (threadIdx.x == 0) op.on_land(k, b, s_aux);
    Sum sum = op.thread_sum(s_data, k, b, warp, lane, s_aux);
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) sum += __shfl_xor_sync(kFull, sum, d);
    if (lane == 0) s_wsum[k][warp] = sum;
    compute_sync();
    if (threadIdx.x == 0) {
      Sum tot = 0;
      for (int w = 0; w < kWarps; ++w) tot += s_wsum[k][w];
      st.publish(tile, tile == 0 ? kStInc : kStAgg, tot);
      if (!ok) {
        atomicOr(&ctl->error, 1u);
        // wait (bounded) once more for the copy, so that none lands in
        // shared memory after the block leaves
        wait_phase(&b_full[k], (fullp >> k) & 1u ^ 1u);
      }
      s_tot[k] = tot;
      s_seen[k] = tile;
      mbar_arrive(&b_agg[k]);
    }
    return true;
  };

  bool more = reduce(0);
  for (int i = 0; more; ++i) {
    const int k = i % kSStages;
    const bool next = reduce((i + 1) % kSStages);  // beside this tile's look-back
    wait_phase(&b_pre[k], (i / kSStages) & 1);      // a timeout is the look-back warp's to report
    const int tile = s_seen[k];
    const long long b = (long long)tile * kTileElems;
    const long long cnt = n - b < kTileElems ? n - b : kTileElems;
    Sum run = s_pre[k];
    for (int w = 0; w < warp; ++w) run += s_wsum[k][w];
    Staged* s_data = stage(k);
    op.finish(s_data, k, b, run, warp, lane, s_aux);
    // the tile's shared-memory writes before the bulk copy reads them (and
    // its reads before the stage's next bulk copy writes it)
    fence_proxy_async();
    compute_sync();
    op.store(s_data, b, cnt, whole(tile));
    compute_sync();  // element stores read the stage before it is refilled
    if (threadIdx.x == 0) fill(k);
    compute_sync();  // s_tile[k]
    more = next;
  }
}

// The integer scan's policy: sums of the elements; the tile is scanned in
// shared memory chunk by chunk (a lane's E elements, a warp scan of the chunk
// totals, the carry of the chunks before) and written back whole.
template <typename T>
struct ScanPass {
  typedef typename Acc<T>::type Staged;
  typedef typename Acc<T>::type Sum;
  static constexpr int E = 16 / (int)sizeof(Staged);
  struct Chunk { Staged e[E]; };
  const Staged* src;
  T* out;
  int exclusive;
  __device__ void on_take(int) const {}
  __device__ void on_land(int, long long, unsigned long long*) const {}
  __device__ Sum thread_sum(Staged* s_data, int, long long, int warp, int lane,
                            const unsigned long long*) const {
    const Chunk* sc = reinterpret_cast<const Chunk*>(lane_chunk0(s_data, warp, lane));
    Sum sum = 0;
#pragma unroll 4
    for (int c = 0; c < kSChunks; ++c) {
      const Chunk x = sc[32 * c];
#pragma unroll
      for (int e = 0; e < E; ++e) sum += x.e[e];
    }
    return sum;
  }
  __device__ void finish(Staged* s_data, int, long long, Sum run, int warp, int lane,
                         const unsigned long long*) const {
    Chunk* sc = reinterpret_cast<Chunk*>(lane_chunk0(s_data, warp, lane));
#pragma unroll 4
    for (int c = 0; c < kSChunks; ++c) {
      Chunk x = sc[32 * c];
      Sum l[E];
      Sum acc = 0;
#pragma unroll
      for (int e = 0; e < E; ++e) {
        l[e] = acc;  // exclusive within the lane's chunk
        acc += x.e[e];
      }
      const Sum ci = warp_inclusive(acc, lane);
      const Sum base = run + ci - acc;
#pragma unroll
      for (int e = 0; e < E; ++e) x.e[e] = base + l[e] + (exclusive ? (Sum)0 : x.e[e]);
      sc[32 * c] = x;
      run += __shfl_sync(kFull, ci, 31);
    }
  }
  __device__ void store(Staged* s_data, long long b, long long cnt, bool whole) const {
    if (whole) {
      if (threadIdx.x == 0) bulk_store_and_wait_read(out + b, s_data, kSTileBytes);
    } else {
      for (int j = threadIdx.x; j < cnt; j += kSThreads) out[b + j] = (T)s_data[j];
    }
  }
};

template <typename T>
__global__ void __launch_bounds__(kSThreads + 32, 1)
    k_scan_single(ScanPass<T> op, long long n, int tiles, ScanCtl* ctl, char* states, int bulk) {
  single_pass(op, n, tiles, ctl, states, bulk);
}

template <typename Staged>
int single_pass_tiles(long long n) {
  const long long per = kSTileBytes / sizeof(Staged);
  return (int)((n + per - 1) / per);
}

template <typename T>
size_t single_scan_bytes(long long n) {
  typedef typename Acc<T>::type A;
  return kScanHead + TileStates<A>::bytes(single_pass_tiles<A>(n));
}

// Clears the scratch's control words and tile states and launches one block
// an SM of `kernel` (the ring is above the 48 KB of shared memory a launch
// gets without opting in: set once per device and kernel; a failure shows
// as the launch's error).
template <class Op>
void launch_single_pass(void (*kernel)(Op, long long, int, ScanCtl*, char*, int), const Op& op,
                        long long n, int bulk, char* scratch, int num_sms, cudaStream_t s) {
  typedef typename Op::Staged Staged;
  typedef typename Op::Sum Sum;
  const size_t smem = (size_t)kSStages * kSTileBytes;
  static int opted[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && !opted[dev]) {
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) ==
            cudaSuccess &&
        cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared) == cudaSuccess)
      opted[dev] = 1;
  }
  const int tiles = single_pass_tiles<Staged>(n);
  const int blocks = tiles < num_sms ? tiles : num_sms;
  cudaMemsetAsync(scratch, 0, kScanHead + TileStates<Sum>::clear_bytes(tiles), s);
  kernel<<<blocks, kSThreads + 32, smem, s>>>(op, n, tiles, reinterpret_cast<ScanCtl*>(scratch),
                                              scratch + kScanHead, bulk);
}

template <typename T>
void scan_single(const T* in, T* out, long long n, bool exclusive, char* scratch, int num_sms,
                 cudaStream_t s) {
  typedef typename Acc<T>::type A;
  const ScanPass<T> op{reinterpret_cast<const A*>(in), out, exclusive ? 1 : 0};
  const int bulk = ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15) == 0;
  launch_single_pass(k_scan_single<T>, op, n, bulk, scratch, num_sms, s);
}

// ---- radix sort -------------------------------------------------------------

// Keys as unsigned integers whose order is the key type's order (ascending);
// descending order is the complement.  Floats: negative values have all bits
// flipped, the others only the sign bit (IEEE total order for non-NaN keys).
template <typename U> struct Bits;
template <> struct Bits<uint32_t> {
  static constexpr uint32_t sign = 0x80000000u;
};
template <> struct Bits<unsigned long long> {
  static constexpr unsigned long long sign = 0x8000000000000000ull;
};

template <typename U>
__device__ __forceinline__ U to_ordered(U x, int kind, bool desc) {
  // kind: 0 unsigned, 1 signed, 2 float
  U t = x;
  if (kind == 1) t = x ^ Bits<U>::sign;
  if (kind == 2) t = (x & Bits<U>::sign) ? (U)~x : (U)(x ^ Bits<U>::sign);
  return desc ? (U)~t : t;
}

template <typename U>
__device__ __forceinline__ U from_ordered(U t, int kind, bool desc) {
  if (desc) t = (U)~t;
  if (kind == 1) return t ^ Bits<U>::sign;
  if (kind == 2) return (t & Bits<U>::sign) ? (U)(t ^ Bits<U>::sign) : (U)~t;
  return t;
}

// The ordering map of a sort pass: keys read from the caller's array are
// mapped to ordered bits as they are loaded (the first pass, `in`), and
// mapped back as the last pass stores them (`out`), so that no pass of its
// own goes over the keys for either.
struct KeyOrder {
  int kind;  // 0 unsigned, 1 signed, 2 float
  int desc;
  int in, out;
  template <typename U>
  __device__ __forceinline__ U load(U x) const {
    return in ? to_ordered(x, kind, desc != 0) : x;
  }
  template <typename U>
  __device__ __forceinline__ U store(U t) const {
    return out ? from_ordered(t, kind, desc != 0) : t;
  }
};

// Digit histogram of each tile, stored digit-major: hist[d * tiles + tile].
template <typename U>
__global__ void __launch_bounds__(kPT) k_digit_hist(const U* __restrict__ keys, long long n,
                                                    int shift, uint32_t* __restrict__ hist,
                                                    int tiles, KeyOrder ord) {
  __shared__ uint32_t s_h[256];
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    s_h[threadIdx.x] = 0;
    __syncthreads();
    const long long b = (long long)tile * kPTile;
#pragma unroll 4
    for (int e = 0; e < kPI; ++e) {
      const long long i = b + e * kPT + threadIdx.x;
      if (i < n) atomicAdd(&s_h[(unsigned)(ord.load(keys[i]) >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[(long long)threadIdx.x * tiles + tile] = s_h[threadIdx.x];
    __syncthreads();
  }
}

// Stable scatter of one pass.  Warp w of a tile owns its 512 consecutive
// elements (tile-local w*512 + e*32 + lane, e = 0..15, loads coalesced) and
// ranks them in element order against warp-private digit counters (warp
// match: equal digits of earlier lanes, plus the warp's earlier rounds).  A
// block-wide prefix over (digit, warp) and over the tile's digits then gives
// every element its place in the tile sorted by digit; keys and source
// indices are staged there in shared memory, and written out in that order:
// consecutive threads write consecutive places of one digit's run (the
// tile's offset for the digit, from the scanned histograms), values gathered
// from the tile's own range.
// VW: 32-bit words a value (0 for Sort).  The tile's 16 keys a thread are
// loaded before any is ranked, and in the write-out each thread gathers its
// 16 values before storing them: each of those loads is otherwise a DRAM
// round trip of its own.
template <typename U, int VW>
__global__ void __launch_bounds__(kPT) k_digit_scatter(const U* __restrict__ kin,
                                                       U* __restrict__ kout,
                                                       const uint32_t* __restrict__ vin,
                                                       uint32_t* __restrict__ vout,
                                                       long long n, int shift,
                                                       const uint32_t* __restrict__ off,
                                                       int tiles, KeyOrder ord) {
  extern __shared__ unsigned long long s_dyn[];
  U* s_key = reinterpret_cast<U*>(s_dyn);                        // [kPTile]
  uint32_t* s_src = reinterpret_cast<uint32_t*>(s_key + kPTile);  // [kPTile]
  uint32_t* s_cnt = s_src + kPTile;                               // [kPT/32][256]
  uint32_t* s_dst = s_cnt + (kPT / 32) * 256;                     // [256] global run start - local start
  uint32_t* s_warp = s_dst + 256;                                 // [kPT/32]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  uint32_t* cnt = s_cnt + warp * 256;
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
#pragma unroll
    for (int w = 0; w < kPT / 32; ++w) s_cnt[w * 256 + threadIdx.x] = 0;
    __syncthreads();
    const long long tb = (long long)tile * kPTile;
    const int lb = warp * (kPI * 32);
    U key[kPI];
    uint32_t rank[kPI];
#pragma unroll
    for (int e = 0; e < kPI; ++e) {
      const long long i = tb + lb + e * 32 + lane;
      key[e] = i < n ? ord.load(kin[i]) : (U)0;
    }
#pragma unroll
    for (int e = 0; e < kPI; ++e) {
      const bool ok = tb + lb + e * 32 + lane < n;
      const unsigned d = ok ? ((unsigned)(key[e] >> shift) & 255u) : 256u;
      const unsigned peers = __match_any_sync(kFull, d);
      const uint32_t before = d < 256u ? cnt[d] : 0u;
      rank[e] = before + __popc(peers & lt);
      __syncwarp();
      if (d < 256u && lane == __ffs(peers) - 1) cnt[d] = before + __popc(peers);
      __syncwarp();
    }
    __syncthreads();
    // thread t = digit: its tile count, prefix over warps, and the tile-local
    // start of its run (exclusive scan over the digits)
    uint32_t tot = 0;
#pragma unroll
    for (int w = 0; w < kPT / 32; ++w) {
      const uint32_t c = s_cnt[w * 256 + threadIdx.x];
      s_cnt[w * 256 + threadIdx.x] = tot;
      tot += c;
    }
    uint32_t x = tot;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(kFull, x, d);
      if (lane >= d) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    uint32_t lstart = x - tot;
    for (int w = 0; w < warp; ++w) lstart += s_warp[w];
#pragma unroll
    for (int w = 0; w < kPT / 32; ++w) s_cnt[w * 256 + threadIdx.x] += lstart;
    s_dst[threadIdx.x] = off[(long long)threadIdx.x * tiles + tile] - lstart;
    __syncthreads();
#pragma unroll
    for (int e = 0; e < kPI; ++e) {
      const int li = lb + e * 32 + lane;
      if (tb + li < n) {
        const unsigned d = (unsigned)(key[e] >> shift) & 255u;
        const uint32_t lp = cnt[d] + rank[e];
        s_key[lp] = key[e];
        s_src[lp] = (uint32_t)li;
      }
    }
    __syncthreads();
    const int valid = (int)min((long long)kPTile, n - tb);
    constexpr int kJ = kPTile / kPT;
    constexpr int kV = VW > 0 ? VW : 1;
    uint32_t at[kJ], v[kJ][kV];
#pragma unroll
    for (int jj = 0; jj < kJ; ++jj) {
      const int j = threadIdx.x + jj * kPT;
      if (j < valid) {
        const U k = s_key[j];
        at[jj] = s_dst[(unsigned)(k >> shift) & 255u] + j;
        kout[at[jj]] = ord.store(k);
        if constexpr (VW > 0) {
          const long long src = tb + s_src[j];
#pragma unroll
          for (int q = 0; q < VW; ++q) v[jj][q] = vin[src * VW + q];
        }
      }
    }
    if constexpr (VW > 0) {
#pragma unroll
      for (int jj = 0; jj < kJ; ++jj)
        if (threadIdx.x + jj * kPT < valid)
#pragma unroll
          for (int q = 0; q < VW; ++q) vout[(long long)at[jj] * VW + q] = v[jj][q];
    }
    __syncthreads();
  }
}

template <typename U>
size_t scatter_smem() {
  return (size_t)kPTile * sizeof(U) + (size_t)kPTile * 4 + (kPT / 32) * 256 * 4 + 256 * 4 +
         (kPT / 32) * 4;
}

// ---- single-pass compaction ------------------------------------------------
//
// StreamCompact and Unique in one read of the stencil (or keys), on the
// single-pass driver: a tile's kept elements are counted as it lands, the
// look-back warp finds its offset, and the compute warps write the tile's
// kept elements at their places: the key itself (Unique), the value gathered
// from its array (StreamCompact with an input), or the element's index.
//
// Unique writes in place: a tile's kept keys go below its own start, into
// tiles that have already loaded (their counts are published before this
// tile's offset is known); the only place it shares with a later read is the
// key before the next tile, which it rewrites only when no key before it was
// dropped, that is with the same key.
struct CompactOp {
  int mode;          // 0 stencil int32 != 0; 1 stencil float != 0; 2 key differs from the previous
  int key_kind;      // mode 2: 0 unsigned, 1 signed, 2 float (compared as values)
  const void* test;  // the staged array: stencil or keys
  const uint32_t* values;  // modes 0 / 1: the values to gather (NULL: the index instead)
  int words;               // 32-bit words a value
  void* out;
};

// S: the staged element (uint32_t or unsigned long long).  W: 32-bit words a
// gathered value (StreamCompact with an input: the tile's values are
// prefetched into L2 by one bulk copy when the tile is taken, and a lane
// loads its chunks' W x 16 bytes of values four chunks at a time, before
// their stores), or 0 (Unique's keys, or indices).  The key before a tile
// (Unique) is read by thread 0 when the tile lands, before this tile writes
// anything, and used by thread 0 alone.
template <typename S, int W>
struct CompactPass {
  typedef S Staged;
  typedef uint32_t Sum;  // counts: fewer than 2^31 elements
  static constexpr int E = 16 / (int)sizeof(S);
  static constexpr int kTileElems = (int)(kSTileBytes / sizeof(S));
  struct Chunk { S e[E]; };
  int mode, key_kind;
  const S* src;
  const uint32_t* values;
  int vec;  // values 16-byte aligned
  void* out;
  long long n;

  __device__ void on_take(int t) const {
    if (W > 0 && vec)  // the tile's values, into L2 ahead of the gather
      asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(
                       values + (long long)t * kTileElems * W),
                   "r"((unsigned)(kTileElems * W * 4))
                   : "memory");
  }
  __device__ void on_land(int k, long long b, unsigned long long* aux) const {
    aux[k] = mode == 2 && b > 0 ? (unsigned long long)src[b - 1] : 0ull;
  }
  __device__ bool keep(S x, S prev, bool first) const {
    if (mode == 0) return (int32_t)x != 0;
    if (mode == 1) return __uint_as_float((uint32_t)x) != 0.0f;
    if (first) return true;
    if (sizeof(S) == 4 && key_kind == 2)
      return __uint_as_float((uint32_t)x) != __uint_as_float((uint32_t)prev);
    return x != prev;
  }
  // kept mask of the lane's chunk c (bit e: element e), and the chunk
  __device__ unsigned kept(const S* s_data, int k, long long b, int c, int warp, int lane,
                           const unsigned long long* aux, Chunk& x) const {
    const S* p = lane_chunk0(s_data, warp, lane) + 32 * c * E;
    const long long idx0 = p - s_data;  // tile-local index of element 0
    x = *reinterpret_cast<const Chunk*>(p);
    S prev = 0;
    if (mode == 2 && b + idx0 > 0) prev = idx0 > 0 ? p[-1] : (S)aux[k];
    unsigned m = 0;
#pragma unroll
    for (int e = 0; e < E; ++e) {
      if (b + idx0 + e < n && keep(x.e[e], prev, b + idx0 + e == 0)) m |= 1u << e;
      prev = x.e[e];
    }
    return m;
  }
  __device__ Sum thread_sum(S* s_data, int k, long long b, int warp, int lane,
                            const unsigned long long* aux) const {
    Sum sum = 0;
#pragma unroll 4
    for (int c = 0; c < kSChunks; ++c) {
      Chunk x;
      sum += __popc(kept(s_data, k, b, c, warp, lane, aux, x));
    }
    return sum;
  }
  // the W words of each of the lane's E elements of chunk c
  __device__ void load_values(long long wb, int c, int lane, uint4* v) const {
    if constexpr (W > 0) {
      const long long i0 = wb + (32 * c + lane) * E;
      if (vec && i0 + E <= n) {
        const uint4* src4 = reinterpret_cast<const uint4*>(values + i0 * W);
#pragma unroll
        for (int q = 0; q < W; ++q) v[q] = __ldcs(src4 + q);
      } else {
        uint32_t* u = reinterpret_cast<uint32_t*>(v);
#pragma unroll
        for (int e = 0; e < E; ++e)
#pragma unroll
          for (int q = 0; q < W; ++q) u[e * W + q] = i0 + e < n ? values[(i0 + e) * W + q] : 0u;
      }
    }
  }
  __device__ void finish(S* s_data, int k, long long b, Sum run, int warp, int lane,
                         const unsigned long long* aux) const {
    constexpr int kV = W > 0 ? W : 1;
    constexpr int kG = 4;  // chunks whose values are loaded before any of their stores
    const long long wb = b + (lane_chunk0(s_data, warp, 0) - s_data);  // the warp's first element
#pragma unroll 1
    for (int c0 = 0; c0 < kSChunks; c0 += kG) {
      uint4 vals[kG][kV];
#pragma unroll
      for (int g = 0; g < kG; ++g) load_values(wb, c0 + g, lane, vals[g]);
#pragma unroll
      for (int g = 0; g < kG; ++g) {
        const int c = c0 + g;
        Chunk x;
        const unsigned m = kept(s_data, k, b, c, warp, lane, aux, x);
        const Sum cm = __popc(m);
        const Sum ci = warp_inclusive(cm, lane);
        unsigned long long pos = run + ci - cm;
        const long long i0 = wb + (32 * c + lane) * E;
        const uint32_t* u = reinterpret_cast<const uint32_t*>(vals[g]);
#pragma unroll
        for (int e = 0; e < E; ++e)
          if ((m >> e) & 1u) {
            if constexpr (W > 0) {
              uint32_t* dst = static_cast<uint32_t*>(out) + pos * W;
#pragma unroll
              for (int q = 0; q < W; ++q) dst[q] = u[e * W + q];
            } else if (mode == 2) {
              static_cast<S*>(out)[pos] = x.e[e];
            } else {
              static_cast<int32_t*>(out)[pos] = (int32_t)(i0 + e);
            }
            ++pos;
          }
        run += __shfl_sync(kFull, ci, 31);
      }
    }
  }
  __device__ void store(S*, long long, long long, bool) const {}
};

template <typename S, int W>
__global__ void __launch_bounds__(kSThreads + 32, 1)
    k_compact_single(CompactPass<S, W> op, long long n, int tiles, ScanCtl* ctl, char* states,
                     int bulk) {
  single_pass(op, n, tiles, ctl, states, bulk);
}

template <typename S, int W>
void compact_single_w(const CompactOp& a, long long n, char* scratch, int num_sms,
                      cudaStream_t s) {
  const CompactPass<S, W> op{a.mode,
                             a.key_kind,
                             static_cast<const S*>(a.test),
                             a.values,
                             (reinterpret_cast<uintptr_t>(a.values) & 15) == 0,
                             a.out,
                             n};
  const int bulk = (reinterpret_cast<uintptr_t>(a.test) & 15) == 0;
  launch_single_pass(k_compact_single<S, W>, op, n, bulk, scratch, num_sms, s);
}

// Kept elements into op.out, the count to ctl->total on the device.
template <typename S>
void compact_single(const CompactOp& op, long long n, char* scratch, int num_sms, cudaStream_t s) {
  switch (op.values ? op.words : 0) {
    case 1: compact_single_w<S, 1>(op, n, scratch, num_sms, s); break;
    case 2: compact_single_w<S, 2>(op, n, scratch, num_sms, s); break;
    case 3: compact_single_w<S, 3>(op, n, scratch, num_sms, s); break;
    case 4: compact_single_w<S, 4>(op, n, scratch, num_sms, s); break;
    default: compact_single_w<S, 0>(op, n, scratch, num_sms, s); break;
  }
}

// ---- sort driver -----------------------------------------------------------

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct SortLayout {
  size_t ktmp, vtmp, hist, sums, total;
};

SortLayout sort_layout(long long n, int key_bytes, int value_bytes) {
  const long long tiles = ptiles(n);
  const long long hn = 256 * tiles;
  SortLayout L;
  L.ktmp = 0;
  L.vtmp = align256(L.ktmp + (size_t)n * key_bytes);
  L.hist = align256(L.vtmp + (size_t)n * value_bytes);
  L.sums = align256(L.hist + (size_t)hn * 4);
  L.total = align256(L.sums + (size_t)sum_slots(hn) * 4);
  return L;
}

// passes: 8-bit digits to sort, least significant first (an even count, so
// the result ends in keys/vals); plain = the keys are unsigned, ascending and
// need no order mapping.
template <typename U>
void radix_sort(U* keys, uint32_t* vals, int vwords, long long n, int kind, bool desc,
                char* scratch, int num_sms, cudaStream_t s, int passes = (int)sizeof(U),
                bool plain = false) {
  const SortLayout L = sort_layout(n, (int)sizeof(U), 4 * vwords);
  U* ktmp = reinterpret_cast<U*>(scratch + L.ktmp);
  uint32_t* vtmp = reinterpret_cast<uint32_t*>(scratch + L.vtmp);
  uint32_t* hist = reinterpret_cast<uint32_t*>(scratch + L.hist);
  void* sums = scratch + L.sums;
  const int tiles = ptiles(n);
  const int bh = resident((const void*)k_digit_hist<U>, kPT, num_sms, tiles);
  const size_t sm = scatter_smem<U>();
  const void* scat = vwords == 0   ? (const void*)k_digit_scatter<U, 0>
                     : vwords == 1 ? (const void*)k_digit_scatter<U, 1>
                     : vwords == 2 ? (const void*)k_digit_scatter<U, 2>
                     : vwords == 3 ? (const void*)k_digit_scatter<U, 3>
                                   : (const void*)k_digit_scatter<U, 4>;
  cudaFuncSetAttribute(scat, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  int per = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, scat, kPT, sm) != cudaSuccess || per < 1)
    per = 1;
  const int bs = (int)(tiles < (long long)num_sms * per ? tiles : (long long)num_sms * per);
  for (int p = 0; p < passes; ++p) {
    const U* ksrc = (p & 1) ? ktmp : keys;
    U* kdst = (p & 1) ? keys : ktmp;
    const uint32_t* vsrc = (p & 1) ? vtmp : vals;
    uint32_t* vdst = (p & 1) ? vals : vtmp;
    KeyOrder ord{kind, desc ? 1 : 0, !plain && p == 0, !plain && p == passes - 1};
    k_digit_hist<U><<<bh, kPT, 0, s>>>(ksrc, n, 8 * p, hist, tiles, ord);
    scan_t<uint32_t>(hist, hist, 256ll * tiles, true, sums, nullptr, num_sms, s);
    int shift = 8 * p;
    void* args[] = {&ksrc, &kdst, &vsrc, &vdst, &n, &shift, &hist, const_cast<int*>(&tiles), &ord};
    cudaLaunchKernel(scat, dim3(bs), dim3(kPT), args, sm, s);
  }
}

// ---- bounds -------------------------------------------------------------------

template <typename T, bool UPPER>
__global__ void k_bounds(const T* __restrict__ sorted, long long n, const T* values, long long m,
                         int32_t* out) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += (long long)gridDim.x * blockDim.x) {
    const T v = values[i];
    long long lo = 0, hi = n;  // first index whose element is >= v (> v for UPPER)
    while (lo < hi) {
      const long long mid = (lo + hi) >> 1;
      const T x = sorted[mid];
      const bool before = UPPER ? !(v < x) : (x < v);
      if (before) lo = mid + 1;
      else hi = mid;
    }
    out[i] = (int32_t)lo;
  }
}

}  // namespace

namespace {

int prim_sms() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms < 1) sms = 1;
  }
  return sms;
}

int bad(const char* msg) {
  set_last_error(msg);
  return DAX_GB300_ERROR_BAD_VALUE;
}

int launched(const char* where) {
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) return DAX_GB300_SUCCESS;
  set_last_error(std::string(where) + ": " + cudaGetErrorString(e));
  return DAX_GB300_ERROR_CUDA;
}

int type_bytes(int t) {
  switch (t) {
    case DAX_GB300_TYPE_I32: case DAX_GB300_TYPE_U32: case DAX_GB300_TYPE_F32: return 4;
    case DAX_GB300_TYPE_I64: case DAX_GB300_TYPE_U64: return 8;
    default: return 0;
  }
}

int type_kind(int t) {
  return (t == DAX_GB300_TYPE_F32) ? 2 : ((t == DAX_GB300_TYPE_I32 || t == DAX_GB300_TYPE_I64) ? 1 : 0);
}

bool size_ok(long long n) { return n >= 0 && n <= 2147483647ll; }

int read_back(void* host, const void* dev, size_t bytes, cudaStream_t s, const char* what) {
  cudaError_t e = cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) return DAX_GB300_SUCCESS;
  set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
  return DAX_GB300_ERROR_CUDA;
}

// The element count of a single-pass compaction (synchronises the stream);
// a look-back wait that ran out is DAX_GB300_ERROR_TIMEOUT.
int read_count(int64_t* h_count, const char* scratch, cudaStream_t s, const char* what) {
  ScanCtl ctl;
  int st = read_back(&ctl, scratch, sizeof(ctl), s, what);
  if (st) return st;
  if (ctl.error) {
    set_last_error(std::string(what) + ": a look-back wait expired on the device");
    return DAX_GB300_ERROR_TIMEOUT;
  }
  *h_count = (int64_t)ctl.total;
  return DAX_GB300_SUCCESS;
}

size_t scan_bytes(long long n) { return align256((size_t)sum_slots(n) * 8); }

// dax_gb300_scan: the reduce-then-scan sums (floats) or the single-pass
// states (integers), whichever is larger.
size_t public_scan_bytes(long long n) {
  const size_t a = scan_bytes(n), b = align256(single_scan_bytes<int64_t>(n));
  return a > b ? a : b;
}

size_t keep_bytes(long long n) { return align256((size_t)sum_slots(n) * 8); }

}  // namespace
}  // namespace daxgb

namespace daxgb {

void sort_unsigned_bits(void* keys, long long n, bool wide, int bits, void* scratch,
                        cudaStream_t s) {
  if (n < 2) return;
  int passes = (bits + 7) / 8;
  passes += passes & 1;
  const int kind = type_kind(wide ? DAX_GB300_TYPE_U64 : DAX_GB300_TYPE_U32);
  if (wide)
    radix_sort<unsigned long long>(static_cast<unsigned long long*>(keys), nullptr, 0, n, kind,
                                   false, static_cast<char*>(scratch), prim_sms(), s,
                                   passes < 8 ? passes : 8, true);
  else
    radix_sort<uint32_t>(static_cast<uint32_t*>(keys), nullptr, 0, n, kind, false,
                         static_cast<char*>(scratch), prim_sms(), s, passes < 4 ? passes : 4,
                         true);
}

}  // namespace daxgb

using daxgb::align256;

extern "C" {

size_t dax_gb300_scan_scratch_bytes(int64_t n) {
  return daxgb::public_scan_bytes(n < 1 ? 1 : n);
}

int dax_gb300_scan(const void* d_in, void* d_out, int64_t n, int type, int exclusive,
                   void* d_scratch, size_t scratch_bytes, void* h_total, void* stream) {
  using namespace daxgb;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!size_ok(n)) return bad("scan length must be in [0, 2^31 - 1]");
  const int tb = type_bytes(type);
  if (!tb) return bad("unknown element type");
  if (n == 0) {
    if (h_total) memset(h_total, 0, (size_t)tb);
    return DAX_GB300_SUCCESS;
  }
  if (!d_in || !d_out || !d_scratch) return bad("NULL input, output or scratch");
  if (scratch_bytes < public_scan_bytes(n))
    return bad("scratch smaller than dax_gb300_scan_scratch_bytes()");
  const int sms = prim_sms();
  char* sc = static_cast<char*>(d_scratch);
  const bool ex = exclusive != 0;
  switch (type) {
    case DAX_GB300_TYPE_I32: scan_single<int32_t>((const int32_t*)d_in, (int32_t*)d_out, n, ex, sc, sms, s); break;
    case DAX_GB300_TYPE_U32: scan_single<uint32_t>((const uint32_t*)d_in, (uint32_t*)d_out, n, ex, sc, sms, s); break;
    case DAX_GB300_TYPE_F32: scan_t<float>((const float*)d_in, (float*)d_out, n, ex, sc, nullptr, sms, s); break;
    case DAX_GB300_TYPE_I64: scan_single<int64_t>((const int64_t*)d_in, (int64_t*)d_out, n, ex, sc, sms, s); break;
    default: scan_single<unsigned long long>((const unsigned long long*)d_in, (unsigned long long*)d_out, n, ex, sc, sms, s); break;
  }
  int st = launched("scan kernels");
  if (st || !h_total) return st;
  if (type == DAX_GB300_TYPE_F32)  // the scanned tile sums end with the grand total
    return read_back(h_total, sc + (size_t)ptiles(n) * tb, (size_t)tb, s, "reading the scan total");
  // the single pass: the error word and the total (little-endian, as wide as the element)
  ScanCtl ctl;
  st = read_back(&ctl, sc, sizeof(ctl), s, "reading the scan total");
  if (st) return st;
  if (ctl.error) {
    set_last_error("scan: a look-back wait expired on the device");
    return DAX_GB300_ERROR_TIMEOUT;
  }
  memcpy(h_total, &ctl.total, (size_t)tb);
  return DAX_GB300_SUCCESS;
}

size_t dax_gb300_sort_scratch_bytes(int64_t n, int key_type, int value_bytes) {
  using namespace daxgb;
  const int kb = type_bytes(key_type);
  if (!kb || n < 0 || value_bytes < 0 || value_bytes > 16 || (value_bytes & 3)) return 0;
  const long long nn = n < 1 ? 1 : n;
  const SortLayout L = sort_layout(nn, kb, value_bytes);
  return L.total + scan_bytes(256ll * ptiles(nn));
}

int dax_gb300_sort_by_key(void* d_keys, void* d_values, int64_t n, int key_type, int value_bytes,
                          int descending, void* d_scratch, size_t scratch_bytes, void* stream) {
  using namespace daxgb;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!size_ok(n)) return bad("sort length must be in [0, 2^31 - 1]");
  const int kb = type_bytes(key_type);
  if (!kb) return bad("unknown key type");
  if (value_bytes < 0 || value_bytes > 16 || (value_bytes & 3))
    return bad("value size must be 0, 4, 8, 12 or 16 bytes");
  if (n < 2) return DAX_GB300_SUCCESS;
  if (!d_keys || (value_bytes && !d_values) || !d_scratch) return bad("NULL keys, values or scratch");
  if (scratch_bytes < dax_gb300_sort_scratch_bytes(n, key_type, value_bytes))
    return bad("scratch smaller than dax_gb300_sort_scratch_bytes()");
  const int kind = type_kind(key_type);
  char* sc = static_cast<char*>(d_scratch);
  if (kb == 4)
    radix_sort<uint32_t>(static_cast<uint32_t*>(d_keys), static_cast<uint32_t*>(d_values),
                         value_bytes / 4, n, kind, descending != 0, sc, prim_sms(), s);
  else
    radix_sort<unsigned long long>(static_cast<unsigned long long*>(d_keys),
                                   static_cast<uint32_t*>(d_values), value_bytes / 4, n, kind,
                                   descending != 0, sc, prim_sms(), s);
  return launched("sort kernels");
}

size_t dax_gb300_compact_scratch_bytes(int64_t n, int element_bytes) {
  using namespace daxgb;
  if (n < 0 || element_bytes < 0) return 0;
  const long long nn = n < 1 ? 1 : n;
  return keep_bytes(nn) + align256((size_t)nn * element_bytes);
}

int dax_gb300_unique(void* d_keys, int64_t n, int key_type, void* d_scratch, size_t scratch_bytes,
                     int64_t* h_count, void* stream) {
  using namespace daxgb;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!size_ok(n)) return bad("unique length must be in [0, 2^31 - 1]");
  const int kb = type_bytes(key_type);
  if (!kb) return bad("unknown key type");
  if (n == 0) {
    if (h_count) *h_count = 0;
    return DAX_GB300_SUCCESS;
  }
  if (!d_keys || !d_scratch) return bad("NULL keys or scratch");
  if (scratch_bytes < dax_gb300_compact_scratch_bytes(n, kb))
    return bad("scratch smaller than dax_gb300_compact_scratch_bytes(n, key bytes)");
  // one pass, in place (the kept keys of a tile go below its start)
  char* sc = static_cast<char*>(d_scratch);
  const CompactOp op{2, type_kind(key_type), d_keys, nullptr, 0, d_keys};
  if (kb == 4)
    compact_single<uint32_t>(op, n, sc, prim_sms(), s);
  else
    compact_single<unsigned long long>(op, n, sc, prim_sms(), s);
  int st = launched("unique kernels");
  if (st || !h_count) return st;
  return read_count(h_count, sc, s, "reading the unique count");
}

int dax_gb300_stream_compact(const void* d_input, int value_bytes, const void* d_stencil,
                             int stencil_type, int64_t n, void* d_output, void* d_scratch,
                             size_t scratch_bytes, int64_t* h_count, void* stream) {
  using namespace daxgb;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!size_ok(n)) return bad("compaction length must be in [0, 2^31 - 1]");
  if (stencil_type != DAX_GB300_TYPE_I32 && stencil_type != DAX_GB300_TYPE_F32)
    return bad("stencil must be int32 or float");
  if (d_input && (value_bytes <= 0 || value_bytes > 16 || (value_bytes & 3)))
    return bad("value size must be 4, 8, 12 or 16 bytes");
  if (n == 0) {
    if (h_count) *h_count = 0;
    return DAX_GB300_SUCCESS;
  }
  if (!d_stencil || !d_output || !d_scratch) return bad("NULL stencil, output or scratch");
  if (scratch_bytes < dax_gb300_compact_scratch_bytes(n, 0))
    return bad("scratch smaller than dax_gb300_compact_scratch_bytes(n, 0)");
  char* sc = static_cast<char*>(d_scratch);
  const CompactOp op{stencil_type == DAX_GB300_TYPE_I32 ? 0 : 1, 0, d_stencil,
                     static_cast<const uint32_t*>(d_input), d_input ? value_bytes / 4 : 1,
                     d_output};
  compact_single<uint32_t>(op, n, sc, prim_sms(), s);
  int st = launched("compaction kernels");
  if (st || !h_count) return st;
  return read_count(h_count, sc, s, "reading the compacted count");
}

int dax_gb300_bounds(const void* d_sorted, int64_t n, const void* d_values, int64_t m,
                     int key_type, int upper, int32_t* d_out, void* stream) {
  using namespace daxgb;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!size_ok(n) || !size_ok(m)) return bad("lengths must be in [0, 2^31 - 1]");
  if (!type_bytes(key_type)) return bad("unknown key type");
  if (m == 0) return DAX_GB300_SUCCESS;
  if ((n && !d_sorted) || !d_values || !d_out) return bad("NULL input, values or output");
  const int b = (int)((m + 255) / 256 < prim_sms() * 8 ? (m + 255) / 256 : prim_sms() * 8);
#define DAXGB_BOUNDS(T)                                                                         \
  (upper ? k_bounds<T, true><<<b, 256, 0, s>>>((const T*)d_sorted, n, (const T*)d_values, m, d_out) \
         : k_bounds<T, false><<<b, 256, 0, s>>>((const T*)d_sorted, n, (const T*)d_values, m, d_out))
  switch (key_type) {
    case DAX_GB300_TYPE_I32: DAXGB_BOUNDS(int32_t); break;
    case DAX_GB300_TYPE_U32: DAXGB_BOUNDS(uint32_t); break;
    case DAX_GB300_TYPE_F32: DAXGB_BOUNDS(float); break;
    case DAX_GB300_TYPE_I64: DAXGB_BOUNDS(int64_t); break;
    default: DAXGB_BOUNDS(unsigned long long); break;
  }
#undef DAXGB_BOUNDS
  return launched("bounds kernel");
}

}  // extern "C"
