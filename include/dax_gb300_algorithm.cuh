/* The device adapter's generic algorithms for any element type and any
 * comparison object (dax/cont/internal/DeviceAdapterAlgorithm.h:44-331; the
 * reference's generic versions are DeviceAdapterAlgorithmGeneral.h), for CUDA
 * C++ callers whose types and functors are templates: dax::Vector3 keys,
 * user structs, SortLess / SortGreater or any strict weak order, Unique with
 * any equivalence.  The C ABI's radix-based entries (dax_gb300_scan,
 * dax_gb300_sort_by_key, ...) remain the fast path for the builtin numeric
 * types.
 *
 *   Copy(in, out, n)                          out[i] = in[i]
 *   ScanInclusive(in, out, n, &total)         T needs T() and operator+
 *   ScanExclusive(in, out, n, &total)
 *   Sort(d, n, comp)                          stable; comp(a, b) = a before b
 *   SortByKey(keys, values, n, comp)          stable, values follow keys
 *   LowerBounds(sorted, n, vals, m, out, comp)   first i with !comp(sorted[i], v)
 *   UpperBounds(sorted, n, vals, m, out, comp)   first i with comp(v, sorted[i])
 *   Unique(d, n, &new_n, same)                keeps the first of every run of
 *                                             neighbours with same(a, b)
 *   StreamCompact(in, stencil, n, out, &m)    keeps in[i] where stencil[i] != U()
 *
 * Every call is stream-ordered on `stream`; the ones returning a count
 * (Unique, StreamCompact, and the totals) wait for it.  Temporary storage is
 * taken from the stream-ordered allocator.  Returns a dax_gb300_status. */
#ifndef DAX_GB300_ALGORITHM_CUH
#define DAX_GB300_ALGORITHM_CUH

#include <stdint.h>

#include <cuda_runtime.h>

#include "dax_gb300.h"

namespace dax_gb300 {

/* dax::math::SortLess / SortGreater for types with < and >. */
struct SortLess {
  template <class T>
  __host__ __device__ bool operator()(const T& a, const T& b) const { return a < b; }
};
struct SortGreater {
  template <class T>
  __host__ __device__ bool operator()(const T& a, const T& b) const { return b < a; }
};
/* Equality for Unique. */
struct Equal {
  template <class T>
  __host__ __device__ bool operator()(const T& a, const T& b) const { return a == b; }
};

namespace detail {

constexpr int kThreads = 256;
constexpr int kItems = 4;
constexpr int kTile = kThreads * kItems;

inline int fail(int code, const char* msg) { return dax_gb300_report_error(code, msg); }

inline int check(cudaError_t e, const char* where) {
  return e == cudaSuccess ? DAX_GB300_SUCCESS : fail(DAX_GB300_ERROR_CUDA, where);
}

inline int grid_for(long long work) {
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long want = (work + kThreads - 1) / kThreads, cap = (long long)sms * 8;
  return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

template <class T>
__global__ void k_copy(const T* __restrict__ in, T* __restrict__ out, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = in[i];
}

// Block-wide inclusive scan of one value per thread (T with operator+).
template <class T>
__device__ T block_inclusive(T v, T* s) {
  s[threadIdx.x] = v;
  __syncthreads();
  for (int d = 1; d < kThreads; d <<= 1) {
    T add = T();
    const bool take = threadIdx.x >= (unsigned)d;
    if (take) add = s[threadIdx.x - d];
    __syncthreads();
    if (take) s[threadIdx.x] = s[threadIdx.x] + add;
    __syncthreads();
  }
  const T r = s[threadIdx.x];
  __syncthreads();
  return r;
}

// Per tile of kTile elements: its sum (thread t sums its kItems in order).
template <class T>
__global__ void __launch_bounds__(kThreads) k_tile_sums(const T* __restrict__ in, long long n,
                                                        T* __restrict__ sums, long long tiles) {
  __shared__ T s[kThreads];
  for (long long tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    T v = T();
    const long long b = tile * kTile + (long long)threadIdx.x * kItems;
    for (int e = 0; e < kItems; ++e)
      if (b + e < n) v = v + in[b + e];
    const T inc = block_inclusive(v, s);
    if (threadIdx.x == kThreads - 1) sums[tile] = inc;
  }
}

// One block: exclusive scan of the tile sums in place, the total at [tiles].
// Thread t sums its own contiguous run of tiles.
template <class T>
__global__ void __launch_bounds__(kThreads) k_scan_sums(T* sums, long long tiles) {
  __shared__ T s[kThreads];
  __shared__ T s_inc[kThreads];
  const long long per = (tiles + kThreads - 1) / kThreads;
  const long long b = threadIdx.x * per, e = b + per < tiles ? b + per : tiles;
  T v = T();
  for (long long i = b; i < e; ++i) v = v + sums[i];
  const T inc = block_inclusive(v, s);
  s_inc[threadIdx.x] = inc;
  __syncthreads();
  T run = threadIdx.x == 0 ? T() : s_inc[threadIdx.x - 1];
  for (long long i = b; i < e; ++i) {
    const T x = sums[i];
    sums[i] = run;
    run = run + x;
  }
  if (threadIdx.x == kThreads - 1) sums[tiles] = inc;
}

// Each tile scanned from its prefix; thread t owns kItems consecutive elements.
template <class T, bool EXCLUSIVE>
__global__ void __launch_bounds__(kThreads) k_tile_scan(const T* __restrict__ in, T* out, long long n,
                                                        const T* __restrict__ prefix, long long tiles) {
  __shared__ T s[kThreads];
  for (long long tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const long long b = tile * kTile + (long long)threadIdx.x * kItems;
    T x[kItems];
    T v = T();
    for (int e = 0; e < kItems; ++e) {
      x[e] = b + e < n ? in[b + e] : T();
      v = v + x[e];
    }
    const T inc = block_inclusive(v, s);
    // exclusive prefix of this thread = inclusive of the previous thread
    s[threadIdx.x] = inc;
    __syncthreads();
    T run = prefix[tile];
    if (threadIdx.x > 0) run = run + s[threadIdx.x - 1];
    __syncthreads();
    for (int e = 0; e < kItems; ++e) {
      if (b + e >= n) break;
      if (EXCLUSIVE) {
        out[b + e] = run;
        run = run + x[e];
      } else {
        run = run + x[e];
        out[b + e] = run;
      }
    }
  }
}

template <class T, bool EXCLUSIVE>
int scan(const T* in, T* out, long long n, T* total, cudaStream_t s) {
  if (n <= 0) {
    if (total) *total = T();
    return DAX_GB300_SUCCESS;
  }
  const long long tiles = (n + kTile - 1) / kTile;
  T* sums = nullptr;
  int st = check(cudaMallocAsync(reinterpret_cast<void**>(&sums), sizeof(T) * (tiles + 1), s),
                 "allocating scan sums");
  if (st) return st;
  const int g = grid_for(tiles * kThreads);
  k_tile_sums<T><<<g, kThreads, 0, s>>>(in, n, sums, tiles);
  k_scan_sums<T><<<1, kThreads, 0, s>>>(sums, tiles);
  k_tile_scan<T, EXCLUSIVE><<<g, kThreads, 0, s>>>(in, out, n, sums, tiles);
  st = check(cudaGetLastError(), "scan kernels");
  if (!st && total) {
    st = check(cudaMemcpyAsync(total, sums + tiles, sizeof(T), cudaMemcpyDeviceToHost, s),
               "reading the scan total");
    if (!st) st = check(cudaStreamSynchronize(s), "scan");
  }
  cudaFreeAsync(sums, s);
  return st;
}

// Keep-flag compaction: out gets the elements with keep(i), in order.
template <class T, class Keep>
__global__ void __launch_bounds__(kThreads) k_keep_counts(long long n, Keep keep,
                                                          long long* __restrict__ sums,
                                                          long long tiles) {
  __shared__ long long s[kThreads];
  for (long long tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const long long b = tile * kTile + (long long)threadIdx.x * kItems;
    long long c = 0;
    for (int e = 0; e < kItems; ++e)
      if (b + e < n && keep(b + e)) ++c;
    const long long inc = block_inclusive(c, s);
    if (threadIdx.x == kThreads - 1) sums[tile] = inc;
  }
}

template <class T, class Keep>
__global__ void __launch_bounds__(kThreads) k_keep_scatter(const T* __restrict__ in, long long n,
                                                           Keep keep, T* __restrict__ out,
                                                           const long long* __restrict__ prefix,
                                                           long long tiles) {
  __shared__ long long s[kThreads];
  for (long long tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const long long b = tile * kTile + (long long)threadIdx.x * kItems;
    int flags = 0;
    long long c = 0;
    for (int e = 0; e < kItems; ++e)
      if (b + e < n && keep(b + e)) {
        flags |= 1 << e;
        ++c;
      }
    const long long inc = block_inclusive(c, s);
    long long pos = prefix[tile] + inc - c;
    for (int e = 0; e < kItems; ++e)
      if (flags & (1 << e)) out[pos++] = in[b + e];
  }
}

template <class T, class Keep>
int compact(const T* in, long long n, Keep keep, T* out, long long* count, cudaStream_t s) {
  *count = 0;
  if (n <= 0) return DAX_GB300_SUCCESS;
  const long long tiles = (n + kTile - 1) / kTile;
  long long* sums = nullptr;
  int st = check(cudaMallocAsync(reinterpret_cast<void**>(&sums), sizeof(long long) * (tiles + 1), s),
                 "allocating compaction sums");
  if (st) return st;
  const int g = grid_for(tiles * kThreads);
  k_keep_counts<T, Keep><<<g, kThreads, 0, s>>>(n, keep, sums, tiles);
  k_scan_sums<long long><<<1, kThreads, 0, s>>>(sums, tiles);
  k_keep_scatter<T, Keep><<<g, kThreads, 0, s>>>(in, n, keep, out, sums, tiles);
  st = check(cudaGetLastError(), "compaction kernels");
  if (!st) st = check(cudaMemcpyAsync(count, sums + tiles, sizeof(long long), cudaMemcpyDeviceToHost, s),
                      "reading the count");
  if (!st) st = check(cudaStreamSynchronize(s), "compaction");
  cudaFreeAsync(sums, s);
  return st;
}

template <class T, class Same>
struct KeepFirstOfRun {
  const T* d;
  Same same;
  __device__ bool operator()(long long i) const { return i == 0 || !same(d[i - 1], d[i]); }
};

template <class U>
struct KeepStencil {
  const U* stencil;
  __device__ bool operator()(long long i) const { return !(stencil[i] == U()); }
};

// ---- comparison sort: tiles sorted in shared memory, then stable merges ----

// Odd-even transposition sort of one tile of kThreads elements (stable: a
// pair is swapped only when the later one comes strictly first).
template <class K, class V, class C, bool VALS>
__global__ void __launch_bounds__(kThreads) k_tile_sort(K* keys, V* vals, long long n, C comp) {
  __shared__ K sk[kThreads];
  __shared__ V sv[VALS ? kThreads : 1];
  const long long b = (long long)blockIdx.x * kThreads;
  const int cnt = (int)(n - b < kThreads ? n - b : kThreads);
  const int t = threadIdx.x;
  if (t < cnt) {
    sk[t] = keys[b + t];
    if (VALS) sv[t] = vals[b + t];
  }
  __syncthreads();
  for (int round = 0; round < cnt; ++round) {
    const int i = 2 * t + (round & 1);
    if (i + 1 < cnt && comp(sk[i + 1], sk[i])) {
      const K k = sk[i];
      sk[i] = sk[i + 1];
      sk[i + 1] = k;
      if (VALS) {
        const V v = sv[i];
        sv[i] = sv[i + 1];
        sv[i + 1] = v;
      }
    }
    __syncthreads();
  }
  if (t < cnt) {
    keys[b + t] = sk[t];
    if (VALS) vals[b + t] = sv[t];
  }
}

// One merge pass of runs of `width`: element i of a left run goes to
// lo + (i - lo) + #(right < x); element j of a right run to
// lo + (j - mid) + #(left <= x), which keeps equal keys in order.
template <class K, class V, class C, bool VALS>
__global__ void __launch_bounds__(kThreads) k_merge(const K* __restrict__ ki, const V* __restrict__ vi,
                                                    K* __restrict__ ko, V* __restrict__ vo,
                                                    long long n, long long width, C comp) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long lo = (i / (2 * width)) * (2 * width);
    const long long mid = lo + width < n ? lo + width : n;
    const long long hi = lo + 2 * width < n ? lo + 2 * width : n;
    const K x = ki[i];
    long long pos;
    if (i < mid) {  // count right-run keys strictly before x
      long long a = mid, c = hi;
      while (a < c) {
        const long long m = (a + c) >> 1;
        if (comp(ki[m], x)) a = m + 1; else c = m;
      }
      pos = lo + (i - lo) + (a - mid);
    } else {        // count left-run keys not after x
      long long a = lo, c = mid;
      while (a < c) {
        const long long m = (a + c) >> 1;
        if (!comp(x, ki[m])) a = m + 1; else c = m;
      }
      pos = lo + (i - mid) + (a - lo);
    }
    ko[pos] = x;
    if (VALS) vo[pos] = vi[i];
  }
}

template <class K, class V, class C, bool VALS>
int merge_sort(K* keys, V* vals, long long n, C comp, cudaStream_t s) {
  if (n < 2) return DAX_GB300_SUCCESS;
  const long long tiles = (n + kThreads - 1) / kThreads;
  k_tile_sort<K, V, C, VALS><<<(unsigned)tiles, kThreads, 0, s>>>(keys, vals, n, comp);
  int st = check(cudaGetLastError(), "tile sort");
  if (st || n <= kThreads) return st;
  K* kt = nullptr;
  V* vt = nullptr;
  st = check(cudaMallocAsync(reinterpret_cast<void**>(&kt), sizeof(K) * n, s), "allocating sort keys");
  if (!st && VALS)
    st = check(cudaMallocAsync(reinterpret_cast<void**>(&vt), sizeof(V) * n, s), "allocating sort values");
  if (st) {
    if (kt) cudaFreeAsync(kt, s);
    return st;
  }
  K *ka = keys, *kb = kt;
  V *va = vals, *vb = vt;
  const int g = grid_for(n);
  for (long long w = kThreads; w < n; w *= 2) {
    k_merge<K, V, C, VALS><<<g, kThreads, 0, s>>>(ka, va, kb, vb, n, w, comp);
    K* tk = ka; ka = kb; kb = tk;
    V* tv = va; va = vb; vb = tv;
  }
  if (ka != keys) {  // the result is in the temporaries: copy it back
    k_copy<K><<<g, kThreads, 0, s>>>(ka, keys, n);
    if (VALS) k_copy<V><<<g, kThreads, 0, s>>>(va, vals, n);
  }
  st = check(cudaGetLastError(), "merge passes");
  cudaFreeAsync(kt, s);
  if (vt) cudaFreeAsync(vt, s);
  return st;
}

template <class T, class C, bool UPPER>
__global__ void k_bounds(const T* __restrict__ sorted, long long n, const T* __restrict__ values,
                         long long m, int32_t* __restrict__ out, C comp) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += (long long)gridDim.x * blockDim.x) {
    const T v = values[i];
    long long a = 0, c = n;
    while (a < c) {
      const long long mid = (a + c) >> 1;
      const bool before = UPPER ? !comp(v, sorted[mid]) : comp(sorted[mid], v);
      if (before) a = mid + 1; else c = mid;
    }
    out[i] = (int32_t)a;
  }
}

}  // namespace detail

template <class T>
int Copy(const T* in, T* out, long long n, cudaStream_t stream = 0) {
  if (n <= 0) return DAX_GB300_SUCCESS;
  detail::k_copy<T><<<detail::grid_for(n), detail::kThreads, 0, stream>>>(in, out, n);
  return detail::check(cudaGetLastError(), "copy");
}

template <class T>
int ScanInclusive(const T* in, T* out, long long n, T* total = nullptr, cudaStream_t stream = 0) {
  return detail::scan<T, false>(in, out, n, total, stream);
}

template <class T>
int ScanExclusive(const T* in, T* out, long long n, T* total = nullptr, cudaStream_t stream = 0) {
  return detail::scan<T, true>(in, out, n, total, stream);
}

template <class T, class C = SortLess>
int Sort(T* d, long long n, C comp = C(), cudaStream_t stream = 0) {
  return detail::merge_sort<T, char, C, false>(d, nullptr, n, comp, stream);
}

template <class K, class V, class C = SortLess>
int SortByKey(K* keys, V* values, long long n, C comp = C(), cudaStream_t stream = 0) {
  return detail::merge_sort<K, V, C, true>(keys, values, n, comp, stream);
}

template <class T, class C = SortLess>
int LowerBounds(const T* sorted, long long n, const T* values, long long m, int32_t* out,
                C comp = C(), cudaStream_t stream = 0) {
  if (m <= 0) return DAX_GB300_SUCCESS;
  detail::k_bounds<T, C, false><<<detail::grid_for(m), detail::kThreads, 0, stream>>>(
      sorted, n, values, m, out, comp);
  return detail::check(cudaGetLastError(), "lower bounds");
}

template <class T, class C = SortLess>
int UpperBounds(const T* sorted, long long n, const T* values, long long m, int32_t* out,
                C comp = C(), cudaStream_t stream = 0) {
  if (m <= 0) return DAX_GB300_SUCCESS;
  detail::k_bounds<T, C, true><<<detail::grid_for(m), detail::kThreads, 0, stream>>>(
      sorted, n, values, m, out, comp);
  return detail::check(cudaGetLastError(), "upper bounds");
}

/* The kept elements are written back to the front of d; *new_n is their count. */
template <class T, class Same = Equal>
int Unique(T* d, long long n, long long* new_n, Same same = Same(), cudaStream_t stream = 0) {
  *new_n = n < 0 ? 0 : n;
  if (n <= 1) return DAX_GB300_SUCCESS;
  T* tmp = nullptr;
  int st = detail::check(cudaMallocAsync(reinterpret_cast<void**>(&tmp), sizeof(T) * n, stream),
                         "allocating unique");
  if (st) return st;
  st = detail::compact(d, n, detail::KeepFirstOfRun<T, Same>{d, same}, tmp, new_n, stream);
  if (!st && *new_n > 0) st = Copy(tmp, d, *new_n, stream);
  if (!st) st = detail::check(cudaStreamSynchronize(stream), "unique");
  cudaFreeAsync(tmp, stream);
  return st;
}

template <class T, class U>
int StreamCompact(const T* in, const U* stencil, long long n, T* out, long long* count,
                  cudaStream_t stream = 0) {
  return detail::compact(in, n, detail::KeepStencil<U>{stencil}, out, count, stream);
}

}  // namespace dax_gb300

#endif  // DAX_GB300_ALGORITHM_CUH
