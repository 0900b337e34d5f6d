// Marching tetrahedra on an unstructured tetrahedral grid
// (dax/worklet/MarchingTetrahedra.h:49-161 driven by DispatcherMapCell and
// DispatcherGenerateInterpolatedCells).
//
// Layout: points float[P][3], field float[P], connectivity int32[C][4]
// (dax::cont::UnstructuredGrid<CellTagTetrahedron>), all caller-owned.
//
//   count   K1 k_mt_count: the case byte of every cell (4 field gathers
//           each), the triangle totals of every chunk of kMtChunk cells and
//           of every tile of kMtTile cells;
//           K2 k_mt_tile_scan: exclusive tile offsets and the total T.
//   emit    K3 k_mt_emit: one warp per chunk of kMtChunk cells, chunks
//           without triangles skipped; each lane takes 16 consecutive cells
//           (one 16-byte load of their cases) and a warp scan of the lanes'
//           triangle counts gives every cell its first output triangle; the
//           case's TriTable edges, lower point id
//           first, weight (iso - f[A]) / (f[B] - f[A]) and Lerp of the two
//           points (MarchingTetrahedra.h:117-161, GenerateWorklets.h:79-92).
//           Unmerged it writes vertices, connectivity and records directly;
//           merged it writes one key (A, B) per record.
//   merge   the reference's ResolveCoordinates on the device adapter's own
//           primitives: Sort and Unique of the keys (radix sort, 32- or
//           64-bit keys as P needs), LowerBounds of every record key
//           (k_mt_merged_conn), and the unique edges' vertices
//           (k_mt_merged_verts).
//
// Point ids outside [0, P) are not dereferenced: the cell counts as case 0
// and Info.error gets kErrBadIndex.
#include "common.cuh"
#include "kernels.cuh"
#include "mc_case.cuh"
#include "mt_tables.h"

namespace daxgb {

// The tables are compile-time constants folded into instructions: lanes of a
// warp index them with different cases, which a constant-memory table would
// serve one address at a time.
constexpr uint32_t kMtWords[16] = DAX_GB300_MT_CASE_WORDS;
__constant__ uint32_t c_mt_case[16] = DAX_GB300_MT_CASE_WORDS;  // copied to shared memory

// NumFaces of case c in bits 2c .. 2c+1.
constexpr uint32_t mt_face_bits() {
  uint32_t b = 0;
  for (int c = 0; c < 16; ++c) b |= (kMtWords[c] >> 28) << (2 * c);
  return b;
}
constexpr uint32_t kMtFaceBits = mt_face_bits();

// cellVertEdges (MarchingTetrahedra.h:126-129), byte e = edge e: low nibble
// first corner, high nibble second.
constexpr unsigned long long kTetEdges = 0x231303022110ull;

__device__ __forceinline__ int mt_faces(int cs) { return (int)((kMtFaceBits >> (2 * cs)) & 3u); }

// GetTetrahedronClassification (MarchingTetrahedra.h:36-46).
__device__ __forceinline__ int mt_classify(const float v[4], float iso) {
  return (v[0] > iso ? 1 : 0) | (v[1] > iso ? 2 : 0) | (v[2] > iso ? 4 : 0) | (v[3] > iso ? 8 : 0);
}

// a[k] for k in 0..3 by selects, so the four values stay in registers.
template <typename T>
__device__ __forceinline__ T pick4(const T a[4], int k) {
  return k == 0 ? a[0] : (k == 1 ? a[1] : (k == 2 ? a[2] : a[3]));
}

// Point ids of cell c; false when one lies outside [0, P).
template <bool VEC>
__device__ __forceinline__ bool load_tet(const int32_t* __restrict__ conn, long long c,
                                         long long P, int id[4]) {
  if (VEC) {
    const int4 q = __ldg(reinterpret_cast<const int4*>(conn) + c);
    id[0] = q.x;
    id[1] = q.y;
    id[2] = q.z;
    id[3] = q.w;
  } else {
#pragma unroll
    for (int n = 0; n < 4; ++n) id[n] = __ldg(conn + 4 * c + n);
  }
  bool ok = true;
#pragma unroll
  for (int n = 0; n < 4; ++n) ok = ok && id[n] >= 0 && (long long)id[n] < P;
  return ok;
}

// Block-wide exclusive sum of small non-negative values; *total gets the sum.
__device__ __forceinline__ unsigned block_excl(unsigned v, unsigned* s_warp, unsigned* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned x = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const unsigned y = __shfl_up_sync(kFull, x, d);
    if (lane >= d) x += y;
  }
  if (lane == 31) s_warp[wid] = x;
  __syncthreads();
  unsigned before = 0, all = 0;
  for (int w = 0; w < kMtThreads / 32; ++w) {
    const unsigned t = s_warp[w];
    before += w < wid ? t : 0u;
    all += t;
  }
  __syncthreads();
  *total = all;
  return before + x - v;
}

// Warp w of a tile takes the kMtChunk consecutive cells of chunk 8 * tile + w
// (lanes interleaved, so every load of ids is 512 contiguous bytes); the
// chunk's and the tile's triangle totals are stored.
template <bool VEC>
__global__ void __launch_bounds__(kMtThreads) k_mt_count(const int32_t* __restrict__ conn,
                                                         long long C,
                                                         const float* __restrict__ f, long long P,
                                                         float iso, uint8_t* __restrict__ cases,
                                                         unsigned* __restrict__ tile_tot,
                                                         unsigned* __restrict__ chunk_tot,
                                                         Info* info, int tiles) {
  __shared__ unsigned s_warp[kMtThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  bool bad = false;
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    unsigned sum = 0;
    const long long cb = (long long)tile * kMtTile + (long long)wid * kMtChunk + lane;
#pragma unroll 4
    for (int r = 0; r < kMtChunk / 32; ++r) {
      const long long c = cb + 32 * r;
      if (c < C) {
        int id[4];
        int cs = 0;
        if (load_tet<VEC>(conn, c, P, id)) {
          const float v[4] = {__ldg(f + id[0]), __ldg(f + id[1]), __ldg(f + id[2]),
                              __ldg(f + id[3])};
          cs = mt_classify(v, iso);
        } else {
          bad = true;
        }
        cases[c] = (uint8_t)cs;
        sum += (unsigned)mt_faces(cs);
      }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) sum += __shfl_xor_sync(kFull, sum, d);
    if (lane == 0) {
      chunk_tot[(long long)tile * (kMtTile / kMtChunk) + wid] = sum;
      s_warp[wid] = sum;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned t = 0;
      for (int w = 0; w < kMtThreads / 32; ++w) t += s_warp[w];
      tile_tot[tile] = t;
    }
    __syncthreads();
  }
  if (bad) atomicOr(&info->error, kErrBadIndex);
}

// One block: exclusive offsets of the tile totals (tile_off[tiles] = T) and
// the total into Info; more than 2^31 - 1 vertex records is an overflow.
// Thread t sums its own contiguous run of tiles, the block scans the 1024
// run totals, then every thread writes its run's offsets.
__global__ void __launch_bounds__(1024) k_mt_tile_scan(const unsigned* __restrict__ tile_tot,
                                                       int tiles,
                                                       unsigned long long* __restrict__ tile_off,
                                                       Info* info) {
  __shared__ unsigned long long s_warp[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int per = (tiles + 1023) / 1024;
  const int b = threadIdx.x * per, e = min(b + per, tiles);
  unsigned long long v = 0;
  for (int i = b; i < e; ++i) v += tile_tot[i];
  unsigned long long x = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const unsigned long long y = __shfl_up_sync(kFull, x, d);
    if (lane >= d) x += y;
  }
  if (lane == 31) s_warp[wid] = x;
  __syncthreads();
  unsigned long long before = 0, all = 0;
  for (int w = 0; w < 32; ++w) {
    const unsigned long long t = s_warp[w];
    before += w < wid ? t : 0ull;
    all += t;
  }
  unsigned long long run = before + x - v;
  for (int i = b; i < e; ++i) {
    tile_off[i] = run;
    run += tile_tot[i];
  }
  if (threadIdx.x == 0) {
    tile_off[tiles] = all;
    info->total_a = (long long)all;
    info->total_b = 0;
    if (3ull * all > 2147483647ull) atomicOr(&info->error, kErrOverflow);
  }
}

// Output sinks of the emit pass.
struct MtOut {
  float* verts;       // unmerged: [3T][3]
  int32_t* tconn;     // unmerged: [3T]
  int32_t* ra;        // unmerged records (optional)
  int32_t* rb;
  float* rw;
  void* keys;         // merged: [3T] keys (A << kbits) | B
  int kbits;
  bool wide;          // 64-bit keys
  long long vcap, tcap;
};

template <bool VEC, bool KEYS>
__global__ void __launch_bounds__(kMtThreads) k_mt_emit(const float* __restrict__ pts,
                                                        const int32_t* __restrict__ conn,
                                                        long long C,
                                                        const float* __restrict__ f, long long P,
                                                        float iso,
                                                        const uint8_t* __restrict__ cases,
                                                        const unsigned long long* __restrict__ tile_off,
                                                        const unsigned* __restrict__ chunk_tot,
                                                        Info* info, MtOut o, long long chunks) {
  // per warp: the chunk's cells with triangles, (cell in chunk | case << 16)
  // and their first triangle relative to the chunk's
  __shared__ uint2 s_act[kMtThreads / 32][kMtChunk];
  __shared__ uint32_t s_case[16];
  if (threadIdx.x < 16) s_case[threadIdx.x] = c_mt_case[threadIdx.x];
  __syncthreads();
  // nothing is written when an earlier pass failed or the outputs are short
  const long long T = info->total_a;
  if (info->error) return;
  if (!KEYS && (T > o.tcap || 3 * T > o.vcap)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&info->error, kErrCapacity);
    return;
  }
  constexpr int kPerTile = kMtTile / kMtChunk;
  const int lane = threadIdx.x & 31;
  uint2* act = s_act[threadIdx.x >> 5];
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long ch = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; ch < chunks;
       ch += nwarps) {
    if (__ldg(chunk_tot + ch) == 0) continue;  // warp-uniform
    // the chunk's first triangle: its tile's offset plus the earlier chunks
    const long long tile = ch / kPerTile;
    unsigned long long t0 = tile_off[tile];
    for (long long k = tile * kPerTile; k < ch; ++k) t0 += __ldg(chunk_tot + k);
    // lane l reads the cases of the kMtPerLane consecutive cells c0 .. c0 + 15
    const long long cbase = ch * kMtChunk;
    const long long c0 = cbase + (long long)lane * kMtPerLane;
    uint32_t cw[kMtPerLane / 4];
    if (c0 + kMtPerLane <= C) {
      const uint4 q = __ldg(reinterpret_cast<const uint4*>(cases + c0));
      cw[0] = q.x;
      cw[1] = q.y;
      cw[2] = q.z;
      cw[3] = q.w;
    } else {
#pragma unroll
      for (int q = 0; q < kMtPerLane / 4; ++q) {
        uint32_t w = 0;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const long long c = c0 + 4 * q + b;
          if (c < C) w |= (uint32_t)cases[c] << (8 * b);
        }
        cw[q] = w;
      }
    }
    // (triangles << 16) | active cells of this lane, scanned over the warp
    unsigned mine = 0;
#pragma unroll
    for (int e = 0; e < kMtPerLane; ++e) {
      const int nf = mt_faces((cw[e >> 2] >> (8 * (e & 3))) & 0xF);
      mine += ((unsigned)nf << 16) | (nf ? 1u : 0u);
    }
    unsigned x = mine;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const unsigned y = __shfl_up_sync(kFull, x, d);
      if (lane >= d) x += y;
    }
    const unsigned nact = __shfl_sync(kFull, x, 31) & 0xFFFFu;
    unsigned slot = (x - mine) & 0xFFFFu, tri = (x - mine) >> 16;
#pragma unroll
    for (int e = 0; e < kMtPerLane; ++e) {
      const int cs = (int)((cw[e >> 2] >> (8 * (e & 3))) & 0xF);
      const int nf = mt_faces(cs);
      if (nf) {
        act[slot++] = make_uint2((unsigned)(lane * kMtPerLane + e) | ((unsigned)cs << 16), tri);
        tri += (unsigned)nf;
      }
    }
    __syncwarp();
    // one active cell per lane
    for (unsigned a = lane; a < nact; a += 32) {
      const uint2 ent = act[a];
      const long long c = cbase + (ent.x & 0xFFFFu);
      const int cs = (int)(ent.x >> 16);
      const int nf = mt_faces(cs);
      const unsigned long long tc = t0 + ent.y;
      int id[4];
      if (!load_tet<VEC>(conn, c, P, id)) continue;  // the count pass saw it: case 0, error set
      const float v[4] = {__ldg(f + id[0]), __ldg(f + id[1]), __ldg(f + id[2]), __ldg(f + id[3])};
      const uint32_t word = s_case[cs];
      for (int m = 0; m < 3 * nf; ++m) {
        const int e = (int)((word >> (4 * m)) & 0xF);
        const int ed = (int)((kTetEdges >> (8 * e)) & 0xFF);
        const int e0 = ed & 0xF, e1 = ed >> 4;
        // the lower point id first (MarchingTetrahedra.h:142-151)
        const int i0 = pick4(id, e0), i1 = pick4(id, e1);
        const bool keep = i0 < i1;
        const int A = keep ? i0 : i1, B = keep ? i1 : i0;
        const long long rec = 3 * (long long)tc + m;
        if (KEYS) {
          if (o.wide)
            static_cast<unsigned long long*>(o.keys)[rec] =
                ((unsigned long long)A << o.kbits) | (unsigned long long)B;
          else
            static_cast<uint32_t*>(o.keys)[rec] = ((uint32_t)A << o.kbits) | (uint32_t)B;
        } else {
          const float fa = keep ? pick4(v, e0) : pick4(v, e1);
          const float fb = keep ? pick4(v, e1) : pick4(v, e0);
          const float w = __fdiv_rn(__fsub_rn(iso, fa), __fsub_rn(fb, fa));
          const float* pa = pts + 3 * (long long)A;
          const float* pb = pts + 3 * (long long)B;
#pragma unroll
          for (int q = 0; q < 3; ++q) o.verts[3 * rec + q] = lerp_rn(__ldg(pa + q), __ldg(pb + q), w);
          o.tconn[rec] = (int32_t)rec;
          if (o.ra) {
            o.ra[rec] = A;
            o.rb[rec] = B;
            o.rw[rec] = w;
          }
        }
      }
    }
    __syncwarp();
  }
}

// The merge scratch starts with a header: the number of unique keys and the
// byte offsets of the record keys and of the unique keys.
// magic marks a header written by dax_gb300_mt_merge; T is the triangle
// count of the count pass it merged.
struct MtMergeHeader {
  unsigned long long magic, V, keys, uniq, T;
};
constexpr unsigned long long kMtMergeMagic = 0x4d54204d45524745ull;

// The header describes keys of this count pass that lie inside the buffer.
template <typename U>
__device__ __forceinline__ bool merge_header_ok(const MtMergeHeader* h, long long T,
                                                unsigned long long mbytes) {
  const unsigned long long n = 3ull * (unsigned long long)T;
  return h->magic == kMtMergeMagic && h->T == (unsigned long long)T && h->V <= n &&
         h->keys <= mbytes && h->uniq <= mbytes && n * sizeof(U) <= mbytes - h->keys &&
         n * sizeof(U) <= mbytes - h->uniq;
}

// conn[r] = LowerBounds(unique keys, key of record r).
template <typename U>
__global__ void __launch_bounds__(256) k_mt_merged_conn(const char* __restrict__ m,
                                                        unsigned long long mbytes, Info* info,
                                                        long long tcap, long long vcap,
                                                        int32_t* __restrict__ tconn) {
  const MtMergeHeader* hdr = reinterpret_cast<const MtMergeHeader*>(m);
  const long long T = info->total_a;
  if (info->error) return;
  if (!merge_header_ok<U>(hdr, T, mbytes)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&info->error, kErrState);
    return;
  }
  const long long V = (long long)hdr->V;
  if (T > tcap || V > vcap) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&info->error, kErrCapacity);
    return;
  }
  const U* __restrict__ keys = reinterpret_cast<const U*>(m + hdr->keys);
  const U* __restrict__ uniq = reinterpret_cast<const U*>(m + hdr->uniq);
  const long long n = 3 * T;
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < n;
       r += (long long)gridDim.x * blockDim.x) {
    const U k = keys[r];
    long long lo = 0, hi = V;
    while (lo < hi) {
      const long long mid = (lo + hi) >> 1;
      if (__ldg(uniq + mid) < k) lo = mid + 1;
      else hi = mid;
    }
    tconn[r] = (int32_t)lo;
  }
}

// Vertex v of the merged output from unique key v: its two point ids, the
// weight from their field values, Lerp of their coordinates.
// (i, j, k) of point p of a uniform grid.
__device__ __forceinline__ void grid_ijk(const Grid& g, int p, int& i, int& j, int& k) {
  const unsigned row = (unsigned)p / (unsigned)g.nx;
  i = p - (int)(row * (unsigned)g.nx);
  split_row(g, row, j, k);
}

// GRID: the points are a uniform grid's (coordinates from the point id),
// else the explicit pts array.
template <typename U, bool GRID>
__global__ void __launch_bounds__(256) k_mt_merged_verts(const char* __restrict__ m,
                                                         unsigned long long mbytes, Grid g,
                                                         const Info* info, long long tcap,
                                                         long long vcap, int kbits,
                                                         const float* __restrict__ pts,
                                                         const float* __restrict__ f, float iso,
                                                         float* __restrict__ verts,
                                                         int32_t* __restrict__ ra,
                                                         int32_t* __restrict__ rb,
                                                         float* __restrict__ rw) {
  const MtMergeHeader* hdr = reinterpret_cast<const MtMergeHeader*>(m);
  const long long T = info->total_a;
  if (info->error || !merge_header_ok<U>(hdr, T, mbytes)) return;
  const long long V = (long long)hdr->V;
  if (T > tcap || V > vcap) return;
  const U* __restrict__ uniq = reinterpret_cast<const U*>(m + hdr->uniq);
  const U mask = (U)((((unsigned long long)1) << kbits) - 1ull);
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V;
       v += (long long)gridDim.x * blockDim.x) {
    const U k = uniq[v];
    const int A = (int)(k >> kbits), B = (int)(k & mask);
    const float fa = __ldg(f + A), fb = __ldg(f + B);
    const float w = __fdiv_rn(__fsub_rn(iso, fa), __fsub_rn(fb, fa));
    if (GRID) {
      int ia, ja, ka, ib, jb, kb;
      grid_ijk(g, A, ia, ja, ka);
      grid_ijk(g, B, ib, jb, kb);
      verts[3 * v + 0] = lerp_rn(coord(g.ox, g.sx, ia, g.mx), coord(g.ox, g.sx, ib, g.mx), w);
      verts[3 * v + 1] = lerp_rn(coord(g.oy, g.sy, ja, g.my), coord(g.oy, g.sy, jb, g.my), w);
      verts[3 * v + 2] = lerp_rn(coord(g.oz, g.sz, ka, g.mz), coord(g.oz, g.sz, kb, g.mz), w);
    } else {
      const float* pa = pts + 3 * (long long)A;
      const float* pb = pts + 3 * (long long)B;
#pragma unroll
      for (int a = 0; a < 3; ++a) verts[3 * v + a] = lerp_rn(__ldg(pa + a), __ldg(pb + a), w);
    }
    if (ra) {
      ra[v] = A;
      rb[v] = B;
      rw[v] = w;
    }
  }
}

// DispatcherMapCell<MarchingTetrahedraCount>: NumFaces of every cell as an
// int32 count array (cells with an id outside [0, P) count 0 and raise
// kErrBadIndex in *err).
__global__ void __launch_bounds__(256) k_mt_cell_count(const int32_t* __restrict__ conn,
                                                       long long C,
                                                       const float* __restrict__ f, long long P,
                                                       float iso, int32_t* __restrict__ count,
                                                       int* err) {
  bool bad = false;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < C;
       c += (long long)gridDim.x * blockDim.x) {
    int id[4];
    int nf = 0;
    if (load_tet<false>(conn, c, P, id)) {
      const float v[4] = {__ldg(f + id[0]), __ldg(f + id[1]), __ldg(f + id[2]), __ldg(f + id[3])};
      nf = mt_faces(mt_classify(v, iso));
    } else {
      bad = true;
    }
    count[c] = nf;
  }
  if (bad && err) atomicOr(err, kErrBadIndex);
}

__global__ void k_mt_set_header(MtMergeHeader* hdr, MtMergeHeader v) { *hdr = v; }

// ---- Marching cubes driven by an arbitrary count array ----------------------
// DispatcherGenerateInterpolatedCells<MarchingCubesGenerate> with any per-cell
// count array (DispatcherGenerateInterpolatedCells.h:158-231): the inclusive
// scan of the counts, UpperBounds(scan, t) for the input cell of output
// triangle t, visit index t - (scan[cell] - count[cell]), then the worklet's
// triangle (MarchingCubes.h:121-168).  A count of 0 drops a cell's
// triangles; a visit index at or beyond the cell's NumFaces (a count the
// worklet cannot honour) raises kErrBadCount and writes nothing for it.

// cellVertEdges (MarchingCubes.h:131-135): byte e = corners of edge e (low
// nibble, high nibble), bytes 0-7 in the first word, 8-11 in the second.
constexpr unsigned long long kHexEdgesLo = 0x7467655430232110ull;
constexpr unsigned int kHexEdgesHi = 0x73625140u;

__device__ __forceinline__ int hex_edge(int e) {
  return e < 8 ? (int)((kHexEdgesLo >> (8 * e)) & 0xFF) : (int)((kHexEdgesHi >> (8 * (e - 8))) & 0xFF);
}

template <bool KEYS>
__global__ void __launch_bounds__(256) k_mc_counted(Grid g, const float* __restrict__ f, float iso,
                                                    const int32_t* __restrict__ count,
                                                    const int32_t* __restrict__ scan, long long C,
                                                    unsigned long long mcx,
                                                    unsigned long long mcy, Info* info, MtOut o) {
  __shared__ uint64_t s_case[256];
  s_case[threadIdx.x] = kMcCase[threadIdx.x];
  __syncthreads();
  const long long T = info->total_a;
  if (info->error) return;
  if (!KEYS && (T > o.tcap || 3 * T > o.vcap)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&info->error, kErrCapacity);
    return;
  }
  const unsigned cx = (unsigned)(g.nx - 1), cy = (unsigned)(g.ny - 1);
  const long long sy = g.nx, sz = (long long)g.nx * g.ny;
  bool bad = false;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < T;
       t += (long long)gridDim.x * blockDim.x) {
    long long lo = 0, hi = C;  // UpperBounds: the first cell whose scan exceeds t
    while (lo < hi) {
      const long long mid = (lo + hi) >> 1;
      if ((long long)__ldg(scan + mid) <= t) lo = mid + 1;
      else hi = mid;
    }
    if (lo >= C) {
      bad = true;
      continue;
    }
    const long long c = lo;
    const long long visit = t - ((long long)__ldg(scan + c) - __ldg(count + c));
    const unsigned r = div_by((unsigned)c, mcx);
    const int i = (int)((unsigned)c - r * cx);
    const unsigned kk = div_by(r, mcy);
    const int k = (int)kk, j = (int)(r - kk * cy);
    const long long p0 = ((long long)k * g.ny + j) * g.nx + i;
    int cs = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int dx = (0x66 >> q) & 1, dy = (0xCC >> q) & 1, dz = q >> 2;
      cs |= (__ldg(f + p0 + dx + dy * sy + dz * sz) > iso ? 1 : 0) << q;
    }
    const uint64_t word = s_case[cs];
    if (visit < 0 || visit >= (long long)(word >> 60)) {
      bad = true;
      continue;
    }
    for (int m = 0; m < 3; ++m) {
      const int e = (int)((word >> (4 * (3 * visit + m))) & 0xF);
      const int ed = hex_edge(e);
      const int q0 = ed & 0xF, q1 = ed >> 4;
      const long long id0 = p0 + ((0x66 >> q0) & 1) + ((0xCC >> q0) & 1) * sy + (q0 >> 2) * sz;
      const long long id1 = p0 + ((0x66 >> q1) & 1) + ((0xCC >> q1) & 1) * sy + (q1 >> 2) * sz;
      // the lower point id first (MarchingCubes.h:148-157)
      const bool keep = id0 < id1;
      const int qa = keep ? q0 : q1, qb = keep ? q1 : q0;
      const int A = (int)(keep ? id0 : id1), B = (int)(keep ? id1 : id0);
      const long long rec = 3 * t + m;
      if (KEYS) {
        if (o.wide)
          static_cast<unsigned long long*>(o.keys)[rec] =
              ((unsigned long long)A << o.kbits) | (unsigned long long)B;
        else
          static_cast<uint32_t*>(o.keys)[rec] = ((uint32_t)A << o.kbits) | (uint32_t)B;
      } else {
        const float fa = __ldg(f + A), fb = __ldg(f + B);
        const float w = __fdiv_rn(__fsub_rn(iso, fa), __fsub_rn(fb, fa));
        const int ia = i + ((0x66 >> qa) & 1), ja = j + ((0xCC >> qa) & 1), ka = k + (qa >> 2);
        const int ib = i + ((0x66 >> qb) & 1), jb = j + ((0xCC >> qb) & 1), kb = k + (qb >> 2);
        o.verts[3 * rec + 0] = lerp_rn(coord(g.ox, g.sx, ia, g.mx), coord(g.ox, g.sx, ib, g.mx), w);
        o.verts[3 * rec + 1] = lerp_rn(coord(g.oy, g.sy, ja, g.my), coord(g.oy, g.sy, jb, g.my), w);
        o.verts[3 * rec + 2] = lerp_rn(coord(g.oz, g.sz, ka, g.mz), coord(g.oz, g.sz, kb, g.mz), w);
        o.tconn[rec] = (int32_t)rec;
        if (o.ra) {
          o.ra[rec] = A;
          o.rb[rec] = B;
          o.rw[rec] = w;
        }
      }
    }
  }
  if (bad) atomicOr(&info->error, kErrBadCount);
}

__global__ void k_set_total(Info* info, long long T, int error) {
  info->total_a = T;
  info->total_b = 0;
  info->total_c = 0;
  info->error = error;
}

void launch_set_total(Info* info, long long T, int error, cudaStream_t s) {
  k_set_total<<<1, 1, 0, s>>>(info, T, error);
}

void launch_mc_counted(const Grid& g, const float* f, float iso, const int32_t* count,
                       const int32_t* scan, Info* info, void* keys, float* verts, long long vcap,
                       int32_t* tconn, long long tcap, int32_t* ra, int32_t* rb, float* rw,
                       long long T_hint, int num_sms, cudaStream_t s) {
  const long long C = (long long)(g.nx - 1) * (g.ny - 1) * (g.nz - 1);
  MtOut o{};
  o.verts = verts;
  o.tconn = tconn;
  o.ra = ra;
  o.rb = rb;
  o.rw = rw;
  o.keys = keys;
  o.kbits = mt_key_bits(g.P);
  o.wide = 2 * o.kbits > 32;
  o.vcap = vcap;
  o.tcap = tcap;
  const unsigned long long mcx = div_multiplier((unsigned)(g.nx - 1));
  const unsigned long long mcy = div_multiplier((unsigned)(g.ny - 1));
  const long long want = (T_hint + 255) / 256;
  if (keys) {
    const int b = resident_blocks(k_mc_counted<true>, 256, 0, num_sms, want);
    k_mc_counted<true><<<b, 256, 0, s>>>(g, f, iso, count, scan, C, mcx, mcy, info, o);
  } else {
    const int b = resident_blocks(k_mc_counted<false>, 256, 0, num_sms, want);
    k_mc_counted<false><<<b, 256, 0, s>>>(g, f, iso, count, scan, C, mcx, mcy, info, o);
  }
}

// ---- Tetrahedralize (the upstream caller: uniform grid -> tetrahedra) -----
// PossibleTetraSplitCases (dax/worklet/Tetrahedralize.h:36-48): rows 0-4
// split even cell ids, rows 5-9 odd ones; entries are voxel corners in
// TopologyUniform order.
constexpr uint8_t kTetSplit[10][4] = {{2, 1, 5, 0}, {0, 2, 3, 7}, {2, 5, 6, 7}, {0, 7, 4, 5},
                                      {0, 2, 7, 5}, {1, 3, 6, 2}, {0, 1, 3, 4}, {1, 4, 5, 6},
                                      {3, 6, 7, 4}, {1, 4, 6, 3}};
// rows r0 .. r0+3 as 16-bit fields of corner nibbles
constexpr unsigned long long tet_split_word(int r0) {
  unsigned long long w = 0;
  for (int r = r0; r < r0 + 4 && r < 10; ++r)
    for (int t = 0; t < 4; ++t)
      w |= (unsigned long long)kTetSplit[r][t] << (16 * (r - r0) + 4 * t);
  return w;
}
constexpr unsigned long long kTetSplit0 = tet_split_word(0), kTetSplit1 = tet_split_word(4),
                             kTetSplit2 = tet_split_word(8);

// One thread per output tetrahedron o: cell o / 5, visit o % 5
// (Tetrahedralize.h:71-80); consecutive threads write consecutive 16 bytes.
template <bool VEC>
__global__ void __launch_bounds__(256) k_tetrahedralize(Grid g, unsigned long long mcx,
                                                        unsigned long long mcy, long long n_out,
                                                        int32_t* __restrict__ out) {
  const unsigned cx = (unsigned)(g.nx - 1), cy = (unsigned)(g.ny - 1);
  for (long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x; o < n_out;
       o += (long long)gridDim.x * blockDim.x) {
    const unsigned c = (unsigned)(o / 5);
    const int visit = (int)(o - 5ll * c);
    const unsigned r = div_by(c, mcx);
    const unsigned i = c - r * cx;
    const unsigned k = div_by(r, mcy);
    const unsigned j = r - k * cy;
    const int first = (int)(i + (unsigned)g.nx * (j + (unsigned)g.ny * k));
    const int sy = g.nx, sz = g.nx * g.ny;
    const int sr = visit + 5 * (int)(c & 1);  // split row
    const unsigned long long sw = sr < 4 ? kTetSplit0 : (sr < 8 ? kTetSplit1 : kTetSplit2);
    const unsigned row = (unsigned)(sw >> (16 * (sr & 3))) & 0xFFFFu;
    // voxel corner n (TopologyUniform order) is +x for n in {1,2,5,6}
    // (0x66), +y for n in {2,3,6,7} (0xCC), +z for n >= 4
    int q4[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int n = (int)((row >> (4 * t)) & 0xF);
      q4[t] = first + ((0x66 >> n) & 1) + sy * ((0xCC >> n) & 1) + sz * (n >> 2);
    }
    const int4 q = make_int4(q4[0], q4[1], q4[2], q4[3]);
    if (VEC) {
      reinterpret_cast<int4*>(out)[o] = q;
    } else {
      out[4 * o + 0] = q.x;
      out[4 * o + 1] = q.y;
      out[4 * o + 2] = q.z;
      out[4 * o + 3] = q.w;
    }
  }
}

// The implicit coordinates of a uniform grid as an explicit [P][3] array
// (UniformGrid::ComputePointCoordinates, dax/cont/UniformGrid.h:82-89).
__global__ void __launch_bounds__(256) k_point_coordinates(Grid g, float* __restrict__ out) {
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < g.P;
       p += (long long)gridDim.x * blockDim.x) {
    const unsigned row = (unsigned)(p / g.nx);
    const int i = (int)(p - (long long)row * g.nx);
    int j, k;
    split_row(g, row, j, k);
    out[3 * p + 0] = coord(g.ox, g.sx, i, g.mx);
    out[3 * p + 1] = coord(g.oy, g.sy, j, g.my);
    out[3 * p + 2] = coord(g.oz, g.sz, k, g.mz);
  }
}

void launch_tetrahedralize(const Grid& g, int32_t* out, int num_sms, cudaStream_t s) {
  const long long C = (long long)(g.nx - 1) * (g.ny - 1) * (g.nz - 1);
  const unsigned long long mcx = div_multiplier((unsigned)(g.nx - 1));
  const unsigned long long mcy = div_multiplier((unsigned)(g.ny - 1));
  const long long n_out = 5 * C;
  if ((reinterpret_cast<uintptr_t>(out) & 15) == 0) {
    const int b = resident_blocks(k_tetrahedralize<true>, 256, 0, num_sms, (n_out + 255) / 256);
    k_tetrahedralize<true><<<b, 256, 0, s>>>(g, mcx, mcy, n_out, out);
  } else {
    const int b = resident_blocks(k_tetrahedralize<false>, 256, 0, num_sms, (n_out + 255) / 256);
    k_tetrahedralize<false><<<b, 256, 0, s>>>(g, mcx, mcy, n_out, out);
  }
}

void launch_point_coordinates(const Grid& g, float* out, int num_sms, cudaStream_t s) {
  const int b = resident_blocks(k_point_coordinates, 256, 0, num_sms, (g.P + 255) / 256);
  k_point_coordinates<<<b, 256, 0, s>>>(g, out);
}

// ---- host side --------------------------------------------------------------

MtLayout mt_layout(long long C) {
  auto a256 = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const long long tiles = (C + kMtTile - 1) / kMtTile;
  MtLayout L;
  L.tiles = (int)tiles;
  L.info = 0;
  L.tile_tot = a256(sizeof(Info));
  L.tile_off = a256(L.tile_tot + 4 * (size_t)(tiles + 1));
  L.chunk_tot = a256(L.tile_off + 8 * (size_t)(tiles + 1));
  L.cases = a256(L.chunk_tot + 4 * (size_t)tiles * (kMtTile / kMtChunk));
  L.total = a256(L.cases + (size_t)(C > 0 ? C : 1));
  return L;
}

int mt_key_bits(long long P) {
  int b = 1;
  while (b < 31 && (1ll << b) < P) ++b;
  return b;
}

void launch_mt_count(const int32_t* conn, long long C, const float* f, long long P, float iso,
                     char* scratch, int num_sms, cudaStream_t s) {
  const MtLayout L = mt_layout(C);
  Info* info = reinterpret_cast<Info*>(scratch + L.info);
  cudaMemsetAsync(info, 0, sizeof(Info), s);
  const bool vec = (reinterpret_cast<uintptr_t>(conn) & 15) == 0;
  uint8_t* cases = reinterpret_cast<uint8_t*>(scratch + L.cases);
  unsigned* tot = reinterpret_cast<unsigned*>(scratch + L.tile_tot);
  unsigned* ctot = reinterpret_cast<unsigned*>(scratch + L.chunk_tot);
  if (vec) {
    const int b = resident_blocks(k_mt_count<true>, kMtThreads, 0, num_sms, L.tiles);
    k_mt_count<true><<<b, kMtThreads, 0, s>>>(conn, C, f, P, iso, cases, tot, ctot, info, L.tiles);
  } else {
    const int b = resident_blocks(k_mt_count<false>, kMtThreads, 0, num_sms, L.tiles);
    k_mt_count<false><<<b, kMtThreads, 0, s>>>(conn, C, f, P, iso, cases, tot, ctot, info,
                                               L.tiles);
  }
  k_mt_tile_scan<<<1, 1024, 0, s>>>(tot, L.tiles,
                                    reinterpret_cast<unsigned long long*>(scratch + L.tile_off),
                                    info);
}

namespace {

template <bool KEYS>
void emit(const float* pts, const int32_t* conn, long long C, const float* f, long long P,
          float iso, char* scratch, const MtOut& o, int num_sms, cudaStream_t s) {
  const MtLayout L = mt_layout(C);
  Info* info = reinterpret_cast<Info*>(scratch + L.info);
  const uint8_t* cases = reinterpret_cast<const uint8_t*>(scratch + L.cases);
  const unsigned long long* off = reinterpret_cast<const unsigned long long*>(scratch + L.tile_off);
  const unsigned* ctot = reinterpret_cast<const unsigned*>(scratch + L.chunk_tot);
  const long long chunks = (C + kMtChunk - 1) / kMtChunk;
  const long long want = (chunks + kMtThreads / 32 - 1) / (kMtThreads / 32);
  if ((reinterpret_cast<uintptr_t>(conn) & 15) == 0) {
    const int b = resident_blocks(k_mt_emit<true, KEYS>, kMtThreads, 0, num_sms, want);
    k_mt_emit<true, KEYS><<<b, kMtThreads, 0, s>>>(pts, conn, C, f, P, iso, cases, off, ctot, info,
                                                   o, chunks);
  } else {
    const int b = resident_blocks(k_mt_emit<false, KEYS>, kMtThreads, 0, num_sms, want);
    k_mt_emit<false, KEYS><<<b, kMtThreads, 0, s>>>(pts, conn, C, f, P, iso, cases, off, ctot,
                                                    info, o, chunks);
  }
}

}  // namespace

void launch_mt_emit_direct(const float* pts, const int32_t* conn, long long C, const float* f,
                           long long P, float iso, char* scratch, float* verts, long long vcap,
                           int32_t* tconn, long long tcap, int32_t* ra, int32_t* rb, float* rw,
                           int num_sms, cudaStream_t s) {
  MtOut o{};
  o.verts = verts;
  o.tconn = tconn;
  o.ra = ra;
  o.rb = rb;
  o.rw = rw;
  o.vcap = vcap;
  o.tcap = tcap;
  emit<false>(pts, conn, C, f, P, iso, scratch, o, num_sms, s);
}

void launch_mt_emit_keys(const int32_t* conn, long long C, const float* f, long long P, float iso,
                         char* scratch, void* keys, int num_sms, cudaStream_t s) {
  MtOut o{};
  o.keys = keys;
  o.kbits = mt_key_bits(P);
  o.wide = 2 * o.kbits > 32;
  emit<true>(nullptr, conn, C, f, P, iso, scratch, o, num_sms, s);
}

void launch_mt_cell_count(const int32_t* conn, long long C, const float* f, long long P,
                          float iso, int32_t* count, int* err, int num_sms, cudaStream_t s) {
  const int b = resident_blocks(k_mt_cell_count, 256, 0, num_sms, (C + 255) / 256);
  k_mt_cell_count<<<b, 256, 0, s>>>(conn, C, f, P, iso, count, err);
}

void launch_mt_set_merged(void* merge, long long T, long long V, size_t keys_off,
                          size_t uniq_off, cudaStream_t s) {
  MtMergeHeader h{kMtMergeMagic, (unsigned long long)V, (unsigned long long)keys_off,
                  (unsigned long long)uniq_off, (unsigned long long)T};
  k_mt_set_header<<<1, 1, 0, s>>>(static_cast<MtMergeHeader*>(merge), h);
}

void launch_mt_merged(const float* pts, const Grid* grid, Info* info, const float* f,
                      long long P, float iso, const void* merge, size_t merge_bytes, float* verts,
                      long long vcap, int32_t* tconn, long long tcap, int32_t* ra, int32_t* rb,
                      float* rw, int num_sms, cudaStream_t s) {
  const Grid g = grid ? *grid : Grid{};
  const unsigned long long mb = (unsigned long long)merge_bytes;
  const char* m = static_cast<const char*>(merge);
  const int kbits = mt_key_bits(P);
  const long long want = (3 * tcap + 255) / 256;  // grid-stride: never more than resident
  if (2 * kbits > 32) {
    typedef unsigned long long U;
    const int b1 = resident_blocks(k_mt_merged_conn<U>, 256, 0, num_sms, want);
    k_mt_merged_conn<U><<<b1, 256, 0, s>>>(m, mb, info, tcap, vcap, tconn);
    if (grid) {
      const int b2 = resident_blocks(k_mt_merged_verts<U, true>, 256, 0, num_sms, want);
      k_mt_merged_verts<U, true><<<b2, 256, 0, s>>>(m, mb, g, info, tcap, vcap, kbits, pts, f, iso,
                                                    verts, ra, rb, rw);
    } else {
      const int b2 = resident_blocks(k_mt_merged_verts<U, false>, 256, 0, num_sms, want);
      k_mt_merged_verts<U, false><<<b2, 256, 0, s>>>(m, mb, g, info, tcap, vcap, kbits, pts, f,
                                                     iso, verts, ra, rb, rw);
    }
  } else {
    typedef uint32_t U;
    const int b1 = resident_blocks(k_mt_merged_conn<U>, 256, 0, num_sms, want);
    k_mt_merged_conn<U><<<b1, 256, 0, s>>>(m, mb, info, tcap, vcap, tconn);
    if (grid) {
      const int b2 = resident_blocks(k_mt_merged_verts<U, true>, 256, 0, num_sms, want);
      k_mt_merged_verts<U, true><<<b2, 256, 0, s>>>(m, mb, g, info, tcap, vcap, kbits, pts, f, iso,
                                                    verts, ra, rb, rw);
    } else {
      const int b2 = resident_blocks(k_mt_merged_verts<U, false>, 256, 0, num_sms, want);
      k_mt_merged_verts<U, false><<<b2, 256, 0, s>>>(m, mb, g, info, tcap, vcap, kbits, pts, f,
                                                     iso, verts, ra, rb, rw);
    }
  }
}

}  // namespace daxgb
