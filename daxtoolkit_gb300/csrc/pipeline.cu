// Pipelined marching cubes on one grid: the whole count + generate of
// dax_gb300_mc_count / dax_gb300_mc_generate in one call, with the grid cut
// into z-ordered slabs so that the passes of different slabs overlap.
//
// One frame runs four passes: K1 streams the field (HBM-bound), K2a/K2b count
// and scan the row words of the bit stream and K3 emits the surface (both
// latency-bound, working from L2).  Run back to back they leave HBM idle for
// more than half of the frame.  Here the row words are cut at scan-tile
// boundaries W_0 = 0 < W_1 < ... < W_S = rowwords, and:
//
//   caller stream : K1(0) K1(1) ... K1(S-1)          (classification of chunks
//                                                     [K_s, K_s+1))
//   stream b      :   count+scan(0)   count+scan(1) ...   (tiles of [W_s, W_s+1),
//                                                     each after K1(s))
//   stream c      :      emit(0)        emit(1)  ...  (active words of
//                                                     [E_s, E_s+1), after scan(s))
//
// so the classification of slab s+1 streams the field while slab s is
// counted, scanned and emitted.  The chunk ranges K are chosen so that K1(0..s)
// has classified every point that count(s) reads (the rows of slab s plus
// one plane and one row).  The emit ranges trail the count ranges by one plane
// plus one row plus two words (E_s = W_s - shift): an emitted word reads the
// offsets of owner words up to that far ahead, and those lie in the scanned
// part.  Every slab's offsets are global (the scan of slab s adds the totals
// of all earlier tiles), so the output is the same as the two-call pipeline's,
// bit for bit.
#include <mutex>
#include <string>

#include "../../include/dax_gb300.h"
#include "common.cuh"
#include "kernels.cuh"

namespace daxgb {

namespace {
int g_pipe_slabs = 1;
PipeOptions g_pipe_opts;
}

void set_pipeline_slabs(int slabs) { g_pipe_slabs = slabs < 1 ? 1 : slabs; }
int pipeline_slabs() { return g_pipe_slabs; }
void set_pipeline_options(const PipeOptions& o) { g_pipe_opts = o; }
PipeOptions pipeline_options() { return g_pipe_opts; }

SlabPlan plan_slabs(const Grid& g, int wanted) {
  SlabPlan p{};
  const long long W = g.R * g.wr;
  const int tiles = word_scan_tiles(W);
  const long long chunks = (g.P + 127) / 128;
  const long long shift = (long long)g.wr * (g.ny + 1) + 2;
  int S = wanted < 1 ? 1 : (wanted > kMaxSlabs ? kMaxSlabs : wanted);
  if (S > tiles) S = tiles;
  if (S < 1) S = 1;
  // every slab but the last must span two shifts, so that the emit ranges
  // E_s = W_s - shift are increasing and start at or after 0
  while (S > 1 && (long long)((tiles + S - 1) / S) * kScanTile < 2 * shift) --S;
  const int tp = (tiles + S - 1) / S;
  S = (tiles + tp - 1) / tp;
  p.S = S;
  for (int s = 0; s <= S; ++s) {
    p.tile[s] = s * tp < tiles ? s * tp : tiles;
    const long long w = (long long)p.tile[s] * kScanTile;
    p.W[s] = w < W ? w : W;
  }
  p.E[0] = 0;
  for (int s = 1; s < S; ++s) p.E[s] = p.W[s] - shift;
  p.E[S] = W;
  p.K[0] = 0;
  for (int s = 0; s < S; ++s) {
    // rows through slab s, then the rows a count of its last row reads
    // (j + 1, k + 1 and the next row word), in points
    const long long rows = (p.W[s + 1] + g.wr - 1) / g.wr;
    const long long pts = (rows + g.ny + 2) * (long long)g.nx + 256;
    long long k = (pts + 127) / 128;
    if (k > chunks) k = chunks;
    p.K[s + 1] = k > p.K[s] ? k : p.K[s];
  }
  p.K[S] = chunks;
  return p;
}

namespace {

constexpr int kMaxDevices = 64;

// Per device: the two streams the count/scan and emit passes run on, and the
// events that order them against the caller's stream.  Created on the first
// pipelined call on the device; the mutex serialises enqueues that reuse
// the events.
struct PipeStreams {
  bool ready = false;
  std::mutex mutex;
  cudaStream_t b = nullptr, c[kMaxEmitStreams] = {};
  cudaEvent_t start = nullptr, bend = nullptr, cend[kMaxEmitStreams] = {};
  cudaEvent_t kdone[kMaxSlabs] = {}, sdone[kMaxSlabs] = {};
  // timeline (timing events): t0, then per slab the ends of K1, of the wait
  // before count, of count, of scan, of the wait before emit, of emit
  bool timeline = false;
  int timeline_slabs = 0;
  cudaEvent_t t0 = nullptr, tl[kMaxSlabs][kTimelinePoints] = {};
};

std::mutex g_pipe_init;
PipeStreams g_pipe[kMaxDevices];

int pipe_fail(cudaError_t e, const char* what) {
  set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
  return DAX_GB300_ERROR_CUDA;
}

int pipe_streams(PipeStreams** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return pipe_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) {
    set_last_error("device index out of range for the pipeline stream table");
    return DAX_GB300_ERROR_UNSUPPORTED;
  }
  PipeStreams& ps = g_pipe[dev];
  std::lock_guard<std::mutex> lock(g_pipe_init);
  if (!ps.ready) {
    int lo = 0, hi = 0;
    e = cudaDeviceGetStreamPriorityRange(&lo, &hi);
    // the latency-bound passes get the higher priority: when a block slot
    // frees, theirs are scheduled before more classification blocks
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&ps.b, cudaStreamNonBlocking, hi);
    const unsigned fl = cudaEventDisableTiming;
    for (int i = 0; i < kMaxEmitStreams && e == cudaSuccess; ++i) {
      e = cudaStreamCreateWithPriority(&ps.c[i], cudaStreamNonBlocking, hi);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ps.cend[i], fl);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ps.start, fl);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ps.bend, fl);
    for (int i = 0; i < kMaxSlabs && e == cudaSuccess; ++i) {
      e = cudaEventCreateWithFlags(&ps.kdone[i], fl);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ps.sdone[i], fl);
    }
    if (e == cudaSuccess) e = cudaEventCreate(&ps.t0);
    for (int i = 0; i < kMaxSlabs && e == cudaSuccess; ++i)
      for (int j = 0; j < kTimelinePoints && e == cudaSuccess; ++j)
        e = cudaEventCreate(&ps.tl[i][j]);
    if (e != cudaSuccess) return pipe_fail(e, "creating the pipeline streams");
    ps.ready = true;
  }
  *out = &ps;
  return DAX_GB300_SUCCESS;
}

}  // namespace

int launch_mc_pipeline(const Grid& g, const float* f, bool aligned, float iso, bool merge,
                       uint32_t* bits, long long nwords, const WordOffsets& o, Info* info,
                       uint32_t* slab_act, float* verts, long long vcap, int32_t* conn,
                       long long tcap, int32_t* ra, int32_t* rb, float* rw, uint32_t* fctl,
                       bool fused, int num_sms, cudaStream_t s) {
  PipeStreams* ps = nullptr;
  int st = pipe_streams(&ps);
  if (st) return st;
  const SlabPlan p = plan_slabs(g, g_pipe_slabs);
  if (p.S == 1 && fused) {
    // one slab: the fused count pass (classification and counts in one
    // launch, then the scan) and the emit, on the caller's stream
    std::lock_guard<std::mutex> lock(ps->mutex);
    const bool tl = ps->timeline;
    ps->timeline_slabs = tl ? 1 : 0;
    if (tl) cudaEventRecord(ps->t0, s);
    const int e = launch_fused_count(0, g, f, iso, 0.0f, bits, nwords, o, info, nullptr, nullptr,
                                     fctl, num_sms, s);
    if (e != 0) return pipe_fail(static_cast<cudaError_t>(e), "fused count pass");
    if (tl)
      for (int j = 0; j < 5; ++j) cudaEventRecord(ps->tl[0][j], s);
    launch_mc_emit(single_set(g, f, iso, 0.0f), merge, bits, o, info, verts, vcap, conn, tcap, ra,
                   rb, rw, num_sms, s);
    if (tl) cudaEventRecord(ps->tl[0][5], s);
    const cudaError_t le = cudaGetLastError();
    return le == cudaSuccess ? DAX_GB300_SUCCESS : pipe_fail(le, "pipelined marching cubes");
  }
  if (p.S == 1) {
    // one slab: nothing to overlap, so the two-call passes run on the
    // caller's stream (no hops to the pipeline's streams): classification
    // (clearing Info), count and scan, emit
    std::lock_guard<std::mutex> lock(ps->mutex);
    const bool tl = ps->timeline;
    ps->timeline_slabs = tl ? 1 : 0;
    if (tl) cudaEventRecord(ps->t0, s);
    const GridSet S1 = single_set(g, f, iso, 0.0f);
    launch_classify_range(0, S1, aligned, bits, nwords, 0, S1.chunks, info, kPassClassify, false,
                          num_sms, s);
    if (tl) cudaEventRecord(ps->tl[0][0], s);
    if (tl) cudaEventRecord(ps->tl[0][1], s);
    launch_mc_scan(S1, bits, o, info, num_sms, s);
    if (tl)
      for (int j = 2; j < 5; ++j) cudaEventRecord(ps->tl[0][j], s);
    launch_mc_emit(S1, merge, bits, o, info, verts, vcap, conn, tcap, ra, rb, rw, num_sms, s);
    if (tl) cudaEventRecord(ps->tl[0][5], s);
    const cudaError_t le = cudaGetLastError();
    return le == cudaSuccess ? DAX_GB300_SUCCESS : pipe_fail(le, "pipelined marching cubes");
  }
  const PipeOptions opt = g_pipe_opts;
  const int ne = opt.emit_streams;
  const GridSet S = single_set(g, f, iso, 0.0f);
  SlabBounds B{};
  B.n = p.S;
  for (int i = 0; i < p.S; ++i) B.e[i] = p.E[i];
  // the slab section: active-word prefixes, then each slab's emit counters
  unsigned* ctr = slab_act + kSlabCounters;
  std::lock_guard<std::mutex> lock(ps->mutex);
  const bool tl = ps->timeline;
  ps->timeline_slabs = tl ? p.S : 0;
  auto mark = [&](int k, int j, cudaStream_t st) {
    if (tl) cudaEventRecord(ps->tl[k][j], st);
  };
  cudaError_t e = cudaMemsetAsync(ctr, 0, 2 * kMaxSlabs * sizeof(unsigned), s);
  if (tl && e == cudaSuccess) e = cudaEventRecord(ps->t0, s);
  if (e == cudaSuccess) e = cudaEventRecord(ps->start, s);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(ps->b, ps->start, 0);
  for (int i = 0; i < ne && e == cudaSuccess; ++i) e = cudaStreamWaitEvent(ps->c[i], ps->start, 0);
  for (int k = 0; k < p.S && e == cudaSuccess; ++k) {
    launch_classify_range(0, S, aligned, bits, nwords, p.K[k], p.K[k + 1], k == 0 ? info : nullptr,
                          kPassPipeClassify, opt.keep_field, num_sms, s);
    mark(k, 0, s);
    e = cudaEventRecord(ps->kdone[k], s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ps->b, ps->kdone[k], 0);
    if (e != cudaSuccess) break;
    mark(k, 1, ps->b);
    launch_mc_scan_slab(S, bits, o, info, p.tile[k], p.tile[k + 1], B, slab_act,
                        kPassPipeCount, num_sms, ps->b,
                        tl ? ps->tl[k][2] : nullptr);
    mark(k, 3, ps->b);
    cudaStream_t c = ps->c[k % ne];
    e = cudaEventRecord(ps->sdone[k], ps->b);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c, ps->sdone[k], 0);
    if (e != cudaSuccess) break;
    mark(k, 4, c);
    launch_mc_emit_range(S, merge, bits, o, info, verts, vcap, conn, tcap, ra, rb, rw, p.E[k],
                         p.E[k + 1], p.E[k + 1], slab_act + k, ctr + 2 * k, ctr + 2 * k + 1,
                         opt.emit_batch, kPassPipeEmit, num_sms, c);
    mark(k, 5, c);
  }
  // join the streams back into the caller's, also after a failed enqueue
  cudaError_t j = cudaEventRecord(ps->bend, ps->b);
  if (j == cudaSuccess) j = cudaStreamWaitEvent(s, ps->bend, 0);
  for (int i = 0; i < ne && j == cudaSuccess; ++i) {
    j = cudaEventRecord(ps->cend[i], ps->c[i]);
    if (j == cudaSuccess) j = cudaStreamWaitEvent(s, ps->cend[i], 0);
  }
  if (e == cudaSuccess) e = j;
  if (e == cudaSuccess) e = cudaGetLastError();
  return e == cudaSuccess ? DAX_GB300_SUCCESS : pipe_fail(e, "pipelined marching cubes");
}

}  // namespace daxgb

namespace daxgb {

int pipeline_timeline(int enable, float* out, int n, int* slabs) {
  PipeStreams* ps = nullptr;
  int st = pipe_streams(&ps);
  if (st) return st;
  std::lock_guard<std::mutex> lock(ps->mutex);
  if (enable >= 0) ps->timeline = enable != 0;
  if (slabs) *slabs = ps->timeline_slabs;
  if (!out) return DAX_GB300_SUCCESS;
  for (int k = 0; k < ps->timeline_slabs; ++k)
    for (int j = 0; j < kTimelinePoints; ++j) {
      const int i = k * kTimelinePoints + j;
      if (i >= n) return DAX_GB300_SUCCESS;
      cudaError_t e = cudaEventSynchronize(ps->tl[k][j]);
      if (e == cudaSuccess) e = cudaEventElapsedTime(&out[i], ps->t0, ps->tl[k][j]);
      if (e != cudaSuccess) return pipe_fail(e, "reading the pipeline timeline");
    }
  return DAX_GB300_SUCCESS;
}

}  // namespace daxgb
