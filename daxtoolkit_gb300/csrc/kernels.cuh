// Launchers shared between the kernel translation units and the C ABI.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace daxgb {

// Bits words allocated for P points: whole 128-point chunks plus padding
// that unaligned 64-bit fetches may touch.
inline long long bit_words(long long P) { return ((P + 127) / 128) * 4 + 8; }

constexpr int kRowsPerTile = 256;   // rows per look-back tile in K2

// Lanes that cooperate on one point row in K2/K3: the power of two >= the
// row's word count, at most a warp.
inline int lanes_per_row(int wr) {
  int g = 1;
  while (g < wr && g < 32) g <<= 1;
  return g;
}

void launch_classify_bits(int mode, const float* f, long long P, float a, float b, uint32_t* bits,
                          long long nwords, int num_sms, cudaStream_t s);
void launch_cell_count(int mode, const Grid& g, const float* f, float a, float b, int32_t* count,
                       uint8_t* cases, int num_sms, cudaStream_t s);

void launch_mc_rows(const Grid& g, const uint32_t* bits, long long* row_t, long long* row_v,
                    unsigned long long* status, Info* info, int tiles, cudaStream_t s);
void launch_mc_emit(const Grid& g, const float* f, float iso, bool merge, const uint32_t* bits,
                    const long long* row_t, const long long* row_v, Info* info, float* verts,
                    long long vcap, int32_t* conn, long long tcap, int32_t* ra, int32_t* rb,
                    float* rw, int num_sms, cudaStream_t s);
void launch_interpolate(const int32_t* ra, const int32_t* rb, const float* rw, long long n,
                        const float* in, float* out, int num_sms, cudaStream_t s);

void launch_thr_rows(const Grid& g, const uint32_t* bits, uint32_t* used, long long* row_k,
                     long long* row_u, unsigned long long* status, Info* info, int tiles,
                     cudaStream_t s);
void launch_thr_emit(const Grid& g, const float* f, const uint32_t* bits, const uint32_t* used,
                     const long long* row_k, const long long* row_u, Info* info, int32_t* conn,
                     long long kcap, float* coords, float* fout, long long ucap, int num_sms,
                     cudaStream_t s);

void launch_cell_gradient(const Grid& g, const float* f, float* out, int num_sms, cudaStream_t s);

}  // namespace daxgb
