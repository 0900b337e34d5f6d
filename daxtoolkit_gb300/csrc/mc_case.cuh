// The packed marching-cubes case table in constant memory (one copy per
// translation unit that includes this header).
#pragma once
#include <cstdint>
#include "mc_tables.h"

namespace daxgb {
static __constant__ uint64_t kMcCase[256] = DAX_GB300_MC_CASE_WORDS;

__device__ __forceinline__ int mc_num_tris(int cs) { return (int)(kMcCase[cs] >> 60); }
__device__ __forceinline__ int mc_edge(uint64_t word, int n) { return (int)((word >> (4 * n)) & 0xF); }
}  // namespace daxgb
