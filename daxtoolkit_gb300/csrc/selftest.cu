// Self-check of div_by_recip against __fdiv_rn: the numerators with bit
// patterns first + i * step (i < count, modulo 2^32) against each given
// divisor, counting the results whose bits differ (NaN results count as
// equal to each other).  Where the numerator and the divisor lie in
// div_fast's domain (x = 0 or 2^-85 <= |x| < 2^87, 2^-30 <= |d| < 2^30),
// div_fast is checked against __fdiv_rn too.  Used by the tests to
// show, exhaustively over the numerators, that the reciprocal-based division
// of the stencil kernels is the correctly rounded one for the divisors a grid
// produces.
#include "../../include/dax_gb300.h"
#include "common.cuh"
#include "kernels.cuh"

namespace daxgb {

__global__ void __launch_bounds__(256) k_division_check(const float* __restrict__ divisors, int nd,
                                                        unsigned first, unsigned long long count,
                                                        unsigned step,
                                                        unsigned long long* __restrict__ mismatches) {
  const unsigned long long total = (unsigned long long)nd * count;
  unsigned long long bad = 0;
  for (unsigned long long t = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (unsigned long long)gridDim.x * blockDim.x) {
    const unsigned long long di = t / count, i = t - di * count;
    const float d = __ldg(divisors + di);
    const float x = __uint_as_float(first + (unsigned)i * step);
    const float r = recip_or_zero(d);
    const float a = div_by_recip(x, d, r);
    const float b = __fdiv_rn(x, d);
    const bool same = __float_as_uint(a) == __float_as_uint(b) || (a != a && b != b);
    bad += same ? 0ull : 1ull;
    const unsigned ux = mag_bits(x);
    if (width_in_band(d) && (ux == 0u || (ux >= 0x15000000u && ux < 0x6b000000u)))
      bad += __float_as_uint(div_fast(x, d, r)) == __float_as_uint(b) ? 0ull : 1ull;
  }
  bad += __shfl_xor_sync(kFull, bad, 16);
  bad += __shfl_xor_sync(kFull, bad, 8);
  bad += __shfl_xor_sync(kFull, bad, 4);
  bad += __shfl_xor_sync(kFull, bad, 2);
  bad += __shfl_xor_sync(kFull, bad, 1);
  if ((threadIdx.x & 31) == 0 && bad) atomicAdd(mismatches, bad);
}

}  // namespace daxgb

extern "C" int dax_gb300_selfcheck_division(const float* d_divisors, int num_divisors,
                                            uint32_t first, uint64_t count, uint32_t step,
                                            unsigned long long* d_mismatches, void* stream) {
  if (num_divisors <= 0 || count == 0) return DAX_GB300_SUCCESS;
  if (count > (1ull << 32)) {
    daxgb::set_last_error("at most 2^32 numerators");
    return DAX_GB300_ERROR_BAD_VALUE;
  }
  if (!d_divisors || !d_mismatches) {
    daxgb::set_last_error("NULL divisors or counter");
    return DAX_GB300_ERROR_BAD_VALUE;
  }
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int b = daxgb::resident_blocks(daxgb::k_division_check, 256, 0, sms, 1ll << 40);
  daxgb::k_division_check<<<b, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      d_divisors, num_divisors, first, count, step, d_mismatches);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    daxgb::set_last_error(cudaGetErrorString(e));
    return DAX_GB300_ERROR_CUDA;
  }
  return DAX_GB300_SUCCESS;
}
