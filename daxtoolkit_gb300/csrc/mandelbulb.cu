// The Mandelbulb benchmark's compute pipeline (Benchmarks/Mandlebulb): the
// escape-iteration point field, the clip-and-count worklet of its cut view,
// and the per-point normals and colours of the extracted surface.  The
// surface itself is the marching-cubes pipeline (extractSurface,
// Mandlebulb.cxx:105-118) or the count-array-driven generate of the cut
// (extractCut, Mandlebulb.cxx:126-157); its GLUT/shader display is replaced
// by the device buffers these kernels write.
//
// Rounding: every add, multiply and divide is spelled out (no fused
// multiply-add) as the reference's float expressions round on the CPU.  The
// transcendental functions of the escape iteration (atan2, pow, sin, tan,
// cos) are CUDA's own; they may differ from the host C library's in the last
// place, so the escape iteration of a point on the fractal's boundary can
// differ between the two.  sqrt and 1/sqrt are correctly rounded on both, so
// normals and colours of the same surface agree bit for bit.
#include "common.cuh"
#include "coolwarm_table.h"
#include "kernels.cuh"
#include "mc_case.cuh"

namespace daxgb {

__constant__ unsigned char c_coolwarm[3 * DAX_GB300_COOLWARM_ENTRIES] = DAX_GB300_COOLWARM_RGB;

__device__ __forceinline__ float magsq3(float x, float y, float z) {
  return __fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z));
}

// worklet::Mandlebulb (Benchmarks/Mandlebulb/Worklets.h:65-109): the escape
// iteration of pos -> pos^10 + c (White and Nylander's power, :92-108), 0
// when c itself is outside radius sqrt(2), at most 35.
__device__ float mandelbulb_value(float cx, float cy, float cz) {
  float x = cx, y = cy, z = cz;
  if (magsq3(x, y, z) > 2.0f) return 0.0f;
  for (int i = 1; i < 35; ++i) {
    const float r2 = magsq3(x, y, z);
    const float t = __fsqrt_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)));
    const float thetaN = __fmul_rn(10.0f, atan2f(t, z));
    const float phiN = __fmul_rn(10.0f, atan2f(y, z));
    const float powR = powf(r2, 5.0f);
    float st, ct;  // sincosf: bit for bit sinf and cosf (checked over every float on GB300)
    sincosf(thetaN, &st, &ct);
    const float px = __fmul_rn(powR, __fmul_rn(st, tanf(phiN)));
    const float py = __fmul_rn(powR, __fmul_rn(st, sinf(phiN)));
    const float pz = __fmul_rn(powR, ct);
    x = __fadd_rn(px, cx);
    y = __fadd_rn(py, cy);
    z = __fadd_rn(pz, cz);
    if (magsq3(x, y, z) > 2.0f) return (float)i;
  }
  return 35.0f;
}

__global__ void __launch_bounds__(256) k_mandelbulb_field(Grid g, float* __restrict__ out) {
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < g.P;
       p += (long long)gridDim.x * blockDim.x) {
    const unsigned row = (unsigned)(p / g.nx);
    const int i = (int)(p - (long long)row * g.nx);
    int j, k;
    split_row(g, row, j, k);
    out[p] = mandelbulb_value(coord(g.ox, g.sx, i, g.mx), coord(g.oy, g.sy, j, g.my),
                              coord(g.oz, g.sz, k, g.mz));
  }
}

// worklet::ColorsAndNorms (Worklets.h:177-209) on an unmerged triangle
// surface: point v belongs to triangle v / 3; its normal is
// Normal(Cross(b - a, c - a)) = (1 / sqrt(dot(x, x))) * x
// (VectorAnalysis.h:182-201, 227-232; RSqrt is 1 / Sqrt off the GPU), its
// colour the cool-warm entry (int)(257 * clamp(|dot(p, (0.09, 0.09, 0.9))|,
// 0, 0.9999)) (CoolWarmColorMap.h:38-45) with alpha 255.
__global__ void __launch_bounds__(256) k_colors_and_norms(const float* __restrict__ verts,
                                                          long long nv, float* __restrict__ norms,
                                                          uint8_t* __restrict__ colors) {
  __shared__ unsigned char s_map[3 * DAX_GB300_COOLWARM_ENTRIES];
  for (int t = threadIdx.x; t < 3 * DAX_GB300_COOLWARM_ENTRIES; t += blockDim.x)
    s_map[t] = c_coolwarm[t];
  __syncthreads();
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < nv;
       v += (long long)gridDim.x * blockDim.x) {
    const float* c0 = verts + 3 * (3 * (v / 3));
    const float ax = __fsub_rn(c0[3], c0[0]), ay = __fsub_rn(c0[4], c0[1]),
                az = __fsub_rn(c0[5], c0[2]);
    const float bx = __fsub_rn(c0[6], c0[0]), by = __fsub_rn(c0[7], c0[1]),
                bz = __fsub_rn(c0[8], c0[2]);
    const float xx = __fsub_rn(__fmul_rn(ay, bz), __fmul_rn(az, by));
    const float xy = __fsub_rn(__fmul_rn(az, bx), __fmul_rn(ax, bz));
    const float xz = __fsub_rn(__fmul_rn(ax, by), __fmul_rn(ay, bx));
    const float r = __fdiv_rn(1.0f, __fsqrt_rn(magsq3(xx, xy, xz)));
    norms[3 * v + 0] = __fmul_rn(r, xx);
    norms[3 * v + 1] = __fmul_rn(r, xy);
    norms[3 * v + 2] = __fmul_rn(r, xz);
    const float* p = verts + 3 * v;
    float s = __fadd_rn(__fadd_rn(__fmul_rn(p[0], 0.09f), __fmul_rn(p[1], 0.09f)),
                        __fmul_rn(p[2], 0.9f));
    s = fminf(0.9999f, fmaxf(0.0f, fabsf(s)));
    const int idx = (int)__fmul_rn(257.0f, s);
    uchar4 c;
    c.x = s_map[3 * idx + 0];
    c.y = s_map[3 * idx + 1];
    c.z = s_map[3 * idx + 2];
    c.w = 255;
    reinterpret_cast<uchar4*>(colors)[v] = c;
  }
}

// worklet::MandlebulbClipCount (Worklets.h:112-170): a cell's marching-cubes
// triangle count when one of its points lies beyond the plane,
// dot(N, p - O) > dot(N, L); otherwise 0.  One thread per cell.
__global__ void __launch_bounds__(256) k_mandelbulb_clip_count(Grid g, const float* __restrict__ f,
                                                               float iso, float3 o, float3 n,
                                                               float loc, unsigned long long mcx,
                                                               unsigned long long mcy,
                                                               long long C,
                                                               int32_t* __restrict__ count) {
  __shared__ unsigned char s_nf[256];
  s_nf[threadIdx.x] = (unsigned char)mc_num_tris(threadIdx.x);
  __syncthreads();
  const unsigned cx = (unsigned)(g.nx - 1), cy = (unsigned)(g.ny - 1);
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < C;
       c += (long long)gridDim.x * blockDim.x) {
    const unsigned r = div_by((unsigned)c, mcx);
    const int i = (int)((unsigned)c - r * cx);
    const unsigned kk = div_by(r, mcy);
    const int k = (int)kk, j = (int)(r - kk * cy);
    const long long p0 = ((long long)k * g.ny + j) * g.nx + i;
    const long long sy = g.nx, sz = (long long)g.nx * g.ny;
    bool in = false;
    int cs = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int dx = (0x66 >> q) & 1, dy = (0xCC >> q) & 1, dz = q >> 2;
      in = in || plane_value(g, o, n, i + dx, j + dy, k + dz) > loc;
      cs |= (__ldg(f + p0 + dx + dy * sy + dz * sz) > iso ? 1 : 0) << q;
    }
    count[c] = in ? (int32_t)s_nf[cs] : 0;
  }
}

void launch_mandelbulb_field(const Grid& g, float* out, int num_sms, cudaStream_t s) {
  const int b = resident_blocks(k_mandelbulb_field, 256, 0, num_sms, (g.P + 255) / 256);
  k_mandelbulb_field<<<b, 256, 0, s>>>(g, out);
}

void launch_colors_and_norms(const float* verts, long long nv, float* norms, uint8_t* colors,
                             int num_sms, cudaStream_t s) {
  const int b = resident_blocks(k_colors_and_norms, 256, 0, num_sms, (nv + 255) / 256);
  k_colors_and_norms<<<b, 256, 0, s>>>(verts, nv, norms, colors);
}

void launch_mandelbulb_clip_count(const Grid& g, const float* f, float iso, float3 o, float3 n,
                                  float loc, int32_t* count, int num_sms, cudaStream_t s) {
  const long long C = (long long)(g.nx - 1) * (g.ny - 1) * (g.nz - 1);
  const int b = resident_blocks(k_mandelbulb_clip_count, 256, 0, num_sms, (C + 255) / 256);
  k_mandelbulb_clip_count<<<b, 256, 0, s>>>(g, f, iso, o, n, loc,
                                            div_multiplier((unsigned)(g.nx - 1)),
                                            div_multiplier((unsigned)(g.ny - 1)), C, count);
}

}  // namespace daxgb
