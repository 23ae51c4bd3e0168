// Headless renderer: the reference's viewer (src/solver.cpp:184-201 and src/example.cpp:55-70,
// a taichi.h X11 canvas) drawn by CUDA kernels into a device RGBA buffer instead of a window.
// The frame is the canvas's: background 0x112F41, the boundary box [0.04, 0.96]^2 outlined in
// 0x4FB99F, every particle a disc of `radius` pixels in its colour, y pointing up.  Particles
// are painted in index order, as the canvas draws them one after another: every covered pixel
// takes the colour of the last particle covering it (an atomicMax of the particle index, then
// one pass per pixel), so the image is deterministic.  3D positions are drawn in the x-y plane
// (a front view).
#include <cuda_runtime.h>
#include <stdint.h>

#include "nclr_gpu.h"

namespace {

constexpr uint32_t kBackground = 0x112F41u;
constexpr uint32_t kBox = 0x4FB99Fu;

__global__ void claim_kernel(const float *__restrict__ x, int64_t n, int dim, int w, int h,
                             float radius, int *__restrict__ winner) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  // explicit roundings (no fused multiply-add): the same pixels as a plain FP32 restatement
  const float px = __fmul_rn(x[p * dim], (float)w);
  const float py = __fmul_rn(__fsub_rn(1.0f, x[p * dim + 1]), (float)h);
  const int r = (int)ceilf(radius);
  const int ci = (int)floorf(px), cj = (int)floorf(py);
  const float r2 = __fmul_rn(radius, radius);
  for (int j = cj - r; j <= cj + r; ++j) {
    if (j < 0 || j >= h) continue;
    for (int i = ci - r; i <= ci + r; ++i) {
      if (i < 0 || i >= w) continue;
      const float dx = __fsub_rn((float)i + 0.5f, px), dy = __fsub_rn((float)j + 0.5f, py);
      if (__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)) <= r2)
        atomicMax(winner + (int64_t)j * w + i, (int)p);
    }
  }
}

// Background, then the box outline (a band of half-width `radius` around each edge), then the
// winning particle's colour.
__global__ void shade_kernel(const int *__restrict__ winner, const uint32_t *__restrict__ colors,
                             uint32_t color, int w, int h, float radius,
                             uint32_t *__restrict__ rgba) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (int64_t)w * h) return;
  const int i = (int)(k % w), j = (int)(k / w);
  const float cx = (float)i + 0.5f, cy = (float)j + 0.5f;
  const float x0 = __fmul_rn(0.04f, (float)w), x1 = __fmul_rn(0.96f, (float)w);
  const float y0 = __fmul_rn(0.04f, (float)h), y1 = __fmul_rn(0.96f, (float)h);
  const bool in_x = cx >= __fsub_rn(x0, radius) && cx <= __fadd_rn(x1, radius);
  const bool in_y = cy >= __fsub_rn(y0, radius) && cy <= __fadd_rn(y1, radius);
  const bool near_v = fabsf(__fsub_rn(cx, x0)) <= radius || fabsf(__fsub_rn(cx, x1)) <= radius;
  const bool near_h = fabsf(__fsub_rn(cy, y0)) <= radius || fabsf(__fsub_rn(cy, y1)) <= radius;
  uint32_t c = ((near_v && in_y) || (near_h && in_x)) ? kBox : kBackground;
  const int p = winner[k];
  if (p >= 0) c = colors ? colors[p] : color;
  rgba[k] = c;
}

}  // namespace

extern "C" {

nclr_status nclr_render_device(const float *x, int64_t n, int dim, const uint32_t *colors,
                               uint32_t color, int width, int height, float radius,
                               uint32_t *rgba, void *stream) {
  if ((dim != 2 && dim != 3) || n < 0 || width < 1 || height < 1 || !rgba || (n > 0 && !x) ||
      !(radius >= 0.0f) || radius > 64.0f || (int64_t)width * height > ((int64_t)1 << 28) ||
      n > (int64_t)0x7fffffff)
    return NCLR_ERR_INVALID;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int64_t pixels = (int64_t)width * height;
  int *winner = nullptr;
  if (cudaMallocAsync((void **)&winner, sizeof(int) * (size_t)pixels, st) != cudaSuccess)
    return NCLR_ERR_CUDA;
  cudaMemsetAsync(winner, 0xff, sizeof(int) * (size_t)pixels, st);  // -1: no particle
  if (n > 0)
    claim_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(x, n, dim, width, height, radius,
                                                              winner);
  shade_kernel<<<(unsigned)((pixels + 255) / 256), 256, 0, st>>>(winner, colors, color, width,
                                                                 height, radius, rgba);
  const cudaError_t e = cudaGetLastError();
  cudaFreeAsync(winner, st);
  return e == cudaSuccess ? NCLR_OK : NCLR_ERR_CUDA;
}

}  // extern "C"
