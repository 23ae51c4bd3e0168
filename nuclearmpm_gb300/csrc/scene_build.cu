// Scene builders on the device: the reference's cube<dim>() lattice (src/nclr_math.h:100-129)
// and the headless solver's generate_cubes (src/solver.cpp:133-149) written straight into
// device memory, so that large scenes are not assembled on the host; the check of a
// device-resident material[] array for nclr_create_device; and the per-particle moduli.
#include <cuda_runtime.h>
#include <stdint.h>

#include "mpm_launch.h"
#include "nclr_gpu.h"

namespace mpm {

namespace {

// Eigen 3.4's LinSpaced(n, low, high) for float, entry i: low + i*step, except that the last
// entry is exactly high, or, when |high| < |low|, high - (n-1-i)*step with the first entry
// exactly low (the same rule as the host builders).  Explicit round-to-nearest operations:
// the host computes the product and the sum separately, so no fused multiply-add here.
__device__ __forceinline__ float linspaced_at(int i, int n, float low, float high) {
  if (n == 1) return high;
  const float step = __fdiv_rn(__fsub_rn(high, low), (float)(n - 1));
  if (fabsf(high) < fabsf(low))
    return i == 0 ? low : __fsub_rn(high, __fmul_rn((float)(n - 1 - i), step));
  return i == n - 1 ? high : __fadd_rn(low, __fmul_rn((float)i, step));
}

// Cube c of `ncubes` lattices of res^dim points each: row c*res^dim + r holds point r of
// cube<dim>(res, lo[c], hi[c]) (x outermost).
__global__ void cubes_kernel(int dim, int res, int ncubes, const float *__restrict__ lo,
                             const float *__restrict__ hi, float *__restrict__ x) {
  const int64_t per = (dim == 3) ? (int64_t)res * res * res : (int64_t)res * res;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= per * ncubes) return;
  const int c = (int)(i / per);
  int64_t r = i - (int64_t)c * per;
  int idx[3];
  for (int d = dim - 1; d >= 0; --d) {
    idx[d] = (int)(r % res);
    r /= res;
  }
  for (int d = 0; d < dim; ++d) x[i * dim + d] = linspaced_at(idx[d], res, lo[c], hi[c]);
}

__global__ void bad_materials_kernel(const uint8_t *__restrict__ mat, int64_t n, int *bad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && mat[i] > 2) atomicAdd(bad, 1);
}

// Slot p takes the moduli of caller row id[p] (row p when id is null): mu_0 = E / (2 (1 + nu)),
// lambda_0 = E nu / ((1 + nu)(1 - 2 nu)) (src/nclr.h:77-78), each operation rounded on its
// own as the host evaluates the simulation's pair (no fused multiply-add).
__global__ void set_lame_kernel(const int *__restrict__ id, int n, const float *__restrict__ E,
                                const float *__restrict__ nu, float2 *__restrict__ lame) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int q = id ? id[p] : p;
  const float e = E[q], v = nu[q];
  const float one_v = __fadd_rn(1.0f, v);
  lame[p] = make_float2(__fdiv_rn(e, __fmul_rn(2.0f, one_v)),
                        __fdiv_rn(__fmul_rn(e, v),
                                  __fmul_rn(one_v, __fsub_rn(1.0f, __fmul_rn(2.0f, v)))));
}

}  // namespace

cudaError_t launch_set_lame(const int *id, int n, const float *E, const float *nu, float2 *lame,
                            cudaStream_t st) {
  if (n > 0) set_lame_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(id, n, E, nu, lame);
  return cudaGetLastError();
}

cudaError_t count_bad_materials(const uint8_t *mat, int64_t n, int *scratch, int *out,
                                cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  if (n > 0) bad_materials_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(mat, n, scratch);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(out, scratch, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
  return cudaStreamSynchronize(st);
}

}  // namespace mpm

extern "C" {

nclr_status nclr_cubes_device(int dim, int ncubes, int res, const float *lo, const float *hi,
                              float *x, void *stream) {
  if ((dim != 2 && dim != 3) || ncubes < 0 || res < 1 || (ncubes > 0 && (!lo || !hi || !x)))
    return NCLR_ERR_INVALID;
  const int64_t per = (dim == 3) ? (int64_t)res * res * res : (int64_t)res * res;
  const int64_t total = per * ncubes;
  if (total == 0) return NCLR_OK;
  if (total > (int64_t)0x7fffffff / 2) return NCLR_ERR_INVALID;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  float *bounds = nullptr;  // lo then hi, on the device
  if (cudaMallocAsync((void **)&bounds, sizeof(float) * 2 * (size_t)ncubes, st) != cudaSuccess)
    return NCLR_ERR_CUDA;
  cudaMemcpyAsync(bounds, lo, sizeof(float) * (size_t)ncubes, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(bounds + ncubes, hi, sizeof(float) * (size_t)ncubes, cudaMemcpyHostToDevice, st);
  mpm::cubes_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(dim, res, ncubes, bounds,
                                                                      bounds + ncubes, x);
  const cudaError_t e = cudaGetLastError();
  cudaFreeAsync(bounds, st);
  if (e != cudaSuccess) return NCLR_ERR_CUDA;
  return cudaStreamSynchronize(st) == cudaSuccess ? NCLR_OK : NCLR_ERR_CUDA;
}

nclr_status nclr_cube_device(int dim, int res, float lo, float hi, float *x, void *stream) {
  return nclr_cubes_device(dim, 1, res, &lo, &hi, x, stream);
}

}  // extern "C"
