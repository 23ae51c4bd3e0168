// nclr_grid_transfer_noalloc: the particle-to-grid transfer and grid update of one step for
// particles that already live in the caller's device memory, written into the caller's
// device grid arrays, without allocating anything.
//
// Who needs it: code that may not call cudaMalloc while it runs -- a host application whose
// own allocator has already reserved the device's memory, a real-time loop where allocation
// (and the device synchronisation cudaMalloc/cudaFree can imply) is forbidden, or a plugin
// living inside another runtime that owns every allocation.  Such callers hand over their
// particle arrays and grid arrays; the only other memory the transfer needs, the float4
// accumulation grid, lives in the file-scope device array below.
//
// The scratch array: kNoallocMaxNodes float4 nodes (16 MiB), allocated when the library's
// device code is loaded on a GPU and held by every GPU that loads it until the process exits.
// Every call on a device shares it and it keeps the last call's contents, so each call clears
// it first; calls whose work overlaps on the GPU (different streams or threads at once) race
// on it and must be serialised by the caller (nothing here serialises them).
//
// The transfer uses the reference's fixed-corotated stress and one material, E and nu for all
// particles; it takes no options.  The physics mode does not matter here: the diag(1,1,0)
// identity of src/nclr_math.h:13-19 and the 2D SVD sign fix enter only G2P, so the grid equals
// grid() after one advance() under either mode.
#include <cuda.h>  // CUcontext / CUresult types only: the two driver calls come through the runtime
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "mpm_device.cuh"
#include "mpm_launch.h"
#include "nclr_gpu.h"

static __device__ __align__(256) float4 g_noalloc_grid[NCLR_NOALLOC_MAX_NODES];
static __device__ int g_noalloc_status;

namespace {

constexpr int64_t kNoallocMaxNodes = NCLR_NOALLOC_MAX_NODES;
constexpr int kMaxDevices = 64;

// Host-side device addresses of the two symbols, looked up once per device and context.  In
// host code the names g_noalloc_grid / g_noalloc_status are host-side stand-ins, not device
// addresses.  A context that is destroyed (cudaDeviceReset, or a caller's own context torn
// down) takes the module and its addresses with it, so each entry remembers the unique id of
// the context it was looked up in, and a call in another context looks the addresses up again.
struct DeviceScratch {
  unsigned long long ctx_id;  // 0: no entry
  float4 *grid;
  int *status;
};
std::mutex g_setup_mutex;  // guards g_scratch and the driver entry points (not the GPU work)
DeviceScratch g_scratch[kMaxDevices] = {};

typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);
bool g_driver_looked_up = false;
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

// Unique id (over the process's life) of the calling thread's current context, 0 when there is
// none yet or the driver cannot say.  Called with g_setup_mutex held.
unsigned long long current_context_id() {
  if (!g_driver_looked_up) {
    g_driver_looked_up = true;
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      g_ctx_get_current = (CtxGetCurrentFn)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      g_ctx_get_id = (CtxGetIdFn)f;
  }
  if (!g_ctx_get_current || !g_ctx_get_id) return 0;
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
  if (g_ctx_get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// Where the current call reports its message (the caller's buffer, may be null).
thread_local char *g_msg = nullptr;
thread_local size_t g_msg_len = 0;

nclr_status noalloc_fail(nclr_status st, const std::string &msg) {
  if (g_msg && g_msg_len > 0) {
    const size_t k = msg.size() < g_msg_len - 1 ? msg.size() : g_msg_len - 1;
    std::memcpy(g_msg, msg.data(), k);
    g_msg[k] = '\0';
  }
  return st;
}

// One particle per thread: stress + APIC affine from the particle's own state (src/nclr.h:
// 313-337), then the 3^dim weighted contributions (src/nclr.h:132-165) reduced into the
// scratch grid.  Rows are particle-major like the C ABI's host layout.
template <int D>
__global__ void __launch_bounds__(128) p2g_rows_kernel(int n, const float *__restrict__ xs,
                                                       const float *__restrict__ vs,
                                                       const float *__restrict__ Fs,
                                                       const float *__restrict__ Cs,
                                                       const float *__restrict__ Jps,
                                                       const float *__restrict__ ms,
                                                       const float *__restrict__ vols,
                                                       mpm::Params P, float4 *__restrict__ grid,
                                                       int *status) {
  using namespace mpm;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  float x[D], v[D];
  Mat<D> F, C;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    x[d] = xs[(size_t)p * D + d];
    v[d] = vs[(size_t)p * D + d];
  }
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      F.a[i][j] = Fs[((size_t)p * D + i) * D + j];
      C.a[i][j] = Cs[((size_t)p * D + i) * D + j];
    }
  const float Jp = Jps[p], m = ms[p], vol = vols[p];
  const Mat<D> A = fused_affine<D>(F, stress_R<D>(F, P, P.model), C, Jp, m, vol, P.model,
                                   make_float2(P.mu0, P.lambda0), P);
  int base[D];
  float fx[D], w[3][D];
  stencil<D>(x, P.inv_dx, base, fx, w);
  const int64_t f0 = flat_index<D>(base, P.N);
  constexpr int S = (D == 3) ? 27 : 9;
#pragma unroll
  for (int o = 0; o < S; ++o) {
    const int oi = (D == 3) ? o / 9 : o / 3;
    const int oj = (D == 3) ? (o / 3) % 3 : o % 3;
    const int ok = (D == 3) ? o % 3 : 0;
    const int oo[3] = {oi, oj, ok};
    const int64_t f = (D == 3) ? f0 + ((int64_t)oi * P.N + oj) * P.N + ok : f0 + (int64_t)oi * P.N + oj;
    if (f < 0 || f >= P.nodes) {
      atomicOr(status, kErrOutOfRange);
      continue;
    }
    float dpos[D];
#pragma unroll
    for (int d = 0; d < D; ++d) dpos[d] = ((float)oo[d] - fx[d]) * P.dx;
    float weight = w[oi][0] * w[oj][1];
    if (D == 3) weight = weight * w[ok][D - 1];
    float c[4] = {0.0f, 0.0f, 0.0f, weight * m};
#pragma unroll
    for (int r = 0; r < D; ++r) {
      float ad = A.a[r][0] * dpos[0];
#pragma unroll
      for (int k = 1; k < D; ++k) ad = ad + A.a[r][k] * dpos[k];
      c[r] = weight * (v[r] * m + ad);
    }
    red_add_v4(grid + f, c[0], c[1], c[2], c[3]);
  }
}

// The device addresses of the scratch symbols on the current device, looked up on the first
// call in the current context of that device (and again after that context was replaced).
nclr_status scratch_for_current_device(int *device, float4 **grid, int **status) {
  cudaError_t e = cudaGetDevice(device);
  if (e != cudaSuccess) return noalloc_fail(NCLR_ERR_NO_DEVICE, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (*device < 0 || *device >= kMaxDevices) return noalloc_fail(NCLR_ERR_INVALID, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  DeviceScratch &ds = g_scratch[*device];
  const unsigned long long id = current_context_id();
  if (id == 0 || ds.ctx_id != id) {
    void *gp = nullptr, *sp = nullptr;
    e = cudaGetSymbolAddress(&gp, g_noalloc_grid);  // also brings up the runtime's context
    if (e != cudaSuccess)
      return noalloc_fail(NCLR_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch grid): ") + cudaGetErrorString(e));
    e = cudaGetSymbolAddress(&sp, g_noalloc_status);
    if (e != cudaSuccess)
      return noalloc_fail(NCLR_ERR_CUDA, std::string("cudaGetSymbolAddress(status): ") + cudaGetErrorString(e));
    // the context the lookup ran in (the runtime may have just created it); 0 keeps no entry,
    // so the next call looks the addresses up again
    ds.ctx_id = current_context_id();
    ds.grid = (float4 *)gp;
    ds.status = (int *)sp;
    *grid = ds.grid;
    *status = ds.status;
    return NCLR_OK;
  }
  *grid = ds.grid;
  *status = ds.status;
  return NCLR_OK;
}

}  // namespace

extern "C" nclr_status nclr_grid_transfer_noalloc(int dim, int64_t n, const float *x, const float *v,
                                                  const float *F, const float *C, const float *Jp,
                                                  const float *mass, const float *volume, int model,
                                                  int res, float dt, float E, float nu, float gravity,
                                                  float *grid_velocity, float *grid_mass,
                                                  void *stream, char *message,
                                                  size_t message_len) {
  g_msg = message;
  g_msg_len = message_len;
  if (message && message_len > 0) message[0] = '\0';
  if (dim != 2 && dim != 3) return noalloc_fail(NCLR_ERR_INVALID, "dim must be 2 or 3");
  if (n < 0 || n > 0x7fffffff) return noalloc_fail(NCLR_ERR_INVALID, "bad particle count");
  if (res < 1) return noalloc_fail(NCLR_ERR_INVALID, "res must be >= 1");
  if (model < 0 || model > 2) return noalloc_fail(NCLR_ERR_INVALID, "unknown material model");
  int64_t nodes = 1;
  for (int d = 0; d < dim && nodes <= kNoallocMaxNodes; ++d) nodes *= (int64_t)res + 1;
  if (nodes > kNoallocMaxNodes)
    return noalloc_fail(NCLR_ERR_INVALID,
                        "grid has " + std::to_string(nodes) + " nodes; the no-allocation entry "
                        "point holds at most " + std::to_string(kNoallocMaxNodes) +
                        " ((res+1)^dim <= NCLR_NOALLOC_MAX_NODES)");
  if (n > 0 && (!x || !v || !F || !C || !Jp || !mass || !volume))
    return noalloc_fail(NCLR_ERR_INVALID, "a particle array is NULL");
  if (!grid_velocity || !grid_mass) return noalloc_fail(NCLR_ERR_INVALID, "a grid array is NULL");

  int device = 0;
  float4 *grid = nullptr;
  int *status = nullptr;
  nclr_status st = scratch_for_current_device(&device, &grid, &status);
  if (st != NCLR_OK) return st;

  mpm::Params P{};
  P.res = res;
  P.N = res + 1;
  P.n = (int)n;
  P.model = model;
  P.dt = dt;
  P.dx = (float)(1.0 / res);  // src/nclr.h:76
  P.inv_dx = 1.0f / P.dx;
  P.gravity = gravity;
  P.allowed = (float)((double)P.dx * 0.9 / (double)dt);  // src/nclr.h:285
  P.mu0 = E / (2.0f * (1.0f + nu));                       // src/nclr.h:77-78
  P.lambda0 = E * nu / ((1.0f + nu) * (1.0f - 2.0f * nu));
  P.Dinv = 4.0f * P.inv_dx * P.inv_dx;
  P.cscale = 4.0f * P.inv_dx;
  P.dt_gravity = dt * gravity;
  P.nodes = nodes;

  cudaStream_t s = (cudaStream_t)stream;
  // The scratch keeps the previous call's sums: clear what this call accumulates into.
  cudaError_t e = cudaMemsetAsync(grid, 0, sizeof(float4) * (size_t)nodes, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(status, 0, sizeof(int), s);
  if (e != cudaSuccess) return noalloc_fail(NCLR_ERR_CUDA, std::string("clear scratch: ") + cudaGetErrorString(e));
  if (n > 0) {
    const unsigned blocks = (unsigned)((n + 127) / 128);
    if (dim == 2)
      p2g_rows_kernel<2><<<blocks, 128, 0, s>>>((int)n, x, v, F, C, Jp, mass, volume, P, grid, status);
    else
      p2g_rows_kernel<3><<<blocks, 128, 0, s>>>((int)n, x, v, F, C, Jp, mass, volume, P, grid, status);
  }
  // Grid update (src/nclr.h:263-310) into the caller's arrays, in the reference's node order.
  if (dim == 2)
    mpm::launch_export_grid<2>(grid, P, grid_velocity, grid_mass, s);
  else
    mpm::launch_export_grid<3>(grid, P, grid_velocity, grid_mass, s);
  e = cudaGetLastError();
  if (e != cudaSuccess) return noalloc_fail(NCLR_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  int flag = 0;
  e = cudaMemcpyAsync(&flag, status, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return noalloc_fail(NCLR_ERR_CUDA, std::string("synchronise: ") + cudaGetErrorString(e));
  if (flag & mpm::kErrOutOfRange)
    return noalloc_fail(NCLR_ERR_OUT_OF_RANGE,
                        "a particle's stencil left the grid (the reference's vector::at throws "
                        "std::out_of_range here)");
  return NCLR_OK;
}
