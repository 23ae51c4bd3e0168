// The 3D fused step with the material fixed at compile time (launch_g2p2g_fixed): a single
// simulation without per-particle materials runs a kernel without the other materials'
// branches.  Kept apart from step3d.cu so that the two compile in parallel.
#include "mpm_step.cuh"
namespace mpm {

template <int D>
void launch_g2p2g_fixed(const PState &s, const Params &P0, const float4 *V, float4 *G,
                        uint8_t *flags, const int *blocks, const int *nactive,
                        const int *bstart, const int *sparse, int *work, int *err, int next_slot,
                        bool ref, int mode, int material, int ctas, cudaStream_t st,
                        const Record &rec, const SnowFix &fix) {
  auto go = [&](auto r, auto m, auto mat) {
    launch_overlapped(
        g2p2g_kernel<D, decltype(r)::value, decltype(m)::value, false, decltype(mat)::value>,
        (unsigned)ctas, kG2P2GThreads, g2p2g_smem_bytes<D, false>(), st, s, P0,
        (const Scene *)nullptr, (const uint16_t *)nullptr, V, G, flags, blocks, nactive, bstart,
        sparse, work, err, next_slot, rec, fix);
  };
  auto by_material = [&](auto r, auto m) {
    if (material == kSnow) go(r, m, std::integral_constant<int, kSnow>{});
    else if (material == kJelly) go(r, m, std::integral_constant<int, kJelly>{});
    else go(r, m, std::integral_constant<int, kLiquid>{});
  };
  auto by_mode = [&](auto r) {
    if (mode == kFinalStep) by_material(r, std::integral_constant<int, kFinalStep>{});
    else by_material(r, std::integral_constant<int, kStep>{});
  };
  if (ref) by_mode(std::true_type{});
  else by_mode(std::false_type{});
}

template <int D>
void g2p2g_fixed_set_smem(int bytes) {
  const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
  auto set = [&](auto r, auto m) {
    constexpr bool R = decltype(r)::value;
    constexpr int M = decltype(m)::value;
    cudaFuncSetAttribute(g2p2g_kernel<D, R, M, false, kSnow>, a, bytes);
    cudaFuncSetAttribute(g2p2g_kernel<D, R, M, false, kJelly>, a, bytes);
    cudaFuncSetAttribute(g2p2g_kernel<D, R, M, false, kLiquid>, a, bytes);
  };
  set(std::true_type{}, std::integral_constant<int, kStep>{});
  set(std::true_type{}, std::integral_constant<int, kFinalStep>{});
  set(std::false_type{}, std::integral_constant<int, kStep>{});
  set(std::false_type{}, std::integral_constant<int, kFinalStep>{});
}

template void g2p2g_fixed_set_smem<3>(int);
template void launch_g2p2g_fixed<3>(const PState &, const Params &, const float4 *, float4 *,
                                    uint8_t *, const int *, const int *, const int *,
                                    const int *, int *, int *, int, bool, int, int, int,
                                    cudaStream_t, const Record &, const SnowFix &);
}  // namespace mpm
