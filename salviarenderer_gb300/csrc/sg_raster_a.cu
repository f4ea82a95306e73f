// sg_raster_a.cu -- k_shade instances for 0 and 1 varyings; the coverage and merge kernels.
#define SG_RASTER_COVER_MERGE
#include "sg_raster.cuh"

namespace sg {

void launch_shade_0(PassParams const& p, uint32_t grid, uint32_t resident, cudaStream_t s) {
  launch_shade_t<0>(p, grid, resident, s);
}
void launch_shade_1(PassParams const& p, uint32_t grid, uint32_t resident, cudaStream_t s) {
  launch_shade_t<1>(p, grid, resident, s);
}

// The EWA table of this translation unit's sampler (each translation unit
// has its own copy of the __constant__ table).
cudaError_t upload_ewa_table_raster_a(float const* tab, cudaStream_t s) {
  return cudaMemcpyToSymbolAsync(c_ewa, tab, 256 * sizeof(float), 0, cudaMemcpyHostToDevice, s);
}

// `max_samples` / `early_z`: the largest sample count of the pass's targets,
// and whether any of them stages depth for early-Z (sizes the shared memory).
void launch_cover(PassParams const& p, uint32_t max_samples, bool early_z, uint32_t grid, cudaStream_t s) {
  size_t smem = cover_smem(max_samples, early_z);
  k_cover<<<grid, COVER_THREADS, smem, s>>>(p);
}

// Raises k_cover's dynamic shared-memory limit to the largest layout (called
// at device creation, outside any stream capture).
cudaError_t init_cover() {
  return cudaFuncSetAttribute(k_cover, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              static_cast<int>(cover_smem(4, true)));
}

void launch_merge(PassParams const& p, uint32_t grid, uint32_t resident, cudaStream_t s) {
  if (resident >= 4)
    launch_pdl(k_merge<4>, grid, RASTER_THREADS, 0, s, p);
  else
    launch_pdl(k_merge<3>, grid, RASTER_THREADS, 0, s, p);
}

}  // namespace sg
