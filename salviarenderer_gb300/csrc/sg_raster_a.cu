// sg_raster_a.cu -- k_shade instances for 0 and 1 varyings; the coverage and merge kernels.
#define SG_RASTER_COVER_MERGE
#include "sg_raster.cuh"

namespace sg {

void launch_shade_0(DrawParams const& p, uint32_t grid, cudaStream_t s) { launch_shade_t<0>(p, grid, s); }
void launch_shade_1(DrawParams const& p, uint32_t grid, cudaStream_t s) { launch_shade_t<1>(p, grid, s); }

// The EWA table of this translation unit's sampler (each translation unit
// has its own copy of the __constant__ table).
cudaError_t upload_ewa_table_raster_a(float const* tab, cudaStream_t s) {
  return cudaMemcpyToSymbolAsync(c_ewa, tab, 256 * sizeof(float), 0, cudaMemcpyHostToDevice, s);
}

void launch_cover(DrawParams const& p, int nreg, uint32_t grid, cudaStream_t s) {
  size_t smem = cover_smem(p.samples, p.early_z && p.ds);
  cudaFuncSetAttribute(k_cover, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  k_cover<<<grid, COVER_THREADS, smem, s>>>(p, nreg);
}

void launch_merge(DrawParams const& p, int nreg, uint32_t grid, cudaStream_t s) {
  k_merge<<<grid, RASTER_THREADS, 0, s>>>(p, nreg);
}

}  // namespace sg
