// sg_raster_c.cu -- k_shade instances for 4 and 5 varyings.
#include "sg_raster.cuh"

namespace sg {

void launch_shade_4(PassParams const& p, uint32_t grid, uint32_t resident, cudaStream_t s) {
  launch_shade_t<4>(p, grid, resident, s);
}
void launch_shade_5(PassParams const& p, uint32_t grid, uint32_t resident, cudaStream_t s) {
  launch_shade_t<5>(p, grid, resident, s);
}

// The EWA table of this translation unit's sampler (each translation unit
// has its own copy of the __constant__ table).
cudaError_t upload_ewa_table_raster_c(float const* tab, cudaStream_t s) {
  return cudaMemcpyToSymbolAsync(c_ewa, tab, 256 * sizeof(float), 0, cudaMemcpyHostToDevice, s);
}

}  // namespace sg
