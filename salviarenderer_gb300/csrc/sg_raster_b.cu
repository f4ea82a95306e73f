// sg_raster_b.cu -- k_shade instances for 2 and 3 varyings.
#include "sg_raster.cuh"

namespace sg {

void launch_shade_2(PassParams const& p, uint32_t grid, uint32_t resident, cudaStream_t s) {
  launch_shade_t<2>(p, grid, resident, s);
}
void launch_shade_3(PassParams const& p, uint32_t grid, uint32_t resident, cudaStream_t s) {
  launch_shade_t<3>(p, grid, resident, s);
}

// The EWA table of this translation unit's sampler (each translation unit
// has its own copy of the __constant__ table).
cudaError_t upload_ewa_table_raster_b(float const* tab, cudaStream_t s) {
  return cudaMemcpyToSymbolAsync(c_ewa, tab, 256 * sizeof(float), 0, cudaMemcpyHostToDevice, s);
}

}  // namespace sg
