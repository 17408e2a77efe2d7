// split_kernels.cu -- placeholder until the tcgen05 split-precision kernel lands.
#include "common.cuh"
namespace rimp2 {
bool split_supported() { return false; }
int split_energy(const SplitEnergyArgs &, cudaStream_t, float *) {
  set_error("split-precision path not built yet");
  return RIMP2_ERR_UNSUPPORTED;
}
}  // namespace rimp2
