// wave_r8.cu -- batched-form kernels with 8 rows per lane (band of 256 rows).
#include "wave_impl.cuh"

namespace nwg {
NWG_DEFINE_WAVE(8)
}  // namespace nwg
