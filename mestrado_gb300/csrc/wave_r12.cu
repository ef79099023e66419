// wave_r12.cu -- batched-form kernels with 12 rows per lane (band of 384 rows).
#include "wave_impl.cuh"

namespace nwg {
NWG_DEFINE_WAVE(12)
}  // namespace nwg
