// wave_r24.cu -- batched-form kernels with 24 rows per lane (band of 768 rows).
#include "wave_impl.cuh"

namespace nwg {
NWG_DEFINE_WAVE(24)
}  // namespace nwg
