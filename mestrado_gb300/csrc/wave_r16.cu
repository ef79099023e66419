// wave_r16.cu -- batched-form kernels with 16 rows per lane (band of 512 rows).
#include "wave_impl.cuh"

namespace nwg {
NWG_DEFINE_WAVE(16)
}  // namespace nwg
