// wave_r4.cu -- batched-form kernels with 4 rows per lane (band of 128 rows).
#include "wave_impl.cuh"

namespace nwg {
NWG_DEFINE_WAVE(4)
}  // namespace nwg
