// wave_r20.cu -- batched-form kernels with 20 rows per lane (band of 640 rows).
#include "wave_impl.cuh"

namespace nwg {
NWG_DEFINE_WAVE(20)
}  // namespace nwg
